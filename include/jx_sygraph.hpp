/*
 * Header-only C++ mirror of the reference's operator surface over the jx C ABI.
 *
 * Reference (vtsynergy/SYCL-Jaccard):
 *   - GraphCSRView<VT,ET,WT>            standalone_csr.hpp:44-105
 *   - sygraph::jaccard<edge_centric>    standalone_algorithms.hpp:67-69 (weighted),
 *                                       standalone_algorithms.hpp:86-87 (unweighted)
 *   - sygraph::detail::Jaccard_*::invoke jaccard.hpp:51-52,104-107,151-156,235-237,256-258,280-283
 *
 * Differences, by design: the graph holds device pointers instead of cl::sycl::buffer, and
 * the queue is a CUDA stream.  Like the reference, the calls return void and report a
 * failure on std::cerr (jaccard.cpp:178-180 and the other catch sites) instead of stopping
 * the program; `sygraph::last_status()` returns the status of the most recent call on this
 * thread.  Only <int32_t, int32_t, float> is supported, the configuration the reference
 * ships (Makefile:33: -DDISABLE_DP_WEIGHT -DDISABLE_DP_INDEX).
 */
#ifndef JX_SYGRAPH_HPP
#define JX_SYGRAPH_HPP

#include <cstdint>
#include <iostream>
#include <type_traits>

#include "jx.h"

namespace sygraph {

/* Non-owning CSR view over device memory (standalone_csr.hpp:44-105). */
template <typename vertex_t, typename edge_t, typename weight_t> class GraphCSRView {
public:
  using vertex_type = vertex_t;
  using edge_type = edge_t;
  using weight_type = weight_t;

  weight_t *edge_data = nullptr; ///< edge weight (unused by Jaccard)
  vertex_t number_of_vertices = 0;
  edge_t number_of_edges = 0;
  edge_t *offsets = nullptr;    ///< CSR offsets, device, V+1
  vertex_t *indices = nullptr;  ///< CSR indices, device, E, rows sorted ascending

  GraphCSRView() = default;
  GraphCSRView(edge_t *offsets_, vertex_t *indices_, weight_t *edge_data_, vertex_t n, edge_t e)
      : edge_data(edge_data_), number_of_vertices(n), number_of_edges(e), offsets(offsets_),
        indices(indices_) {}
};

namespace detail {
inline jx_status &status_slot() {
  static thread_local jx_status s = JX_OK;
  return s;
}
inline void report(jx_status s, const char *where) {
  status_slot() = s;
  if (s != JX_OK) std::cerr << "jx error during " << where << "\n\t" << jx_status_string(s) << std::endl;
}
template <typename VT, typename ET, typename WT> constexpr void check_types() {
  static_assert(std::is_same<VT, int32_t>::value && std::is_same<ET, int32_t>::value &&
                    std::is_same<WT, float>::value,
                "jx supports GraphCSRView<int32_t, int32_t, float> only");
}
template <typename VT, typename ET, typename WT>
inline jx_csr to_c(const GraphCSRView<VT, ET, WT> &g) {
  return jx_csr{g.number_of_vertices, g.number_of_edges, g.offsets, g.indices};
}
} // namespace detail

/* Status of the last call made through this header on this thread. */
inline jx_status last_status() { return detail::status_slot(); }

/* sygraph::jaccard<edge_centric>(graph, weights, result, q): weights = per-vertex, device. */
template <bool edge_centric, typename VT, typename ET, typename WT>
void jaccard(GraphCSRView<VT, ET, WT> &graph, const WT *weights, WT *result,
             jx_stream_t stream = nullptr) {
  detail::check_types<VT, ET, WT>();
  const jx_csr g = detail::to_c(graph);
  detail::report(jx_jaccard(&g, weights, result,
                            edge_centric ? JX_ALGO_EDGE_CENTRIC : JX_ALGO_VERTEX_CENTRIC, stream),
                 edge_centric ? "EC Jaccard" : "VC Jaccard");
}

/* sygraph::jaccard<edge_centric>(graph, result, q): unweighted. */
template <bool edge_centric, typename VT, typename ET, typename WT>
void jaccard(GraphCSRView<VT, ET, WT> &graph, WT *result, jx_stream_t stream = nullptr) {
  jaccard<edge_centric, VT, ET, WT>(graph, static_cast<const WT *>(nullptr), result, stream);
}

namespace detail {

/* Kernel-level calls (the static invoke functions of jaccard.hpp). */
template <bool weighted, typename vertex_t, typename edge_t, typename weight_t>
struct Jaccard_RowSumKernel {
  static void invoke(vertex_t n, edge_t e, const edge_t *csrPtr, const vertex_t *csrInd,
                     const weight_t *weight_in, weight_t *work, jx_stream_t s = nullptr) {
    check_types<vertex_t, edge_t, weight_t>();
    report(jx_rowsum(n, e, csrPtr, csrInd, weighted ? weight_in : nullptr, work, s), "VC RowSum");
  }
};

template <bool weighted, typename vertex_t, typename edge_t, typename weight_t>
struct Jaccard_IsKernel {
  static void invoke(vertex_t n, edge_t e, const edge_t *csrPtr, const vertex_t *csrInd,
                     const weight_t *weight_in, const weight_t *work, weight_t *weight_i,
                     weight_t *weight_s, jx_stream_t s = nullptr) {
    check_types<vertex_t, edge_t, weight_t>();
    report(jx_intersect(n, e, csrPtr, csrInd, weighted ? weight_in : nullptr, work, weight_i,
                        weight_s, s),
           "VC Intersection");
  }
};

template <typename vertex_t, typename edge_t, typename weight_t> struct Jaccard_JwKernel {
  static void invoke(edge_t e, const weight_t *weight_i, const weight_t *weight_s,
                     weight_t *weight_j, jx_stream_t s = nullptr) {
    check_types<vertex_t, edge_t, weight_t>();
    report(jx_weight(e, weight_i, weight_s, weight_j, s), "VC Weights");
  }
};

template <typename vertex_t, typename edge_t, typename weight_t> struct Jaccard_ec_scan {
  static void invoke(edge_t e, vertex_t n, const edge_t *csrPtr, vertex_t *dest_ind,
                     weight_t *weight_j, jx_stream_t s = nullptr) {
    check_types<vertex_t, edge_t, weight_t>();
    report(jx_ec_scan(e, n, csrPtr, dest_ind, weight_j, s), "EC-Scan");
  }
};

template <typename vertex_t, typename edge_t, typename weight_t> struct Jaccard_ec_unweighted {
  static void invoke(edge_t e, vertex_t n, const edge_t *csrPtr, const vertex_t *csrInd,
                     const vertex_t *dest_ind, weight_t *weight_j, jx_stream_t s = nullptr) {
    check_types<vertex_t, edge_t, weight_t>();
    report(jx_ec_unweighted(e, n, csrPtr, csrInd, dest_ind, weight_j, s), "EC-unweighted");
  }
};

} // namespace detail
} // namespace sygraph

/* FillKernel<T>::invoke (jaccard.hpp:40-53) lives at global scope in the reference. */
template <typename T> struct FillKernel {
  static void invoke(size_t n, T *x, T value, jx_stream_t s = nullptr) {
    static_assert(std::is_same<T, float>::value, "jx FillKernel supports float only");
    sygraph::detail::report(jx_fill((int64_t)n, x, value, s), "Fill");
  }
};

#endif /* JX_SYGRAPH_HPP */
