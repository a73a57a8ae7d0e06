/*
 * C entry points around the reference's own Jaccard code -- TEST INFRASTRUCTURE ONLY.
 *
 * This translation unit includes the reference's `jaccard.cpp` (vtsynergy/SYCL-Jaccard)
 * unmodified, compiled against the host SYCL subset in oracle/syclshim with the reference's
 * shipped flags (Makefile:33: -DDISABLE_DP_WEIGHT -DDISABLE_LIST -DDISABLE_DP_INDEX, plus
 * -DSTANDALONE -DSYCL_1_2_1 as its Makefile:387 and ICX flags give).  The source directory
 * is put on the include path by oracle/build_ref.py; no reference source lives in this
 * repository.
 *
 * Entry points mirror the reference's public and kernel-level calls:
 *   jxref_jaccard        sygraph::jaccard<edge_centric>(graph, [weights,] result, q)
 *                        (standalone_algorithms.hpp:67-87, jaccard.cpp:926-955)
 *   jxref_rowsum         detail::Jaccard_RowSumKernel<w>::invoke   (jaccard.cpp:263-313)
 *   jxref_fill           FillKernel<float>::invoke                  (jaccard.cpp:161-182)
 *   jxref_intersect      detail::Jaccard_IsKernel<w>::invoke       (jaccard.cpp:402-458)
 *   jxref_weight         detail::Jaccard_JwKernel::invoke           (jaccard.cpp:622-653)
 *   jxref_ec_scan        detail::Jaccard_ec_scan::invoke            (jaccard.cpp:666-700)
 *   jxref_ec_unweighted  detail::Jaccard_ec_unweighted::invoke      (jaccard.cpp:745-782)
 *   jxref_csr_write      CSRToFile<int32_t,int32_t,float>        (readMtxToCSR.cpp:285-337)
 *   jxref_csr_read       FileToCSR                                 (readMtxToCSR.cpp:388-395)
 *   jxref_remove_reverse CSRToMtx + removeReverseEdges             (readMtxToCSR.cpp:134-147, 211-248)
 *   jxref_csr_from_edges MTX set + invertDirection + mtxSetToCSR    (main.cpp:99-118,
 *                        readMtxToCSR.cpp:117-132, 153-208)
 * The edge-centric driver prints a line to std::cout (jaccard.cpp:819); it is discarded.
 */
#include "jaccard.cpp"

#include "readMtxToCSR.hpp"

#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <streambuf>

namespace {
struct NullBuf : std::streambuf {
  int overflow(int c) override { return c; }
};

struct MuteCout {
  NullBuf nb;
  std::streambuf *old;
  MuteCout() : old(std::cout.rdbuf(&nb)) {}
  ~MuteCout() { std::cout.rdbuf(old); }
};

template <typename T> cl::sycl::buffer<T> wrap(const T *p, int64_t n) {
  return cl::sycl::buffer<T>(const_cast<T *>(p), cl::sycl::range<1>((size_t)n));
}
} // namespace

extern "C" {

void jxref_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Execute only work-groups g with g % k == residue in each launch (timing samples);
 * k = 1 runs everything. */
void jxref_set_group_sample(long long k, long long residue) { jxshim::set_group_sample(k, residue); }

/* Execute only work-groups g < len with mask[g] != 0 in each launch (timing samples); a NULL
 * mask restores the stride sample.  The mask must stay valid while calls run. */
void jxref_set_group_mask(const unsigned char *mask, long long len) { jxshim::set_group_mask(mask, len); }

int jxref_jaccard(int edge_centric, int32_t n, int32_t e, const int32_t *row_ptr,
                  const int32_t *col, const float *vertex_w, float *out) {
  MuteCout mute;
  cl::sycl::queue q;
  GraphCSRView<int32_t, int32_t, float> g(wrap(row_ptr, (int64_t)n + 1), wrap(col, e),
                                          cl::sycl::buffer<float>(nullptr), n, e);
  cl::sycl::buffer<float> result(out, cl::sycl::range<1>((size_t)e));
  if (vertex_w) {
    cl::sycl::buffer<float> wb = wrap(vertex_w, n);
    if (edge_centric)
      sygraph::jaccard<true, int32_t, int32_t, float>(g, wb, result, q);
    else
      sygraph::jaccard<false, int32_t, int32_t, float>(g, wb, result, q);
  } else {
    if (edge_centric)
      sygraph::jaccard<true, int32_t, int32_t, float>(g, result, q);
    else
      sygraph::jaccard<false, int32_t, int32_t, float>(g, result, q);
  }
  return 0;
}

int jxref_rowsum(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *ind,
                 const float *w, float *work) {
  cl::sycl::queue q;
  auto rp = wrap(row_ptr, (int64_t)n + 1);
  auto ci = wrap(ind, e);
  cl::sycl::buffer<float> wk(work, cl::sycl::range<1>((size_t)n));
  if (w) {
    auto wb = wrap(w, e); /* the vertex-weight array must cover every index in `ind` */
    sygraph::detail::Jaccard_RowSumKernel<true, int32_t, int32_t, float>::invoke(n, e, rp, ci, &wb,
                                                                                wk, q);
  } else {
    sygraph::detail::Jaccard_RowSumKernel<false, int32_t, int32_t, float>::invoke(n, e, rp, ci,
                                                                                 nullptr, wk, q);
  }
  return 0;
}

int jxref_fill(int64_t n, float *x, float value) {
  cl::sycl::queue q;
  cl::sycl::buffer<float> xb(x, cl::sycl::range<1>((size_t)n));
  FillKernel<float>::invoke((size_t)n, xb, value, q);
  return 0;
}

int jxref_intersect(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *col,
                    const float *w, const float *work, float *weight_i, float *weight_s) {
  cl::sycl::queue q;
  auto rp = wrap(row_ptr, (int64_t)n + 1);
  auto ci = wrap(col, e);
  auto wk = wrap(work, n);
  cl::sycl::buffer<float> wi(weight_i, cl::sycl::range<1>((size_t)e));
  cl::sycl::buffer<float> ws(weight_s, cl::sycl::range<1>((size_t)e));
  if (w) {
    auto wb = wrap(w, n);
    sygraph::detail::Jaccard_IsKernel<true, int32_t, int32_t, float>::invoke(n, e, rp, ci, &wb, wk,
                                                                            wi, ws, q);
  } else {
    sygraph::detail::Jaccard_IsKernel<false, int32_t, int32_t, float>::invoke(n, e, rp, ci, nullptr,
                                                                             wk, wi, ws, q);
  }
  return 0;
}

int jxref_weight(int32_t e, const float *weight_i, const float *weight_s, float *weight_j) {
  cl::sycl::queue q;
  auto wi = wrap(weight_i, e);
  auto ws = wrap(weight_s, e);
  cl::sycl::buffer<float> wj(weight_j, cl::sycl::range<1>((size_t)e));
  sygraph::detail::Jaccard_JwKernel<int32_t, int32_t, float>::invoke(e, wi, ws, wj, q);
  return 0;
}

int jxref_ec_scan(int32_t e, int32_t n, const int32_t *row_ptr, int32_t *dest_ind,
                  float *weight_j) {
  cl::sycl::queue q;
  auto rp = wrap(row_ptr, (int64_t)n + 1);
  cl::sycl::buffer<int32_t> di(dest_ind, cl::sycl::range<1>((size_t)e));
  cl::sycl::buffer<float> wj(weight_j, cl::sycl::range<1>((size_t)e));
  sygraph::detail::Jaccard_ec_scan<int32_t, int32_t, float>::invoke(e, n, rp, di, wj, q);
  return 0;
}

int jxref_ec_unweighted(int32_t e, int32_t n, const int32_t *row_ptr, const int32_t *col,
                        const int32_t *dest_ind, float *weight_j) {
  cl::sycl::queue q;
  auto rp = wrap(row_ptr, (int64_t)n + 1);
  auto ci = wrap(col, e);
  auto di = wrap(dest_ind, e);
  cl::sycl::buffer<float> wj(weight_j, cl::sycl::range<1>((size_t)e));
  sygraph::detail::Jaccard_ec_unweighted<int32_t, int32_t, float>::invoke(e, n, rp, ci, di, wj, q);
  return 0;
}

/* CSRToFile with weights (the reference writes its weight copy through an unallocated pointer
 * when isWeighted is false, readMtxToCSR.cpp:295-314, so only the weighted form is usable). */
int jxref_csr_write(const char *path, int32_t n, int32_t e, const int32_t *offsets,
                    const int32_t *indices, const float *weights, int zero_indexed, int directed,
                    int reverse_edges) {
  GraphCSRView<int32_t, int32_t, float> g(wrap(offsets, (int64_t)n + 1), wrap(indices, e), wrap(weights, e),
                                          n, e);
  std::ofstream f(path, std::ios_base::out | std::ios_base::trunc | std::ios_base::binary);
  if (!f) return 1;
  CSRToFile<int32_t, int32_t, float>(f, g, zero_indexed != 0, true, directed != 0, reverse_edges != 0);
  return f.good() ? 0 : 2;
}

/* FileToCSR: header fields and arrays (caller sizes them from jxref_csr_header). */
int jxref_csr_header(const char *path, int64_t *nv, int64_t *ne, uint64_t *flags) {
  std::ifstream f(path, std::ios_base::in | std::ios_base::binary);
  if (!f) return 1;
  CSRFileHeader h;
  f.read(reinterpret_cast<char *>(&h), sizeof h);
  *nv = h.numVerts;
  *ne = h.numEdges;
  uint64_t bits;
  std::memcpy(&bits, &h.flags, sizeof bits);
  *flags = bits;
  return 0;
}

int jxref_csr_read(const char *path, int32_t *offsets, int32_t *indices, float *weights) {
  std::ifstream f(path, std::ios_base::in | std::ios_base::binary);
  if (!f) return 1;
  CSRFileHeader h;
  void *gv = FileToCSR(f, &h);
  if (h.flags.isVertexT64 || h.flags.isEdgeT64 || h.flags.isWeightT64) return 2;
  auto *g = static_cast<GraphCSRView<int32_t, int32_t, float> *>(gv);
  auto o = g->offsets.get_access<cl::sycl::access::mode::read>();
  auto ix = g->indices.get_access<cl::sycl::access::mode::read>();
  std::memcpy(offsets, &o[0], sizeof(int32_t) * (h.numVerts + 1));
  std::memcpy(indices, &ix[0], sizeof(int32_t) * h.numEdges);
  if (h.flags.isWeighted && weights) {
    auto wa = g->edge_data.get_access<cl::sycl::access::mode::read>();
    std::memcpy(weights, &wa[0], sizeof(float) * h.numEdges);
  }
  delete g;
  return 0;
}

/* The reference program's result post-processing (main.cpp:307-309): CSR + per-edge values to an MTX set,
 * then removeReverseEdges.  Writes the surviving (src, dst, value) triples (zero-based) in the
 * set's order; returns their number, or -1 when `cap` is too small. */
int64_t jxref_remove_reverse(int32_t n, int32_t e, const int32_t *offsets, const int32_t *indices,
                             const float *values, int32_t *src, int32_t *dst, float *val, int64_t cap) {
  GraphCSRView<int32_t, int32_t, float> g(wrap(offsets, (int64_t)n + 1), wrap(indices, e), wrap(values, e),
                                          n, e);
  std::set<std::tuple<int32_t, int32_t, float>> *m = CSRToMtx(g, true, true);
  {
    NullBuf nb;
    std::streambuf *old = std::cerr.rdbuf(&nb);
    removeReverseEdges(*m);
    std::cerr.rdbuf(old);
  }
  if ((int64_t)m->size() > cap) {
    delete m;
    return -1;
  }
  int64_t k = 0;
  for (const auto &t : *m) {
    src[k] = std::get<0>(t) - 1;
    dst[k] = std::get<1>(t) - 1;
    val[k] = std::get<2>(t);
    ++k;
  }
  delete m;
  return k;
}

/* The reference program's graph preparation (main.cpp:99-118) on a zero-based edge list: the edges as
 * an MTX set (one-based ids, weight 1), the set's invertDirection inserted when symmetrising,
 * then mtxSetToCSR (self loops dropped unless keep_self).  Writes the CSR's offsets and
 * indices; *nv receives its number of rows (the reference's rows run from the first source to
 * the last).  Returns the number of edges, or -1 when a capacity is too small, -2 when the
 * list is empty. */
int64_t jxref_csr_from_edges(int64_t m, const int32_t *src, const int32_t *dst, int symmetrize, int keep_self,
                             int32_t *offsets, int64_t offsets_cap, int32_t *indices, int64_t cap,
                             int32_t *nv) {
  if (m <= 0) return -2;
  std::set<std::tuple<int32_t, int32_t, float>> mtx;
  for (int64_t i = 0; i < m; ++i) mtx.insert(std::tuple<int32_t, int32_t, float>(src[i] + 1, dst[i] + 1, 1.0f));
  if (symmetrize) {
    std::set<std::tuple<int32_t, int32_t, float>> *rev = invertDirection(mtx);
    mtx.insert(rev->begin(), rev->end());
    delete rev;
  }
  GraphCSRView<int32_t, int32_t, float> *g = mtxSetToCSR(mtx, !keep_self, false);
  const int64_t n = g->number_of_vertices, e = g->number_of_edges;
  if (n + 1 > offsets_cap || e > cap) {
    delete g;
    return -1;
  }
  {
    auto o = g->offsets.get_access<cl::sycl::access::mode::read>();
    std::memcpy(offsets, &o[0], sizeof(int32_t) * (size_t)(n + 1));
    if (e > 0) {
      auto ix = g->indices.get_access<cl::sycl::access::mode::read>();
      std::memcpy(indices, &ix[0], sizeof(int32_t) * (size_t)e);
    }
  }
  *nv = (int32_t)n;
  delete g;
  return e;
}

} /* extern "C" */
