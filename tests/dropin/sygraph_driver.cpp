// C++ caller of the drop-in header include/jx_sygraph.hpp, linked against libjx.so.
//
// It makes the calls the reference's driver program makes on the hot path, in the same order
// and with the same arguments (main.cpp:205-282):
//   - sygraph::jaccard<true>(graph, results)                    edge-centric, main.cpp:207
//   - pseudo indices 0..e-1, then Jaccard_RowSumKernel<true>::invoke over the edge data to
//     build per-vertex weights                                   main.cpp:213-257
//   - sygraph::jaccard<false>(graph, vertWeights, results)      weighted VC, main.cpp:274-275
//   - sygraph::jaccard<false>(graph, results)                   unweighted VC, main.cpp:278
// and then drives the stage kernels the way detail::jaccard does (jaccard.cpp:784-897):
// RowSum -> Fill -> IsKernel -> JwKernel, and ec_scan -> ec_unweighted.  One call with a
// missing result buffer checks the error path (sygraph::last_status()).
//
// Input file:  int32 n, int32 e, int32 offsets[n + 1], int32 indices[e], float edge_data[e]
// Output file: float J_ec[e], vertWeights[n], J_vcw[e], J_vc[e], J_stages_vcw[e], J_stages_ec[e],
//              then int32 statuses: the error call's status, the status of the call after it.
#include "jx_sygraph.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <vector>

#define CHECK(x)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess) {                                                                       \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                                \
      return 3;                                                                                    \
    }                                                                                              \
  } while (0)

template <typename T> static T *to_device(const std::vector<T> &h) {
  T *d = nullptr;
  if (cudaMalloc(&d, sizeof(T) * (h.size() ? h.size() : 1)) != cudaSuccess) return nullptr;
  if (!h.empty()) cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
  return d;
}

template <typename T> static bool put(std::FILE *f, const T *d, size_t count) {
  std::vector<T> h(count);
  if (count && cudaMemcpy(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
  return std::fwrite(h.data(), sizeof(T), count, f) == count;
}

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s input output\n", argv[0]);
    return 2;
  }
  std::FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  int32_t n = 0, e = 0;
  if (std::fread(&n, 4, 1, in) != 1 || std::fread(&e, 4, 1, in) != 1) return 2;
  std::vector<int32_t> offsets(n + 1), indices(e);
  std::vector<float> edge_data(e);
  if (std::fread(offsets.data(), 4, n + 1, in) != (size_t)n + 1 || std::fread(indices.data(), 4, e, in) != (size_t)e ||
      std::fread(edge_data.data(), 4, e, in) != (size_t)e)
    return 2;
  std::fclose(in);

  int32_t *d_off = to_device(offsets), *d_ind = to_device(indices);
  float *d_edge = to_device(edge_data);
  float *d_res = nullptr, *d_vw = nullptr, *d_wi = nullptr, *d_ws = nullptr, *d_work = nullptr;
  int32_t *d_presum = nullptr, *d_dest = nullptr;
  CHECK(cudaMalloc(&d_res, sizeof(float) * e));
  CHECK(cudaMalloc(&d_vw, sizeof(float) * n));
  CHECK(cudaMalloc(&d_wi, sizeof(float) * e));
  CHECK(cudaMalloc(&d_ws, sizeof(float) * e));
  CHECK(cudaMalloc(&d_work, sizeof(float) * n));
  CHECK(cudaMalloc(&d_dest, sizeof(int32_t) * e));
  if (!d_off || !d_ind || !d_edge) return 3;
  sygraph::GraphCSRView<int32_t, int32_t, float> graph(d_off, d_ind, d_edge, n, e);

  std::FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  bool ok = true;

  // main.cpp:207
  sygraph::jaccard<true, int32_t, int32_t, float>(graph, d_res);
  CHECK(cudaDeviceSynchronize());
  ok &= sygraph::last_status() == JX_OK && put(out, d_res, e);

  // main.cpp:213-257: pseudo indices 0..e-1 and the row sums of the edge data as vertex weights
  std::vector<int32_t> iota(e);
  std::iota(iota.begin(), iota.end(), 0);
  d_presum = to_device(iota);
  if (!d_presum) return 3;
  sygraph::detail::Jaccard_RowSumKernel<true, int32_t, int32_t, float>::invoke(
      graph.number_of_vertices, graph.number_of_edges, graph.offsets, d_presum, graph.edge_data, d_vw);
  CHECK(cudaDeviceSynchronize());
  ok &= sygraph::last_status() == JX_OK && put(out, d_vw, n);

  // main.cpp:274-275
  sygraph::jaccard<false, int32_t, int32_t, float>(graph, d_vw, d_res);
  CHECK(cudaDeviceSynchronize());
  ok &= sygraph::last_status() == JX_OK && put(out, d_res, e);

  // main.cpp:278
  sygraph::jaccard<false, int32_t, int32_t, float>(graph, d_res);
  CHECK(cudaDeviceSynchronize());
  ok &= sygraph::last_status() == JX_OK && put(out, d_res, e);

  // the stages of detail::jaccard (jaccard.cpp:820-897), weighted vertex-centric
  using namespace sygraph::detail;
  Jaccard_RowSumKernel<true, int32_t, int32_t, float>::invoke(n, e, d_off, d_ind, d_vw, d_work);
  FillKernel<float>::invoke((size_t)e, d_wi, 0.0f);
  Jaccard_IsKernel<true, int32_t, int32_t, float>::invoke(n, e, d_off, d_ind, d_vw, d_work, d_wi, d_ws);
  Jaccard_JwKernel<int32_t, int32_t, float>::invoke(e, d_wi, d_ws, d_res);
  CHECK(cudaDeviceSynchronize());
  ok &= sygraph::last_status() == JX_OK && put(out, d_res, e);

  // edge-centric stages (jaccard.cpp:791-797)
  Jaccard_ec_scan<int32_t, int32_t, float>::invoke(e, n, d_off, d_dest, d_res);
  Jaccard_ec_unweighted<int32_t, int32_t, float>::invoke(e, n, d_off, d_ind, d_dest, d_res);
  CHECK(cudaDeviceSynchronize());
  ok &= sygraph::last_status() == JX_OK && put(out, d_res, e);

  // error path: no result buffer.  Reported on std::cerr and kept in last_status(), and the
  // next call runs normally.
  sygraph::jaccard<false, int32_t, int32_t, float>(graph, static_cast<float *>(nullptr));
  const int32_t st_err = sygraph::last_status();
  sygraph::jaccard<false, int32_t, int32_t, float>(graph, d_res);
  CHECK(cudaDeviceSynchronize());
  const int32_t st_next = sygraph::last_status();
  ok &= std::fwrite(&st_err, 4, 1, out) == 1 && std::fwrite(&st_next, 4, 1, out) == 1;
  std::fclose(out);

  for (void *p : {(void *)d_off, (void *)d_ind, (void *)d_edge, (void *)d_res, (void *)d_vw, (void *)d_wi,
                  (void *)d_ws, (void *)d_work, (void *)d_presum, (void *)d_dest})
    cudaFree(p);
  return ok ? 0 : 1;
}
