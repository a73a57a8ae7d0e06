// Batched mode: many graphs packed into one offset-indexed super-CSR on the device.
//
// The graphs are disjoint components of the super-CSR (graph g's vertices are shifted by the
// number of vertices before it, its edges by the number of edges before it), so the operator
// run once on the union gives, for every graph, exactly its own per-edge results, as a
// contiguous slice of the output.  The operator's launch sequence for the super-CSR is
// captured once as a CUDA graph and replayed by jx_batch_run, so a pass over the whole batch
// costs one graph launch instead of one operator call (about ten kernels plus a workspace
// allocation) per graph.  jx_batch_create can also time candidate schedules on the batch
// itself and keep the fastest (the autotuner): one kernel per degree bin against the persistent
// row launch, the hub kernel beside or before the rows, bin limits, the hub fetch cap and grid
// sizes.
#include "jx_common.cuh"
#include "jx_plan.h"

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

struct jx_batch_s {
  int32_t ngraphs = 0;
  int64_t nv = 0, ne = 0;
  jx_algo algo = JX_ALGO_VERTEX_CENTRIC;
  bool weighted = false;
  std::vector<int64_t> vbase, ebase; // ngraphs + 1 entries
  int32_t *row_ptr = nullptr, *col = nullptr;
  float *w = nullptr, *out = nullptr;
  void *ws = nullptr;
  int64_t *d_vbase = nullptr, *d_ebase = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels_per_run = 0;
  jx::Plan plan{};
  std::string plan_desc;
};

namespace jx {

// Shift graph-local indices to super-CSR indices: rows of graph g get +ebase[g], columns of
// graph g get +vbase[g].  The graph of a row / edge is found by binary search over the bases.
__global__ void shift_rows_kernel(int64_t nv, int32_t ngraphs, const int64_t *__restrict__ vbase,
                                  const int64_t *__restrict__ ebase, int32_t *__restrict__ row_ptr) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nv; r += (int64_t)gridDim.x * blockDim.x) {
    int32_t lo = 0, hi = ngraphs - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) >> 1;
      if (vbase[mid] <= r) lo = mid; else hi = mid - 1;
    }
    row_ptr[r] += (int32_t)ebase[lo];
  }
}

__global__ void shift_cols_kernel(int64_t ne, int32_t ngraphs, const int64_t *__restrict__ vbase,
                                  const int64_t *__restrict__ ebase, int32_t *__restrict__ col) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ne; k += (int64_t)gridDim.x * blockDim.x) {
    int32_t lo = 0, hi = ngraphs - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) >> 1;
      if (ebase[mid] <= k) lo = mid; else hi = mid - 1;
    }
    col[k] += (int32_t)vbase[lo];
  }
}

jx_status shift_to_super(int64_t nv, int64_t ne, int32_t ngraphs, const int64_t *vbase, const int64_t *ebase,
                         int32_t *row_ptr, int32_t *col, cudaStream_t s) {
  const int sms = sm_count();
  jx_status st = JX_OK;
  if (nv > 0) {
    shift_rows_kernel<<<sms * 8, 256, 0, s>>>(nv, ngraphs, vbase, ebase, row_ptr);
    if ((st = check_launch()) != JX_OK) return st;
  }
  if (ne > 0) {
    shift_cols_kernel<<<sms * 8, 256, 0, s>>>(ne, ngraphs, vbase, ebase, col);
    st = check_launch();
  }
  return st;
}

static void free_batch(jx_batch_s *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->row_ptr);
  cudaFree(b->col);
  cudaFree(b->w);
  cudaFree(b->out);
  cudaFree(b->ws);
  cudaFree(b->d_vbase);
  cudaFree(b->d_ebase);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

static std::string describe(const Plan &P) {
  char buf[256];
  std::snprintf(buf, sizeof buf,
                "%s b0_ctas=%d b1_ctas=%s b2_ctas=%d hub_clusters=%dx%d%s lane_max=%d warp_max=%d cta_max=%d "
                "hub_unit=%d hub_batch=%d%s",
                P.persistent ? "persistent-rows" : "per-bin", P.b0_ctas,
                P.b1_ctas > 0 ? std::to_string(P.b1_ctas).c_str() : "resident", P.b2_ctas, P.hub_clusters,
                P.hub_cluster, P.hub_beside ? " (beside)" : "", P.b0_max, P.b1_max, P.b2_max, P.hub_unit,
                P.hub_batch, P.relabel ? " relabelled" : "");
  return buf;
}

} // namespace jx

using namespace jx;

extern "C" {

jx_status jx_batch_create(const jx_host_graph *graphs, int32_t ngraphs, jx_algo algo, int weighted, int tune,
                          jx_batch *out) {
  if (!graphs || ngraphs <= 0 || !out) return JX_ERR_INVALID;
  if (algo != JX_ALGO_VERTEX_CENTRIC && algo != JX_ALGO_EDGE_CENTRIC) return JX_ERR_INVALID;
  *out = nullptr;
  jx_batch b = new jx_batch_s();
  b->ngraphs = ngraphs;
  b->algo = algo;
  b->weighted = weighted && algo == JX_ALGO_VERTEX_CENTRIC;
  b->vbase.assign(ngraphs + 1, 0);
  b->ebase.assign(ngraphs + 1, 0);
  int64_t max_deg = 0; // sizes the class streams (fit_plan)
  for (int32_t g = 0; g < ngraphs; ++g) {
    const jx_host_graph &h = graphs[g];
    if (h.n < 0 || h.e < 0 || (h.n == 0 && h.e > 0) || (h.n > 0 && !h.row_ptr) || (h.e > 0 && !h.col_idx) ||
        (b->weighted && h.n > 0 && !h.vertex_w)) {
      free_batch(b);
      return JX_ERR_INVALID;
    }
    b->vbase[g + 1] = b->vbase[g] + h.n;
    b->ebase[g + 1] = b->ebase[g] + h.e;
    for (int32_t r = 0; r < h.n; ++r) max_deg = std::max<int64_t>(max_deg, (int64_t)h.row_ptr[r + 1] - h.row_ptr[r]);
  }
  b->nv = b->vbase[ngraphs];
  b->ne = b->ebase[ngraphs];
  if (b->nv >= INT32_MAX || b->ne > INT32_MAX) {
    free_batch(b);
    return JX_ERR_TOO_LARGE;
  }
  cudaError_t ce;
  jx_status st = JX_OK;
#define JX_TRY(x)                                                                                  \
  if ((ce = (x)) != cudaSuccess) {                                                                 \
    st = set_cuda_error(ce);                                                                       \
    free_batch(b);                                                                                 \
    return st;                                                                                     \
  }
  JX_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  JX_TRY(cudaMalloc(&b->row_ptr, sizeof(int32_t) * (size_t)(b->nv + 1)));
  JX_TRY(cudaMalloc(&b->col, sizeof(int32_t) * (size_t)std::max<int64_t>(b->ne, 1)));
  JX_TRY(cudaMalloc(&b->out, sizeof(float) * (size_t)std::max<int64_t>(b->ne, 1)));
  if (b->weighted) JX_TRY(cudaMalloc(&b->w, sizeof(float) * (size_t)std::max<int64_t>(b->nv, 1)));
  JX_TRY(cudaMalloc(&b->d_vbase, sizeof(int64_t) * (ngraphs + 1)));
  JX_TRY(cudaMalloc(&b->d_ebase, sizeof(int64_t) * (ngraphs + 1)));
  // pack: graph-local arrays into their slots, then shift to super-CSR indices
  for (int32_t g = 0; g < ngraphs; ++g) {
    const jx_host_graph &h = graphs[g];
    if (h.n > 0)
      JX_TRY(cudaMemcpyAsync(b->row_ptr + b->vbase[g], h.row_ptr, sizeof(int32_t) * (size_t)h.n,
                             cudaMemcpyHostToDevice, b->stream));
    if (h.e > 0)
      JX_TRY(cudaMemcpyAsync(b->col + b->ebase[g], h.col_idx, sizeof(int32_t) * (size_t)h.e,
                             cudaMemcpyHostToDevice, b->stream));
    if (b->weighted && h.n > 0)
      JX_TRY(cudaMemcpyAsync(b->w + b->vbase[g], h.vertex_w, sizeof(float) * (size_t)h.n,
                             cudaMemcpyHostToDevice, b->stream));
  }
  const int32_t total_e = (int32_t)b->ne;
  JX_TRY(cudaMemcpyAsync(b->row_ptr + b->nv, &total_e, sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
  JX_TRY(cudaMemcpyAsync(b->d_vbase, b->vbase.data(), sizeof(int64_t) * (ngraphs + 1), cudaMemcpyHostToDevice,
                         b->stream));
  JX_TRY(cudaMemcpyAsync(b->d_ebase, b->ebase.data(), sizeof(int64_t) * (ngraphs + 1), cudaMemcpyHostToDevice,
                         b->stream));
  const int sms = sm_count();
  if ((st = shift_to_super(b->nv, b->ne, ngraphs, b->d_vbase, b->d_ebase, b->row_ptr, b->col, b->stream)) != JX_OK) {
    free_batch(b);
    return st;
  }
  JX_TRY(cudaStreamSynchronize(b->stream)); // host arrays may be released after create
  const jx_csr csr{(int32_t)b->nv, (int32_t)b->ne, b->row_ptr, b->col};
  const float *wp = b->weighted ? b->w : nullptr;

  // candidate plans (the default first); the autotuner keeps the fastest on this batch: one
  // kernel per bin against the persistent row launch, the hub kernel beside or before the rows,
  // the graph's own vertex ids or relabelled ones, bin limits (which rows take the lane, warp,
  // CTA or hub path), the hub fetch cap, and the grids of the lane and warp kernels
  const Plan base = fit_plan(default_plan(), b->ne, max_deg);
  std::vector<Plan> plans{base};
  if (tune) {
    auto add = [&](Plan P) { plans.push_back(fit_plan(P, b->ne, max_deg)); };
    Plan Q = base;
    Q.hub_beside = !base.hub_beside;
    add(Q);
    Q = base;
    Q.relabel = !base.relabel;
    add(Q);
    Q = base;
    Q.persistent = true;
    add(Q);
    Q = base;
    Q.hub_cluster = base.hub_cluster == 4 ? 8 : 4;
    Q.hub_clusters = hub_cluster_count(Q.hub_cluster);
    add(Q);
    for (int32_t b1 : {128, 256}) {
      Q = base;
      Q.b1_max = b1;
      add(Q);
    }
    for (int32_t b2 : {4096, 12288}) {
      Q = base;
      Q.b2_max = b2;
      add(Q);
    }
    for (int32_t hb : {1, 8}) {
      Q = base;
      Q.hub_batch = hb;
      add(Q);
    }
    for (int m0 : {4, 16}) {
      Q = base;
      Q.b0_ctas = sms * m0;
      add(Q);
    }
    for (int m1 : {2, 4}) {
      Q = base;
      Q.b1_ctas = sms * m1;
      add(Q);
    }
  }
  size_t ws_bytes = 0;
  for (const Plan &P : plans) ws_bytes = std::max(ws_bytes, plan_workspace(csr.n, csr.e, b->weighted, P));
  JX_TRY(cudaMalloc(&b->ws, std::max<size_t>(ws_bytes, 256)));
  b->plan = plans[0];
  if (b->ne > 0) {
    // warm-up (also sets kernel attributes outside any capture)
    if ((st = run_plan(csr, wp, b->out, algo, b->ws, b->plan, b->stream)) != JX_OK) { free_batch(b); return st; }
    if (plans.size() > 1) {
      cudaEvent_t e0, e1;
      JX_TRY(cudaEventCreate(&e0));
      JX_TRY(cudaEventCreate(&e1));
      float best = 1e30f;
      for (const Plan &P : plans) {
        float total = 0.0f;
        for (int rep = 0; rep < 2; ++rep) {
          cudaEventRecord(e0, b->stream);
          if ((st = run_plan(csr, wp, b->out, algo, b->ws, P, b->stream)) != JX_OK) break;
          cudaEventRecord(e1, b->stream);
          cudaEventSynchronize(e1);
          float ms = 0.0f;
          cudaEventElapsedTime(&ms, e0, e1);
          total += ms;
        }
        if (st != JX_OK) break;
        if (total < best) {
          best = total;
          b->plan = P;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (st != JX_OK) { free_batch(b); return st; }
    }
    // capture the operator under the chosen plan
    const uint64_t before = jx_launch_count();
    JX_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    st = run_plan(csr, wp, b->out, algo, b->ws, b->plan, b->stream);
    cudaGraph_t graph = nullptr;
    ce = cudaStreamEndCapture(b->stream, &graph);
    if (st != JX_OK) { if (graph) cudaGraphDestroy(graph); free_batch(b); return st; }
    JX_TRY(ce);
    b->graph = graph;
    b->kernels_per_run = jx_launch_count() - before;
    jx_launch_count_reset(); // the capture itself launched nothing
    count_launches(before);
    JX_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
    // the warm-up pass ran on the batch's own stream: it must end before a replay on the
    // caller's stream touches the same workspace and outputs
    JX_TRY(cudaStreamSynchronize(b->stream));
  }
  b->plan_desc = describe(b->plan);
#undef JX_TRY
  *out = b;
  return JX_OK;
}

jx_status jx_batch_run(jx_batch b, jx_stream_t stream) {
  if (!b) return JX_ERR_INVALID;
  if (!b->exec) return JX_OK;
  const cudaError_t ce = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  count_launches(b->kernels_per_run);
  return JX_OK;
}

jx_status jx_batch_result(jx_batch b, int32_t g, const float **device_out, int64_t *count) {
  if (!b || g < 0 || g >= b->ngraphs || !device_out || !count) return JX_ERR_INVALID;
  *device_out = b->out + b->ebase[g];
  *count = b->ebase[g + 1] - b->ebase[g];
  return JX_OK;
}

jx_status jx_batch_download(jx_batch b, int32_t g, float *host_out, jx_stream_t stream) {
  if (!b || g < -1 || g >= b->ngraphs || !host_out) return JX_ERR_INVALID;
  const int64_t first = g < 0 ? 0 : b->ebase[g];
  const int64_t cnt = g < 0 ? b->ne : b->ebase[g + 1] - b->ebase[g];
  if (cnt == 0) return JX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce = cudaMemcpyAsync(host_out, b->out + first, sizeof(float) * (size_t)cnt,
                                   cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  return ce == cudaSuccess ? JX_OK : set_cuda_error(ce);
}

jx_status jx_batch_info(jx_batch b, int64_t *vertices, int64_t *edges, uint64_t *kernels_per_run,
                        char *plan_desc, size_t len) {
  if (!b) return JX_ERR_INVALID;
  if (vertices) *vertices = b->nv;
  if (edges) *edges = b->ne;
  if (kernels_per_run) *kernels_per_run = b->kernels_per_run;
  if (plan_desc && len) {
    const size_t k = std::min(len - 1, b->plan_desc.size());
    std::copy(b->plan_desc.begin(), b->plan_desc.begin() + k, plan_desc);
    plan_desc[k] = 0;
  }
  return JX_OK;
}

void jx_batch_destroy(jx_batch b) { free_batch(b); }

} // extern "C"
