// Fused Jaccard operator: intersection and weight in one pass, J written once per edge, no
// atomics on results.  Drop-in for sygraph::jaccard<edge_centric> (jaccard.cpp:926-955).
//
// Work decomposition ("tasks").  An intersection |N(x) n N(y)| is computed by staging the
// longer list N(u) in shared memory as an open-addressing hash set and streaming the shorter
// list N(v) through it.  Row u (the "cur" list) owns a task for every neighbour v with
// d_v <= d_u (v's list is the "ref" list, the one the reference walks element by element).
// The reference picks the ref list per directed edge (VC: jaccard.cpp:333-336, EC:
// jaccard.cpp:716-719), so one task serves two directed edges:
//   VC: (u,v) always (ref = v when d_u >= d_v);      (v,u) when d_v < d_u
//   EC: (u,v) when d_v < d_u;                         (v,u) always (ref = v when d_v <= d_u)
// The reverse edge (v,u) is located for free: it is the position of u inside N(v), which
// the task streams anyway.  Its result is bit-identical because both edges use the same ref
// list, the same cur set and a commutative S_u + S_v.  Edges that no task covers (graphs
// that are not symmetric) keep a sentinel and are computed by a fix-up pass.
//
// Degree bins (by d_u, the staged list):
//   B0: d_u <= 32        one warp per row, 64-slot table per warp
//   B1: d_u <= 512       one warp per row, 1024-slot table per warp
//   B2: d_u <= 24576     one 1024-thread CTA per row, table of 2*d_u slots (<= 192 KB)
//   B3: larger (hubs)    one CTA per row, ref elements binary-searched in N(u)
//
// Weighted sums follow the reference's accumulation order exactly: ref positions are taken
// in the order il, il+8, il+16, ... for il = 0..7 (jaccard.cpp:343) and folded one by one.
#include "jx_common.cuh"

#include <algorithm>

namespace jx {

constexpr int kBins = 4;
constexpr int32_t kB0Max = 32, kB1Max = 512, kB2Max = 24576;
constexpr int kB0Slots = 64, kB1Slots = 1024;
constexpr int kB2Threads = 1024;
constexpr int kRowThreads = 256; // warps-per-row kernels
constexpr int32_t kEmpty = -1;

// Counters in the workspace (int32 each).
enum { kCntBin0 = 0, kWorkBin2 = kBins, kWorkBin3 = kBins + 1, kCounters = 16 };

struct Workspace {
  float *S;        // weighted row sums, n floats (weighted VC only)
  int32_t *rows;   // bin row lists: bin b starts at rows + b * n ... packed by offsets below
  int32_t *cnt;    // counters
};

// ---------------------------------------------------------------- hash set in shared memory
__device__ __forceinline__ uint32_t hslot(int32_t key, uint32_t size) {
  return __umulhi((uint32_t)key * 0x9E3779B1u, size);
}

__device__ __forceinline__ void hset_insert(int32_t *t, uint32_t size, int32_t key) {
  uint32_t s = hslot(key, size);
  for (;;) {
    const int32_t old = atomicCAS(t + s, kEmpty, key);
    if (old == kEmpty || old == key) return;
    if (++s == size) s = 0;
  }
}

__device__ __forceinline__ bool hset_find(const int32_t *t, uint32_t size, int32_t key) {
  uint32_t s = hslot(key, size);
  for (;;) {
    const int32_t k = t[s];
    if (k == key) return true;
    if (k == kEmpty) return false;
    if (++s == size) s = 0;
  }
}

struct HashProbe {
  const int32_t *t;
  uint32_t size;
  __device__ bool operator()(int32_t key) const { return hset_find(t, size, key); }
};

struct SearchProbe { // sorted cur list in global memory (hub fallback)
  const int32_t *col;
  int32_t lo, hi; // inclusive range
  __device__ bool operator()(int32_t key) const { return bsearch_found(col, lo, hi, key); }
};

// ---------------------------------------------------------------- one task, one warp
// Streams N(v) (positions [vs, vs+dv)) through `probe` (membership in N(u)).
// Returns the reference-order intersection value (count for unweighted) and the position
// of u inside N(v) (or -1; -2 when u occurs more than once).
template <bool kWeighted, class Probe>
__device__ __forceinline__ float warp_task(const Probe &probe, const int32_t *__restrict__ col,
                                           const float *__restrict__ w, int32_t u, int32_t vs,
                                           int32_t dv, int32_t &mirror) {
  const int lane = threadIdx.x & 31;
  mirror = -1;
  if (!kWeighted) {
    int32_t cnt = 0;
    for (int32_t p0 = 0; p0 < dv; p0 += 32) {
      const int32_t p = p0 + lane;
      int32_t x = kEmpty;
      bool found = false;
      if (p < dv) {
        x = __ldg(col + vs + p);
        found = probe(x);
      }
      cnt += __popc(__ballot_sync(kFull, found));
      const unsigned mb = __ballot_sync(kFull, x == u);
      if (mb) mirror = (mirror == -1 && __popc(mb) == 1) ? p0 + __ffs(mb) - 1 : -2;
    }
    return (float)cnt;
  } else {
    float acc = 0.0f;
    for (int il = 0; il < kIsILanes; ++il) {
      const int32_t cntc = dv > il ? (dv - il + kIsILanes - 1) / kIsILanes : 0;
      for (int32_t m0 = 0; m0 < cntc; m0 += 32) {
        const int32_t m = m0 + lane;
        int32_t x = kEmpty;
        bool found = false;
        float val = 0.0f;
        if (m < cntc) {
          x = __ldg(col + vs + il + kIsILanes * m);
          found = probe(x);
          if (found) val = __ldg(w + x);
        }
        acc = warp_ordered_fold(__ballot_sync(kFull, found), val, acc);
        const unsigned mb = __ballot_sync(kFull, x == u);
        if (mb) mirror = (mirror == -1 && __popc(mb) == 1) ? il + kIsILanes * (m0 + __ffs(mb) - 1) : -2;
      }
    }
    return acc;
  }
}

// Result for a task and the two directed edges it may serve.
template <bool kEC, bool kWeighted>
__device__ __forceinline__ void write_task(float I, int32_t du, int32_t dv, float Su, float Sv,
                                           int64_t e_uv, int64_t e_vu, float *__restrict__ out) {
  float J;
  if (kEC) {
    J = I / ((float)(dv + du) - I); // jaccard.cpp:741, Ni = d_v (csrInd[tid]), Nj = d_u
  } else {
    const float Ws = kWeighted ? (Su + Sv) : ((float)du + (float)dv); // jaccard.cpp:258,339
    const float Wu = Ws - I;                                           // jaccard.cpp:617
    J = I / Wu;                                                        // jaccard.cpp:618
  }
  const bool strict = dv < du;
  if (kEC) {
    if (strict) out[e_uv] = J;
    if (e_vu >= 0) out[e_vu] = J;
  } else {
    out[e_uv] = J;
    if (strict && e_vu >= 0) out[e_vu] = J;
  }
}

// ---------------------------------------------------------------- plan: bin the rows
__global__ void plan_kernel(int32_t n, const int32_t *__restrict__ row_ptr, int32_t *__restrict__ rows,
                            int32_t *__restrict__ cnt) {
  // rows: four regions of n entries (row lists per bin)
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = __ldg(row_ptr + u + 1) - __ldg(row_ptr + u);
    if (d == 0) continue;
    const int b = d <= kB0Max ? 0 : (d <= kB1Max ? 1 : (d <= kB2Max ? 2 : 3));
    const int32_t slot = atomicAdd(cnt + kCntBin0 + b, 1);
    rows[(int64_t)b * n + slot] = (int32_t)u;
  }
}

__global__ void fill_bits_kernel(int64_t n, uint32_t *__restrict__ x, uint32_t bits) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = bits;
}

// ---------------------------------------------------------------- B0/B1: one warp per row
template <bool kEC, bool kWeighted, int kSlots>
__global__ void __launch_bounds__(kRowThreads) warp_rows_kernel(
    int32_t n, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
    const float *__restrict__ w, const float *__restrict__ S, const int32_t *__restrict__ rows,
    const int32_t *__restrict__ count, float *__restrict__ out) {
  __shared__ int32_t tables[kRowThreads / 32][kSlots];
  const int lane = threadIdx.x & 31;
  int32_t *t = tables[threadIdx.x >> 5];
  const int32_t nrows = *count;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nrows; i += nwarps) {
    const int32_t u = rows[i];
    const int32_t us = __ldg(row_ptr + u), du = __ldg(row_ptr + u + 1) - us;
    uint32_t size = 2u * (uint32_t)du;
    size = size < 32u ? 32u : size;
    for (uint32_t k = lane; k < size; k += 32) t[k] = kEmpty;
    __syncwarp();
    for (int32_t k = lane; k < du; k += 32) hset_insert(t, size, __ldg(col + us + k));
    __syncwarp();
    const float Su = kWeighted ? __ldg(S + u) : 0.0f;
    const HashProbe probe{t, size};
    for (int32_t k = 0; k < du; ++k) {
      const int32_t v = __ldg(col + us + k);
      const int32_t vs = __ldg(row_ptr + v), dv = __ldg(row_ptr + v + 1) - vs;
      if (dv > du) continue;
      int32_t mirror;
      const float I = warp_task<kWeighted>(probe, col, w, u, vs, dv, mirror);
      if (lane == 0)
        write_task<kEC, kWeighted>(I, du, dv, Su, kWeighted ? __ldg(S + v) : 0.0f, (int64_t)us + k,
                                   mirror >= 0 ? (int64_t)vs + mirror : -1, out);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- B2/B3: one CTA per row
template <bool kEC, bool kWeighted, bool kHub>
__global__ void __launch_bounds__(kB2Threads) cta_rows_kernel(
    int32_t n, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
    const float *__restrict__ w, const float *__restrict__ S, const int32_t *__restrict__ rows,
    const int32_t *__restrict__ count, int32_t *__restrict__ work_ctr, float *__restrict__ out) {
  extern __shared__ int32_t table[];
  __shared__ int32_t s_row;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int32_t nrows = *count;
  for (;;) {
    if (threadIdx.x == 0) s_row = atomicAdd(work_ctr, 1);
    __syncthreads();
    const int32_t i = s_row;
    __syncthreads();
    if (i >= nrows) break;
    const int32_t u = rows[i];
    const int32_t us = __ldg(row_ptr + u), du = __ldg(row_ptr + u + 1) - us;
    const uint32_t size = 2u * (uint32_t)du;
    if (!kHub) {
      for (uint32_t k = threadIdx.x; k < size; k += blockDim.x) table[k] = kEmpty;
      __syncthreads();
      for (int32_t k = threadIdx.x; k < du; k += blockDim.x) hset_insert(table, size, __ldg(col + us + k));
      __syncthreads();
    }
    const float Su = kWeighted ? __ldg(S + u) : 0.0f;
    for (int32_t k = warp; k < du; k += nw) {
      const int32_t v = __ldg(col + us + k);
      const int32_t vs = __ldg(row_ptr + v), dv = __ldg(row_ptr + v + 1) - vs;
      if (dv > du) continue;
      int32_t mirror;
      float I;
      if (kHub)
        I = warp_task<kWeighted>(SearchProbe{col, us, us + du - 1}, col, w, u, vs, dv, mirror);
      else
        I = warp_task<kWeighted>(HashProbe{table, size}, col, w, u, vs, dv, mirror);
      if (lane == 0)
        write_task<kEC, kWeighted>(I, du, dv, Su, kWeighted ? __ldg(S + v) : 0.0f, (int64_t)us + k,
                                   mirror >= 0 ? (int64_t)vs + mirror : -1, out);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- fix-up of uncovered edges
// Any edge still holding the sentinel is computed on its own, with the reference's own
// ref/cur choice (VC jaccard.cpp:333-336, EC jaccard.cpp:716-719) and binary search.
template <bool kEC, bool kWeighted>
__global__ void __launch_bounds__(256) fixup_kernel(int32_t n, const int32_t *__restrict__ row_ptr,
                                                    const int32_t *__restrict__ col,
                                                    const float *__restrict__ w,
                                                    const float *__restrict__ S,
                                                    float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  uint32_t *outb = reinterpret_cast<uint32_t *>(out);
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += nwarps) {
    const int32_t us = __ldg(row_ptr + u), ue = __ldg(row_ptr + u + 1), du = ue - us;
    for (int32_t j0 = us; j0 < ue; j0 += 32) {
      const int32_t j = j0 + lane;
      unsigned todo = __ballot_sync(kFull, j < ue && outb[j] == kUnwritten);
      while (todo) {
        const int32_t jj = j0 + __ffs(todo) - 1;
        todo &= todo - 1;
        const int32_t v = __ldg(col + jj);
        const int32_t vs = __ldg(row_ptr + v), dv = __ldg(row_ptr + v + 1) - vs;
        // ref/cur per the reference rule for this directed edge
        const bool u_is_ref = kEC ? !(dv < du) : (du < dv);
        const int32_t rs = u_is_ref ? us : vs, rl = u_is_ref ? du : dv;
        const int32_t cs = u_is_ref ? vs : us, cl = u_is_ref ? dv : du;
        int32_t dummy;
        const float I = warp_task<kWeighted && !kEC>(SearchProbe{col, cs, cs + cl - 1}, col, w,
                                                      -1, rs, rl, dummy);
        if (lane == 0) {
          float J;
          if (kEC) {
            J = I / ((float)(dv + du) - I);
          } else {
            const float Ws = kWeighted ? (__ldg(S + u) + __ldg(S + v)) : ((float)du + (float)dv);
            J = I / (Ws - I);
          }
          out[jj] = J;
        }
      }
    }
  }
}

// ---------------------------------------------------------------- host driver
size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t workspace_bytes(int32_t n, bool weighted_vc) {
  return align256(sizeof(int32_t) * kCounters) + align256(sizeof(int32_t) * (size_t)n * kBins) +
         (weighted_vc ? align256(sizeof(float) * (size_t)n) : 0);
}

template <bool kEC, bool kWeighted>
jx_status run_fused(const jx_csr &g, const float *w, float *out, char *ws, cudaStream_t s) {
  const int32_t n = g.n;
  int32_t *cnt = reinterpret_cast<int32_t *>(ws);
  int32_t *rows = reinterpret_cast<int32_t *>(ws + align256(sizeof(int32_t) * kCounters));
  float *S = kWeighted ? reinterpret_cast<float *>(ws + align256(sizeof(int32_t) * kCounters) +
                                                   align256(sizeof(int32_t) * (size_t)n * kBins))
                       : nullptr;
  const int sms = sm_count();
  cudaError_t ce = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * kCounters, s);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  jx_status st;
  plan_kernel<<<sms * 8, 256, 0, s>>>(n, g.row_ptr, rows, cnt);
  if ((st = check_launch()) != JX_OK) return st;
  if (kWeighted) {
    if ((st = jx_rowsum(n, g.e, g.row_ptr, g.col_idx, w, S, (jx_stream_t)s)) != JX_OK) return st;
  }
  fill_bits_kernel<<<sms * 8, 256, 0, s>>>(g.e, reinterpret_cast<uint32_t *>(out), kUnwritten);
  if ((st = check_launch()) != JX_OK) return st;

  const size_t smem_b2 = sizeof(int32_t) * 2 * (size_t)kB2Max;
  ce = cudaFuncSetAttribute(cta_rows_kernel<kEC, kWeighted, false>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b2);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  // hubs first (longest rows), then the CTA bin, then the warp bins
  cta_rows_kernel<kEC, kWeighted, true><<<sms, kB2Threads, 0, s>>>(
      n, g.row_ptr, g.col_idx, w, S, rows + 3 * (size_t)n, cnt + kCntBin0 + 3, cnt + kWorkBin3, out);
  if ((st = check_launch()) != JX_OK) return st;
  cta_rows_kernel<kEC, kWeighted, false><<<sms, kB2Threads, smem_b2, s>>>(
      n, g.row_ptr, g.col_idx, w, S, rows + 2 * (size_t)n, cnt + kCntBin0 + 2, cnt + kWorkBin2, out);
  if ((st = check_launch()) != JX_OK) return st;
  warp_rows_kernel<kEC, kWeighted, kB1Slots><<<sms * 4, kRowThreads, 0, s>>>(
      n, g.row_ptr, g.col_idx, w, S, rows + 1 * (size_t)n, cnt + kCntBin0 + 1, out);
  if ((st = check_launch()) != JX_OK) return st;
  warp_rows_kernel<kEC, kWeighted, kB0Slots><<<sms * 8, kRowThreads, 0, s>>>(
      n, g.row_ptr, g.col_idx, w, S, rows, cnt + kCntBin0, out);
  if ((st = check_launch()) != JX_OK) return st;
  fixup_kernel<kEC, kWeighted><<<sms * 8, 256, 0, s>>>(n, g.row_ptr, g.col_idx, w, S, out);
  return check_launch();
}

} // namespace jx

using namespace jx;

extern "C" {

size_t jx_jaccard_workspace_size(const jx_csr *g, int weighted, jx_algo algo) {
  if (!g || g->n < 0) return 0;
  return workspace_bytes(g->n, weighted && algo == JX_ALGO_VERTEX_CENTRIC);
}

jx_status jx_jaccard_ws(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                        void *workspace, size_t workspace_bytes_, jx_stream_t stream) {
  if (!g || g->n < 0 || g->e < 0) return JX_ERR_INVALID;
  if (algo != JX_ALGO_VERTEX_CENTRIC && algo != JX_ALGO_EDGE_CENTRIC) return JX_ERR_INVALID;
  if (g->n == 0 || g->e == 0) return JX_OK;
  if (!g->row_ptr || !g->col_idx || !out_j) return JX_ERR_INVALID;
  const bool ec = algo == JX_ALGO_EDGE_CENTRIC;
  const bool weighted = vertex_w != nullptr && !ec; // EC ignores weights (jaccard.cpp:790)
  if (!workspace || workspace_bytes_ < workspace_bytes(g->n, weighted) ||
      (reinterpret_cast<uintptr_t>(workspace) & 255u))
    return JX_ERR_INVALID;
  char *ws = static_cast<char *>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  if (ec) return run_fused<true, false>(*g, nullptr, out_j, ws, s);
  if (weighted) return run_fused<false, true>(*g, vertex_w, out_j, ws, s);
  return run_fused<false, false>(*g, nullptr, out_j, ws, s);
}

jx_status jx_jaccard(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                     jx_stream_t stream) {
  if (!g || g->n < 0 || g->e < 0) return JX_ERR_INVALID;
  if (g->n == 0 || g->e == 0) return JX_OK;
  const size_t bytes = jx_jaccard_workspace_size(g, vertex_w != nullptr, algo);
  cudaStream_t s = (cudaStream_t)stream;
  void *ws = nullptr;
  cudaError_t ce = cudaMallocAsync(&ws, bytes, s);
  if (ce != cudaSuccess) return ce == cudaErrorMemoryAllocation ? JX_ERR_NOMEM : set_cuda_error(ce);
  const jx_status st = jx_jaccard_ws(g, vertex_w, out_j, algo, ws, bytes, stream);
  ce = cudaFreeAsync(ws, s);
  if (st != JX_OK) return st;
  return ce == cudaSuccess ? JX_OK : set_cuda_error(ce);
}

} // extern "C"
