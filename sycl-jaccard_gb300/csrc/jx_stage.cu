// Stage-level kernels: one per kernel of the reference's vertex-centric and edge-centric
// pipelines (jaccard.hpp), with bit-identical results.  These serve stage parity and callers
// that drive the stages themselves; the fused operator (jx_fused.cu) is the fast path.
#include "jx_common.cuh"

namespace jx {

// ---------------------------------------------------------------- RowSum
// Jaccard_RowSumKernel (jaccard.cpp:236-261) + parallel_prefix_sum (jaccard.cpp:53-137).
// Each 32-element chunk is reduced with the scan's tree (lanes past the row end hold 0.0,
// jaccard.cpp:98), then the carry (the previous chunk's total) is added:
// T = tree(chunk) + T_prev (jaccard.cpp:119).  The row total is lane 31's final value.
// A row of at most 32 elements is one chunk: one thread evaluates the 32-leaf tree itself
// (pairs (2i+1, 2i), then pairs of pairs, ...; zeros past the end), which is the same set of
// additions the scan performs for lane 31.  Longer rows are taken by the whole warp.
// A warp takes 32 consecutive rows.  When they hold at most 1024 elements and none is longer
// than 32, the warp loads their contiguous index span coalesced, gathers the weights into
// shared memory, and each thread evaluates its own row's tree from there.  Otherwise each
// short row is loaded by its own thread and rows longer than 32 go to the whole warp, which
// loads and reduces 8 chunks at a time (independent loads and trees; only the carry is
// serial).  Rows of more than max_len entries are skipped (left to the caller).
constexpr int kRowSumSpan = 1024;

template <bool kWeighted>
__global__ void __launch_bounds__(256) rowsum_kernel(int32_t n, const int32_t *__restrict__ row_ptr,
                                                      const int32_t *__restrict__ ind,
                                                      const float *__restrict__ w,
                                                      float *__restrict__ work, int32_t max_len) {
  __shared__ float span_buf[kWeighted ? 256 / 32 : 1][kWeighted ? kRowSumSpan : 1];
  const int lane = threadIdx.x & 31;
  float *buf = span_buf[kWeighted ? (threadIdx.x >> 5) : 0];
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = base + threadIdx.x;
    int32_t start = 0, len = 0;
    if (r < n) {
      start = __ldg(row_ptr + r);
      len = __ldg(row_ptr + r + 1) - start;
    }
    if (!kWeighted) {
      if (r < n) work[r] = (float)len;
      continue;
    }
    const int32_t s0 = __shfl_sync(kFull, start, 0);
    const int32_t last = __reduce_max_sync(kFull, r < n ? start + len : 0);
    const bool staged = __all_sync(kFull, len <= 32) && last - s0 <= kRowSumSpan;
    if (staged) {
      for (int32_t i = lane; i < last - s0; i += 32) buf[i] = __ldg(w + __ldg(ind + s0 + i));
      __syncwarp();
    }
    if (r < n && len <= 32) {
      float x[32];
#pragma unroll
      for (int i = 0; i < 32; ++i)
        x[i] = i < len ? (staged ? buf[start - s0 + i] : __ldg(w + __ldg(ind + start + i))) : 0.0f;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
#pragma unroll
        for (int i = 0; i < 32; i += 2 * o) x[i] = x[i + o] + x[i];
      work[r] = x[0] + 0.0f;
    }
    __syncwarp();
    unsigned longs = __ballot_sync(kFull, r < n && len > 32 && len <= max_len);
    while (longs) {
      const int b = __ffs(longs) - 1;
      longs &= longs - 1;
      const int32_t sb = __shfl_sync(kFull, start, b), lb = __shfl_sync(kFull, len, b);
      float total = 0.0f;
      for (int64_t i0 = 0; i0 < lb; i0 += 8 * 32) {
        float x[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int64_t i = i0 + 32 * c + lane;
          x[c] = i < lb ? __ldg(w + __ldg(ind + sb + i)) : 0.0f;
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = warp_tree_sum(x[c]);
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (i0 + 32 * c < lb) total = x[c] + total; // chunks of the row only
      }
      if (lane == b) work[r] = total;
    }
  }
}

// ---------------------------------------------------------------- Fill
__global__ void fill_kernel(int64_t n, float *__restrict__ x, float value) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = value;
}

// ---------------------------------------------------------------- IS
// Jaccard_IsKernel (jaccard.cpp:315-400).  One warp per row; for each edge j of the row the
// warp walks the ref list in the order the reference's 8 i-lanes add on a CPU device:
// positions il, il+8, il+16, ... for il = 0..7 (jaccard.cpp:343), each found element adding
// ref_val onto weight_i[j] (jaccard.cpp:385-388: val + old).
template <bool kWeighted>
__global__ void __launch_bounds__(256) intersect_kernel(
    int32_t n, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
    const float *__restrict__ w, const float *__restrict__ work, float *__restrict__ weight_i,
    float *__restrict__ weight_s) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < n; row += nwarps) {
    const int32_t rs = __ldg(row_ptr + row), re = __ldg(row_ptr + row + 1);
    const int32_t Ni = re - rs;
    for (int32_t j = rs; j < re; ++j) {
      const int32_t c = __ldg(col + j);
      const int32_t cs = __ldg(row_ptr + c), ce = __ldg(row_ptr + c + 1);
      const int32_t Nj = ce - cs;
      const bool row_is_ref = Ni < Nj;                 // jaccard.cpp:335-336
      const int32_t ref_s = row_is_ref ? rs : cs, ref_len = row_is_ref ? Ni : Nj;
      const int32_t cur_s = row_is_ref ? cs : rs, cur_e = (row_is_ref ? ce : re) - 1;
      float acc = weight_i[j];
      for (int il = 0; il < kIsILanes; ++il) {
        const int32_t cnt = ref_len > il ? (ref_len - il + kIsILanes - 1) / kIsILanes : 0;
        for (int32_t m0 = 0; m0 < cnt; m0 += 32) {
          const int32_t m = m0 + lane;
          bool found = false;
          float val = 1.0f;
          if (m < cnt) {
            const int32_t key = __ldg(col + ref_s + il + kIsILanes * m);
            found = bsearch_found(col, cur_s, cur_e, key);
            if (kWeighted && found) val = __ldg(w + key);
          }
          acc = warp_ordered_fold(__ballot_sync(kFull, found), val, acc);
        }
      }
      if (lane == 0) {
        weight_i[j] = acc;
        weight_s[j] = __ldg(work + row) + __ldg(work + c); // jaccard.cpp:339
      }
    }
  }
}

// ---------------------------------------------------------------- JW
// Jaccard_JwKernel (jaccard.cpp:608-620).
__global__ void weight_kernel(int64_t e, const float *__restrict__ wi, const float *__restrict__ ws,
                              float *__restrict__ wj) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < e;
       j += (int64_t)gridDim.x * blockDim.x) {
    const float Wi = wi[j], Ws = ws[j];
    const float Wu = Ws - Wi;
    wj[j] = Wi / Wu;
  }
}

// ---------------------------------------------------------------- EC scan
// Jaccard_ec_scan (jaccard.cpp:654-664): one warp per row, coalesced writes.
__global__ void ec_scan_kernel(int32_t n, const int32_t *__restrict__ row_ptr,
                               int32_t *__restrict__ dest_ind, float *__restrict__ weight_j) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < n; row += nwarps) {
    const int32_t rs = __ldg(row_ptr + row), re = __ldg(row_ptr + row + 1);
    for (int32_t i = rs + lane; i < re; i += 32) {
      dest_ind[i] = (int32_t)row;
      weight_j[i] = 0.0f;
    }
  }
}

// ---------------------------------------------------------------- EC unweighted
// Jaccard_ec_unweighted (jaccard.cpp:703-743).  One warp per edge; the count keeps the
// reference's float accumulator semantics (weight_j[tid] + 1 per match, from the current
// value), then J = c / ((float)(Ni + Nj) - c).
__global__ void __launch_bounds__(256) ec_unweighted_kernel(
    int64_t e, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
    const int32_t *__restrict__ dest_ind, float *__restrict__ weight_j) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t tid = warp; tid < e; tid += nwarps) {
    const int32_t row = __ldg(col + tid);      // jaccard.cpp:712
    const int32_t colv = __ldg(dest_ind + tid); // jaccard.cpp:713
    const int32_t rs = __ldg(row_ptr + row), re = __ldg(row_ptr + row + 1);
    const int32_t cs = __ldg(row_ptr + colv), ce = __ldg(row_ptr + colv + 1);
    const int32_t Ni = re - rs, Nj = ce - cs;
    const bool row_is_ref = Ni < Nj;
    const int32_t ref_s = row_is_ref ? rs : cs, ref_len = row_is_ref ? Ni : Nj;
    const int32_t cur_s = row_is_ref ? cs : rs, cur_e = (row_is_ref ? ce : re) - 1;
    int32_t matches = 0;
    for (int32_t i0 = 0; i0 < ref_len; i0 += 32) {
      bool found = false;
      if (i0 + lane < ref_len) found = bsearch_found(col, cur_s, cur_e, __ldg(col + ref_s + i0 + lane));
      matches += __popc(__ballot_sync(kFull, found));
    }
    if (lane == 0) {
      float c = weight_j[tid];
      // c + 1 repeated `matches` times; exact in one step while c stays an integer < 2^24.
      if (c == truncf(c) && fabsf(c) + (float)matches < 16777216.0f)
        c = c + (float)matches;
      else
        for (int32_t k = 0; k < matches; ++k) c = c + 1.0f;
      weight_j[tid] = c / ((float)(Ni + Nj) - c);
    }
  }
}

// ---------------------------------------------------------------- launch helpers
static int grid_for(int64_t work_items, int threads, int per_sm = 16) {
  const int64_t want = (work_items + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * per_sm;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

jx_status rowsum_upto(int32_t n, const int32_t *row_ptr, const int32_t *ind, const float *w, float *work,
                      int32_t max_len, cudaStream_t s) {
  if (n == 0) return JX_OK;
  rowsum_kernel<true><<<grid_for(n, 256), 256, 0, s>>>(n, row_ptr, ind, w, work, max_len);
  return check_launch();
}
} // namespace jx

using namespace jx;

extern "C" {

jx_status jx_rowsum(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *ind,
                    const float *w, float *work, jx_stream_t stream) {
  if (n < 0 || e < 0 || (n > 0 && (!row_ptr || !work)) || (w && e > 0 && !ind))
    return JX_ERR_INVALID;
  if (n == 0) return JX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (w)
    rowsum_kernel<true><<<grid_for(n, 256), 256, 0, s>>>(n, row_ptr, ind, w, work, INT32_MAX);
  else
    rowsum_kernel<false><<<grid_for(n, 256), 256, 0, s>>>(n, row_ptr, ind, w, work, INT32_MAX);
  return check_launch();
}

jx_status jx_fill(int64_t n, float *x, float value, jx_stream_t stream) {
  if (n < 0 || (n > 0 && !x)) return JX_ERR_INVALID;
  if (n == 0) return JX_OK;
  fill_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, x, value);
  return check_launch();
}

jx_status jx_intersect(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *col_idx,
                       const float *w, const float *work, float *weight_i, float *weight_s,
                       jx_stream_t stream) {
  if (n < 0 || e < 0 || (n > 0 && (!row_ptr || !work)) || (e > 0 && (!col_idx || !weight_i || !weight_s)))
    return JX_ERR_INVALID;
  if (n == 0 || e == 0) return JX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int g = grid_for((int64_t)n * 32, 256);
  if (w)
    intersect_kernel<true><<<g, 256, 0, s>>>(n, row_ptr, col_idx, w, work, weight_i, weight_s);
  else
    intersect_kernel<false><<<g, 256, 0, s>>>(n, row_ptr, col_idx, w, work, weight_i, weight_s);
  return check_launch();
}

jx_status jx_weight(int32_t e, const float *weight_i, const float *weight_s, float *weight_j,
                    jx_stream_t stream) {
  if (e < 0 || (e > 0 && (!weight_i || !weight_s || !weight_j))) return JX_ERR_INVALID;
  if (e == 0) return JX_OK;
  weight_kernel<<<grid_for(e, 256), 256, 0, (cudaStream_t)stream>>>(e, weight_i, weight_s, weight_j);
  return check_launch();
}

jx_status jx_ec_scan(int32_t e, int32_t n, const int32_t *row_ptr, int32_t *dest_ind,
                     float *weight_j, jx_stream_t stream) {
  if (n < 0 || e < 0 || (n > 0 && !row_ptr) || (e > 0 && (!dest_ind || !weight_j)))
    return JX_ERR_INVALID;
  if (n == 0 || e == 0) return JX_OK;
  ec_scan_kernel<<<grid_for((int64_t)n * 32, 256), 256, 0, (cudaStream_t)stream>>>(n, row_ptr, dest_ind,
                                                                                  weight_j);
  return check_launch();
}

jx_status jx_ec_unweighted(int32_t e, int32_t n, const int32_t *row_ptr, const int32_t *col_idx,
                           const int32_t *dest_ind, float *weight_j, jx_stream_t stream) {
  if (n < 0 || e < 0 || (n > 0 && !row_ptr) || (e > 0 && (!col_idx || !dest_ind || !weight_j)))
    return JX_ERR_INVALID;
  if (e == 0) return JX_OK;
  ec_unweighted_kernel<<<grid_for((int64_t)e * 32, 256), 256, 0, (cudaStream_t)stream>>>(
      e, row_ptr, col_idx, dest_ind, weight_j);
  return check_launch();
}

} // extern "C"
