// Result post-processing of the reference's driver, on the device:
//   - the edge-centric "non zero pairs" count (jaccard.cpp:810-819): values above a threshold;
//   - reverse-edge removal before MTX output (main.cpp:307-309, readMtxToCSR.cpp:134-147):
//     the reference program turns (row, col, J) into a std::set and, walking it from the largest tuple
//     down, erases the reverse (col, row, J) of every tuple still present.  The survivors are
//     every (a, b) with a > b, and every (a, b) with a < b whose reverse is missing or holds a
//     different value (equal, or either a NaN -- std::set treats NaN as equivalent); self
//     loops erase themselves.  Output is the surviving edges in CSR order, which is the set's
//     ascending order when rows are sorted.
#include "jx_common.cuh"

namespace jx {

constexpr int kPostThreads = 256;

__global__ void count_above_kernel(int64_t e, const float *__restrict__ v, float thresh,
                                   unsigned long long *__restrict__ count) {
  unsigned long long c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < e; i += (int64_t)gridDim.x * blockDim.x)
    c += v[i] > thresh;
  c = __reduce_add_sync(kFull, (unsigned)c);
  __shared__ unsigned long long s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s, c);
  __syncthreads();
  if (threadIdx.x == 0 && s) atomicAdd(count, s);
}

// keep[k] = 1 when edge k survives reverse-edge removal.  One warp per row.
__global__ void keep_kernel(int32_t n, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
                            const float *__restrict__ v, uint8_t *__restrict__ keep) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n; a += nwarps) {
    const int32_t s = row_ptr[a], t = row_ptr[a + 1];
    for (int32_t k = s + lane; k < t; k += 32) {
      const int32_t b = col[k];
      bool keep_it;
      if (b < a) {
        keep_it = true;
      } else if (b == a) {
        keep_it = false;
      } else {
        // reverse (b, a): binary search a in N(b)
        int32_t lo = row_ptr[b], hi = row_ptr[b + 1] - 1, pos = -1;
        while (lo <= hi) {
          const int32_t mid = (lo + hi) >> 1;
          const int32_t c = col[mid];
          if (c < a) lo = mid + 1;
          else if (c > a) hi = mid - 1;
          else { pos = mid; break; }
        }
        if (pos < 0) {
          keep_it = true;
        } else {
          const float x = v[k], y = v[pos];
          keep_it = !(x == y || isnan(x) || isnan(y));
        }
      }
      keep[k] = keep_it;
    }
  }
}

// Per-block counts of kept edges over consecutive tiles of kPostThreads * 4 edges.
constexpr int kTile = kPostThreads * 4;

__global__ void tile_count_kernel(int64_t e, const uint8_t *__restrict__ keep, int64_t *__restrict__ tiles) {
  const int64_t t0 = (int64_t)blockIdx.x * kTile;
  int c = 0;
  for (int q = 0; q < 4; ++q) {
    const int64_t i = t0 + q * kPostThreads + threadIdx.x;
    c += i < e ? keep[i] : 0;
  }
  c = __reduce_add_sync(kFull, c);
  __shared__ int s[kPostThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t tot = 0;
    for (int w = 0; w < kPostThreads / 32; ++w) tot += s[w];
    tiles[blockIdx.x] = tot;
  }
}

// Exclusive scan of the tile counts in one block (sequential over chunks of the block size).
__global__ void tile_scan_kernel(int64_t ntiles, int64_t *__restrict__ tiles, int64_t *__restrict__ total) {
  __shared__ int64_t s[1024];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const int64_t x = i < ntiles ? tiles[i] : 0;
    s[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      const int64_t y = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += y;
      __syncthreads();
    }
    if (i < ntiles) tiles[i] = carry + s[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += s[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// Scatter the kept edges as (src, dst, value) in CSR order.
__global__ void scatter_kernel(int32_t n, int64_t e, const int32_t *__restrict__ row_ptr,
                               const int32_t *__restrict__ col, const float *__restrict__ v,
                               const uint8_t *__restrict__ keep, const int64_t *__restrict__ tiles,
                               int32_t *__restrict__ src, int32_t *__restrict__ dst, float *__restrict__ val) {
  __shared__ int s[kTile];
  const int64_t t0 = (int64_t)blockIdx.x * kTile;
  for (int q = 0; q < 4; ++q) {
    const int64_t i = t0 + q * kPostThreads + threadIdx.x;
    s[q * kPostThreads + threadIdx.x] = i < e ? keep[i] : 0;
  }
  __syncthreads();
  // inclusive scan of the tile in shared memory (Hillis-Steele, 1024 entries)
  for (int o = 1; o < kTile; o <<= 1) {
    int y[4];
    for (int q = 0; q < 4; ++q) {
      const int j = q * kPostThreads + threadIdx.x;
      y[q] = j >= o ? s[j - o] : 0;
    }
    __syncthreads();
    for (int q = 0; q < 4; ++q) s[q * kPostThreads + threadIdx.x] += y[q];
    __syncthreads();
  }
  for (int q = 0; q < 4; ++q) {
    const int j = q * kPostThreads + threadIdx.x;
    const int64_t i = t0 + j;
    if (i < e && keep[i]) {
      const int64_t o = tiles[blockIdx.x] + s[j] - 1;
      // source row of edge i: last row with row_ptr[row] <= i
      int32_t lo = 0, hi = n - 1;
      while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (row_ptr[mid] <= i) lo = mid; else hi = mid - 1;
      }
      src[o] = lo;
      dst[o] = col[i];
      val[o] = v[i];
    }
  }
}

} // namespace jx

using namespace jx;

extern "C" {

jx_status jx_count_above(int64_t e, const float *values, float thresh, unsigned long long *count,
                         jx_stream_t stream) {
  if (e < 0 || !count || (e > 0 && !values)) return JX_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  if (e == 0) return JX_OK;
  const int64_t want = (e + kPostThreads - 1) / kPostThreads;
  const int grid = (int)(want < (int64_t)sm_count() * 8 ? want : (int64_t)sm_count() * 8);
  count_above_kernel<<<grid, kPostThreads, 0, s>>>(e, values, thresh, count);
  return check_launch();
}

jx_status jx_remove_reverse_edges(const jx_csr *g, const float *values, int32_t *src, int32_t *dst,
                                  float *out_values, int64_t *count, jx_stream_t stream) {
  if (!g || g->n < 0 || g->e < 0 || !count) return JX_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce;
  if (g->e == 0 || g->n == 0) {
    ce = cudaMemsetAsync(count, 0, sizeof(int64_t), s);
    return ce == cudaSuccess ? JX_OK : set_cuda_error(ce);
  }
  if (!g->row_ptr || !g->col_idx || !values || !src || !dst || !out_values) return JX_ERR_INVALID;
  const int64_t e = g->e;
  const int64_t ntiles = (e + kTile - 1) / kTile;
  uint8_t *keep = nullptr;
  int64_t *tiles = nullptr;
  if ((ce = cudaMallocAsync(&keep, (size_t)e, s)) != cudaSuccess) return set_cuda_error(ce);
  if ((ce = cudaMallocAsync(&tiles, sizeof(int64_t) * (size_t)ntiles, s)) != cudaSuccess) {
    cudaFreeAsync(keep, s);
    return set_cuda_error(ce);
  }
  jx_status st = JX_OK;
  do {
    keep_kernel<<<sm_count() * 8, kPostThreads, 0, s>>>(g->n, g->row_ptr, g->col_idx, values, keep);
    if ((st = check_launch()) != JX_OK) break;
    tile_count_kernel<<<(unsigned)ntiles, kPostThreads, 0, s>>>(e, keep, tiles);
    if ((st = check_launch()) != JX_OK) break;
    tile_scan_kernel<<<1, 1024, 0, s>>>(ntiles, tiles, count);
    if ((st = check_launch()) != JX_OK) break;
    scatter_kernel<<<(unsigned)ntiles, kPostThreads, 0, s>>>(g->n, e, g->row_ptr, g->col_idx, values, keep,
                                                             tiles, src, dst, out_values);
    st = check_launch();
  } while (0);
  cudaFreeAsync(keep, s);
  cudaFreeAsync(tiles, s);
  return st;
}

} // extern "C"
