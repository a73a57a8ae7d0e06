// Device CSR builder: the graph preparation the reference's driver does on the host
// (main.cpp:99-118, readMtxToCSR.cpp:117-208): edge list -> optional reverse edges -> sorted,
// deduplicated set -> CSR rows without self loops.  Here as device passes:
//   1. keys: every edge (u, v) becomes the key u * n + v (and v * n + u when symmetrising);
//      dropped self loops and padding become the sentinel n * n, which sorts last;
//   2. an LSD radix sort of the 64-bit keys over the bits n * n needs (8 bits per pass; each
//      pass = tile histograms, one exclusive scan of the digit-major counts, a stable scatter
//      that ranks keys inside a tile in order);
//   3. first-of-run flags -> exclusive scan -> compaction into col, row counts -> scan ->
//      row_ptr.
// The scans are reduce-then-scan over 4096-element tiles, recursive over the tile sums.
#include "jx_common.cuh"

#include <vector>

namespace jx {
namespace {

constexpr int kBuildThreads = 256;
constexpr int kPerThread = 16;
constexpr int kTileKeys = kBuildThreads * kPerThread; // 4096 keys per tile

// ---------------------------------------------------------------- scan (int64)
__global__ void tile_sum_kernel(int64_t n, const int64_t *__restrict__ in, int64_t *__restrict__ sums) {
  __shared__ int64_t s[kBuildThreads / 32];
  const int64_t t0 = (int64_t)blockIdx.x * kTileKeys;
  int64_t acc = 0;
  for (int q = 0; q < kPerThread; ++q) {
    const int64_t i = t0 + (int64_t)q * kBuildThreads + threadIdx.x;
    if (i < n) acc += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t tot = 0;
    for (int w = 0; w < kBuildThreads / 32; ++w) tot += s[w];
    sums[blockIdx.x] = tot;
  }
}

// Exclusive scan of one tile in shared memory plus the tile's offset.  Thread t owns the 16
// consecutive elements t*16 .. t*16+15 of the tile.
__global__ void tile_scan_kernel(int64_t n, const int64_t *__restrict__ in, const int64_t *__restrict__ offs,
                                 int64_t *__restrict__ out) {
  __shared__ int64_t s[kBuildThreads];
  const int64_t t0 = (int64_t)blockIdx.x * kTileKeys + (int64_t)threadIdx.x * kPerThread;
  int64_t v[kPerThread];
  int64_t local = 0;
#pragma unroll
  for (int q = 0; q < kPerThread; ++q) {
    const int64_t i = t0 + q;
    v[q] = i < n ? in[i] : 0;
    local += v[q];
  }
  s[threadIdx.x] = local;
  __syncthreads();
  for (int o = 1; o < kBuildThreads; o <<= 1) {
    const int64_t y = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += y;
    __syncthreads();
  }
  int64_t run = (offs ? offs[blockIdx.x] : 0) + s[threadIdx.x] - local;
#pragma unroll
  for (int q = 0; q < kPerThread; ++q) {
    const int64_t i = t0 + q;
    if (i < n) out[i] = run;
    run += v[q];
  }
}

// out[i] = sum of in[0..i) for i < n (in and out may alias); *total = sum of all (device).
jx_status scan_exclusive(const int64_t *in, int64_t *out, int64_t n, int64_t *total, cudaStream_t s) {
  if (n <= 0) {
    if (total) {
      const cudaError_t ce = cudaMemsetAsync(total, 0, sizeof(int64_t), s);
      if (ce != cudaSuccess) return set_cuda_error(ce);
    }
    return JX_OK;
  }
  const int64_t tiles = (n + kTileKeys - 1) / kTileKeys;
  int64_t *sums = nullptr;
  cudaError_t ce = cudaMallocAsync(&sums, sizeof(int64_t) * (size_t)(tiles + 1), s);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  jx_status st = JX_OK;
  do {
    if (tiles > 1 || total) {
      tile_sum_kernel<<<(unsigned)tiles, kBuildThreads, 0, s>>>(n, in, sums);
      if ((st = check_launch()) != JX_OK) break;
    }
    if (tiles > 1) {
      // offsets of the tiles: an exclusive scan of their sums (recursive), total in sums[tiles]
      if ((st = scan_exclusive(sums, sums, tiles, sums + tiles, s)) != JX_OK) break;
    } else if (total) {
      // one tile: its sum is the total
      if ((ce = cudaMemcpyAsync(sums + 1, sums, sizeof(int64_t), cudaMemcpyDeviceToDevice, s)) != cudaSuccess) {
        st = set_cuda_error(ce);
        break;
      }
    }
    if (total && (ce = cudaMemcpyAsync(total, sums + tiles, sizeof(int64_t), cudaMemcpyDeviceToDevice, s)) !=
                     cudaSuccess) {
      st = set_cuda_error(ce);
      break;
    }
    tile_scan_kernel<<<(unsigned)tiles, kBuildThreads, 0, s>>>(n, in, tiles > 1 ? sums : nullptr, out);
    st = check_launch();
  } while (0);
  cudaFreeAsync(sums, s);
  return st;
}

// ---------------------------------------------------------------- keys
__global__ void keys_kernel(int64_t m, int32_t n, const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
                            bool symmetrize, bool keep_self, uint64_t *__restrict__ keys,
                            uint32_t *__restrict__ bad) {
  const uint64_t sentinel = (uint64_t)n * (uint64_t)n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = src[i], v = dst[i];
    uint64_t a = sentinel, b = sentinel;
    if (u < 0 || u >= n || v < 0 || v >= n) {
      atomicOr(bad, 1u);
    } else if (u != v || keep_self) {
      a = (uint64_t)u * (uint64_t)n + (uint64_t)v;
      b = (uint64_t)v * (uint64_t)n + (uint64_t)u;
    }
    keys[i] = a;
    if (symmetrize) keys[m + i] = b;
  }
}

// ---------------------------------------------------------------- radix sort (8-bit digits)
__global__ void digit_hist_kernel(int64_t nk, const uint64_t *__restrict__ keys, int shift, int64_t ntiles,
                                  int64_t *__restrict__ counts) {
  __shared__ int32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t t0 = (int64_t)blockIdx.x * kTileKeys;
  for (int q = 0; q < kPerThread; ++q) {
    const int64_t i = t0 + (int64_t)q * kBuildThreads + threadIdx.x;
    if (i < nk) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x]; // digit-major
}

// Stable scatter of one tile: rounds of 256 keys in tile order; inside a round, warps rank
// their keys per digit with match_any, and the warps' counts are combined in warp order.
__global__ void digit_scatter_kernel(int64_t nk, const uint64_t *__restrict__ keys, int shift, int64_t ntiles,
                                     const int64_t *__restrict__ offs, uint64_t *__restrict__ out) {
  __shared__ int64_t base[256];
  __shared__ int32_t wc[kBuildThreads / 32][256];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  base[threadIdx.x] = offs[(int64_t)threadIdx.x * ntiles + blockIdx.x];
  const int64_t t0 = (int64_t)blockIdx.x * kTileKeys;
  for (int r = 0; r < kPerThread; ++r) {
    for (int k = threadIdx.x; k < (kBuildThreads / 32) * 256; k += kBuildThreads) (&wc[0][0])[k] = 0;
    __syncthreads();
    const int64_t i = t0 + (int64_t)r * kBuildThreads + threadIdx.x;
    const bool valid = i < nk;
    const uint64_t key = valid ? keys[i] : 0;
    const int d = valid ? (int)((key >> shift) & 255u) : 256 + lane; // invalid lanes match only themselves
    const unsigned peers = __match_any_sync(kFull, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wc[wid][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int32_t before = 0;
      for (int w = 0; w < wid; ++w) before += wc[w][d];
      out[base[d] + before + rank] = key;
    }
    __syncthreads();
    int32_t sum = 0;
    for (int w = 0; w < kBuildThreads / 32; ++w) sum += wc[w][threadIdx.x];
    base[threadIdx.x] += sum;
    __syncthreads();
  }
}

// ---------------------------------------------------------------- compaction and rows
__global__ void run_flags_kernel(int64_t nk, const uint64_t *__restrict__ keys, uint64_t sentinel,
                                 int64_t *__restrict__ flags) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    flags[i] = (k != sentinel && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
  }
}

__global__ void compact_kernel(int64_t nk, const uint64_t *__restrict__ keys, const int64_t *__restrict__ pos,
                               uint64_t sentinel, int32_t n, int32_t *__restrict__ col,
                               int64_t *__restrict__ row_count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    if (k != sentinel && (i == 0 || keys[i - 1] != k)) {
      col[pos[i]] = (int32_t)(k % (uint64_t)n);
      atomicAdd(reinterpret_cast<unsigned long long *>(row_count + k / (uint64_t)n), 1ull);
    }
  }
}

__global__ void to_int32_kernel(int64_t n, const int64_t *__restrict__ in, int32_t *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)in[i];
}

unsigned grid_of(int64_t work) {
  const int64_t g = (work + kBuildThreads - 1) / kBuildThreads;
  const int64_t cap = (int64_t)sm_count() * 16;
  return (unsigned)(g < 1 ? 1 : (g < cap ? g : cap));
}

} // namespace
} // namespace jx

using namespace jx;

extern "C" {

jx_status jx_csr_build(int32_t n, int64_t m, const int32_t *src, const int32_t *dst, uint32_t flags,
                       int32_t *row_ptr, int32_t *col, int64_t cap, int64_t *e_out, jx_stream_t stream) {
  if (n < 0 || m < 0 || !row_ptr || !e_out || cap < 0 || (m > 0 && (!src || !dst)) ||
      (flags & ~(uint32_t)(JX_BUILD_SYMMETRIZE | JX_BUILD_KEEP_SELF_LOOPS)))
    return JX_ERR_INVALID;
  if (n == 0 && m > 0) return JX_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce;
  *e_out = 0;
  if (n == 0) return JX_OK;
  const bool sym = (flags & JX_BUILD_SYMMETRIZE) != 0;
  const bool keep_self = (flags & JX_BUILD_KEEP_SELF_LOOPS) != 0;
  const int64_t nk = sym ? 2 * m : m;
  if (m == 0) { // no edges: every row empty
    ce = cudaMemsetAsync(row_ptr, 0, sizeof(int32_t) * ((size_t)n + 1), s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    return ce == cudaSuccess ? JX_OK : set_cuda_error(ce);
  }
  const uint64_t sentinel = (uint64_t)n * (uint64_t)n;
  int bits = 0;
  while (bits < 64 && (sentinel >> bits) != 0) ++bits;
  const int passes = (bits + 7) / 8;
  const int64_t ntiles = (nk + kTileKeys - 1) / kTileKeys;

  uint64_t *ka = nullptr, *kb = nullptr;
  int64_t *counts = nullptr, *pos = nullptr, *rows = nullptr, *dev_total = nullptr;
  uint32_t *bad = nullptr;
  jx_status st = JX_OK;
  auto release = [&]() {
    cudaFreeAsync(ka, s);
    cudaFreeAsync(kb, s);
    cudaFreeAsync(counts, s);
    cudaFreeAsync(pos, s);
    cudaFreeAsync(rows, s);
    cudaFreeAsync(dev_total, s);
    cudaFreeAsync(bad, s);
  };
  do {
    if ((ce = cudaMallocAsync(&ka, sizeof(uint64_t) * (size_t)nk, s)) != cudaSuccess ||
        (ce = cudaMallocAsync(&kb, sizeof(uint64_t) * (size_t)nk, s)) != cudaSuccess ||
        (ce = cudaMallocAsync(&counts, sizeof(int64_t) * 256 * (size_t)ntiles, s)) != cudaSuccess ||
        (ce = cudaMallocAsync(&pos, sizeof(int64_t) * (size_t)nk, s)) != cudaSuccess ||
        (ce = cudaMallocAsync(&rows, sizeof(int64_t) * ((size_t)n + 1), s)) != cudaSuccess ||
        (ce = cudaMallocAsync(&dev_total, sizeof(int64_t) * 2, s)) != cudaSuccess ||
        (ce = cudaMallocAsync(&bad, sizeof(uint32_t), s)) != cudaSuccess) {
      st = set_cuda_error(ce);
      break;
    }
    if ((ce = cudaMemsetAsync(bad, 0, sizeof(uint32_t), s)) != cudaSuccess) { st = set_cuda_error(ce); break; }
    keys_kernel<<<grid_of(m), kBuildThreads, 0, s>>>(m, n, src, dst, sym, keep_self, ka, bad);
    if ((st = check_launch()) != JX_OK) break;
    uint32_t h_bad = 0;
    if ((ce = cudaMemcpyAsync(&h_bad, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess) {
      st = set_cuda_error(ce);
      break;
    }
    if (h_bad) { st = JX_ERR_INVALID; break; } // a vertex id outside [0, n)
    for (int p = 0; p < passes && st == JX_OK; ++p) {
      digit_hist_kernel<<<(unsigned)ntiles, kBuildThreads, 0, s>>>(nk, ka, 8 * p, ntiles, counts);
      if ((st = check_launch()) != JX_OK) break;
      if ((st = scan_exclusive(counts, counts, 256 * ntiles, nullptr, s)) != JX_OK) break;
      digit_scatter_kernel<<<(unsigned)ntiles, kBuildThreads, 0, s>>>(nk, ka, 8 * p, ntiles, counts, kb);
      if ((st = check_launch()) != JX_OK) break;
      std::swap(ka, kb);
    }
    if (st != JX_OK) break;
    run_flags_kernel<<<grid_of(nk), kBuildThreads, 0, s>>>(nk, ka, sentinel, pos);
    if ((st = check_launch()) != JX_OK) break;
    if ((st = scan_exclusive(pos, pos, nk, dev_total, s)) != JX_OK) break;
    int64_t e = 0;
    if ((ce = cudaMemcpyAsync(&e, dev_total, sizeof(int64_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess) {
      st = set_cuda_error(ce);
      break;
    }
    *e_out = e;
    if (e > INT32_MAX || e > cap || (e > 0 && !col)) { st = JX_ERR_TOO_LARGE; break; }
    if ((ce = cudaMemsetAsync(rows, 0, sizeof(int64_t) * ((size_t)n + 1), s)) != cudaSuccess) {
      st = set_cuda_error(ce);
      break;
    }
    compact_kernel<<<grid_of(nk), kBuildThreads, 0, s>>>(nk, ka, pos, sentinel, n, col, rows);
    if ((st = check_launch()) != JX_OK) break;
    if ((st = scan_exclusive(rows, rows, (int64_t)n + 1, nullptr, s)) != JX_OK) break;
    to_int32_kernel<<<grid_of((int64_t)n + 1), kBuildThreads, 0, s>>>((int64_t)n + 1, rows, row_ptr);
    if ((st = check_launch()) != JX_OK) break;
  } while (0);
  release();
  ce = cudaStreamSynchronize(s);
  if (st == JX_OK && ce != cudaSuccess) st = set_cuda_error(ce);
  return st;
}

} // extern "C"
