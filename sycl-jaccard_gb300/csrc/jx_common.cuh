// Shared device helpers and host plumbing for the jx engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/jx.h"

namespace jx {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarp = 32;
// Reference launch constants (standalone_csr.hpp:27-28): kept only where a stage kernel's
// result could depend on them; it never does here.
constexpr int kIsILanes = 8; // jaccard.cpp:409,414 (i-lanes of Jaccard_IsKernel)

// Marks an output slot not yet written by the fused kernel (a quiet NaN with a payload no
// CUDA arithmetic produces: GPU NaN results are always 0x7fffffff).
constexpr uint32_t kUnwritten = 0x7fc0deadu;

// -------------------------------------------------------------- host plumbing
jx_status set_cuda_error(cudaError_t e);
void count_launches(uint64_t k);
inline jx_status check_launch() {
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? JX_OK : set_cuda_error(e);
}
int sm_count();

// Optional per-launch timing (jx_profile_begin / jx_profile_end): when enabled on this
// thread, prof_mark records an event on `s` after a launch; durations are the gaps between
// consecutive marks.  A no-op when disabled.
void prof_mark(const char *name, cudaStream_t s);

// Weighted row sums (jx_rowsum) of the rows of at most max_len entries; longer rows are left to
// the caller.
jx_status rowsum_upto(int32_t n, const int32_t *row_ptr, const int32_t *ind, const float *w, float *work,
                      int32_t max_len, cudaStream_t s);

// -------------------------------------------------------------- device helpers

// Binary search of `key` in col[left .. right] (inclusive), jaccard.cpp:353-367.
__device__ __forceinline__ bool bsearch_found(const int32_t *__restrict__ col, int32_t left,
                                              int32_t right, int32_t key) {
  while (left <= right) {
    int32_t middle = (left + right) >> 1;
    int32_t c = __ldg(col + middle);
    if (c > key)
      right = middle - 1;
    else if (c < key)
      left = middle + 1;
    else
      return true;
  }
  return false;
}

// Lane 31's value of a 32-wide inclusive Hillis-Steele scan (jaccard.cpp:101-117).  For the
// last lane the scan is a balanced pairwise tree, which the xor butterfly reproduces
// operation for operation (float addition is commutative).
__device__ __forceinline__ float warp_tree_sum(float x) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) x += __shfl_xor_sync(kFull, x, o);
  return x;
}

// Fibonacci hashing into a table of 2^(32 - shift) slots.
__device__ __forceinline__ uint32_t hash_slot(int32_t key, int shift) {
  return ((uint32_t)key * 0x9E3779B1u) >> shift;
}

// Fold the values of the lanes set in `mask` into acc in ascending lane order:
// acc = val[b] + acc for each set bit b (the reference's atomic add computes val + old,
// jaccard.cpp:196).  Every lane returns the same acc.
__device__ __forceinline__ float warp_ordered_fold(unsigned mask, float val, float acc) {
  while (mask) {
    const int b = __ffs(mask) - 1;
    acc = __shfl_sync(kFull, val, b) + acc;
    mask &= mask - 1;
  }
  return acc;
}

} // namespace jx
