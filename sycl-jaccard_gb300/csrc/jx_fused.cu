// Fused Jaccard operator: intersection and weight in one pass, J written once per edge, no
// atomics on results.  Drop-in for sygraph::jaccard<edge_centric> (jaccard.cpp:926-955).
//
// Work decomposition ("tasks").  An intersection is computed by staging the longer list
// N(u) as a membership structure and streaming the shorter list N(v) through it.  Row u
// owns a task for every neighbour v with d_v <= d_u; v's list is the "ref" list, the one the
// reference walks element by element.  The reference picks the ref list per directed edge
// (VC: jaccard.cpp:333-336, EC: jaccard.cpp:716-719), so one task serves two directed edges:
//   VC: (u,v) always (ref = v when d_u >= d_v);      (v,u) when d_v < d_u
//   EC: (u,v) when d_v < d_u;                         (v,u) always (ref = v when d_v <= d_u)
// The reverse edge (v,u) is found for free: it is the position of u inside N(v), which the
// task streams anyway.  Its result is bit-identical: same ref list, same cur set, and a
// commutative S_u + S_v.  Edges no task covers (graphs that are not symmetric, repeated
// neighbours) keep a sentinel and are computed by the fix-up pass.
//
// Bins by d_u (the staged list), each row list sorted by degree, largest first:
//   B0  d_u <= 32      one warp per row, one lane per task, 64-slot hash per warp
//   B1  d_u <= 512     one warp per row, cuckoo hash of <= 1280 slots per warp (shared)
//   B2  d_u <= 24576   one 1024-thread CTA per row, cuckoo hash of <= 58000 slots (227 KB)
//   hub d_u >  24576   4-CTA clusters; N(u) as a bitmap over [0, n) in global memory (L2)
//
// Streaming: a warp reads the ref list in 256-element chunks, lane k holding positions
// k + 32j (j = 0..7): eight independent coalesced loads in flight per lane.
//
// Weighted sums follow the reference's accumulation order exactly.  On a CPU SYCL device its
// 8 i-lanes add their matches one lane after another (jaccard.cpp:343, 370-396): ref
// positions 0, 8, 16, ..., then 1, 9, 17, ..., i.e. "class" c = position mod 8 major,
// position minor.  While streaming, the matches' weights of each class are appended to
// per-warp class streams (shared memory for B1, global scratch otherwise); after the list
// ends the warp adds them up class by class.  A class that outgrows its stream resumes with a
// strided walk over its remaining positions (same order).
#include "jx_common.cuh"
#include "jx_plan.h"

#include <cooperative_groups.h>
#include <cuda.h>

#include <algorithm>
#include <mutex>
#include <vector>

namespace cg = cooperative_groups;

namespace jx {

constexpr int32_t kB0Max = 32, kB1Max = 512, kB2Max = 24576;
constexpr int kB0Slots = 64;
constexpr int kB1Slots = 1280;   // cuckoo, 2.5 slots per element at d = 512
constexpr int kB2Slots = 58000;  // cuckoo, <= 227 KB; load factor <= 0.424 at d = kB2Max
constexpr int kB2FoldWords = (1024 / 32) * 128; // fold buffers of the 32 warps of a B2 CTA
constexpr int kCuckooMaxEvict = 64;
constexpr int kCuckooSeeds = 4;
constexpr int kB2Threads = 1024;
constexpr int kRowThreads = 256;
constexpr int kHubThreads = 1024;
constexpr int kCluster = 4; // CTAs per hub cluster by default (R-MAT 24 weighted hub kernel: 4 -> 153 ms, 8 -> 189 ms)
constexpr int32_t kEmpty = -1;
constexpr int kChunk = 256;
constexpr int kB1Cap = kB1Max / 8;   // class-stream capacity per class, B1 (exact bound)
constexpr int kCap = (kB2Max + 7) / 8; // class-stream capacity per class, B2 (no overflow)
constexpr int kHubCap = 8192;          // class-stream capacity per class, hubs (overflow resumes)
constexpr int kKeys = 128;           // plan sort keys: 4 bins x 32 log2 buckets
constexpr unsigned kClass0 = 0x01010101u;

// Counters in the workspace (int32).
enum {
  kCntKeys = 0,                // [0, 128)   per-key counts, then cursors
  kOffKeys = kKeys,            // [128, 257) key offsets (exclusive scan, 129 entries)
  kCtrB2 = 2 * kKeys + 8,      // work counter, B2 rows
  kCtrHub,                     // work counter, hub units
  kNumHubUnits,                // number of hub units
  kCtrB1,                      // work counter, B1 rows (persistent kernel)
  kCtrB0,                      // work counter, B0 rows (persistent kernel)
  kHubUnitSize,                // tasks per hub work unit of this call
  kCtrIsolated,                // vertices without neighbours placed after the plan's rows (relabel)
  kCounters = 2 * kKeys + 32
};

// ---------------------------------------------------------------- membership probes
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

// Open-addressing hash set of N(u) in shared memory (load factor <= 1/2: every probe loop
// ends at an empty slot).
struct HashProbe {
  const int32_t *t;
  uint32_t size;
  __device__ __forceinline__ bool operator()(int32_t key) const {
    uint32_t s = hslot(key, size);
    for (;;) {
      const int32_t k = t[s];
      if (k == key) return true;
      if (k == kEmpty) return false;
      if (++s == size) s = 0;
    }
  }
};

// Two-choice cuckoo hash set of N(u) in shared memory: table halves [0, m) and [m, 2m), a key
// lives at h1(key) or at m + h2(key).  A lookup is two independent loads and no branch, so all
// lanes of a warp stay converged (linear probing made lanes wait on each other's collision
// chains).  Inserts run in parallel with atomicExch and a bounded eviction walk; a failed
// build (an eviction cycle) is retried with other multipliers.  (Reading h2 only when h1 holds
// another key -- an empty h1 proves absence, since slots are never emptied -- saves
// shared-memory wavefronts but makes the second load wait for the first: R-MAT 24 weighted CTA
// rows 562 ms against 439 ms with both loads; not used.)
struct CuckooProbe {
  const int32_t *t;
  uint32_t m, a1, a2;
  __device__ __forceinline__ uint32_t h1(int32_t k) const { return __umulhi((uint32_t)k * a1, m); }
  __device__ __forceinline__ uint32_t h2(int32_t k) const { return m + __umulhi((uint32_t)k * a2, m); }
  __device__ __forceinline__ bool operator()(int32_t key) const {
    const int32_t k1 = t[h1(key)], k2 = t[h2(key)];
    return (k1 == key) | (k2 == key);
  }
};

// The cuckoo set with the weight of each key beside it (wt[s] = w[t[s]] for every filled slot
// s, in shared memory): a weighted lookup returns a match's weight without a global gather.
struct CuckooWProbe {
  CuckooProbe c;
  const float *wt;
  __device__ __forceinline__ bool operator()(int32_t key) const { return c(key); }
  __device__ __forceinline__ bool lookup(int32_t key, float &v) const {
    const uint32_t s1 = c.h1(key), s2 = c.h2(key);
    const int32_t k1 = c.t[s1], k2 = c.t[s2];
    const bool f = (k1 == key) | (k2 == key);
    v = f ? wt[k1 == key ? s1 : s2] : 0.0f;
    return f;
  }
};
template <class P> struct HasWeights { static constexpr bool value = false; };
template <> struct HasWeights<CuckooWProbe> { static constexpr bool value = true; };

// Odd multipliers for attempt `seed` (xor with an even number keeps them odd).
__device__ __forceinline__ CuckooProbe cuckoo_params(const int32_t *t, uint32_t slots, int seed) {
  return CuckooProbe{t, slots / 2, 0x9E3779B1u ^ ((uint32_t)seed * 0x6A09E668u),
                     0x85EBCA77u ^ ((uint32_t)seed * 0xBB67AE86u)};
}

// Inserts `key`; false when the eviction walk gave up (the table then misses a key).
__device__ __forceinline__ bool cuckoo_insert(const CuckooProbe &c, int32_t *t, int32_t key) {
  uint32_t loc = c.h1(key);
  for (int it = 0; it < kCuckooMaxEvict; ++it) {
    const int32_t old = atomicExch(t + loc, key);
    if (old == kEmpty || old == key) return true;
    key = old;
    const uint32_t l1 = c.h1(key);
    loc = (loc == l1) ? c.h2(key) : l1;
  }
  return false;
}

// Bitmap of N(u) over [0, n) in global memory, rebuilt per hub: read through L2 only
// (ld.global.cg), never from a possibly stale L1 line.
struct BitmapProbe {
  const uint32_t *bm;
  __device__ __forceinline__ bool operator()(int32_t key) const {
    return (__ldcg(bm + (key >> 5)) >> (key & 31)) & 1u;
  }
};

// A hub's neighbour set through a one-hash bit filter of it in shared memory first: most
// non-members are turned away on chip, and only the rest read the exact bitmap in L2.
// Filter words per hub CTA (dynamic shared memory).  Measured on R-MAT 24: the unweighted hub
// kernel drops from 93 to 76 ms with 96 or 192 KB; the weighted one is slower with any filter
// (32 / 64 / 192 KB: 197 / 196 / 238 ms against 189 ms without), so it keeps none.
constexpr uint32_t kHubFilterWordsU = 48 * 1024;
constexpr uint32_t kHubFilterWordsW = 0;
template <bool kWeighted> __host__ __device__ constexpr uint32_t hub_filter_words() { return kWeighted ? kHubFilterWordsW : kHubFilterWordsU; }
__device__ __forceinline__ uint32_t filter_bit(int32_t key, uint32_t bits) {
  return __umulhi((uint32_t)key * 0x9E3779B1u, bits);
}
struct FilterProbe {
  const uint32_t *filt; // shared memory, bits / 32 words
  const uint32_t *bm;   // global bitmap over [0, n)
  uint32_t bits;
  __device__ __forceinline__ bool operator()(int32_t key) const {
    const uint32_t h = filter_bit(key, bits);
    if (!((filt[h >> 5] >> (h & 31)) & 1u)) return false;
    return (__ldcg(bm + (key >> 5)) >> (key & 31)) & 1u;
  }
};

// Sorted cur list in global memory (fix-up path).
struct SearchProbe {
  const int32_t *col;
  int32_t lo, hi; // inclusive
  __device__ __forceinline__ bool operator()(int32_t key) const { return bsearch_found(col, lo, hi, key); }
};

// ---------------------------------------------------------------- class streams
// Per-warp class streams of a weighted task: class c's entries from base + c * cap, in
// ascending ref position.  An entry is the weight of a match (its bit pattern), gathered by
// vertex id when the match is found, so that the gather's latency overlaps the rest of the
// chunk and the fold reads the stream alone.  cap is a multiple of 4, so no int4 read leaves
// its class.
template <bool kGlobal, bool kExactCap = false> struct Streams {
  static constexpr bool kExact = kExactCap; // capacity holds every match: no overflow handling
  int32_t *base;
  int cap;
  float *fbuf = nullptr; // shared memory, 128 floats of this warp for the fold, or none
  __device__ __forceinline__ void put(int c, int pos, int32_t x) const {
    if (kGlobal) __stcg(base + c * cap + pos, x); else base[c * cap + pos] = x;
  }
  __device__ __forceinline__ int4 load4(const int32_t *p) const {
    if (kGlobal) return __ldcg(reinterpret_cast<const int4 *>(p));
    return *reinterpret_cast<const int4 *>(p);
  }
  // acc = v0 + acc, v1 + acc, ... over the first n entries of class c; acc uniform.
  __device__ __forceinline__ float fold(int c, int n, float acc) const {
    const int lane = threadIdx.x & 31;
    const int32_t *p = base + c * cap;
    int4 cur = make_int4(0, 0, 0, 0);
    if (4 * lane < n) cur = load4(p + 4 * lane);
    for (int t = 0; t < n; t += 128) {
      int4 nxt = make_int4(0, 0, 0, 0);
      if (t + 128 + 4 * lane < n) nxt = load4(p + t + 128 + 4 * lane);
      const int k = n - t < 128 ? n - t : 128;
      const int i0 = 4 * lane;
      const float va = i0 < k ? __int_as_float(cur.x) : 0.0f;
      const float vb = i0 + 1 < k ? __int_as_float(cur.y) : 0.0f;
      const float vc = i0 + 2 < k ? __int_as_float(cur.z) : 0.0f;
      const float vd = i0 + 3 < k ? __int_as_float(cur.w) : 0.0f;
#pragma unroll
      for (int L = 0; L < 32; ++L) {
        if (4 * L < k) {
          const float a = __shfl_sync(kFull, va, L), b = __shfl_sync(kFull, vb, L);
          const float q = __shfl_sync(kFull, vc, L), d = __shfl_sync(kFull, vd, L);
          acc = a + acc;
          if (4 * L + 1 < k) acc = b + acc;
          if (4 * L + 2 < k) acc = q + acc;
          if (4 * L + 3 < k) acc = d + acc;
        }
      }
      cur = nxt;
    }
    return acc;
  }
};
template <class S> struct kIsGlobal;
template <bool G, bool E> struct kIsGlobal<Streams<G, E>> { static constexpr bool value = G; };

// All classes at once when none overflowed.  The entries are taken in class-major order
// (class c starts at the prefix sum of the counts of classes < c) 128 per round: lane L holds
// entries 4L .. 4L+3 of the round; the entries of the next round are loaded before the
// current round is folded.  The warp then adds the 128 values in order: from a shared-memory copy
// (one broadcast 16-byte read per 4 values) when the warp has a fold buffer, else through
// shuffles with constant lane indices; values are added in whole groups of 4 (see below).
// counts: lane c (c < 8) holds class c's count, other lanes 0.  acc: +0.0 on entry.
//
// Entry i of class c sits at c * cap + (i - start[c]); with d[q] = cap - count[q - 1] that is
// i + the sum of d[q] over the classes q >= 1 that start at or before i.
template <class S>
__device__ __forceinline__ int32_t class_entry(const S &cls, const int32_t (&start)[8], const int32_t (&d)[8],
                                               int32_t i, int32_t total) {
  if (i >= total) return 0; // never used: the fold tests the index
  int32_t off = i;
#pragma unroll
  for (int q = 1; q < 8; ++q) off += i >= start[q] ? d[q] : 0;
  return kIsGlobal<S>::value ? __ldcg(cls.base + off) : cls.base[off];
}

template <class S>
__device__ __forceinline__ float fold_all(const S &cls, int32_t my_count, float acc) {
  const int lane = threadIdx.x & 31;
  int32_t incl = my_count;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const int32_t y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  const int32_t total = __shfl_sync(kFull, incl, 7);
  int32_t start[8], d[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) start[c] = __shfl_sync(kFull, incl - my_count, c);
  d[0] = 0;
#pragma unroll
  for (int q = 1; q < 8; ++q) d[q] = cls.cap - (start[q] - start[q - 1]);
  // Values past the total are +0.0 and are added in groups of 4 without tests: acc starts at
  // +0.0 and a round-to-nearest sum is -0.0 only when both addends are, so acc is never -0.0
  // and acc + 0.0 is acc bit for bit (a NaN acc is already the canonical NaN).
  if (total <= 32) { // one entry per lane, added in lane order from registers
    const float v = lane < total ? __int_as_float(class_entry(cls, start, d, lane, total)) : 0.0f;
    for (int32_t L = 0; L < total; L += 4) {
      const float a = __shfl_sync(kFull, v, L), b = __shfl_sync(kFull, v, L + 1);
      const float c = __shfl_sync(kFull, v, L + 2), e = __shfl_sync(kFull, v, L + 3);
      acc = a + acc;
      acc = b + acc;
      acc = c + acc;
      acc = e + acc;
    }
    return acc;
  }
  int32_t ent[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) ent[m] = class_entry(cls, start, d, 4 * lane + m, total);
  float4 *const buf = reinterpret_cast<float4 *>(cls.fbuf);
  for (int32_t t = 0; t < total; t += 128) {
    float v[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) v[m] = t + 4 * lane + m < total ? __int_as_float(ent[m]) : 0.0f;
    if (t + 128 < total) { // the next round's entries (most tasks have one round)
#pragma unroll
      for (int m = 0; m < 4; ++m) ent[m] = class_entry(cls, start, d, t + 128 + 4 * lane + m, total);
    }
    const int32_t k = total - t < 128 ? total - t : 128;
    if (buf) {
      __syncwarp(); // the previous round's reads are done
      buf[lane] = make_float4(v[0], v[1], v[2], v[3]);
      __syncwarp();
      if (k == 128) {
#pragma unroll
        for (int L = 0; L < 32; ++L) {
          const float4 q = buf[L];
          acc = q.x + acc;
          acc = q.y + acc;
          acc = q.z + acc;
          acc = q.w + acc;
        }
      } else {
        for (int L = 0; 4 * L < k; ++L) {
          const float4 q = buf[L];
          acc = q.x + acc;
          acc = q.y + acc;
          acc = q.z + acc;
          acc = q.w + acc;
        }
      }
    } else if (k == 128) {
#pragma unroll
      for (int L = 0; L < 32; ++L) {
        const float a = __shfl_sync(kFull, v[0], L), b = __shfl_sync(kFull, v[1], L);
        const float c = __shfl_sync(kFull, v[2], L), e = __shfl_sync(kFull, v[3], L);
        acc = a + acc;
        acc = b + acc;
        acc = c + acc;
        acc = e + acc;
      }
    } else {
#pragma unroll
      for (int L = 0; L < 32; ++L) {
        if (4 * L < k) {
          const float a = __shfl_sync(kFull, v[0], L), b = __shfl_sync(kFull, v[1], L);
          const float c = __shfl_sync(kFull, v[2], L), e = __shfl_sync(kFull, v[3], L);
          acc = a + acc;
          acc = b + acc;
          acc = c + acc;
          acc = e + acc;
        }
      }
    }
  }
  if (buf) __syncwarp();
  return acc;
}

using ClassStreams = Streams<true>;
using SmemClassStreams = Streams<false, true>; // warp-per-row kernel: capacity kB1Max / 8 is exact

// ---------------------------------------------------------------- one task, one warp
// Class-major strided walk (the reference's order with no buffering); used for overflowing
// weighted tasks and by the fix-up pass.
template <bool kWeighted, class Probe>
__device__ __forceinline__ float task_strided(const Probe &probe, const int32_t *__restrict__ col,
                                              const float *__restrict__ w, int32_t u, int32_t vs,
                                              int32_t dv, int32_t &mirror) {
  const int lane = threadIdx.x & 31;
  mirror = -1;
  float acc = 0.0f;
  for (int il = 0; il < kIsILanes; ++il) {
    const int32_t cntc = dv > il ? (dv - il + kIsILanes - 1) / kIsILanes : 0;
    for (int32_t m0 = 0; m0 < cntc; m0 += 32) {
      const int32_t m = m0 + lane;
      int32_t x = kEmpty;
      bool found = false;
      float val = 1.0f;
      if (m < cntc) {
        x = __ldg(col + vs + il + kIsILanes * m);
        found = probe(x);
        if (kWeighted && found) val = __ldg(w + x);
      }
      acc = warp_ordered_fold(__ballot_sync(kFull, found), val, acc);
      const unsigned mb = __ballot_sync(kFull, x == u && x != kEmpty);
      if (mb) mirror = (mirror == -1 && __popc(mb) == 1) ? il + kIsILanes * (m0 + __ffs(mb) - 1) : -2;
    }
  }
  return acc;
}

// The remaining positions of class c, from p0 (p0 = c mod 8) to the end of the ref list,
// folded in order onto acc (uniform across the warp): the tail of an overflowing class.
template <class Probe>
__device__ __forceinline__ float class_tail(const Probe &probe, const int32_t *__restrict__ col,
                                            const float *__restrict__ w, int32_t vs, int32_t dv,
                                            int32_t p0, float acc) {
  const int lane = threadIdx.x & 31;
  for (int32_t q = p0; q < dv; q += 32 * kIsILanes) {
    const int32_t p = q + kIsILanes * lane;
    bool found = false;
    float val = 0.0f;
    if (p < dv) {
      const int32_t x = __ldg(col + vs + p);
      found = probe(x);
      if (found) val = __ldg(w + x);
    }
    acc = warp_ordered_fold(__ballot_sync(kFull, found), val, acc);
  }
  return acc;
}

// One 256-element chunk at `base`: lane k takes positions base + k + 32j.  kTail: the chunk
// may run past the end of the list (bounds checks; padding lanes probe vertex 0, always a
// valid key, and drop the answer).
template <bool kWeighted, bool kTail, class Probe, class Streams>
__device__ __forceinline__ void task_chunk(const Probe &probe, const int32_t *__restrict__ col,
                                           const float *__restrict__ w, int32_t u, int32_t vs,
                                           int32_t dv, int32_t base, const Streams &cls, int32_t &cnt,
                                           int32_t &upos, int32_t &ccount, int32_t &lastp) {
  const int lane = threadIdx.x & 31;
  // weighted probes that carry the weights: the lookup returns a match's weight
  constexpr bool kW = kWeighted && HasWeights<Probe>::value;
  int32_t x[8];
  bool f[8];
  float wv[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int32_t p = base + lane + 32 * j;
    x[j] = (!kTail || p < dv) ? __ldg(col + vs + p) : kEmpty;
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    wv[j] = 0.0f;
    if (kTail) {
      // rows of the tail past the end of the list (warp-uniform test) probe nothing
      f[j] = false;
      if (base + 32 * j < dv) {
        const int32_t key = x[j] != kEmpty ? x[j] : 0;
        bool hit;
        if constexpr (kW) hit = probe.lookup(key, wv[j]); else hit = probe(key);
        f[j] = (x[j] != kEmpty) & hit;
      }
    } else {
      if constexpr (kW) f[j] = probe.lookup(x[j], wv[j]); else f[j] = probe(x[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (x[j] == u) upos = base + lane + 32 * j;
  if (!kWeighted) {
#pragma unroll
    for (int j = 0; j < 8; ++j) cnt += f[j];
  } else {
    // the matches' weights (from the probe, or gathered before the ballots so that the loads
    // overlap them)
    int32_t val[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) val[j] = f[j] ? __float_as_int(kW ? wv[j] : __ldg(w + x[j])) : 0;
    // position base + lane + 32j has class (lane & 7); within a class, ascending positions
    // are j-major, lane-minor: the order of these ballots.
    const unsigned lt = (1u << lane) - 1u;
    const int my_class = lane & 7;
    const unsigned my_cmask = kClass0 << my_class;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const unsigned m = __ballot_sync(kFull, f[j]);
      if (f[j]) {
        const int32_t pos = ccount + __popc(m & my_cmask & lt);
        if (Streams::kExact || pos < cls.cap) {
          cls.put(my_class, pos, val[j]);
          if (!Streams::kExact) lastp = base + lane + 32 * j;
        }
      }
      ccount += __popc(m & my_cmask);
    }
  }
}

// Weighted task whose list fits one warp row (dv <= 32): lane k holds position k, gathers its
// weight when it matches, and the warp adds the matches class by class (lanes c, c+8, c+16,
// c+24 for class c: the reference's order) straight from registers -- no class streams.
template <class Probe>
__device__ __forceinline__ float task_tiny_weighted(const Probe &probe, const int32_t *__restrict__ col,
                                                    const float *__restrict__ w, int32_t u, int32_t vs,
                                                    int32_t dv, int32_t &mirror) {
  const int lane = threadIdx.x & 31;
  const bool in = lane < dv;
  const int32_t x = in ? __ldg(col + vs + lane) : 0; // lanes past the list probe vertex 0, a valid key
  const bool f = probe(x) && in;
  const float val = f ? __ldg(w + x) : 0.0f;
  const unsigned m = __ballot_sync(kFull, f);
  mirror = __reduce_max_sync(kFull, (in && x == u) ? lane : -1);
  float acc = 0.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c) acc = warp_ordered_fold(m & (kClass0 << c), val, acc);
  return acc;
}

// Chunked stream of N(v) = col[vs, vs+dv) through `probe`.  Returns the intersection value in
// the reference's order (count when unweighted) and a position of u in N(v) in `mirror`
// (-1 absent).  Counts and the position of u are kept per lane and reduced once per task.
template <bool kWeighted, class Probe, class Streams>
__device__ __forceinline__ float task_stream(const Probe &probe, const int32_t *__restrict__ col,
                                             const float *__restrict__ w, int32_t u, int32_t vs,
                                             int32_t dv, int32_t &mirror, const Streams &cls) {
  if (kWeighted && dv <= 32) return task_tiny_weighted(probe, col, w, u, vs, dv, mirror);
  const int lane = threadIdx.x & 31;
  const int my_class = lane & 7;
  int32_t cnt = 0, upos = -1;
  int32_t ccount = 0; // matches so far in this lane's class (same value in all lanes of a class)
  int32_t lastp = -1; // ref position of the last value this lane stored
  int32_t base = 0;
  for (; base + kChunk <= dv; base += kChunk)
    task_chunk<kWeighted, false>(probe, col, w, u, vs, dv, base, cls, cnt, upos, ccount, lastp);
  if (base < dv)
    task_chunk<kWeighted, true>(probe, col, w, u, vs, dv, base, cls, cnt, upos, ccount, lastp);
  // Position of u in N(v).  If u occurs more than once (a repeated neighbour), the task's
  // value is right for every occurrence; the one written here is the last, the others keep
  // the sentinel and the fix-up pass computes them.
  mirror = __reduce_max_sync(kFull, upos);
  if (!kWeighted) return (float)__reduce_add_sync(kFull, cnt);
  __syncwarp();
  float acc = 0.0f;
  if (Streams::kExact || !__any_sync(kFull, ccount > cls.cap)) {
    acc = fold_all(cls, lane < 8 ? ccount : 0, acc);
    __syncwarp();
    return acc;
  }
  for (int c = 0; c < 8; ++c) {
    const int32_t nc = __shfl_sync(kFull, ccount, c);
    acc = cls.fold(c, nc < cls.cap ? nc : cls.cap, acc);
    if (nc > cls.cap) { // resume class c after its last stored value
      const int32_t lp = __reduce_max_sync(kFull, my_class == c ? lastp : -1);
      acc = class_tail(probe, col, w, vs, dv, lp + kIsILanes, acc);
    }
  }
  __syncwarp();
  return acc;
}

// J for a task and the directed edges it serves (see the header comment).
template <bool kEC, bool kWeighted>
__device__ __forceinline__ void write_task(float I, int32_t du, int32_t dv, float Su, float Sv,
                                           int64_t e_uv, int64_t e_vu, float *__restrict__ out) {
  float J;
  if (kEC) {
    J = I / ((float)(dv + du) - I); // jaccard.cpp:741 with Ni = d_v (csrInd[tid]), Nj = d_u
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

// ---------------------------------------------------------------- plan: degree-sorted rows
// Degree bins of one call (a plan's choice, at most the limits of the header comment) and the
// hub kernel's work split.
// Where each vertex's list lies in col: [start(v), end(v)).  For a call on the graph's own ids
// these are the CSR offsets (start = row_ptr, end = row_ptr + 1); for a call on relabelled ids
// (see relabel in run_fused) they are arrays by new id, the lists staying where they are.
struct Rows {
  const int32_t *start, *end;
  __device__ __forceinline__ int32_t s(int32_t v) const { return __ldg(start + v); }
  __device__ __forceinline__ int32_t e(int32_t v) const { return __ldg(end + v); }
};

struct Bins {
  int32_t b0_max, b1_max, b2_max; // lane rows d <= b0_max, warp rows <= b1_max, CTA rows <= b2_max
  int32_t hub_unit;               // tasks per hub work unit at most (hub_units_kernel may use fewer)
  int32_t hub_batch;              // tasks a hub warp takes per fetch
};

// Sort key = bin * 32 + (31 - ceil(log2 d)): hubs, then B2, B1, B0, each largest first.
__device__ __forceinline__ int plan_key(int32_t d, const Bins &b) {
  const int bin = d > b.b2_max ? 0 : (d > b.b1_max ? 1 : (d > b.b0_max ? 2 : 3));
  const int lg = d <= 1 ? 0 : 32 - __clz(d - 1);
  return bin * 32 + (31 - lg);
}

template <bool kScatter>
__global__ void plan_kernel(int32_t n, Rows rp, int32_t *__restrict__ cnt, int32_t *__restrict__ rows,
                            Bins bins) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = base + threadIdx.x;
    int key = -1;
    if (u < n) {
      const int32_t d = rp.e((int32_t)u) - rp.s((int32_t)u);
      if (d > 0) key = plan_key(d, bins);
    }
    const unsigned peers = __match_any_sync(kFull, key);
    if (key >= 0) {
      const int leader = __ffs(peers) - 1;
      int32_t b = 0;
      if (lane == leader) b = atomicAdd(cnt + kCntKeys + key, __popc(peers));
      b = __shfl_sync(peers, b, leader);
      if (kScatter) rows[cnt[kOffKeys + key] + b + __popc(peers & ((1u << lane) - 1u))] = (int32_t)u;
    }
  }
}

// Exclusive scan of the key counts; resets the counts to serve as scatter cursors.
__global__ void plan_offsets_kernel(int32_t *__restrict__ cnt) {
  __shared__ int32_t s[kKeys];
  const int t = threadIdx.x;
  s[t] = cnt[kCntKeys + t];
  __syncthreads();
  if (t == 0) {
    int32_t run = 0;
    for (int k = 0; k < kKeys; ++k) {
      cnt[kOffKeys + k] = run;
      run += s[k];
    }
    cnt[kOffKeys + kKeys] = run;
  }
  cnt[kCntKeys + t] = 0;
}

// Hub work units: a hub row with d tasks gives ceil(d / unit) units.  unit = hub_unit, or less
// when the hubs hold fewer than kHubUnitsPerCluster units of hub_unit tasks per cluster, so that
// every cluster gets work (not below kHubUnitMin).  Measured: R-MAT 20 weighted has 21 hubs
// (617,517 tasks), one unit each at 65536 -- 21 of 36 clusters busy; its hub kernel took 4.2 ms
// against 2.8 ms with 15 clusters of 8.  R-MAT 24 (21.0M hub tasks) keeps units of 65536.
constexpr int32_t kHubUnitsPerCluster = 4;
constexpr int32_t kHubUnitMin = 4096;
__global__ void hub_units_kernel(Rows rp, const int32_t *__restrict__ rows, int32_t *__restrict__ cnt,
                                 int32_t *__restrict__ unit_off, int32_t hub_unit, int32_t clusters) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int32_t h0 = cnt[kOffKeys + 0], h1 = cnt[kOffKeys + 32];
  int64_t tasks = 0;
  for (int32_t i = h0; i < h1; ++i) tasks += rp.e(rows[i]) - rp.s(rows[i]);
  const int64_t want = (int64_t)kHubUnitsPerCluster * (clusters > 0 ? clusters : 1);
  const int64_t fit = (tasks + want - 1) / want;
  const int64_t floor_unit = hub_unit < kHubUnitMin ? hub_unit : kHubUnitMin;
  const int64_t cap_unit = fit < hub_unit ? fit : hub_unit;
  const int32_t unit = (int32_t)(cap_unit > floor_unit ? cap_unit : floor_unit);
  int32_t run = 0;
  for (int32_t i = h0; i < h1; ++i) {
    unit_off[i - h0] = run;
    const int32_t u = rows[i];
    const int32_t d = rp.e(u) - rp.s(u);
    run += (d + unit - 1) / unit;
  }
  unit_off[h1 - h0] = run;
  cnt[kNumHubUnits] = run;
  cnt[kHubUnitSize] = unit;
}

__global__ void fill_bits_kernel(int64_t n, uint32_t *__restrict__ x, uint32_t bits) {
  const int64_t n4 = (reinterpret_cast<uintptr_t>(x) & 15u) ? 0 : n >> 2; // vector stores need 16 B alignment
  uint4 *x4 = reinterpret_cast<uint4 *>(x);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x)
    x4[i] = make_uint4(bits, bits, bits, bits);
  for (int64_t i = (n4 << 2) + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = bits;
}

// ---------------------------------------------------------------- relabelling
// A call can run on relabelled vertex ids (schedule field `relabel`): new id i = position of
// the vertex in the plan's row list (hubs first, then each bin by descending log2 degree,
// vertices without neighbours last), every list staying where it is in col with its entries
// mapped to new ids in the same order.  Results do not change -- membership, list positions
// and degrees are the same -- but the vertices that appear in most lists (the high-degree ones)
// get the smallest ids, so their weights, row sums, offsets and hub-bitmap words share fewer
// cache lines whatever the input's numbering.  Measured on R-MAT 24 weighted: 689 ms against
// 744 ms when the input's ids are a random bijection, but 660 against 615 ms on R-MAT's own ids,
// which already put high degrees first and keep neighbours' ids close; the plan's order within a
// bucket is not the ids' order, and the lists stay where they are.  Off by default.

// Vertices without neighbours, after the plan's R rows: rows[R .. n).
__global__ void relabel_isolated_kernel(int32_t n, const int32_t *__restrict__ row_ptr, int32_t *__restrict__ cnt,
                                        int32_t *__restrict__ rows) {
  const int lane = threadIdx.x & 31;
  const int32_t R = cnt[kOffKeys + kKeys];
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = base + threadIdx.x;
    const bool iso = u < n && __ldg(row_ptr + u + 1) == __ldg(row_ptr + u);
    const unsigned m = __ballot_sync(kFull, iso);
    if (!m) continue;
    int32_t b = 0;
    if (lane == __ffs(m) - 1) b = atomicAdd(cnt + kCtrIsolated, __popc(m));
    b = __shfl_sync(kFull, b, __ffs(m) - 1);
    if (iso) rows[R + b + __popc(m & ((1u << lane) - 1u))] = (int32_t)u;
  }
}

// perm[old] = new; the new ids' list bounds, weights and row sums.
__global__ void relabel_build_kernel(int32_t n, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ rows,
                                     const float *__restrict__ w, const float *__restrict__ S,
                                     int32_t *__restrict__ perm, int32_t *__restrict__ start2,
                                     int32_t *__restrict__ end2, float *__restrict__ w2, float *__restrict__ S2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = rows[i];
    perm[u] = (int32_t)i;
    start2[i] = __ldg(row_ptr + u);
    end2[i] = __ldg(row_ptr + u + 1);
    if (w2) {
      w2[i] = __ldg(w + u);
      S2[i] = __ldg(S + u);
    }
  }
}

// col2[k] = perm[col[k]]: every list entry as a new id, in place.
__global__ void relabel_col_kernel(int64_t e, const int32_t *__restrict__ col, const int32_t *__restrict__ perm,
                                   int32_t *__restrict__ col2) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < e; k += (int64_t)gridDim.x * blockDim.x)
    col2[k] = __ldg(perm + __ldg(col + k));
}

// ---------------------------------------------------------------- row sums of long rows
// Row sums of the rows of more than kB1Max entries, which the row-sum kernel leaves out, taken
// from the plan's row lists so that no warp walks several long rows in a row.  The reference's
// order for a row is T = tree(chunk k) + T over its 32-entry chunks in order
// (jaccard.cpp:101-119, the tree being lane 31's scan value).  Hub rows (> kB2Max): one CTA
// per row; the warps reduce the chunks' trees in parallel, 8 chunks per warp at a time, into
// shared memory, and thread 0 adds the chunk totals in order, kRsSeg chunks per pass.  CTA-bin
// rows: one warp per row, 8 chunks at a time (independent loads and trees, serial carry).
constexpr int kRsSeg = 8192;
__global__ void __launch_bounds__(1024) rowsum_long_kernel(const int32_t *__restrict__ row_ptr,
                                                           const int32_t *__restrict__ col,
                                                           const float *__restrict__ w,
                                                           const int32_t *__restrict__ rows,
                                                           const int32_t *__restrict__ cnt, float *__restrict__ S) {
  __shared__ float tot[kRsSeg];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int32_t h0 = cnt[kOffKeys + 0], h1 = cnt[kOffKeys + 32], b2_end = cnt[kOffKeys + 64];
  for (int32_t i = h0 + blockIdx.x; i < h1; i += gridDim.x) {
    const int32_t u = rows[i];
    const int64_t us = __ldg(row_ptr + u);
    const int64_t du = __ldg(row_ptr + u + 1) - us;
    const int64_t nch = (du + 31) / 32;
    float T = 0.0f;
    for (int64_t c0 = 0; c0 < nch; c0 += kRsSeg) {
      const int nseg = (int)(nch - c0 < kRsSeg ? nch - c0 : kRsSeg);
      for (int k = wid * 8; k < nseg; k += (1024 / 32) * 8) {
        float x[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int64_t p = (c0 + k + c) * 32 + lane;
          x[c] = (k + c < nseg && p < du) ? __ldg(w + __ldg(col + us + p)) : 0.0f;
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = warp_tree_sum(x[c]);
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (lane == c && k + c < nseg) tot[k + c] = x[c];
      }
      __syncthreads();
      if (threadIdx.x == 0)
        for (int k = 0; k < nseg; ++k) T = tot[k] + T;
      __syncthreads();
    }
    if (threadIdx.x == 0) S[u] = T;
  }
  for (int64_t i = h1 + (int64_t)blockIdx.x * (1024 / 32) + wid; i < b2_end; i += (int64_t)gridDim.x * (1024 / 32)) {
    const int32_t u = rows[i];
    const int32_t us = __ldg(row_ptr + u), du = __ldg(row_ptr + u + 1) - us;
    float T = 0.0f;
    for (int32_t i0 = 0; i0 < du; i0 += 8 * 32) {
      float x[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int32_t p = i0 + 32 * c + lane; // du <= kB2Max (CTA-bin rows): no overflow
        x[c] = p < du ? __ldg(w + __ldg(col + us + p)) : 0.0f;
      }
#pragma unroll
      for (int c = 0; c < 8; ++c) x[c] = warp_tree_sum(x[c]);
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (i0 + 32 * c < du) T = x[c] + T; // chunks of the row only
    }
    if (lane == 0) S[u] = T;
  }
}

// ---------------------------------------------------------------- B0: lane per task
// Row u (du <= 32): its neighbours in a 64-slot hash set `t` (this warp's), then lane k runs the
// task of neighbour k alone.
template <bool kEC, bool kWeighted>
__device__ __forceinline__ void lane_row(int32_t *t, int32_t u, Rows rp, const int32_t *__restrict__ col,
                                         const float *__restrict__ w, const float *__restrict__ S,
                                         float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int32_t us = rp.s(u), du = rp.e(u) - us;
  const uint32_t size = 2u * kB0Max;
  t[lane] = kEmpty;
  t[lane + 32] = kEmpty;
  __syncwarp();
  if (lane < du) hset_insert(t, size, __ldg(col + us + lane));
  __syncwarp();
  if (lane < du) {
    const HashProbe probe{t, size};
    const int32_t v = __ldg(col + us + lane);
    const int32_t vs = rp.s(v), dv = rp.e(v) - vs;
    if (dv <= du) {
      int32_t mirror = -1;
      float I;
      if (!kWeighted) {
        int32_t c = 0;
        for (int32_t p = 0; p < dv; ++p) {
          const int32_t x = __ldg(col + vs + p);
          c += probe(x);
          if (x == u) mirror = mirror == -1 ? p : -2;
        }
        I = (float)c;
      } else {
        float acc = 0.0f;
        for (int il = 0; il < kIsILanes; ++il)
          for (int32_t p = il; p < dv; p += kIsILanes) {
            const int32_t x = __ldg(col + vs + p);
            if (probe(x)) acc = __ldg(w + x) + acc;
            if (x == u) mirror = mirror == -1 ? p : -2;
          }
        I = acc;
      }
      write_task<kEC, kWeighted>(I, du, dv, kWeighted ? __ldg(S + u) : 0.0f,
                                 kWeighted ? __ldg(S + v) : 0.0f, (int64_t)us + lane,
                                 mirror >= 0 ? (int64_t)vs + mirror : -1, out);
    }
  }
  __syncwarp();
}

template <bool kEC, bool kWeighted>
__global__ void __launch_bounds__(kRowThreads) b0_kernel(
    Rows rp, const int32_t *__restrict__ col, const float *__restrict__ w,
    const float *__restrict__ S, const int32_t *__restrict__ rows, const int32_t *__restrict__ cnt,
    float *__restrict__ out) {
  __shared__ int32_t tables[kRowThreads / 32][kB0Slots];
  const int32_t r0 = cnt[kOffKeys + 96], r1 = cnt[kOffKeys + 128];
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = r0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < r1; i += nwarps)
    lane_row<kEC, kWeighted>(tables[threadIdx.x >> 5], rows[i], rp, col, w, S, out);
}

// ---------------------------------------------------------------- task batches
// Lanes fetch up to 32 candidate tasks (neighbours k0 .. k_end of row u) at once; the warp
// then runs the ones with d_v <= d_u one by one.  (Packing tasks of at most 8 or 16 elements 4
// or 2 to a warp pass changed R-MAT 24 weighted by -1.5 ms and the 2000-graph batch by -0.5 %;
// not kept.  Running the tasks of at most 16 / 32 / 64 elements one per lane, 32 at once in the
// reference's order: R-MAT 24 weighted 612 / 620 / 627 ms against 606 ms, unweighted 293 / 297 /
// 301 against 293 ms; a 250-graph batch pass unweighted 58.2 / 58.2 / 54.2 ms against 58.5 ms,
// weighted 126.7 (32) against 122.1 ms -- uncoalesced per-lane loads and divergence cost more
// than the latency they hide; not kept.  Prefetching the first 2 / 4 / 8 lines of each task's
// list to L2 when the batch is fetched: R-MAT 24 unchanged (615 / 616 / 617 against 615 ms),
// the batch pass 1-2 % shorter; not kept.)
template <bool kEC, bool kWeighted, class Probe, class Streams>
__device__ __forceinline__ void run_batch(const Probe &probe, const Streams &cls, Rows rp,
                                          const int32_t *__restrict__ col, const float *__restrict__ w,
                                          const float *__restrict__ S, int32_t u, int32_t us, int32_t du,
                                          float Su, int32_t k0, int32_t k_end, float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  int32_t v = -1, vs = 0, dv = 0;
  float Sv = 0.0f; // weighted: S[v], loaded with the degrees rather than after each task
  if (k0 + lane < k_end) {
    v = __ldg(col + us + k0 + lane);
    vs = rp.s(v);
    dv = rp.e(v) - vs;
    if (kWeighted) Sv = __ldg(S + v);
  }
  unsigned todo = __ballot_sync(kFull, v >= 0 && dv <= du);
  while (todo) {
    const int b = __ffs(todo) - 1;
    todo &= todo - 1;
    const int32_t tvs = __shfl_sync(kFull, vs, b), tdv = __shfl_sync(kFull, dv, b);
    const float tSv = kWeighted ? __shfl_sync(kFull, Sv, b) : 0.0f;
    int32_t mirror;
    const float I = task_stream<kWeighted>(probe, col, w, u, tvs, tdv, mirror, cls);
    if (lane == 0)
      write_task<kEC, kWeighted>(I, du, tdv, Su, tSv, (int64_t)us + k0 + b,
                                 mirror >= 0 ? (int64_t)tvs + mirror : -1, out);
  }
}

// Tasks a warp takes at once from a row (or hub unit) shared by `warps` warps, `rem` tasks
// left: 32 while plenty remain, then smaller batches so that the warps finish the row close
// together (they meet at a barrier before the next row).
__device__ __forceinline__ int32_t guided_batch(int32_t rem, int warps) {
  const int32_t g = rem / (2 * warps);
  return g >= 32 ? 32 : (g < 2 ? 2 : g);
}

// Cuckoo table size for d keys: 2.5 slots per key (even), at most `cap` slots.
__device__ __forceinline__ uint32_t cuckoo_slots(int32_t d, uint32_t cap) {
  uint32_t s = ((5u * (uint32_t)d + 3u) / 2u + 1u) & ~1u;
  s = s < 4u ? 4u : s;
  return s > cap ? cap : s;
}

// ---------------------------------------------------------------- B1: warp per row
// Shared memory of a warp: kB1Slots table slots, then (weighted) 8 * kB1Cap class-stream entries.
// (Folds here are short -- at most 512 matches -- and use shuffles, not a fold buffer.)
template <bool kWeighted> __host__ __device__ constexpr int b1_warp_words() {
  return kB1Slots + (kWeighted ? 8 * kB1Cap : 0);
}

// Row u (du <= kB1Max) by one warp: cuckoo hash of N(u) in the warp's area `t`, then its tasks.
template <bool kEC, bool kWeighted>
__device__ __forceinline__ void warp_row(int32_t *t, int32_t u, Rows rp,
                                         const int32_t *__restrict__ col, const float *__restrict__ w,
                                         const float *__restrict__ S, float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const SmemClassStreams cls{t + kB1Slots, kB1Cap};
  const int32_t us = rp.s(u), du = rp.e(u) - us;
  const float Su = kWeighted ? __ldg(S + u) : 0.0f;
  const uint32_t slots = cuckoo_slots(du, kB1Slots);
  int seed = 0;
  for (; seed < kCuckooSeeds; ++seed) {
    for (uint32_t k = lane; k < slots; k += 32) t[k] = kEmpty;
    __syncwarp();
    const CuckooProbe cp = cuckoo_params(t, slots, seed);
    bool fail = false;
    for (int32_t k = lane; k < du; k += 32) fail |= !cuckoo_insert(cp, t, __ldg(col + us + k));
    fail = __any_sync(kFull, fail);
    __syncwarp();
    if (!fail) break;
  }
  if (seed < kCuckooSeeds) {
    const CuckooProbe probe = cuckoo_params(t, slots, seed);
    for (int32_t k0 = 0; k0 < du; k0 += 32)
      run_batch<kEC, kWeighted>(probe, cls, rp, col, w, S, u, us, du, Su, k0, du, out);
  } else { // eviction cycles with every multiplier: linear probing (load <= 0.4)
    for (uint32_t k = lane; k < slots; k += 32) t[k] = kEmpty;
    __syncwarp();
    for (int32_t k = lane; k < du; k += 32) hset_insert(t, slots, __ldg(col + us + k));
    __syncwarp();
    const HashProbe probe{t, slots};
    for (int32_t k0 = 0; k0 < du; k0 += 32)
      run_batch<kEC, kWeighted>(probe, cls, rp, col, w, S, u, us, du, Su, k0, du, out);
  }
  __syncwarp();
}

template <bool kEC, bool kWeighted>
__global__ void __launch_bounds__(kRowThreads, 4) b1_kernel(
    Rows rp, const int32_t *__restrict__ col, const float *__restrict__ w,
    const float *__restrict__ S, const int32_t *__restrict__ rows, const int32_t *__restrict__ cnt,
    float *__restrict__ out) {
  extern __shared__ int32_t b1_smem[];
  int32_t *t = b1_smem + (threadIdx.x >> 5) * b1_warp_words<kWeighted>();
  const int32_t r0 = cnt[kOffKeys + 64], r1 = cnt[kOffKeys + 96];
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = r0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < r1; i += nwarps)
    warp_row<kEC, kWeighted>(t, rows[i], rp, col, w, S, out);
}

// ---------------------------------------------------------------- B2: CTA per row
template <bool kEC, bool kWeighted, class Probe, class CS>
__device__ __forceinline__ void b2_tasks(const Probe &probe, const CS &cls, int32_t *s_task, Rows rp,
                                         const int32_t *__restrict__ col,
                                         const float *__restrict__ w, const float *__restrict__ S, int32_t u,
                                         int32_t us, int32_t du, float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const float Su = kWeighted ? __ldg(S + u) : 0.0f;
  for (;;) {
    int32_t k0 = 0, g = 0;
    if (lane == 0) {
      g = guided_batch(du - *(volatile int32_t *)s_task, kB2Threads / 32);
      k0 = atomicAdd(s_task, g);
    }
    k0 = __shfl_sync(kFull, k0, 0);
    g = __shfl_sync(kFull, g, 0);
    if (k0 >= du) break;
    run_batch<kEC, kWeighted>(probe, cls, rp, col, w, S, u, us, du, Su, k0, min(du, k0 + g), out);
  }
}

// CTA rows from the plan's list until it runs out: one row at a time per CTA, its cuckoo table in
// `table` (kB2Slots words of shared memory), its tasks handed out to the warps.  s_row, s_task,
// s_fail: the CTA's shared bookkeeping words.  The class streams of warp `wid` (8 classes of
// `cap` entries) start at scratch + (blockIdx.x * 32 + wid) * 8 * cap.
template <bool kEC, bool kWeighted, bool kExact>
__device__ __forceinline__ void cta_rows_phase(int32_t *table, int32_t *s_row, int32_t *s_task, int32_t *s_fail,
                                               Rows rp, const int32_t *__restrict__ col, const float *__restrict__ w,
                                               const float *__restrict__ S, const int32_t *__restrict__ rows,
                                               int32_t *__restrict__ cnt, float *__restrict__ out,
                                               int32_t *__restrict__ scratch, int cap) {
  const int wid = threadIdx.x >> 5;
  using CS = Streams<true, kExact>;
  const CS cls{scratch + ((int64_t)blockIdx.x * (kB2Threads / 32) + wid) * 8 * cap, cap};
  const int32_t r0 = cnt[kOffKeys + 32], r1 = cnt[kOffKeys + 64];
  for (;;) {
    if (threadIdx.x == 0) {
      *s_row = r0 + atomicAdd(cnt + kCtrB2, 1);
      *s_task = 0;
    }
    __syncthreads();
    const int32_t i = *(volatile int32_t *)s_row;
    if (i >= r1) break;
    const int32_t u = rows[i];
    const int32_t us = rp.s(u), du = rp.e(u) - us;
    const uint32_t slots = cuckoo_slots(du, kB2Slots);
    int seed = 0;
    for (; seed < kCuckooSeeds; ++seed) {
      for (uint32_t k = threadIdx.x; k < slots; k += blockDim.x) table[k] = kEmpty;
      if (threadIdx.x == 0) *s_fail = 0;
      __syncthreads();
      const CuckooProbe cp = cuckoo_params(table, slots, seed);
      bool fail = false;
      for (int32_t k = threadIdx.x; k < du; k += blockDim.x) fail |= !cuckoo_insert(cp, table, __ldg(col + us + k));
      if (fail) *s_fail = 1;
      __syncthreads();
      const bool failed = *(volatile int32_t *)s_fail != 0;
      __syncthreads();
      if (!failed) break;
    }
    // the table uses `slots` words; the last 32 x 128 words of the area, when free, hold the
    // warps' fold buffers
    CS rcls = cls;
    if (kWeighted && slots + kB2FoldWords <= (uint32_t)kB2Slots)
      rcls.fbuf = reinterpret_cast<float *>(table + kB2Slots - kB2FoldWords) + wid * 128;
    // weighted rows whose table leaves room: each slot's weight right after the table, below the
    // fold buffers
    const bool wtab = kWeighted && seed < kCuckooSeeds && 2 * slots + kB2FoldWords <= (uint32_t)kB2Slots;
    if (wtab) {
      float *wt = reinterpret_cast<float *>(table + slots);
      for (uint32_t k = threadIdx.x; k < slots; k += blockDim.x) {
        const int32_t key = table[k];
        wt[k] = key != kEmpty ? __ldg(w + key) : 0.0f;
      }
      __syncthreads();
    }
    if (seed < kCuckooSeeds) {
      if constexpr (kWeighted) {
        if (wtab) {
          const CuckooWProbe probe{cuckoo_params(table, slots, seed), reinterpret_cast<const float *>(table + slots)};
          b2_tasks<kEC, kWeighted>(probe, rcls, s_task, rp, col, w, S, u, us, du, out);
        } else {
          b2_tasks<kEC, kWeighted>(cuckoo_params(table, slots, seed), rcls, s_task, rp, col, w, S, u, us, du, out);
        }
      } else {
        b2_tasks<kEC, kWeighted>(cuckoo_params(table, slots, seed), rcls, s_task, rp, col, w, S, u, us, du, out);
      }
    } else { // eviction cycles with every multiplier: linear probing (load <= 0.43)
      for (uint32_t k = threadIdx.x; k < slots; k += blockDim.x) table[k] = kEmpty;
      __syncthreads();
      for (int32_t k = threadIdx.x; k < du; k += blockDim.x) hset_insert(table, slots, __ldg(col + us + k));
      __syncthreads();
      b2_tasks<kEC, kWeighted>(HashProbe{table, slots}, rcls, s_task, rp, col, w, S, u, us, du, out);
    }
    __syncthreads();
  }
}

template <bool kEC, bool kWeighted, bool kExact>
__global__ void __launch_bounds__(kB2Threads, 1) b2_kernel(
    Rows rp, const int32_t *__restrict__ col, const float *__restrict__ w,
    const float *__restrict__ S, const int32_t *__restrict__ rows, int32_t *__restrict__ cnt,
    float *__restrict__ out, int32_t *__restrict__ scratch, int cap) {
  extern __shared__ int32_t table[];
  __shared__ int32_t s_row, s_task, s_fail;
  cta_rows_phase<kEC, kWeighted, kExact>(table, &s_row, &s_task, &s_fail, rp, col, w, S, rows, cnt, out,
                                         scratch, cap);
}

// ---------------------------------------------------------------- hubs: CTA clusters
// A cluster of kCl CTAs takes one hub unit (hub row u, task range) at a time: its CTAs build
// N(u) as a bitmap over [0, n) in the cluster's own global slot, all warps stream the unit's
// tasks against it (L2 hits), then the bits are cleared again.  Cluster barriers separate the
// phases; the unit index and task counter live in rank 0's shared memory.
template <bool kEC, bool kWeighted, int kCl>
__global__ void __launch_bounds__(kHubThreads, 1) hub_kernel(
    Rows rp, const int32_t *__restrict__ col, const float *__restrict__ w,
    const float *__restrict__ S, const int32_t *__restrict__ rows, int32_t *__restrict__ cnt,
    const int32_t *__restrict__ unit_off, uint32_t *__restrict__ bitmaps, int64_t words,
    float *__restrict__ out, int32_t *__restrict__ scratch, int cap, Bins bins) {
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ uint32_t filt[]; // hub_filter_words(): this CTA's filter of the unit's hub
  constexpr uint32_t kWords = hub_filter_words<kWeighted>();
  __shared__ int32_t s_unit, s_task;
  __shared__ __align__(16) float s_fold[kWeighted ? kHubThreads / 32 : 1][128];
  const unsigned rank = cluster.block_rank();
  const int64_t cid = blockIdx.x / kCl;
  uint32_t *bm = bitmaps + cid * words;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const ClassStreams cls{scratch + ((int64_t)blockIdx.x * (kHubThreads / 32) + wid) * 8 * cap, cap,
                         kWeighted ? s_fold[kWeighted ? wid : 0] : nullptr};
  int32_t *unit_p = cluster.map_shared_rank(&s_unit, 0);
  int32_t *task_p = cluster.map_shared_rank(&s_task, 0);
  const int32_t h0 = cnt[kOffKeys + 0];
  const int32_t nunits = cnt[kNumHubUnits];
  const int32_t unit_size = cnt[kHubUnitSize];
  const int32_t nhubs = cnt[kOffKeys + 32] - h0;
  if (rank == 0 && threadIdx.x == 0) {
    s_unit = atomicAdd(cnt + kCtrHub, 1);
    s_task = 0;
  }
  cluster.sync();
  for (;;) {
    const int32_t unit = *unit_p;
    if (unit >= nunits) break;
    // locate the hub of this unit
    int32_t lo = 0, hi = nhubs - 1;
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) >> 1;
      if (unit_off[mid] <= unit) lo = mid; else hi = mid - 1;
    }
    const int32_t u = rows[h0 + lo];
    const int32_t us = rp.s(u), du = rp.e(u) - us;
    const int32_t k_begin = (unit - unit_off[lo]) * unit_size;
    const int32_t k_end = min(du, k_begin + unit_size);
    if constexpr (kWords != 0) {
      for (uint32_t k = threadIdx.x; k < kWords; k += blockDim.x) filt[k] = 0u;
      __syncthreads();
      for (int32_t k = threadIdx.x; k < du; k += blockDim.x) { // every CTA filters all of N(u)
        const uint32_t h = filter_bit(__ldg(col + us + k), kWords * 32);
        atomicOr(filt + (h >> 5), 1u << (h & 31));
      }
    }
    for (int32_t k = rank * blockDim.x + threadIdx.x; k < du; k += kCl * blockDim.x) {
      const int32_t x = __ldg(col + us + k);
      atomicOr(bm + (x >> 5), 1u << (x & 31));
    }
    cluster.sync();
    const float Su = kWeighted ? __ldg(S + u) : 0.0f;
    for (;;) {
      int32_t k0 = 0, g = 0;
      if (lane == 0) {
        // hub tasks include whole hub-to-hub intersections: a warp takes at most hub_batch of them
        // at a time, so the biggest ones spread over many warps instead of queueing in one
        g = min(bins.hub_batch, guided_batch(k_end - k_begin - *(volatile int32_t *)task_p, kCl * (kHubThreads / 32)));
        k0 = k_begin + atomicAdd(task_p, g);
      }
      k0 = __shfl_sync(kFull, k0, 0);
      g = __shfl_sync(kFull, g, 0);
      if (k0 >= k_end) break;
      if constexpr (kWords != 0)
        run_batch<kEC, kWeighted>(FilterProbe{filt, bm, kWords * 32}, cls, rp, col, w, S, u, us, du, Su, k0,
                                  min(k_end, k0 + g), out);
      else
        run_batch<kEC, kWeighted>(BitmapProbe{bm}, cls, rp, col, w, S, u, us, du, Su, k0, min(k_end, k0 + g),
                                  out);
    }
    cluster.sync();
    for (int32_t k = rank * blockDim.x + threadIdx.x; k < du; k += kCl * blockDim.x)
      __stcg(bm + (__ldg(col + us + k) >> 5), 0u);
    if (rank == 0 && threadIdx.x == 0) {
      s_unit = atomicAdd(cnt + kCtrHub, 1);
      s_task = 0;
    }
    cluster.sync();
  }
  // no CTA may exit while another can still read rank 0's shared memory
  cluster.sync();
}

// ---------------------------------------------------------------- the row bins in one launch
// Persistent form: one 1024-thread CTA per SM, every CTA walking the bins in turn -- CTA rows,
// then warp rows and lane rows (its 32 warps independently) -- each from a device counter, so a
// bin's last items overlap the next bin's work instead of ending a kernel.  (Hub units stay in
// the cluster kernel: an 8-CTA cluster needs 8 free SMs of one GPC, and a persistent grid of
// clusters -- measured on R-MAT 24: 908 ms against 650 ms -- leaves SMs idle that CTA rows use.)
// The shared-memory area (kB2Slots words) holds the CTA row's table, then one part per warp for
// its warp-row table and later its lane-row table.
constexpr int kB1Fetch = 4;  // warp rows a warp takes per fetch
constexpr int kB0Fetch = 32; // lane rows a warp takes per fetch

template <bool kEC, bool kWeighted, bool kExact>
__global__ void __launch_bounds__(kB2Threads, 1) rows_kernel(
    Rows rp, const int32_t *__restrict__ col, const float *__restrict__ w,
    const float *__restrict__ S, const int32_t *__restrict__ rows, int32_t *__restrict__ cnt,
    float *__restrict__ out, int32_t *__restrict__ scratch, int cap_b2) {
  extern __shared__ int32_t area[];
  __shared__ int32_t s_row, s_task, s_fail;
  static_assert((kB2Threads / 32) * b1_warp_words<kWeighted>() <= kB2Slots, "warp-row tables");
  cta_rows_phase<kEC, kWeighted, kExact>(area, &s_row, &s_task, &s_fail, rp, col, w, S, rows, cnt, out, scratch,
                                         cap_b2);
  // warp rows, then lane rows: each warp in its own part of the area (no barrier between them;
  // every thread left the CTA-row phase together)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t *t = area + wid * b1_warp_words<kWeighted>();
  {
    const int32_t r0 = cnt[kOffKeys + 64], r1 = cnt[kOffKeys + 96];
    for (;;) {
      int32_t i = 0;
      if (lane == 0) i = r0 + atomicAdd(cnt + kCtrB1, kB1Fetch);
      i = __shfl_sync(kFull, i, 0);
      if (i >= r1) break;
      for (int32_t j = i; j < min(r1, i + kB1Fetch); ++j) warp_row<kEC, kWeighted>(t, rows[j], rp, col, w, S, out);
    }
  }
  {
    const int32_t r0 = cnt[kOffKeys + 96], r1 = cnt[kOffKeys + 128];
    for (;;) {
      int32_t i = 0;
      if (lane == 0) i = r0 + atomicAdd(cnt + kCtrB0, kB0Fetch);
      i = __shfl_sync(kFull, i, 0);
      if (i >= r1) break;
      for (int32_t j = i; j < min(r1, i + kB0Fetch); ++j) lane_row<kEC, kWeighted>(t, rows[j], rp, col, w, S, out);
    }
  }
}

// ---------------------------------------------------------------- fix-up of uncovered edges
// Any edge still holding the sentinel is computed on its own with the reference's ref/cur
// choice (VC jaccard.cpp:333-336, EC jaccard.cpp:716-719) and binary search.
template <bool kEC, bool kWeighted>
__global__ void __launch_bounds__(256) fixup_kernel(int32_t n, int64_t e, const int32_t *__restrict__ row_ptr,
                                                    const int32_t *__restrict__ col,
                                                    const float *__restrict__ w,
                                                    const float *__restrict__ S,
                                                    float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t *outb = reinterpret_cast<const uint32_t *>(out);
  for (int64_t j0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 128; j0 < e; j0 += nwarps * 128) {
    uint32_t b[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t j = j0 + lane + 32 * q;
      b[q] = j < e ? outb[j] : 0u;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      unsigned todo = __ballot_sync(kFull, b[q] == kUnwritten);
      while (todo) {
        const int64_t jj = j0 + 32 * q + __ffs(todo) - 1;
        todo &= todo - 1;
        // source row: the last u with row_ptr[u] <= jj
        int32_t lo = 0, hi = n - 1;
        while (lo < hi) {
          const int32_t mid = (lo + hi + 1) >> 1;
          if (__ldg(row_ptr + mid) <= jj) lo = mid; else hi = mid - 1;
        }
        const int32_t u = lo;
        const int32_t us = __ldg(row_ptr + u), du = __ldg(row_ptr + u + 1) - us;
        const int32_t v = __ldg(col + jj);
        const int32_t vs = __ldg(row_ptr + v), dv = __ldg(row_ptr + v + 1) - vs;
        const bool u_is_ref = kEC ? !(dv < du) : (du < dv);
        const int32_t rs = u_is_ref ? us : vs, rl = u_is_ref ? du : dv;
        const int32_t cs = u_is_ref ? vs : us, cl = u_is_ref ? dv : du;
        int32_t dummy;
        const float I = task_strided<kWeighted && !kEC>(SearchProbe{col, cs, cs + cl - 1}, col, w, -1, rs, rl, dummy);
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

// ---------------------------------------------------------------- pair list
// jaccard_list (standalone_algorithms.hpp:109-133, jaccard.cpp:957-988): J for explicit vertex
// pairs (first[p], second[p]).  The pair is treated like the edge (first, second) of the
// vertex-centric path: the shorter list is ref (ties: second), the sum is taken in the
// 8-i-lane order, J = I / (S_first + S_second - I).  The reference's pair kernel
// (Jaccard_IsPairsKernel, jaccard.cpp:462-540) accumulates into weight_i[i], the ref position,
// instead of weight_i[idx] (jaccard.cpp:517, 528), so its results are not usable; this is the
// intended computation.  One warp per pair; vertices must lie in [0, n).
template <bool kWeighted>
__global__ void __launch_bounds__(256) pairs_kernel(int64_t np, const int32_t *__restrict__ row_ptr,
                                                    const int32_t *__restrict__ col, const float *__restrict__ w,
                                                    const float *__restrict__ S, const int32_t *__restrict__ first,
                                                    const int32_t *__restrict__ second, float *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < np; p += nwarps) {
    const int32_t a = __ldg(first + p), b = __ldg(second + p);
    const int32_t as = __ldg(row_ptr + a), Ni = __ldg(row_ptr + a + 1) - as;
    const int32_t bs = __ldg(row_ptr + b), Nj = __ldg(row_ptr + b + 1) - bs;
    const bool a_is_ref = Ni < Nj; // jaccard.cpp:476-477
    const int32_t rs = a_is_ref ? as : bs, rl = a_is_ref ? Ni : Nj;
    const int32_t cs = a_is_ref ? bs : as, cl = a_is_ref ? Nj : Ni;
    int32_t dummy;
    const float I = task_strided<kWeighted>(SearchProbe{col, cs, cs + cl - 1}, col, w, -1, rs, rl, dummy);
    if (lane == 0) {
      const float Ws = kWeighted ? (__ldg(S + a) + __ldg(S + b)) : ((float)Ni + (float)Nj); // jaccard.cpp:480
      out[p] = I / (Ws - I);
    }
  }
}

// ---------------------------------------------------------------- host side
static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Grid sizes and class-stream capacities of one operator call.  The default plan fills the
// GPU; the fixed-scratch entry point uses a small plan whose workspace fits its array.
// Hub clusters of `cl` CTAs that can be resident at once on the current device: a cluster of
// these one-CTA-per-SM kernels needs `cl` free SMs of one GPC, so fewer than SMs / cl clusters
// may fit (a cluster launched beyond them would only start when another has finished; on GB300
// 15 clusters of 8 fit, leaving 32 of 152 SMs idle).  Both hub kernel variants are asked (their
// shared memory differs); cached per device and cluster size.
template <int kCl> static int query_resident_clusters() {
  const int most = std::max(1, sm_count() / kCl);
  int fit = most;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(most * kCl);
  cfg.blockDim = dim3(kHubThreads);
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  cfg.dynamicSmemBytes = sizeof(uint32_t) * hub_filter_words<false>();
  if (cudaFuncSetAttribute(hub_kernel<false, false, kCl>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)cfg.dynamicSmemBytes) == cudaSuccess &&
      cudaOccupancyMaxActiveClusters(&n, hub_kernel<false, false, kCl>, &cfg) == cudaSuccess && n > 0)
    fit = std::min(fit, n);
  cfg.dynamicSmemBytes = sizeof(uint32_t) * hub_filter_words<true>();
  if (cudaOccupancyMaxActiveClusters(&n, hub_kernel<false, true, kCl>, &cfg) == cudaSuccess && n > 0)
    fit = std::min(fit, n);
  cudaGetLastError(); // a failed query leaves the SM-count bound
  return fit;
}

static int resident_hub_clusters(int cl) {
  static std::mutex mu;
  static std::vector<int> cache; // [device * 2 + (cl == 4)]
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mu);
  const size_t k = (size_t)dev * 2 + (cl == 4 ? 1 : 0);
  if (cache.size() <= k) cache.resize(k + 1, 0);
  if (cache[k] == 0) cache[k] = cl == 4 ? query_resident_clusters<4>() : query_resident_clusters<8>();
  return cache[k];
}

int hub_cluster_count(int cluster_size) { return resident_hub_clusters(cluster_size); }

Plan default_plan() {
  const int sms = sm_count();
  Plan P{sms, resident_hub_clusters(kCluster), kCap, kHubCap, 0, sms * 8}; // b1_ctas 0: by occupancy
  P.hub_cluster = kCluster;
  P.b2_exact = true; // 8 * kCap >= kB2Max
  return P;
}

// Class-stream capacities no larger than a graph can fill: a class of a task holds at most
// ceil(d / 8) entries, d the length of the list it walks (<= the maximum degree, <= e), and no row
// of more than kB2Max tasks means no hub units.  max_degree must be an upper bound of the
// graph's largest degree (or -1: unknown, e is used): when 8 * cap_b2 covers it, the plan is
// marked exact and the CTA-row kernel drops its overflow checks, so a hint below the real
// maximum would let a class write past its stream.  Capacities stay multiples of 4 (int4
// reads of a class).
Plan fit_plan(Plan P, int64_t e, int64_t max_degree) {
  P.b0_max = std::max(1, std::min(P.b0_max, kB0Max));
  P.b1_max = std::max(P.b0_max, std::min(P.b1_max, kB1Max));
  P.b2_max = std::max(P.b1_max, std::min(P.b2_max, kB2Max));
  P.hub_unit = std::max(1, P.hub_unit);
  P.hub_batch = std::max(1, std::min(P.hub_batch, 32));
  const int64_t bound = max_degree >= 0 ? std::min<int64_t>(max_degree, e) : e;
  const int64_t d = std::min<int64_t>(bound, P.b2_max);
  const int cap = (int)(((d + 7) / 8 + 3) / 4 * 4);
  P.cap_b2 = std::max(4, std::min(P.cap_b2, cap));
  P.b2_exact = 8 * (int64_t)P.cap_b2 >= d; // no CTA-bin row exceeds d edges
  if (bound <= P.b2_max) P.cap_hub = std::min(P.cap_hub, 4);
  return P;
}

Plan apply_schedule(Plan P, const jx_schedule *sch, int64_t e, int64_t max_degree) {
  if (sch) {
    P.persistent = sch->persistent != 0;
    if (sch->lane_max > 0) P.b0_max = sch->lane_max;
    if (sch->warp_max > 0) P.b1_max = sch->warp_max;
    if (sch->cta_max > 0) P.b2_max = sch->cta_max;
    if (sch->hub_unit > 0) P.hub_unit = sch->hub_unit;
    if (sch->hub_batch > 0) P.hub_batch = sch->hub_batch;
    if (sch->hub_beside) P.hub_beside = sch->hub_beside > 0;
    if (sch->relabel) P.relabel = sch->relabel > 0;
    if (sch->hub_cluster == 4 || sch->hub_cluster == 8) {
      P.hub_cluster = sch->hub_cluster;
      P.hub_clusters = resident_hub_clusters(P.hub_cluster);
    }
  }
  return fit_plan(P, e, max_degree);
}

static Bins bins_of(const Plan &P) { return Bins{P.b0_max, P.b1_max, P.b2_max, P.hub_unit, P.hub_batch}; }

struct Layout {
  size_t cnt, rows, unit_off, S, scratch, bitmaps, total;
  size_t perm, start2, end2, w2, S2, col2; // relabelled ids (P.relabel)
  size_t hub_scratch; // byte offset of the hub kernel's class streams inside the scratch region
  int64_t words;
};

static Layout layout(int32_t n, int32_t e, bool weighted_vc, const Plan &P) {
  Layout L;
  L.words = ((int64_t)n + 31) / 32;
  size_t off = 0;
  L.cnt = off;      off += align256(sizeof(int32_t) * kCounters);
  L.rows = off;     off += align256(sizeof(int32_t) * (size_t)n);
  // every hub row holds more than b2_max edges
  const size_t max_hubs = std::min<size_t>((size_t)n, (size_t)e / ((size_t)P.b2_max + 1));
  L.unit_off = off; off += align256(sizeof(int32_t) * (max_hubs + 2));
  L.S = off;        off += weighted_vc ? align256(sizeof(float) * (size_t)n) : 0;
  // class streams: one region per warp of the CTA-row grid and of the hub grid; the hub region
  // follows the CTA-row region when the two kernels run side by side, else they share one
  const size_t b2_ids = (size_t)P.b2_ctas * (kB2Threads / 32) * 8 * P.cap_b2;
  const size_t hub_ids = (size_t)P.hub_clusters * P.hub_cluster * (kHubThreads / 32) * 8 * P.cap_hub;
  L.hub_scratch = P.hub_beside ? sizeof(int32_t) * b2_ids : 0;
  L.scratch = off;
  off += weighted_vc ? align256(sizeof(int32_t) * (P.hub_beside ? b2_ids + hub_ids : std::max(b2_ids, hub_ids))) : 0;
  L.bitmaps = off;  off += align256(sizeof(uint32_t) * (size_t)L.words * P.hub_clusters);
  L.perm = L.start2 = L.end2 = L.w2 = L.S2 = L.col2 = 0;
  if (P.relabel) {
    L.perm = off;   off += align256(sizeof(int32_t) * (size_t)n);
    L.start2 = off; off += align256(sizeof(int32_t) * (size_t)n);
    L.end2 = off;   off += align256(sizeof(int32_t) * (size_t)n);
    L.w2 = off;     off += weighted_vc ? align256(sizeof(float) * (size_t)n) : 0;
    L.S2 = off;     off += weighted_vc ? align256(sizeof(float) * (size_t)n) : 0;
    L.col2 = off;   off += align256(sizeof(int32_t) * (size_t)e);
  }
  L.total = off;
  return L;
}

// The second stream of a call (the hub kernel's, beside the row kernels) with its fork and join
// events: one set per host thread and device, created on first use.  A call records `fork` on
// its stream, makes the second stream wait for it, launches there, records `join` there and
// makes its own stream wait for that -- also valid inside a stream capture.
struct HubStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
struct HubStreams {
  std::vector<HubStream> v;
  ~HubStreams() {
    for (HubStream &h : v) {
      if (h.fork) cudaEventDestroy(h.fork);
      if (h.join) cudaEventDestroy(h.join);
      if (h.s) cudaStreamDestroy(h.s);
    }
  }
};
static thread_local HubStreams tl_hub_streams;

static jx_status hub_stream(HubStream **out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  auto &v = tl_hub_streams.v;
  if ((int)v.size() <= dev) v.resize(dev + 1);
  HubStream &h = v[dev];
  if (!h.s) {
    if ((ce = cudaStreamCreateWithFlags(&h.s, cudaStreamNonBlocking)) != cudaSuccess ||
        (ce = cudaEventCreateWithFlags(&h.fork, cudaEventDisableTiming)) != cudaSuccess ||
        (ce = cudaEventCreateWithFlags(&h.join, cudaEventDisableTiming)) != cudaSuccess) {
      if (h.fork) cudaEventDestroy(h.fork);
      if (h.s) cudaStreamDestroy(h.s);
      h = HubStream{};
      return set_cuda_error(ce);
    }
  }
  *out = &h;
  return JX_OK;
}

template <bool kEC, bool kWeighted>
static jx_status run_fused(const jx_csr &g, const float *w, float *out, char *ws, const Plan &P,
                           cudaStream_t s, const float *row_sums) {
  const int32_t n = g.n;
  const Layout L = layout(n, g.e, kWeighted, P);
  int32_t *cnt = reinterpret_cast<int32_t *>(ws + L.cnt);
  int32_t *rows = reinterpret_cast<int32_t *>(ws + L.rows);
  int32_t *unit_off = reinterpret_cast<int32_t *>(ws + L.unit_off);
  // row sums: computed into the workspace, or given (kept resident by the caller)
  float *S_ws = kWeighted ? reinterpret_cast<float *>(ws + L.S) : nullptr;
  const float *S = kWeighted ? (row_sums ? row_sums : S_ws) : nullptr;
  int32_t *scratch = kWeighted ? reinterpret_cast<int32_t *>(ws + L.scratch) : nullptr;
  uint32_t *bitmaps = reinterpret_cast<uint32_t *>(ws + L.bitmaps);
  const int sms = sm_count();
  jx_status st;
  cudaError_t ce;
  prof_mark("start", s);
  if ((ce = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * kCounters, s)) != cudaSuccess) return set_cuda_error(ce);
  if ((ce = cudaMemsetAsync(bitmaps, 0, sizeof(uint32_t) * (size_t)L.words * P.hub_clusters, s)) != cudaSuccess)
    return set_cuda_error(ce);
  const Bins bins = bins_of(P);
  const Rows orig{g.row_ptr, g.row_ptr + 1};
  auto plan = [&](Rows rp) -> jx_status {
    plan_kernel<false><<<sms * 4, 256, 0, s>>>(n, rp, cnt, rows, bins);
    jx_status r = check_launch();
    if (r != JX_OK) return r;
    plan_offsets_kernel<<<1, kKeys, 0, s>>>(cnt);
    if ((r = check_launch()) != JX_OK) return r;
    plan_kernel<true><<<sms * 4, 256, 0, s>>>(n, rp, cnt, rows, bins);
    return check_launch();
  };
  if ((st = plan(orig)) != JX_OK) return st;
  if (kWeighted && !row_sums) {
    // rows of the warp and lane bins, then the longer ones from the plan's row lists
    if ((st = rowsum_upto(n, g.row_ptr, g.col_idx, w, S_ws, P.b1_max, s)) != JX_OK) return st;
    rowsum_long_kernel<<<sms, 1024, 0, s>>>(g.row_ptr, g.col_idx, w, rows, cnt, S_ws);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("rowsum", s);
  }
  // the arrays the row kernels work on: the graph's own, or relabelled (ids by plan position)
  Rows rp = orig;
  const int32_t *colA = g.col_idx;
  const float *wA = w, *SA = S;
  if (P.relabel) {
    int32_t *perm = reinterpret_cast<int32_t *>(ws + L.perm);
    int32_t *start2 = reinterpret_cast<int32_t *>(ws + L.start2);
    int32_t *end2 = reinterpret_cast<int32_t *>(ws + L.end2);
    float *w2 = kWeighted ? reinterpret_cast<float *>(ws + L.w2) : nullptr;
    float *S2 = kWeighted ? reinterpret_cast<float *>(ws + L.S2) : nullptr;
    int32_t *col2 = reinterpret_cast<int32_t *>(ws + L.col2);
    relabel_isolated_kernel<<<sms * 4, 256, 0, s>>>(n, g.row_ptr, cnt, rows);
    if ((st = check_launch()) != JX_OK) return st;
    relabel_build_kernel<<<sms * 4, 256, 0, s>>>(n, g.row_ptr, rows, w, S, perm, start2, end2, w2, S2);
    if ((st = check_launch()) != JX_OK) return st;
    relabel_col_kernel<<<sms * 8, 256, 0, s>>>(g.e, g.col_idx, perm, col2);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("relabel", s);
    rp = Rows{start2, end2};
    colA = col2;
    wA = w2;
    SA = S2;
    // the plan again, on the new ids (the same rows in the same bins, now numbered in order)
    if ((ce = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * kCounters, s)) != cudaSuccess) return set_cuda_error(ce);
    if ((st = plan(rp)) != JX_OK) return st;
  }
  hub_units_kernel<<<1, 32, 0, s>>>(rp, rows, cnt, unit_off, bins.hub_unit, P.hub_clusters);
  if ((st = check_launch()) != JX_OK) return st;
  prof_mark("plan", s);
  fill_bits_kernel<<<sms * 4, 256, 0, s>>>(g.e, reinterpret_cast<uint32_t *>(out), kUnwritten);
  if ((st = check_launch()) != JX_OK) return st;
  prof_mark("sentinel_fill", s);

  // hub units: the cluster kernel, on a second stream beside the row kernels (P.hub_beside) or
  // first on the call's stream
  cudaStream_t hs = s;
  HubStream *fork = nullptr;
  if (P.hub_beside) {
    if ((st = hub_stream(&fork)) != JX_OK) return st;
    hs = fork->s;
    if ((ce = cudaEventRecord(fork->fork, s)) != cudaSuccess || (ce = cudaStreamWaitEvent(hs, fork->fork, 0)) != cudaSuccess)
      return set_cuda_error(ce);
    prof_mark("_fork", hs);
  }
  {
    cudaLaunchAttribute cluster_attr[1];
    cluster_attr[0].id = cudaLaunchAttributeClusterDimension;
    const int cl = P.hub_cluster == 4 ? 4 : 8;
    cluster_attr[0].val.clusterDim.x = cl;
    cluster_attr[0].val.clusterDim.y = 1;
    cluster_attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.hub_clusters * cl);
    cfg.blockDim = dim3(kHubThreads);
    cfg.dynamicSmemBytes = sizeof(uint32_t) * hub_filter_words<kWeighted>();
    auto hub = cl == 4 ? hub_kernel<kEC, kWeighted, 4> : hub_kernel<kEC, kWeighted, 8>;
    ce = cudaFuncSetAttribute(hub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.dynamicSmemBytes);
    if (ce != cudaSuccess) return set_cuda_error(ce);
    cfg.stream = hs;
    cfg.attrs = cluster_attr;
    cfg.numAttrs = 1;
    int32_t *hub_scratch = scratch ? scratch + L.hub_scratch / sizeof(int32_t) : nullptr;
    ce = cudaLaunchKernelEx(&cfg, hub, rp, colA, wA, SA, (const int32_t *)rows, cnt,
                            (const int32_t *)unit_off, bitmaps, (int64_t)L.words, out, hub_scratch, P.cap_hub, bins);
    if (ce != cudaSuccess) return set_cuda_error(ce);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("hub_rows", hs);
  }
  const size_t smem_b2 = sizeof(int32_t) * (size_t)kB2Slots;
  if (P.persistent) {
    // CTA, warp and lane rows in one launch (rows_kernel)
    auto kern = (kWeighted && P.b2_exact) ? rows_kernel<kEC, kWeighted, true> : rows_kernel<kEC, kWeighted, false>;
    ce = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b2);
    if (ce != cudaSuccess) return set_cuda_error(ce);
    kern<<<P.b2_ctas, kB2Threads, smem_b2, s>>>(rp, colA, wA, SA, rows, cnt, out, scratch, P.cap_b2);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("row_bins", s);
  } else {
    auto b2 = (kWeighted && P.b2_exact) ? b2_kernel<kEC, kWeighted, true> : b2_kernel<kEC, kWeighted, false>;
    ce = cudaFuncSetAttribute(b2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b2);
    if (ce != cudaSuccess) return set_cuda_error(ce);
    b2<<<P.b2_ctas, kB2Threads, smem_b2, s>>>(rp, colA, wA, SA, rows, cnt, out, scratch, P.cap_b2);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("cta_rows", s);
    const size_t smem_b1 = sizeof(int32_t) * (kRowThreads / 32) * b1_warp_words<kWeighted>();
    ce = cudaFuncSetAttribute(b1_kernel<kEC, kWeighted>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b1);
    if (ce != cudaSuccess) return set_cuda_error(ce);
    int b1_grid = P.b1_ctas;
    if (b1_grid <= 0) { // every CTA that fits at once (registers and shared memory: 4 per SM on GB300)
      int per_sm = 0;
      ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b1_kernel<kEC, kWeighted>, kRowThreads, smem_b1);
      if (ce != cudaSuccess) return set_cuda_error(ce);
      b1_grid = std::max(1, per_sm) * sms;
    }
    b1_kernel<kEC, kWeighted><<<b1_grid, kRowThreads, smem_b1, s>>>(rp, colA, wA, SA, rows, cnt, out);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("warp_rows", s);
    b0_kernel<kEC, kWeighted><<<P.b0_ctas, kRowThreads, 0, s>>>(rp, colA, wA, SA, rows, cnt, out);
    if ((st = check_launch()) != JX_OK) return st;
    prof_mark("lane_rows", s);
  }
  if (fork) {
    if ((ce = cudaEventRecord(fork->join, hs)) != cudaSuccess || (ce = cudaStreamWaitEvent(s, fork->join, 0)) != cudaSuccess)
      return set_cuda_error(ce);
    prof_mark("join", s);
  }
  fixup_kernel<kEC, kWeighted><<<sms * 8, 256, 0, s>>>(n, g.e, g.row_ptr, g.col_idx, w, S, out);
  if ((st = check_launch()) != JX_OK) return st;
  prof_mark("fixup", s);
  return JX_OK;
}

// Argument checks shared by the entry points; JX_OK with *run = false means "nothing to do".
static jx_status check_args(const jx_csr *g, jx_algo algo, const float *out_j, bool *run) {
  *run = false;
  if (!g || g->n < 0 || g->e < 0) return JX_ERR_INVALID;
  if (algo != JX_ALGO_VERTEX_CENTRIC && algo != JX_ALGO_EDGE_CENTRIC) return JX_ERR_INVALID;
  if (g->n == 0 || g->e == 0) return JX_OK;
  if (!g->row_ptr || !g->col_idx || !out_j) return JX_ERR_INVALID;
  *run = true;
  return JX_OK;
}

static jx_status dispatch(const jx_csr &g, const float *vertex_w, float *out_j, jx_algo algo, char *ws,
                          const Plan &P, cudaStream_t s, const float *row_sums = nullptr) {
  if (algo == JX_ALGO_EDGE_CENTRIC) return run_fused<true, false>(g, nullptr, out_j, ws, P, s, nullptr);
  if (vertex_w) return run_fused<false, true>(g, vertex_w, out_j, ws, P, s, row_sums);
  return run_fused<false, false>(g, nullptr, out_j, ws, P, s, nullptr);
}

size_t plan_workspace(int32_t n, int32_t e, bool weighted_vc, const Plan &P) {
  return layout(n, e, weighted_vc, P).total;
}

jx_status run_plan(const jx_csr &g, const float *vertex_w, float *out, jx_algo algo, void *workspace,
                   const Plan &P, cudaStream_t s, const float *row_sums) {
  bool run;
  const jx_status st = check_args(&g, algo, out, &run);
  if (!run) return st;
  if (!workspace || (reinterpret_cast<uintptr_t>(workspace) & 255u)) return JX_ERR_INVALID;
  const bool weighted = vertex_w != nullptr && algo == JX_ALGO_VERTEX_CENTRIC;
  return dispatch(g, weighted ? vertex_w : nullptr, out, algo, static_cast<char *>(workspace), P, s,
                  weighted ? row_sums : nullptr);
}

// ---------------------------------------------------------------- fixed-scratch entry point
// Workspace for jx_jaccard_noalloc: a file-scope device array, so that entry point never
// allocates.  Every GPU that loads this library holds it until the process exits.  All
// calls share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[JX_NOALLOC_SCRATCH_BYTES];

// A small grid whose workspace for any graph of at most JX_NOALLOC_MAX_VERTICES vertices fits
// the array: 8 B2 CTAs, one hub cluster, 1024 entries per class stream (overflows resume).
static Plan noalloc_plan() {
  const int sms = sm_count();
  Plan P{8, 1, 1024, 1024, sms * 3, sms * 8};
  P.hub_beside = false; // one stream: no second stream or events to create
  P.relabel = false;    // no room for a relabelled copy of the lists
  return P;
}

// Device address of g_noalloc_scratch on the current device.  In host code the symbol names a
// host-side stand-in, not device memory, so the address is looked up with that device current
// (cudaGetSymbolAddress, which also loads the module on the device's first use) and cached per
// device together with the id of the context it belongs to.  A device reset destroys that
// context and the module with it; the next call sees a new context id and looks the address
// up again instead of using a stale one.  The driver's context calls are reached through the
// runtime's entry-point query, so the library needs no link to the driver library.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

static jx_status current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, id) != CUDA_SUCCESS)
    return JX_ERR_CUDA;
  return JX_OK;
}

static jx_status noalloc_scratch(char **ptr) {
  struct Entry {
    unsigned long long ctx_id = 0;
    void *addr = nullptr;
  };
  static std::mutex mu;
  static std::vector<Entry> cache;
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  // makes the device's primary context current (and creates it after a reset); allocates nothing
  if ((ce = cudaSetDevice(dev)) != cudaSuccess) return set_cuda_error(ce);
  unsigned long long id = 0;
  if (current_context_id(&id) != JX_OK) return JX_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1);
  Entry &en = cache[dev];
  if (!en.addr || en.ctx_id != id) {
    void *p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess) return set_cuda_error(ce);
    en.addr = p;
    en.ctx_id = id;
  }
  *ptr = static_cast<char *>(en.addr);
  return JX_OK;
}

} // namespace jx

using namespace jx;

extern "C" {

size_t jx_jaccard_workspace_size(const jx_csr *g, int weighted, jx_algo algo) {
  if (!g || g->n < 0) return 0;
  return layout(g->n, g->e, weighted && algo == JX_ALGO_VERTEX_CENTRIC, fit_plan(default_plan(), g->e, -1)).total;
}

jx_status jx_jaccard_ws(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                        void *workspace, size_t workspace_bytes, jx_stream_t stream) {
  bool run;
  const jx_status st = check_args(g, algo, out_j, &run);
  if (!run) return st;
  const bool weighted = vertex_w != nullptr && algo == JX_ALGO_VERTEX_CENTRIC; // EC ignores weights
  const Plan P = fit_plan(default_plan(), g->e, -1);
  if (!workspace || workspace_bytes < layout(g->n, g->e, weighted, P).total ||
      (reinterpret_cast<uintptr_t>(workspace) & 255u))
    return JX_ERR_INVALID;
  return dispatch(*g, weighted ? vertex_w : nullptr, out_j, algo, static_cast<char *>(workspace), P,
                  (cudaStream_t)stream);
}

size_t jx_jaccard_schedule_workspace_size(const jx_csr *g, int weighted, jx_algo algo, const jx_schedule *sch) {
  if (!g || g->n < 0) return 0;
  return layout(g->n, g->e, weighted && algo == JX_ALGO_VERTEX_CENTRIC,
                apply_schedule(default_plan(), sch, g->e, -1)).total;
}

jx_status jx_jaccard_schedule(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                              const jx_schedule *sch, void *workspace, size_t workspace_bytes,
                              jx_stream_t stream) {
  bool run;
  const jx_status st = check_args(g, algo, out_j, &run);
  if (!run) return st;
  if (sch && (sch->lane_max < 0 || sch->warp_max < 0 || sch->cta_max < 0 || sch->hub_unit < 0 ||
              sch->hub_batch < 0))
    return JX_ERR_INVALID;
  const bool weighted = vertex_w != nullptr && algo == JX_ALGO_VERTEX_CENTRIC;
  const Plan P = apply_schedule(default_plan(), sch, g->e, -1);
  if (!workspace || workspace_bytes < layout(g->n, g->e, weighted, P).total ||
      (reinterpret_cast<uintptr_t>(workspace) & 255u))
    return JX_ERR_INVALID;
  return dispatch(*g, weighted ? vertex_w : nullptr, out_j, algo, static_cast<char *>(workspace), P,
                  (cudaStream_t)stream);
}

jx_status jx_jaccard(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                     jx_stream_t stream) {
  if (!g || g->n < 0 || g->e < 0) return JX_ERR_INVALID;
  if (g->n == 0 || g->e == 0) return JX_OK;
  const size_t bytes = jx_jaccard_workspace_size(g, vertex_w != nullptr, algo);
  cudaStream_t s = (cudaStream_t)stream;
  void *ws = nullptr;
  cudaError_t ce = cudaMallocAsync(&ws, bytes, s);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  const jx_status st = jx_jaccard_ws(g, vertex_w, out_j, algo, ws, bytes, stream);
  ce = cudaFreeAsync(ws, s);
  if (st != JX_OK) return st;
  return ce == cudaSuccess ? JX_OK : set_cuda_error(ce);
}

// Same operator and results as jx_jaccard, with its workspace in g_noalloc_scratch instead
// of allocated memory.  Rejects graphs above JX_NOALLOC_MAX_VERTICES with JX_ERR_TOO_LARGE.
jx_status jx_jaccard_noalloc(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                             jx_stream_t stream) {
  bool run;
  const jx_status st0 = check_args(g, algo, out_j, &run);
  if (!run) return st0;
  if (g->n > JX_NOALLOC_MAX_VERTICES) return JX_ERR_TOO_LARGE;
  const bool weighted = vertex_w != nullptr && algo == JX_ALGO_VERTEX_CENTRIC;
  const Plan P = noalloc_plan();
  if (layout(g->n, g->e, weighted, P).total > (size_t)JX_NOALLOC_SCRATCH_BYTES) return JX_ERR_TOO_LARGE;
  char *ws = nullptr;
  const jx_status st = noalloc_scratch(&ws);
  if (st != JX_OK) return st;
  return dispatch(*g, weighted ? vertex_w : nullptr, out_j, algo, ws, P, (cudaStream_t)stream);
}

jx_status jx_jaccard_list(const jx_csr *g, const float *vertex_w, int64_t num_pairs, const int32_t *first,
                          const int32_t *second, float *out, jx_stream_t stream) {
  if (!g || g->n < 0 || g->e < 0 || num_pairs < 0) return JX_ERR_INVALID;
  if (num_pairs == 0) return JX_OK;
  if (!g->row_ptr || (g->e > 0 && !g->col_idx) || !first || !second || !out) return JX_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t want = (num_pairs * 32 + 255) / 256;
  const int grid = (int)(want < (int64_t)sm_count() * 16 ? want : (int64_t)sm_count() * 16);
  if (!vertex_w) {
    pairs_kernel<false><<<grid, 256, 0, s>>>(num_pairs, g->row_ptr, g->col_idx, nullptr, nullptr, first, second, out);
    return check_launch();
  }
  float *S = nullptr;
  cudaError_t ce = cudaMallocAsync(&S, sizeof(float) * ((size_t)g->n + 1), s);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  jx_status st = jx_rowsum(g->n, g->e, g->row_ptr, g->col_idx, vertex_w, S, stream);
  if (st == JX_OK) {
    pairs_kernel<true><<<grid, 256, 0, s>>>(num_pairs, g->row_ptr, g->col_idx, vertex_w, S, first, second, out);
    st = check_launch();
  }
  cudaFreeAsync(S, s);
  return st;
}

} // extern "C"
