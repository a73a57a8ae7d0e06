/*
 * Synthetic graph generator for the Jaccard engine (host side, OpenMP).
 *
 * Produces the int32 CSR graphs the reference's driver feeds to `sygraph::jaccard`
 * (main.cpp:99-120 symmetrises through a std::set, which also deduplicates and sorts;
 * readMtxToCSR.cpp drops self loops).  Here the same shape of CSR is built directly:
 *   - every undirected sample (u, v) contributes (u, v) and (v, u);
 *   - self loops are dropped;
 *   - each adjacency list is sorted ascending and deduplicated.
 * Unlike the reference's MTX path, vertex ids are never renumbered and isolated vertices
 * (including trailing ones) are kept, so V is exactly the requested vertex count.
 *
 * Every random choice is a pure function of the seed (jx_rng.h), so the graph does not
 * depend on the thread count or on the host architecture.
 */
#include "../jx_rng.h"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Graph {
  int64_t n = 0;
  int64_t e = 0;
  std::vector<int64_t> row_ptr; // n + 1
  std::vector<int32_t> col;     // e
};

static inline void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* Build a symmetric, loop-free, deduplicated, row-sorted CSR from undirected samples. */
static Graph *build_symmetric(int64_t n, const std::vector<uint32_t> &src,
                              const std::vector<uint32_t> &dst) {
  Graph *g = new Graph();
  g->n = n;
  const int64_t m = (int64_t)src.size();
  std::vector<std::atomic<int64_t>> deg(n);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < n; ++v) deg[v].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    uint32_t a = src[i], b = dst[i];
    if (a == b) continue;
    deg[a].fetch_add(1, std::memory_order_relaxed);
    deg[b].fetch_add(1, std::memory_order_relaxed);
  }
  std::vector<int64_t> off(n + 1);
  off[0] = 0;
  for (int64_t v = 0; v < n; ++v) off[v + 1] = off[v] + deg[v].load(std::memory_order_relaxed);
  const int64_t total = off[n];
  std::vector<int32_t> raw(total);
  std::vector<std::atomic<int64_t>> pos(n);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < n; ++v) pos[v].store(off[v], std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    uint32_t a = src[i], b = dst[i];
    if (a == b) continue;
    raw[pos[a].fetch_add(1, std::memory_order_relaxed)] = (int32_t)b;
    raw[pos[b].fetch_add(1, std::memory_order_relaxed)] = (int32_t)a;
  }
  std::vector<int64_t> ndeg(n);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; ++v) {
    int32_t *b = raw.data() + off[v];
    int32_t *e = raw.data() + off[v + 1];
    std::sort(b, e);
    ndeg[v] = std::unique(b, e) - b;
  }
  g->row_ptr.resize(n + 1);
  g->row_ptr[0] = 0;
  for (int64_t v = 0; v < n; ++v) g->row_ptr[v + 1] = g->row_ptr[v] + ndeg[v];
  g->e = g->row_ptr[n];
  g->col.resize(g->e);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; ++v)
    std::memcpy(g->col.data() + g->row_ptr[v], raw.data() + off[v], sizeof(int32_t) * ndeg[v]);
  return g;
}

static inline uint32_t threshold32(double p) {
  if (p <= 0.0) return 0u;
  if (p >= 1.0) return 0xFFFFFFFFu;
  return (uint32_t)(p * 4294967296.0);
}

} // namespace

extern "C" {

/*
 * R-MAT graph: 2^scale vertices, edge_factor * 2^scale undirected samples with quadrant
 * probabilities (a, b, c, 1-a-b-c), then symmetrised / deduplicated / loop-free.
 * With perm_seed == 0 no vertex relabelling is applied (high-degree vertices keep small ids);
 * otherwise every id v becomes jx_permute_bits(v, scale, perm_seed), a seeded bijection, so
 * the graph is the same up to the names of its vertices.
 */
void *jxg_rmat(int scale, int64_t edge_factor, double a, double b, double c, uint64_t seed,
               uint64_t perm_seed, int nthreads) {
  if (scale < 1 || scale > 30 || edge_factor < 1) return nullptr;
  set_threads(nthreads);
  const int64_t n = (int64_t)1 << scale;
  const int64_t m = edge_factor * n;
  const uint32_t t0 = threshold32(a), t1 = threshold32(a + b), t2 = threshold32(a + b + c);
  try {
    std::vector<uint32_t> src(m), dst(m);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; ++i) {
      jx_rmat_sample(seed, (uint64_t)i, scale, t0, t1, t2, &src[i], &dst[i]);
      if (perm_seed) {
        src[i] = jx_permute_bits(src[i], scale, perm_seed);
        dst[i] = jx_permute_bits(dst[i], scale, perm_seed);
      }
    }
    return build_symmetric(n, src, dst);
  } catch (const std::bad_alloc &) {
    return nullptr;
  }
}

/* Erdos-Renyi G(n, p): each unordered pair {i < j} is an edge with probability p. */
void *jxg_er_gnp(int64_t n, double p, uint64_t seed, int nthreads) {
  if (n < 1 || n > (int64_t)1 << 20) return nullptr; /* O(n^2) pair tests */
  set_threads(nthreads);
  const uint32_t thr = threshold32(p);
  try {
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<std::vector<uint32_t>> ps(nt), pd(nt);
#pragma omp parallel
    {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
#pragma omp for schedule(dynamic, 16)
      for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i + 1; j < n; ++j)
          if ((uint32_t)(jx_draw(seed, (uint64_t)i, (uint64_t)j) >> 32) < thr) {
            ps[t].push_back((uint32_t)i);
            pd[t].push_back((uint32_t)j);
          }
    }
    std::vector<uint32_t> src, dst;
    for (int t = 0; t < nt; ++t) {
      src.insert(src.end(), ps[t].begin(), ps[t].end());
      dst.insert(dst.end(), pd[t].begin(), pd[t].end());
    }
    return build_symmetric(n, src, dst);
  } catch (const std::bad_alloc &) {
    return nullptr;
  }
}

/* Erdos-Renyi G(n, m): m uniform undirected samples, then symmetrised / deduplicated. */
void *jxg_er_gnm(int64_t n, int64_t m, uint64_t seed, int nthreads) {
  if (n < 1 || n > ((int64_t)1 << 31) - 1 || m < 0) return nullptr;
  set_threads(nthreads);
  try {
    std::vector<uint32_t> src(m), dst(m);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; ++i) {
      src[i] = jx_bounded32(jx_draw(seed, (uint64_t)i, 0), (uint32_t)n);
      dst[i] = jx_bounded32(jx_draw(seed, (uint64_t)i, 1), (uint32_t)n);
    }
    return build_symmetric(n, src, dst);
  } catch (const std::bad_alloc &) {
    return nullptr;
  }
}

int64_t jxg_num_vertices(const void *h) { return h ? ((const Graph *)h)->n : -1; }
int64_t jxg_num_edges(const void *h) { return h ? ((const Graph *)h)->e : -1; }

/* Copy the CSR out; row_ptr receives n + 1 int32 offsets (E must be < 2^31). */
int jxg_export(const void *h, int32_t *row_ptr, int32_t *col) {
  if (!h) return -1;
  const Graph *g = (const Graph *)h;
  if (g->e > 0x7FFFFFFFll) return -2;
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v <= g->n; ++v) row_ptr[v] = (int32_t)g->row_ptr[v];
  const int64_t chunk = 1 << 20;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < g->e; s += chunk)
    std::memcpy(col + s, g->col.data() + s, sizeof(int32_t) * std::min(chunk, g->e - s));
  return 0;
}

void jxg_free(void *h) { delete (Graph *)h; }

/* Per-vertex weights uniform on the grid {k * 2^-24 : k = 1 .. 2^24}, i.e. in (0, 1]. */
void jxg_uniform_weights(int64_t n, uint64_t seed, float *out, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < n; ++v) {
    uint32_t k = (uint32_t)(jx_draw(seed, 0x57E16u, (uint64_t)v) >> 40) + 1u; /* 1 .. 2^24 */
    out[v] = (float)k * (1.0f / 16777216.0f);
  }
}

} /* extern "C" */
