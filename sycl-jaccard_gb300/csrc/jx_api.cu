// C-ABI plumbing: status strings, error/launch bookkeeping, the host-buffer entry point and
// the CSR validator.
#include "jx_common.cuh"

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace jx {

static thread_local int tl_last_cuda = 0;
static thread_local uint64_t tl_launches = 0;

jx_status set_cuda_error(cudaError_t e) {
  tl_last_cuda = (int)e;
  return e == cudaErrorMemoryAllocation ? JX_ERR_NOMEM : JX_ERR_CUDA;
}

void count_launches(uint64_t k) { tl_launches += k; }

struct ProfMark {
  const char *name;
  cudaEvent_t ev;
  cudaStream_t s;
};
static thread_local bool tl_prof = false;
static thread_local std::vector<ProfMark> tl_marks;

void prof_mark(const char *name, cudaStream_t s) {
  if (!tl_prof) return;
  cudaEvent_t ev;
  if (cudaEventCreate(&ev) != cudaSuccess) return;
  cudaEventRecord(ev, s);
  tl_marks.push_back({name, ev, s});
}

int sm_count() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = v > 0 ? v : 1;
  }
  return cache[dev];
}

// ---------------------------------------------------------------- CSR validation
__global__ void check_rows_kernel(int32_t n, int32_t e, const int32_t *__restrict__ row_ptr,
                                  const int32_t *__restrict__ col, uint32_t *__restrict__ flags) {
  uint32_t f = 0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u <= n;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = row_ptr[u];
    if (u == 0 && a != 0) f |= JX_CSR_OFFSETS_BAD;
    if (u == n) {
      if (a != e) f |= JX_CSR_OFFSETS_BAD;
      continue;
    }
    const int32_t b = row_ptr[u + 1];
    if (b < a || a < 0 || b > e) {
      f |= JX_CSR_OFFSETS_BAD;
      continue;
    }
    int32_t prev = -1;
    for (int32_t k = a; k < b; ++k) {
      const int32_t c = col[k];
      if (c < 0 || c >= n) f |= JX_CSR_INDEX_RANGE;
      if (c == (int32_t)u) f |= JX_CSR_SELF_LOOP;
      if (k > a) {
        if (c < prev) f |= JX_CSR_UNSORTED;
        if (c == prev) f |= JX_CSR_DUPLICATE;
      }
      prev = c;
    }
  }
  if (f) atomicOr(flags, f);
}

// Requires offsets valid, indices in range and rows sorted.
__global__ void check_symmetry_kernel(int32_t n, const int32_t *__restrict__ row_ptr,
                                      const int32_t *__restrict__ col, uint32_t *__restrict__ flags) {
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  bool bad = false;
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += nwarps) {
    const int32_t a = row_ptr[u], b = row_ptr[u + 1];
    for (int32_t k = a + lane; k < b; k += 32) {
      const int32_t v = col[k];
      if (!bsearch_found(col, row_ptr[v], row_ptr[v + 1] - 1, (int32_t)u)) bad = true;
    }
  }
  if (__any_sync(kFull, bad) && lane == 0) atomicOr(flags, JX_CSR_ASYMMETRIC);
}

// ---------------------------------------------------------------- host-buffer entry point state
// Device memory of jx_jaccard_host comes from a pool this library owns, one per device, whose
// release threshold keeps freed blocks mapped: calls after the first reuse their device memory
// instead of mapping gigabytes again (the default pool returns it at every synchronisation).
// jx_host_release() hands it back.  Each host thread has its own stream per device.
static std::mutex g_host_mu;
static std::vector<cudaMemPool_t> g_host_pools;

struct HostStreams {
  std::vector<cudaStream_t> s;
  ~HostStreams() {
    for (cudaStream_t x : s)
      if (x) cudaStreamDestroy(x);
  }
};
static thread_local HostStreams tl_host_streams;

static jx_status host_stream_and_pool(cudaStream_t *s, cudaMemPool_t *pool) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  {
    std::lock_guard<std::mutex> lock(g_host_mu);
    if ((int)g_host_pools.size() <= dev) g_host_pools.resize(dev + 1, nullptr);
    if (!g_host_pools[dev]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t p = nullptr;
      if ((ce = cudaMemPoolCreate(&p, &props)) != cudaSuccess) return set_cuda_error(ce);
      uint64_t keep = UINT64_MAX;
      if ((ce = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
        cudaMemPoolDestroy(p);
        return set_cuda_error(ce);
      }
      g_host_pools[dev] = p;
    }
    *pool = g_host_pools[dev];
  }
  auto &v = tl_host_streams.s;
  if ((int)v.size() <= dev) v.resize(dev + 1, nullptr);
  if (!v[dev] && (ce = cudaStreamCreateWithFlags(&v[dev], cudaStreamNonBlocking)) != cudaSuccess) {
    v[dev] = nullptr;
    return set_cuda_error(ce);
  }
  *s = v[dev];
  return JX_OK;
}

} // namespace jx

using namespace jx;

extern "C" {

const char *jx_status_string(jx_status s) {
  switch (s) {
  case JX_OK: return "ok";
  case JX_ERR_INVALID: return "invalid argument";
  case JX_ERR_CUDA: return "CUDA error";
  case JX_ERR_NOMEM: return "out of memory";
  case JX_ERR_BAD_GRAPH: return "invalid CSR graph";
  case JX_ERR_UNSUPPORTED: return "unsupported request";
  case JX_ERR_TOO_LARGE: return "size above the supported maximum";
  case JX_ERR_CANCELLED: return "request cancelled";
  }
  return "unknown status";
}

int jx_version(void) { return 10000; }

void jx_profile_begin(void) {
  for (auto &m : tl_marks) cudaEventDestroy(m.ev);
  tl_marks.clear();
  tl_prof = true;
}

int jx_profile_end(char *buf, size_t len) {
  tl_prof = false;
  std::string out;
  int count = 0;
  // a mark's time runs from the previous mark on its own stream (from the previous mark of any
  // stream for the first mark of a stream); marks named "_..." only anchor the next interval
  for (size_t i = 1; i < tl_marks.size(); ++i) {
    size_t j = i - 1;
    for (size_t k = i; k-- > 0;)
      if (tl_marks[k].s == tl_marks[i].s) {
        j = k;
        break;
      }
    float ms = 0.0f;
    cudaEventSynchronize(tl_marks[i].ev);
    if (tl_marks[i].name[0] == '_') continue;
    if (cudaEventElapsedTime(&ms, tl_marks[j].ev, tl_marks[i].ev) != cudaSuccess) continue;
    char line[160];
    snprintf(line, sizeof line, "%s%s=%.6f", count ? ";" : "", tl_marks[i].name, ms);
    out += line;
    ++count;
  }
  for (auto &m : tl_marks) cudaEventDestroy(m.ev);
  tl_marks.clear();
  if (buf && len) {
    size_t k = out.size() < len - 1 ? out.size() : len - 1;
    memcpy(buf, out.data(), k);
    buf[k] = 0;
  }
  return count;
}
int jx_last_cuda_error(void) { return tl_last_cuda; }
uint64_t jx_launch_count(void) { return tl_launches; }
void jx_launch_count_reset(void) { tl_launches = 0; }

jx_status jx_csr_check(const jx_csr *g, uint32_t *flags, jx_stream_t stream) {
  if (!g || !flags || g->n < 0 || g->e < 0) return JX_ERR_INVALID;
  *flags = 0;
  if (g->n == 0) return JX_OK;
  if (!g->row_ptr || (g->e > 0 && !g->col_idx)) return JX_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t *d = nullptr;
  cudaError_t ce = cudaMallocAsync(&d, sizeof(uint32_t), s);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  jx_status st = JX_OK;
  uint32_t h = 0;
  do {
    if ((ce = cudaMemsetAsync(d, 0, sizeof(uint32_t), s)) != cudaSuccess) { st = set_cuda_error(ce); break; }
    check_rows_kernel<<<sm_count() * 8, 256, 0, s>>>(g->n, g->e, g->row_ptr, g->col_idx, d);
    if ((st = check_launch()) != JX_OK) break;
    if ((ce = cudaMemcpyAsync(&h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess) { st = set_cuda_error(ce); break; }
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) { st = set_cuda_error(ce); break; }
    if (h & (JX_CSR_OFFSETS_BAD | JX_CSR_INDEX_RANGE | JX_CSR_UNSORTED)) break; // symmetry test needs them
    check_symmetry_kernel<<<sm_count() * 8, 256, 0, s>>>(g->n, g->row_ptr, g->col_idx, d);
    if ((st = check_launch()) != JX_OK) break;
    if ((ce = cudaMemcpyAsync(&h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess) { st = set_cuda_error(ce); break; }
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) { st = set_cuda_error(ce); break; }
  } while (0);
  cudaFreeAsync(d, s);
  *flags = h;
  return st;
}

jx_status jx_jaccard_host(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *col_idx,
                          const float *vertex_w, float *out_j, jx_algo algo) {
  if (n < 0 || e < 0) return JX_ERR_INVALID;
  if (n == 0 || e == 0) return JX_OK;
  if (!row_ptr || !col_idx || !out_j) return JX_ERR_INVALID;
  if (algo != JX_ALGO_VERTEX_CENTRIC && algo != JX_ALGO_EDGE_CENTRIC) return JX_ERR_INVALID;
  cudaStream_t s = nullptr;
  cudaMemPool_t pool = nullptr;
  jx_status st = host_stream_and_pool(&s, &pool);
  if (st != JX_OK) return st;
  const bool weighted = vertex_w && algo == JX_ALGO_VERTEX_CENTRIC;
  const jx_csr shape{n, e, nullptr, nullptr};
  const size_t ws_bytes = jx_jaccard_workspace_size(&shape, weighted, algo);
  int32_t *d_rp = nullptr, *d_col = nullptr;
  float *d_w = nullptr, *d_out = nullptr;
  void *d_ws = nullptr;
  cudaError_t ce;
  prof_mark("host_call", s);
  do {
    if ((ce = cudaMallocFromPoolAsync(&d_rp, sizeof(int32_t) * ((size_t)n + 1), pool, s)) != cudaSuccess ||
        (ce = cudaMallocFromPoolAsync(&d_col, sizeof(int32_t) * (size_t)e, pool, s)) != cudaSuccess ||
        (ce = cudaMallocFromPoolAsync(&d_out, sizeof(float) * (size_t)e, pool, s)) != cudaSuccess ||
        (ce = cudaMallocFromPoolAsync(&d_ws, ws_bytes, pool, s)) != cudaSuccess ||
        (weighted && (ce = cudaMallocFromPoolAsync(&d_w, sizeof(float) * (size_t)n, pool, s)) != cudaSuccess)) {
      st = set_cuda_error(ce);
      break;
    }
    prof_mark("alloc", s);
    if ((ce = cudaMemcpyAsync(d_rp, row_ptr, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_col, col_idx, sizeof(int32_t) * (size_t)e, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (weighted && (ce = cudaMemcpyAsync(d_w, vertex_w, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, s)) != cudaSuccess)) {
      st = set_cuda_error(ce);
      break;
    }
    prof_mark("h2d", s);
    const jx_csr g{n, e, d_rp, d_col};
    if ((st = jx_jaccard_ws(&g, weighted ? d_w : nullptr, d_out, algo, d_ws, ws_bytes, (jx_stream_t)s)) != JX_OK) break;
    if ((ce = cudaMemcpyAsync(out_j, d_out, sizeof(float) * (size_t)e, cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
      st = set_cuda_error(ce);
      break;
    }
    prof_mark("d2h", s);
  } while (0);
  for (void *p : {(void *)d_rp, (void *)d_col, (void *)d_out, (void *)d_ws, (void *)d_w})
    if (p) cudaFreeAsync(p, s);
  ce = cudaStreamSynchronize(s);
  if (st == JX_OK && ce != cudaSuccess) st = set_cuda_error(ce);
  return st;
}

jx_status jx_host_alloc(size_t bytes, void **ptr) {
  if (!ptr) return JX_ERR_INVALID;
  *ptr = nullptr;
  const cudaError_t ce = cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault);
  if (ce != cudaSuccess) {
    *ptr = nullptr;
    return set_cuda_error(ce);
  }
  return JX_OK;
}

jx_status jx_host_free(void *ptr) {
  if (!ptr) return JX_OK;
  const cudaError_t ce = cudaFreeHost(ptr);
  return ce == cudaSuccess ? JX_OK : set_cuda_error(ce);
}

jx_status jx_host_release(void) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  std::lock_guard<std::mutex> lock(g_host_mu);
  if (dev < (int)g_host_pools.size() && g_host_pools[dev]) {
    if ((ce = cudaDeviceSynchronize()) != cudaSuccess) return set_cuda_error(ce);
    if ((ce = cudaMemPoolTrimTo(g_host_pools[dev], 0)) != cudaSuccess) return set_cuda_error(ce);
  }
  return JX_OK;
}

} // extern "C"
