// Serving: a request loop on one GPU with admission by device-memory budget, resident graphs,
// folding of queued small requests into one super-CSR pass, and several passes in flight.
//
// Threads: the caller submits (non-blocking) into a FIFO queue; one dispatcher thread admits
// requests in arrival order -- a request waits until its device bytes fit the budget and a
// slot is free -- and forms passes; `slots` worker threads each own a CUDA stream and run one
// pass at a time (uploads, the fused operator, result copies), so passes of different slots
// overlap on the device.  A pass is either one request on its own graph (a resident graph
// runs in place, with its resident row sums) or several small requests of the same kind
// packed into one super-CSR (disjoint components: each request's results are exactly its
// own, see the batched mode).  Device memory comes from a pool owned by the server; the
// budget is enforced by reservation before a pass starts.
#include "jx_common.cuh"
#include "jx_plan.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace jx {
namespace {

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

struct Resident {
  int32_t n = 0, e = 0;
  int32_t max_deg = 0;
  int32_t *row_ptr = nullptr, *col = nullptr;
  float *w = nullptr, *S = nullptr; // weights and their row sums (weighted graphs)
  size_t bytes = 0;
};

struct Req {
  uint64_t ticket = 0;
  int32_t graph_id = -1;
  jx_host_graph up{};
  jx_algo algo = JX_ALGO_VERTEX_CENTRIC;
  bool weighted = false;
  float *host_out = nullptr;
  int64_t arrival_ns = 0, done_ns = 0;
  int32_t n = 0, e = 0, max_deg = 0;
  Resident res{};  // the resident graph's device arrays (graph_id >= 0), copied at submit
  size_t need = 0; // device bytes of this request alone
  jx_status status = JX_OK;
  bool done = false;
};

struct Pass {
  std::vector<Req *> reqs;
  size_t reserved = 0;
};

} // namespace
} // namespace jx

using namespace jx;

struct jx_server_s {
  jx_server_config cfg{};
  int device = 0;
  cudaMemPool_t pool = nullptr;

  std::mutex mu;
  std::condition_variable cv_queue; // dispatcher: new request / slot or memory freed / stop
  std::condition_variable cv_done;  // waiters: a request completed
  std::deque<Req *> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  uint64_t next_ticket = 1;
  uint64_t submitted = 0, finished = 0;
  size_t reserved = 0, peak_reserved = 0, resident_bytes = 0;
  std::vector<Resident> graphs;
  bool stop = false;
  bool paused = false;                  // admission held (jx_server_set_paused)
  std::atomic<int32_t> inject_alloc{0}; // allocations still to fail (jx_server_inject_alloc_failures)

  // slots
  struct Slot {
    std::thread th;
    cudaStream_t stream = nullptr;
    std::unique_ptr<Pass> pass; // guarded by mu: the pass handed to this slot, until it starts
    bool busy = false;          // guarded by mu: a pass is handed over or running
    std::condition_variable cv;
  };
  std::vector<std::unique_ptr<Slot>> slots;
  int free_slots = 0;
  std::thread dispatcher;

  // statistics (guarded by mu)
  std::vector<double> lat_ms;
  uint64_t completed = 0, failed = 0, cancelled = 0, passes = 0, folded = 0;
  int64_t edges = 0;
  int64_t first_arrival = 0, last_done = 0;
  std::atomic<uint64_t> kernels{0};
};

namespace jx {
namespace {

// Device bytes one request needs on its own (inputs it uploads, results, workspace).
size_t request_bytes(const jx_server_s *S, const Req &r) {
  size_t b = align_up(sizeof(float) * (size_t)r.e); // results
  if (r.graph_id < 0) {
    b += align_up(sizeof(int32_t) * ((size_t)r.n + 1)) + align_up(sizeof(int32_t) * (size_t)r.e);
    if (r.weighted) b += align_up(sizeof(float) * (size_t)r.n);
  }
  b += align_up(plan_workspace(r.n, r.e, r.weighted, apply_schedule(default_plan(), &S->cfg.schedule, r.e, r.max_deg)));
  return b;
}

// The plan of a folded pass: the default grid, class streams for the largest degree in it.
Plan fold_plan(const jx_server_s *S, const std::vector<Req *> &reqs, int64_t e) {
  int64_t d = 0;
  for (const Req *r : reqs) d = std::max<int64_t>(d, r->max_deg);
  return apply_schedule(default_plan(), &S->cfg.schedule, e, d);
}

// Device bytes of a folded pass over `reqs` (everything is packed, resident graphs copied).
size_t fold_bytes(const jx_server_s *S, const std::vector<Req *> &reqs) {
  int64_t n = 0, e = 0;
  bool weighted = false;
  for (const Req *r : reqs) {
    n += r->n;
    e += r->e;
    weighted = r->weighted;
  }
  size_t b = align_up(sizeof(int32_t) * (size_t)(n + 1)) + 2 * align_up(sizeof(int32_t) * (size_t)e);
  if (weighted) b += align_up(sizeof(float) * (size_t)n);
  b += 2 * align_up(sizeof(int64_t) * (reqs.size() + 1));
  b += align_up(plan_workspace((int32_t)n, (int32_t)e, weighted, fold_plan(S, reqs, e)));
  return b;
}

bool foldable(const jx_server_s *S, const Req *r) { return r->e <= S->cfg.fold_edges; }
bool same_kind(const Req *a, const Req *b) { return a->algo == b->algo && a->weighted == b->weighted; }

// Take one injected allocation failure, if any are left.
bool take_injected(std::atomic<int32_t> *left) {
  int32_t v = left ? left->load() : 0;
  while (v > 0 && !left->compare_exchange_weak(v, v - 1)) {
  }
  return v > 0;
}

struct DevBuf {
  cudaMemPool_t pool;
  cudaStream_t s;
  std::atomic<int32_t> *inject = nullptr;
  std::vector<void *> ptrs;
  cudaError_t err = cudaSuccess;
  template <class T> T *get(size_t count) {
    void *p = nullptr;
    if (err != cudaSuccess) return nullptr;
    if (take_injected(inject)) {
      err = cudaErrorMemoryAllocation;
      return nullptr;
    }
    err = cudaMallocFromPoolAsync(&p, std::max<size_t>(align_up(sizeof(T) * count), 256), pool, s);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T *>(p);
  }
  ~DevBuf() {
    for (void *p : ptrs) cudaFreeAsync(p, s);
  }
};

#define JX_SRV_TRY(x)                                                                               \
  do {                                                                                               \
    cudaError_t ce_ = (x);                                                                           \
    if (ce_ != cudaSuccess) return set_cuda_error(ce_);                                              \
  } while (0)

// One request on its own graph.
jx_status run_single(jx_server_s *S, Req &r, cudaStream_t s) {
  if (r.e == 0) return JX_OK;
  DevBuf buf{S->pool, s, &S->inject_alloc};
  const Plan P = apply_schedule(default_plan(), &S->cfg.schedule, r.e, r.max_deg);
  jx_csr g{r.n, r.e, nullptr, nullptr};
  const float *w = nullptr, *row_sums = nullptr;
  if (r.graph_id >= 0) {
    const Resident &R = r.res;
    g.row_ptr = R.row_ptr;
    g.col_idx = R.col;
    if (r.weighted) {
      w = R.w;
      row_sums = R.S;
    }
  } else {
    int32_t *rp = buf.get<int32_t>((size_t)r.n + 1);
    int32_t *col = buf.get<int32_t>((size_t)r.e);
    float *wd = r.weighted ? buf.get<float>((size_t)r.n) : nullptr;
    JX_SRV_TRY(buf.err);
    JX_SRV_TRY(cudaMemcpyAsync(rp, r.up.row_ptr, sizeof(int32_t) * ((size_t)r.n + 1), cudaMemcpyHostToDevice, s));
    JX_SRV_TRY(cudaMemcpyAsync(col, r.up.col_idx, sizeof(int32_t) * (size_t)r.e, cudaMemcpyHostToDevice, s));
    if (wd) JX_SRV_TRY(cudaMemcpyAsync(wd, r.up.vertex_w, sizeof(float) * (size_t)r.n, cudaMemcpyHostToDevice, s));
    g.row_ptr = rp;
    g.col_idx = col;
    w = wd;
  }
  float *out = buf.get<float>((size_t)r.e);
  void *ws = buf.get<char>(plan_workspace(r.n, r.e, r.weighted, P));
  JX_SRV_TRY(buf.err);
  jx_status st = run_plan(g, w, out, r.algo, ws, P, s, row_sums);
  if (st != JX_OK) return st;
  JX_SRV_TRY(cudaMemcpyAsync(r.host_out, out, sizeof(float) * (size_t)r.e, cudaMemcpyDeviceToHost, s));
  JX_SRV_TRY(cudaStreamSynchronize(s));
  return JX_OK;
}

// Several small requests of one kind packed into one super-CSR pass.
jx_status run_fold(jx_server_s *S, std::vector<Req *> &reqs, cudaStream_t s) {
  const int32_t k = (int32_t)reqs.size();
  std::vector<int64_t> vb(k + 1, 0), eb(k + 1, 0);
  for (int32_t i = 0; i < k; ++i) {
    vb[i + 1] = vb[i] + reqs[i]->n;
    eb[i + 1] = eb[i] + reqs[i]->e;
  }
  const int64_t nv = vb[k], ne = eb[k];
  if (ne == 0) return JX_OK;
  const bool weighted = reqs[0]->weighted;
  const jx_algo algo = reqs[0]->algo;
  const Plan P = fold_plan(S, reqs, ne);
  DevBuf buf{S->pool, s, &S->inject_alloc};
  int32_t *rp = buf.get<int32_t>((size_t)nv + 1);
  int32_t *col = buf.get<int32_t>((size_t)ne);
  float *w = weighted ? buf.get<float>((size_t)nv) : nullptr;
  int64_t *dvb = buf.get<int64_t>((size_t)k + 1);
  int64_t *deb = buf.get<int64_t>((size_t)k + 1);
  float *out = buf.get<float>((size_t)ne);
  void *ws = buf.get<char>(plan_workspace((int32_t)nv, (int32_t)ne, weighted, P));
  JX_SRV_TRY(buf.err);
  for (int32_t i = 0; i < k; ++i) {
    const Req &r = *reqs[i];
    const bool res = r.graph_id >= 0;
    const Resident *R = res ? &r.res : nullptr;
    const cudaMemcpyKind kind = res ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (r.n > 0)
      JX_SRV_TRY(cudaMemcpyAsync(rp + vb[i], res ? R->row_ptr : r.up.row_ptr, sizeof(int32_t) * (size_t)r.n, kind, s));
    if (r.e > 0)
      JX_SRV_TRY(cudaMemcpyAsync(col + eb[i], res ? R->col : r.up.col_idx, sizeof(int32_t) * (size_t)r.e, kind, s));
    if (weighted && r.n > 0)
      JX_SRV_TRY(cudaMemcpyAsync(w + vb[i], res ? R->w : r.up.vertex_w, sizeof(float) * (size_t)r.n, kind, s));
  }
  const int32_t total = (int32_t)ne;
  JX_SRV_TRY(cudaMemcpyAsync(rp + nv, &total, sizeof(int32_t), cudaMemcpyHostToDevice, s));
  JX_SRV_TRY(cudaMemcpyAsync(dvb, vb.data(), sizeof(int64_t) * (k + 1), cudaMemcpyHostToDevice, s));
  JX_SRV_TRY(cudaMemcpyAsync(deb, eb.data(), sizeof(int64_t) * (k + 1), cudaMemcpyHostToDevice, s));
  jx_status st = shift_to_super(nv, ne, k, dvb, deb, rp, col, s);
  if (st != JX_OK) return st;
  const jx_csr g{(int32_t)nv, (int32_t)ne, rp, col};
  if ((st = run_plan(g, w, out, algo, ws, P, s)) != JX_OK) return st;
  for (int32_t i = 0; i < k; ++i)
    if (reqs[i]->e > 0)
      JX_SRV_TRY(cudaMemcpyAsync(reqs[i]->host_out, out + eb[i], sizeof(float) * (size_t)reqs[i]->e,
                                 cudaMemcpyDeviceToHost, s));
  // the host copies of the row-offset total and the bases must outlive their copies
  JX_SRV_TRY(cudaStreamSynchronize(s));
  return JX_OK;
}

#undef JX_SRV_TRY

void finish(jx_server_s *S, jx_server_s::Slot *slot, Pass &pass, jx_status st) {
  const int64_t t = now_ns();
  std::lock_guard<std::mutex> lock(S->mu);
  slot->busy = false;
  for (Req *r : pass.reqs) {
    r->status = st;
    r->done_ns = t;
    r->done = true;
    if (st == JX_OK) {
      ++S->completed;
      S->edges += r->e;
      S->lat_ms.push_back((double)(t - r->arrival_ns) * 1e-6);
      if (S->first_arrival == 0 || r->arrival_ns < S->first_arrival) S->first_arrival = r->arrival_ns;
      S->last_done = std::max(S->last_done, t);
    } else {
      ++S->failed;
    }
    ++S->finished;
  }
  ++S->passes;
  if (pass.reqs.size() > 1) S->folded += pass.reqs.size();
  S->reserved -= pass.reserved;
  ++S->free_slots;
  S->cv_queue.notify_all();
  S->cv_done.notify_all();
}

void slot_main(jx_server_s *S, jx_server_s::Slot *slot) {
  cudaSetDevice(S->device);
  for (;;) {
    std::unique_ptr<Pass> pass;
    {
      std::unique_lock<std::mutex> lock(S->mu);
      slot->cv.wait(lock, [&] { return slot->pass || S->stop; });
      if (!slot->pass) return; // stop with nothing to do
      pass = std::move(slot->pass);
    }
    jx_launch_count_reset();
    jx_status st;
    if (pass->reqs.size() == 1) st = run_single(S, *pass->reqs[0], slot->stream);
    else st = run_fold(S, pass->reqs, slot->stream);
    if (st != JX_OK) cudaStreamSynchronize(slot->stream);
    S->kernels += jx_launch_count();
    finish(S, slot, *pass, st);
  }
}

void dispatcher_main(jx_server_s *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lock(S->mu);
  for (;;) {
    S->cv_queue.wait(lock, [&] { return S->stop || (!S->paused && !S->queue.empty() && S->free_slots > 0); });
    if (S->queue.empty() && S->stop) return;
    if (S->queue.empty() || S->free_slots == 0 || (S->paused && !S->stop)) continue;
    Req *head = S->queue.front();
    const size_t budget = S->cfg.memory_budget;
    if (S->resident_bytes + head->need > budget) { // can never fit
      S->queue.pop_front();
      head->status = JX_ERR_TOO_LARGE;
      head->done = true;
      head->done_ns = now_ns();
      ++S->failed;
      ++S->finished;
      S->cv_done.notify_all();
      continue;
    }
    if (S->resident_bytes + S->reserved + head->need > budget) { // wait for memory, in arrival order
      // (or for the head to be cancelled: the queue front then changes)
      S->cv_queue.wait(lock, [&] {
        return S->stop || S->queue.empty() || S->queue.front() != head ||
               S->resident_bytes + S->reserved + head->need <= budget;
      });
      continue;
    }
    auto pass = std::make_unique<Pass>();
    pass->reqs.push_back(head);
    S->queue.pop_front();
    size_t bytes = head->need;
    if (foldable(S, head)) {
      // fold every queued small request of the same kind that still fits
      int64_t fe = head->e;
      int64_t fv = head->n;
      for (auto it = S->queue.begin(); it != S->queue.end();) {
        Req *r = *it;
        if (!foldable(S, r) || !same_kind(head, r) || fe + r->e > S->cfg.fold_max_edges ||
            fv + r->n >= INT32_MAX) {
          ++it;
          continue;
        }
        pass->reqs.push_back(r);
        const size_t fb = fold_bytes(S, pass->reqs);
        if (S->resident_bytes + S->reserved + fb > budget) {
          pass->reqs.pop_back();
          break;
        }
        bytes = fb;
        fe += r->e;
        fv += r->n;
        it = S->queue.erase(it);
      }
    }
    pass->reserved = bytes;
    S->reserved += bytes;
    S->peak_reserved = std::max(S->peak_reserved, S->resident_bytes + S->reserved);
    --S->free_slots;
    for (auto &sl : S->slots)
      if (!sl->busy) {
        sl->busy = true;
        sl->pass = std::move(pass);
        sl->cv.notify_one();
        break;
      }
  }
}

} // namespace
} // namespace jx

extern "C" {

int64_t jx_server_clock_ns(void) { return now_ns(); }

jx_status jx_server_create(const jx_server_config *cfg, jx_server *out) {
  if (!cfg || !out || cfg->slots < 1 || cfg->slots > 64 || cfg->memory_budget == 0 || cfg->fold_edges < 0 ||
      cfg->fold_max_edges < 0 || cfg->schedule.lane_max < 0 || cfg->schedule.warp_max < 0 ||
      cfg->schedule.cta_max < 0 || cfg->schedule.hub_unit < 0 || cfg->schedule.hub_batch < 0)
    return JX_ERR_INVALID;
  *out = nullptr;
  auto S = std::make_unique<jx_server_s>();
  S->cfg = *cfg;
  S->cfg.fold_max_edges = std::min<int64_t>(cfg->fold_max_edges, INT32_MAX);
  cudaError_t ce = cudaGetDevice(&S->device);
  if (ce != cudaSuccess) return set_cuda_error(ce);
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = S->device;
  if ((ce = cudaMemPoolCreate(&S->pool, &props)) != cudaSuccess) return set_cuda_error(ce);
  uint64_t keep = UINT64_MAX; // freed blocks stay in the pool for the next pass
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  for (int i = 0; i < cfg->slots; ++i) {
    auto sl = std::make_unique<jx_server_s::Slot>();
    if ((ce = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking)) != cudaSuccess) {
      for (auto &x : S->slots) cudaStreamDestroy(x->stream);
      cudaMemPoolDestroy(S->pool);
      return set_cuda_error(ce);
    }
    S->slots.push_back(std::move(sl));
  }
  S->free_slots = cfg->slots;
  jx_server_s *raw = S.get();
  for (auto &sl : S->slots) sl->th = std::thread(slot_main, raw, sl.get());
  S->dispatcher = std::thread(dispatcher_main, raw);
  *out = S.release();
  return JX_OK;
}

jx_status jx_server_add_graph(jx_server S, const jx_host_graph *h, int32_t weighted, int32_t *graph_id) {
  if (!S || !h || !graph_id || h->n < 0 || h->e < 0 || (h->n == 0 && h->e > 0) || (h->n > 0 && !h->row_ptr) ||
      (h->e > 0 && !h->col_idx) || (weighted && h->n > 0 && !h->vertex_w))
    return JX_ERR_INVALID;
  Resident R;
  R.n = h->n;
  R.e = h->e;
  for (int32_t v = 0; v < h->n; ++v) R.max_deg = std::max(R.max_deg, h->row_ptr[v + 1] - h->row_ptr[v]);
  R.bytes = align_up(sizeof(int32_t) * ((size_t)h->n + 1)) + align_up(sizeof(int32_t) * (size_t)h->e) +
            (weighted ? 2 * align_up(sizeof(float) * (size_t)h->n) : 0);
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->resident_bytes + S->reserved + R.bytes > S->cfg.memory_budget) return JX_ERR_TOO_LARGE;
    S->resident_bytes += R.bytes;
    S->peak_reserved = std::max(S->peak_reserved, S->resident_bytes + S->reserved);
  }
  cudaStream_t s = nullptr;
  cudaError_t ce = cudaSuccess;
  jx_status st = JX_OK;
  auto fail = [&](jx_status why) {
    cudaFree(R.row_ptr);
    cudaFree(R.col);
    cudaFree(R.w);
    cudaFree(R.S);
    if (s) cudaStreamDestroy(s);
    std::lock_guard<std::mutex> lock(S->mu);
    S->resident_bytes -= R.bytes;
    S->cv_queue.notify_all();
    return why;
  };
  if ((ce = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return fail(set_cuda_error(ce));
  if ((ce = cudaMalloc(&R.row_ptr, sizeof(int32_t) * ((size_t)h->n + 1))) != cudaSuccess ||
      (ce = cudaMalloc(&R.col, sizeof(int32_t) * std::max<size_t>(h->e, 1))) != cudaSuccess ||
      (weighted && (ce = cudaMalloc(&R.w, sizeof(float) * std::max<size_t>(h->n, 1))) != cudaSuccess) ||
      (weighted && (ce = cudaMalloc(&R.S, sizeof(float) * std::max<size_t>(h->n, 1))) != cudaSuccess))
    return fail(set_cuda_error(ce));
  if (h->n > 0)
    ce = cudaMemcpyAsync(R.row_ptr, h->row_ptr, sizeof(int32_t) * ((size_t)h->n + 1), cudaMemcpyHostToDevice, s);
  else
    ce = cudaMemsetAsync(R.row_ptr, 0, sizeof(int32_t), s);
  if (ce == cudaSuccess && h->e > 0)
    ce = cudaMemcpyAsync(R.col, h->col_idx, sizeof(int32_t) * (size_t)h->e, cudaMemcpyHostToDevice, s);
  if (ce == cudaSuccess && weighted && h->n > 0)
    ce = cudaMemcpyAsync(R.w, h->vertex_w, sizeof(float) * (size_t)h->n, cudaMemcpyHostToDevice, s);
  if (ce != cudaSuccess) return fail(set_cuda_error(ce));
  if (weighted && h->n > 0 && (st = jx_rowsum(h->n, h->e, R.row_ptr, R.col, R.w, R.S, (jx_stream_t)s)) != JX_OK)
    return fail(st);
  if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return fail(set_cuda_error(ce));
  cudaStreamDestroy(s);
  std::lock_guard<std::mutex> lock(S->mu);
  S->graphs.push_back(R);
  *graph_id = (int32_t)S->graphs.size() - 1;
  return JX_OK;
}

jx_status jx_server_submit(jx_server S, const jx_request *q, uint64_t *ticket) {
  if (!S || !q || !ticket) return JX_ERR_INVALID;
  if (q->algo != JX_ALGO_VERTEX_CENTRIC && q->algo != JX_ALGO_EDGE_CENTRIC) return JX_ERR_INVALID;
  auto r = std::make_unique<Req>();
  r->graph_id = q->graph_id;
  r->algo = q->algo;
  r->weighted = q->weighted && q->algo == JX_ALGO_VERTEX_CENTRIC;
  r->host_out = q->host_out;
  r->arrival_ns = q->arrival_ns ? q->arrival_ns : now_ns();
  if (q->graph_id < 0) { // an upload: checked and scanned outside the lock
    const jx_host_graph *h = q->graph;
    if (!h || h->n < 0 || h->e < 0 || (h->n == 0 && h->e > 0) || (h->n > 0 && !h->row_ptr) ||
        (h->e > 0 && !h->col_idx) || (r->weighted && h->n > 0 && !h->vertex_w))
      return JX_ERR_INVALID;
    r->up = *h;
    r->n = h->n;
    r->e = h->e;
    for (int32_t v = 0; v < h->n; ++v) r->max_deg = std::max(r->max_deg, h->row_ptr[v + 1] - h->row_ptr[v]);
  }
  std::lock_guard<std::mutex> lock(S->mu);
  if (S->stop) return JX_ERR_INVALID;
  if (q->graph_id >= 0) {
    if (q->graph_id >= (int32_t)S->graphs.size()) return JX_ERR_INVALID;
    r->res = S->graphs[q->graph_id];
    if (r->weighted && !r->res.w) return JX_ERR_INVALID; // resident without weights
    r->n = r->res.n;
    r->e = r->res.e;
    r->max_deg = r->res.max_deg;
  }
  if (r->e > 0 && !r->host_out) return JX_ERR_INVALID;
  r->need = request_bytes(S, *r);
  r->ticket = S->next_ticket++;
  *ticket = r->ticket;
  ++S->submitted;
  Req *raw = r.get();
  S->reqs.emplace(raw->ticket, std::move(r));
  S->queue.push_back(raw);
  S->cv_queue.notify_all();
  return JX_OK;
}

jx_status jx_server_wait(jx_server S, uint64_t ticket, double *latency_ms) {
  if (!S) return JX_ERR_INVALID;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return JX_ERR_INVALID;
  Req *r = it->second.get();
  S->cv_done.wait(lock, [&] { return r->done; });
  const jx_status st = r->status;
  if (latency_ms) *latency_ms = (double)(r->done_ns - r->arrival_ns) * 1e-6;
  S->reqs.erase(it);
  return st;
}

jx_status jx_server_set_paused(jx_server S, int32_t paused) {
  if (!S) return JX_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  S->paused = paused != 0;
  S->cv_queue.notify_all();
  return JX_OK;
}

jx_status jx_server_cancel(jx_server S, uint64_t ticket) {
  if (!S) return JX_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return JX_ERR_INVALID;
  Req *r = it->second.get();
  auto q = std::find(S->queue.begin(), S->queue.end(), r);
  if (r->done || q == S->queue.end()) return JX_ERR_UNSUPPORTED; // started or finished
  S->queue.erase(q);
  r->status = JX_ERR_CANCELLED;
  r->done_ns = now_ns();
  r->done = true;
  ++S->cancelled;
  ++S->finished;
  S->cv_queue.notify_all();
  S->cv_done.notify_all();
  return JX_OK;
}

jx_status jx_server_inject_alloc_failures(jx_server S, int32_t count) {
  if (!S || count < 0) return JX_ERR_INVALID;
  S->inject_alloc.store(count);
  return JX_OK;
}

jx_status jx_server_drain(jx_server S) {
  if (!S) return JX_ERR_INVALID;
  std::unique_lock<std::mutex> lock(S->mu);
  S->cv_done.wait(lock, [&] { return S->finished == S->submitted; });
  return JX_OK;
}

jx_status jx_server_get_stats(jx_server S, jx_server_stats *o) {
  if (!S || !o) return JX_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  *o = jx_server_stats{};
  o->completed = S->completed;
  o->failed = S->failed;
  o->cancelled = S->cancelled;
  o->passes = S->passes;
  o->folded_requests = S->folded;
  o->kernels = S->kernels.load();
  o->edges = S->edges;
  o->peak_reserved = S->peak_reserved;
  if (!S->lat_ms.empty()) {
    std::vector<double> v = S->lat_ms;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
      const size_t i = (size_t)std::min<double>((double)v.size() - 1, std::ceil(p * (double)v.size()) - 1);
      return v[i];
    };
    o->p50_ms = pct(0.50);
    o->p99_ms = pct(0.99);
    o->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    o->mean_ms = sum / (double)v.size();
    o->span_s = (double)(S->last_done - S->first_arrival) * 1e-9;
  }
  return JX_OK;
}

void jx_server_reset_stats(jx_server S) {
  if (!S) return;
  std::lock_guard<std::mutex> lock(S->mu);
  S->lat_ms.clear();
  S->completed = S->failed = S->cancelled = S->passes = S->folded = 0;
  S->edges = 0;
  S->first_arrival = S->last_done = 0;
  S->peak_reserved = S->resident_bytes + S->reserved;
  S->kernels = 0;
}

void jx_server_destroy(jx_server S) {
  if (!S) return;
  jx_server_set_paused(S, 0); // queued requests run before the server goes away
  jx_server_drain(S);
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    S->cv_queue.notify_all();
    for (auto &sl : S->slots) sl->cv.notify_all();
  }
  if (S->dispatcher.joinable()) S->dispatcher.join();
  for (auto &sl : S->slots) {
    if (sl->th.joinable()) sl->th.join();
    cudaStreamDestroy(sl->stream);
  }
  for (Resident &R : S->graphs) {
    cudaFree(R.row_ptr);
    cudaFree(R.col);
    cudaFree(R.w);
    cudaFree(R.S);
  }
  cudaMemPoolDestroy(S->pool);
  delete S;
}

} // extern "C"
