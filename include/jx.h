/*
 * jx -- GB300-native Jaccard engine: C ABI.
 *
 * Plain C, plain pointers and sizes.  Every pointer argument documented as "device" must be
 * device (or managed) memory of the current CUDA device; "host" pointers are host memory.
 * All calls are asynchronous on the given stream unless documented otherwise; a NULL stream
 * is the legacy default stream.  Calls return a status code and never exit the process.
 *
 * Graph model (reference: standalone_csr.hpp:44-105, GraphCSRView<int32_t,int32_t,float>):
 *   row_ptr  int32[n + 1]  CSR offsets, row_ptr[0] = 0, non-decreasing, row_ptr[n] = e
 *   col_idx  int32[e]      neighbours of each row, each row sorted ascending, values in [0, n)
 * Results are per stored directed edge, in CSR order (out[k] belongs to edge k).
 *
 * Numerics follow the reference bit for bit:
 *   - unweighted: J = c / (d_u + d_v - c) with the reference's float expressions
 *     (edge-centric jaccard.cpp:741, vertex-centric jaccard.cpp:258,339,617-618);
 *   - weighted: row sums S in the reference's 32-wide scan order (jaccard.cpp:53-137) and the
 *     intersection weight I accumulated in the order a CPU SYCL device gives the reference's
 *     8 i-lanes (jaccard.cpp:343, 370-396): ref positions 0,8,16,..., then 1,9,17,..., ...
 *     The reference adds those lanes with unordered atomics, so this is one legal schedule of
 *     it (work-items in linear-id order, as its CPU device runs them): a runtime that schedules
 *     the lanes differently gives other weighted results, which can differ from these by more
 *     than 1e-6 relative (the reference order's own error against FP64 reaches 2.5e-6).
 *   - IEEE float division (no fast math).
 */
#ifndef JX_H
#define JX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t. */
typedef struct CUstream_st *jx_stream_t;

typedef enum {
  JX_OK = 0,
  JX_ERR_INVALID = 1,     /* bad argument (NULL pointer, negative size, ...) */
  JX_ERR_CUDA = 2,        /* a CUDA call failed; jx_last_cuda_error() has the code */
  JX_ERR_NOMEM = 3,       /* device or host allocation failed */
  JX_ERR_BAD_GRAPH = 4,   /* jx_csr_check found an invalid CSR */
  JX_ERR_UNSUPPORTED = 5, /* valid request outside what this library supports */
  JX_ERR_TOO_LARGE = 6,   /* size above a documented maximum */
  JX_ERR_CANCELLED = 7    /* a server request was cancelled before it started */
} jx_status;

typedef enum {
  JX_ALGO_VERTEX_CENTRIC = 0, /* sygraph::jaccard<false, ...>  RowSum -> IS -> JW */
  JX_ALGO_EDGE_CENTRIC = 1    /* sygraph::jaccard<true, ...>   ec_scan -> ec_unweighted */
} jx_algo;

/* Device-pointer view of an int32 CSR graph (GraphCSRView, standalone_csr.hpp:44-105). */
typedef struct {
  int32_t n;              /* number_of_vertices */
  int32_t e;              /* number_of_edges (stored directed edges) */
  const int32_t *row_ptr; /* offsets, device, n + 1 */
  const int32_t *col_idx; /* indices, device, e */
} jx_csr;

/* Bits reported by jx_csr_check. */
#define JX_CSR_OFFSETS_BAD 0x1u /* row_ptr[0] != 0, decreasing, or row_ptr[n] != e */
#define JX_CSR_INDEX_RANGE 0x2u /* some col_idx outside [0, n) */
#define JX_CSR_UNSORTED 0x4u    /* some row not sorted ascending */
#define JX_CSR_DUPLICATE 0x8u   /* some row holds the same neighbour twice */
#define JX_CSR_SELF_LOOP 0x10u  /* some row lists itself */
#define JX_CSR_ASYMMETRIC 0x20u /* some edge (u,v) has no (v,u) */

const char *jx_status_string(jx_status s);
int jx_version(void);        /* 10000 * major + 100 * minor + patch */
int jx_last_cuda_error(void); /* cudaError_t of the last JX_ERR_CUDA on this thread */

/* ------------------------------------------------------------------ whole-operator calls */

/*
 * Jaccard for every stored edge: the drop-in for
 *   sygraph::jaccard<edge_centric, int32_t, int32_t, float>(graph, [weights,] result, q)
 * (standalone_algorithms.hpp:67-69 weighted, :86-87 unweighted; jaccard.cpp:926-955).
 *
 *   vertex_w  device float[n] per-vertex weights, or NULL for unweighted.  The edge-centric
 *             algorithm ignores weights, as the reference does (jaccard.cpp:790).
 *   out_j     device float[e], written once per edge.
 * Temporaries are taken from the stream-ordered allocator and released before return
 * (stream-ordered); use jx_jaccard_ws to supply them instead.  Asynchronous.
 */
jx_status jx_jaccard(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                     jx_stream_t stream);

/* Bytes of device workspace jx_jaccard_ws needs for this graph (a host-side bound). */
size_t jx_jaccard_workspace_size(const jx_csr *g, int weighted, jx_algo algo);

/* jx_jaccard with caller-provided device workspace (256-byte aligned, >= the size above). */
jx_status jx_jaccard_ws(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                        void *workspace, size_t workspace_bytes, jx_stream_t stream);

/*
 * Schedule of one operator call: how the rows are split into degree bins and launched.  (This
 * library's addition: the reference has one fixed launch shape per kernel.)  Results never
 * depend on the schedule, only the speed does.  A zero field takes its default.
 */
typedef struct {
  int32_t persistent; /* 1: one persistent launch walks the CTA, warp and lane rows; 0 (default):
                         one kernel per bin */
  int32_t lane_max;   /* rows of at most this many neighbours: one lane per task (1..32, default 32) */
  int32_t warp_max;   /* ... one warp per row (lane_max..512, default 512) */
  int32_t cta_max;    /* ... one 1024-thread CTA per row (warp_max..24576, default 24576); longer
                         rows are split into hub work units run by CTA clusters */
  int32_t hub_unit;   /* largest tasks per hub work unit (default 65536); units shrink, to no
                         less than 4096 tasks, until every resident hub cluster has 4 */
  int32_t hub_batch;  /* tasks a hub warp takes per fetch (1..32, default 2) */
  int32_t hub_beside; /* 1: the hub kernel runs on a second stream beside the row kernels;
                         -1: before them on the call's stream; 0: the library default */
  int32_t hub_cluster;/* CTAs per hub cluster, 4 or 8 (default 4); 0: the library default */
  int32_t relabel;    /* 1: the row kernels work on vertex ids renumbered by degree (high-degree
                         vertices first; the lists stay in place, their entries mapped), at the
                         cost of a copy of col_idx in the workspace -- faster on graphs whose own
                         ids scatter the high-degree vertices; -1 or 0 (default): the graph's
                         own ids */
} jx_schedule;

/* jx_jaccard_ws under a given schedule (NULL: the default one), and its workspace size. */
size_t jx_jaccard_schedule_workspace_size(const jx_csr *g, int weighted, jx_algo algo, const jx_schedule *sch);
jx_status jx_jaccard_schedule(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                              const jx_schedule *sch, void *workspace, size_t workspace_bytes,
                              jx_stream_t stream);

/*
 * Host-buffer form of jx_jaccard: the reference's buffers wrap host memory
 * (main.cpp:196-200), so this entry point takes host arrays, copies them to the device,
 * runs the operator and copies the results back.  Synchronous.  Pinned host memory gives
 * the fastest copies; pageable memory works.  The device buffers come from a memory pool this
 * library owns (one per device) that keeps freed memory mapped for the next call, on a stream
 * of the calling thread's own; jx_host_release() returns that memory to the device.
 */
jx_status jx_jaccard_host(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *col_idx,
                          const float *vertex_w, float *out_j, jx_algo algo);

/* Pinned (page-locked) host memory for jx_jaccard_host's arrays, from the CUDA runtime this
 * library uses: copies from and to it run at the host link's rate.  (Host memory pinned by other
 * means can sit far from the GPU: on the GB300 host, arrays pinned by PyTorch uploaded at about
 * 16 GB/s against 37 GB/s for this memory, and downloaded at 14 against 189 GB/s.)  Free with
 * jx_host_free.  Synchronous. */
jx_status jx_host_alloc(size_t bytes, void **ptr);
jx_status jx_host_free(void *ptr);

/* Waits for the device, then frees the device memory jx_jaccard_host keeps between calls on the
 * current device.  (The reference frees its temporaries at every call's end,
 * jaccard.cpp:931-938; keeping them is this library's choice for repeated calls.) */
jx_status jx_host_release(void);

/*
 * jx_jaccard without any device allocation.  (No counterpart in the reference.)
 *
 * For callers that cannot allocate device memory while they run: services that reserve their
 * whole device-memory budget up front and own no allocator, and pipelines in which an
 * allocation call, with the device synchronisation it may bring, is not acceptable between
 * launches.  The operator, its arguments and its results are those of jx_jaccard; the
 * workspace is a fixed array of JX_NOALLOC_SCRATCH_BYTES inside this library (every GPU that
 * loads the library holds it until the process exits), sized for graphs of at most
 * JX_NOALLOC_MAX_VERTICES vertices; larger graphs are rejected with JX_ERR_TOO_LARGE.
 * The first call on a device looks up the array's device address (a host-side set-up step),
 * and so does the first call after the device's context was reset (cudaDeviceReset); make
 * those calls before any stream capture.  Every call shares the one array: calls
 * that overlap on the GPU (on different streams, or from different threads) race and must be
 * serialised by the caller.  Asynchronous on `stream`; the work is smaller-grid than
 * jx_jaccard and so slower on large graphs.
 */
#define JX_NOALLOC_MAX_VERTICES (1 << 20)
#define JX_NOALLOC_SCRATCH_BYTES (32u << 20)
jx_status jx_jaccard_noalloc(const jx_csr *g, const float *vertex_w, float *out_j, jx_algo algo,
                             jx_stream_t stream);

/* ------------------------------------------------------------------ stage-level calls
 * One call per reference kernel (the static invoke functions of jaccard.hpp), for stage
 * parity and for callers that, like main.cpp:255-257, drive the kernels themselves.
 */

/* Jaccard_RowSumKernel<w>::invoke (jaccard.hpp:104-107, jaccard.cpp:263-313).
 * work[r] = (float)(row_ptr[r+1]-row_ptr[r]) when w == NULL, else the reference-order sum of
 * w[ind[k]] over the row.  `ind` is any int32[e] index array (main.cpp:213-257 passes
 * 0..e-1 with edge weights to build vertex weights).  device pointers. */
jx_status jx_rowsum(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *ind,
                    const float *w, float *work, jx_stream_t stream);

/* FillKernel<float>::invoke (jaccard.hpp:51-52, jaccard.cpp:161-182): x[0..n) = value. */
jx_status jx_fill(int64_t n, float *x, float value, jx_stream_t stream);

/* Jaccard_IsKernel<w>::invoke (jaccard.hpp:151-156, jaccard.cpp:402-458):
 *   weight_s[j]  = work[row] + work[col]
 *   weight_i[j] += sum over common neighbours (1 or w[k]), starting from weight_i[j]'s
 *                  current value, in the reference's order.
 * w may be NULL (unweighted).  device pointers. */
jx_status jx_intersect(int32_t n, int32_t e, const int32_t *row_ptr, const int32_t *col_idx,
                       const float *w, const float *work, float *weight_i, float *weight_s,
                       jx_stream_t stream);

/* Jaccard_JwKernel::invoke (jaccard.hpp:235-237, jaccard.cpp:622-653):
 * weight_j[j] = weight_i[j] / (weight_s[j] - weight_i[j]). */
jx_status jx_weight(int32_t e, const float *weight_i, const float *weight_s, float *weight_j,
                    jx_stream_t stream);

/* Jaccard_ec_scan::invoke (jaccard.hpp:256-258, jaccard.cpp:666-700):
 * dest_ind[k] = row of edge k, weight_j[k] = 0. */
jx_status jx_ec_scan(int32_t e, int32_t n, const int32_t *row_ptr, int32_t *dest_ind,
                     float *weight_j, jx_stream_t stream);

/* Jaccard_ec_unweighted::invoke (jaccard.hpp:280-283, jaccard.cpp:745-782):
 * weight_j[k] += matches, then weight_j[k] = c / ((float)(Ni + Nj) - c). */
jx_status jx_ec_unweighted(int32_t e, int32_t n, const int32_t *row_ptr, const int32_t *col_idx,
                           const int32_t *dest_ind, float *weight_j, jx_stream_t stream);

/* ------------------------------------------------------------------ next to the path */

/* jaccard_list (standalone_algorithms.hpp:109-133, jaccard.cpp:957-988): J for explicit pairs
 * (first[p], second[p]), p < num_pairs, computed like the vertex-centric edge (first, second)
 * (same ref/cur rule, same accumulation order, J = I / (S_first + S_second - I)).  The
 * reference's pair kernel accumulates into the wrong slot (jaccard.cpp:517, 528); this is the
 * intended result.  vertex_w NULL = unweighted.  Pair vertices must lie in [0, n).
 * device pointers; asynchronous. */
jx_status jx_jaccard_list(const jx_csr *g, const float *vertex_w, int64_t num_pairs,
                          const int32_t *first, const int32_t *second, float *out,
                          jx_stream_t stream);

/* The reference's edge-centric driver's "non zero pairs" count (jaccard.cpp:810-819): *count (device,
 * unsigned long long) = number of values[k] > thresh (the reference uses 0.00001). */
jx_status jx_count_above(int64_t e, const float *values, float thresh, unsigned long long *count,
                         jx_stream_t stream);

/* Reverse-edge removal of the reference program's output path (main.cpp:307-309,
 * readMtxToCSR.cpp:134-147): keeps (a,b,v) when a > b, or a < b and the reverse edge is absent
 * or holds a different value; drops self loops.  Writes the survivors in CSR order to
 * src/dst/out_values (device, capacity e) and their number to *count (device int64). */
jx_status jx_remove_reverse_edges(const jx_csr *g, const float *values, int32_t *src, int32_t *dst,
                                  float *out_values, int64_t *count, jx_stream_t stream);

/* Graph preparation of the reference's driver on the device (main.cpp:99-118: reverse edges
 * added to the MTX set, then mtxSetToCSR, readMtxToCSR.cpp:117-208): from an edge list to a
 * CSR with every row sorted ascending, no repeated neighbour and, unless kept, no self loop.
 *   src, dst   device int32[m], zero-based vertex ids in [0, n) (else JX_ERR_INVALID);
 *   flags      JX_BUILD_SYMMETRIZE adds (v, u) for every (u, v) (the reference's
 *              invertDirection for undirected input); JX_BUILD_KEEP_SELF_LOOPS keeps (u, u);
 *   row_ptr    device int32[n + 1] out; col device int32[cap] out (cap >= m, or 2m when
 *              symmetrising, always suffices); *e_out (host) the number of stored edges.
 * Unlike the reference, every vertex in [0, n) keeps its row (the reference's rows start at the
 * first source and end at the last, readMtxToCSR.cpp:158-179), and edge values are not
 * carried (the operators use per-vertex weights).  JX_ERR_TOO_LARGE when the result exceeds
 * cap or 2^31 - 1 edges.  Synchronous on `stream` (it reads back the edge count);
 * temporaries (about 40 bytes per input edge) from the stream-ordered allocator. */
#define JX_BUILD_SYMMETRIZE 0x1u
#define JX_BUILD_KEEP_SELF_LOOPS 0x2u
jx_status jx_csr_build(int32_t n, int64_t m, const int32_t *src, const int32_t *dst, uint32_t flags,
                       int32_t *row_ptr, int32_t *col, int64_t cap, int64_t *e_out, jx_stream_t stream);

/* ------------------------------------------------------------------ batched mode
 * Many graphs packed into one offset-indexed super-CSR on the device (graph g's vertex ids
 * shifted by the vertices before it, its edges by the edges before it; at most 2^31 - 1
 * edges and vertices in total, larger batches are split by the caller).  The graphs are
 * disjoint components, so one operator pass over the super-CSR gives each graph its own
 * results as a contiguous slice.  The pass is captured once as a CUDA graph and replayed by
 * jx_batch_run.  tune != 0 times candidate schedules on the batch and keeps the fastest: one
 * kernel per degree bin against the persistent row launch, bin limits, the hub fetch cap, the
 * hub kernel beside or before the row kernels, and the grids of the lane and warp kernels
 * (jx_batch_info names the one kept).  (Batching is this library's addition; the reference scores one graph
 * per call.) */
typedef struct {
  int32_t n, e;
  const int32_t *row_ptr; /* host, n + 1 */
  const int32_t *col_idx; /* host, e */
  const float *vertex_w;  /* host, n; required when the batch is weighted */
} jx_host_graph;

typedef struct jx_batch_s *jx_batch;

/* Copies the graphs to the device (synchronous; the host arrays may be freed afterwards). */
jx_status jx_batch_create(const jx_host_graph *graphs, int32_t ngraphs, jx_algo algo, int weighted,
                          int tune, jx_batch *out);
/* One pass over every graph of the batch (asynchronous on `stream`).  Passes of one batch
 * share its workspace and outputs: do not let two of them overlap (issue them on one stream,
 * or synchronise between streams). */
jx_status jx_batch_run(jx_batch b, jx_stream_t stream);
/* Device slice of graph g's results (valid until destroy). */
jx_status jx_batch_result(jx_batch b, int32_t g, const float **device_out, int64_t *count);
/* Copy graph g's results to host memory (synchronous on `stream`); g = -1 copies the results
 * of every graph, concatenated in batch order (the whole super-CSR output). */
jx_status jx_batch_download(jx_batch b, int32_t g, float *host_out, jx_stream_t stream);
jx_status jx_batch_info(jx_batch b, int64_t *vertices, int64_t *edges, uint64_t *kernels_per_run,
                        char *plan_desc, size_t len);
void jx_batch_destroy(jx_batch b);

/* ------------------------------------------------------------------ serving
 * A request loop on one GPU (this library's addition; the reference has no server).  A
 * request scores every edge of one graph: a graph kept resident on the device by
 * jx_server_add_graph (with its row sums when weighted), or a host CSR uploaded with the
 * request.  Requests are admitted in arrival order while the device-memory budget allows
 * (resident graphs count against it); small requests that are queued together are folded into
 * one super-CSR pass (disjoint components, so every request's results are exactly its own);
 * up to `slots` passes are in flight at once, each on its own stream, so requests that arrive
 * while others run overlap with them on the device.  Results are written to the request's
 * host buffer. */
typedef struct {
  size_t memory_budget;   /* device bytes for resident graphs + admitted requests */
  int32_t slots;          /* passes in flight at once (>= 1), one stream and host thread each */
  int64_t fold_edges;     /* requests of at most this many edges may be folded together */
  int64_t fold_max_edges; /* edges of one folded pass at most */
  jx_schedule schedule;   /* launch schedule of every pass (zero fields: defaults) */
} jx_server_config;

typedef struct {
  int32_t graph_id;            /* >= 0: a resident graph; -1: upload `graph` */
  const jx_host_graph *graph;  /* host CSR (weights too when weighted), graph_id == -1 only;
                                  must stay valid until the request completes */
  jx_algo algo;
  int32_t weighted;            /* vertex-centric only: use the graph's vertex weights */
  float *host_out;             /* e floats, the graph's CSR edge order; written on completion */
  int64_t arrival_ns;          /* arrival time on jx_server_clock_ns() (0: at submit) */
} jx_request;

typedef struct {
  uint64_t completed, failed;
  uint64_t passes;          /* operator passes run (single or folded) */
  uint64_t folded_requests; /* requests that shared a pass with others */
  uint64_t kernels;         /* kernels launched by the passes */
  int64_t edges;            /* edges scored by completed requests */
  double p50_ms, p99_ms, mean_ms, max_ms; /* arrival -> results in host memory */
  double span_s;            /* first arrival -> last completion */
  size_t peak_reserved;     /* most device bytes admitted at once (resident graphs included) */
  uint64_t cancelled;       /* requests cancelled before they started (not in `failed`) */
} jx_server_stats;

typedef struct jx_server_s *jx_server;

jx_status jx_server_create(const jx_server_config *cfg, jx_server *out);
/* Upload a graph to stay resident (row sums computed now when weighted); synchronous. */
jx_status jx_server_add_graph(jx_server s, const jx_host_graph *g, int32_t weighted, int32_t *graph_id);
/* Queue a request; returns at once.  JX_ERR_TOO_LARGE (at wait) when it alone exceeds the
 * budget. */
jx_status jx_server_submit(jx_server s, const jx_request *r, uint64_t *ticket);
/* Wait for one request; returns its status, *latency_ms its arrival -> completion time. */
jx_status jx_server_wait(jx_server s, uint64_t ticket, double *latency_ms);
/* Wait for every request submitted so far. */
jx_status jx_server_drain(jx_server s);
jx_status jx_server_get_stats(jx_server s, jx_server_stats *out);
void jx_server_reset_stats(jx_server s);
/* The server's clock (monotonic, nanoseconds) for jx_request.arrival_ns. */
int64_t jx_server_clock_ns(void);
/* paused != 0: admit nothing new (passes already started run to completion; submitted requests
 * wait in the queue); paused == 0: resume admission. */
jx_status jx_server_set_paused(jx_server s, int32_t paused);
/* Cancel a request that has not started: JX_OK, its jx_server_wait returns JX_ERR_CANCELLED and
 * its host buffer is not written.  JX_ERR_UNSUPPORTED when it has already started or finished
 * (it runs to completion); JX_ERR_INVALID for an unknown ticket.  (The reference reports a
 * failed kernel and carries on, jaccard.cpp:178-180; a request here fails alone likewise.) */
jx_status jx_server_cancel(jx_server s, uint64_t ticket);
/* Failure injection for tests of the server's error handling, on the host: the next `count`
 * device allocations made for passes fail as if the device were out of memory, without calling
 * the allocator.  The requests of an affected pass complete with JX_ERR_NOMEM; other passes
 * and requests are unaffected. */
jx_status jx_server_inject_alloc_failures(jx_server s, int32_t count);
/* Drains, then releases every resident graph and the server's threads and streams. */
void jx_server_destroy(jx_server s);

/* ------------------------------------------------------------------ utilities */

/* Validate a CSR on the device; *flags receives JX_CSR_* bits (0 = valid, sorted, symmetric).
 * Synchronous on `stream`. */
jx_status jx_csr_check(const jx_csr *g, uint32_t *flags, jx_stream_t stream);

/* Per-launch timing of the fused operator on this thread: jx_profile_begin() starts
 * recording an event after each kernel the operator launches (and, in jx_jaccard_host, after
 * its copies in and out); jx_profile_end() waits for them and writes "name=ms;name=ms;..."
 * into buf (NUL-terminated, truncated to len), each time measured from the previous event on
 * the same stream.  Returns the number of timed launches.  Diagnostic only; adds event records
 * to the stream. */
void jx_profile_begin(void);
int jx_profile_end(char *buf, size_t len);

/* Number of kernels this library launched on this thread since the last reset. */
uint64_t jx_launch_count(void);
void jx_launch_count_reset(void);

#ifdef __cplusplus
}
#endif

#endif /* JX_H */
