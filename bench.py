"""Benchmark: edges scored per second by the fused Jaccard operator on one GB300.

Workload (default): the large weighted configuration -- R-MAT scale 24, edge factor 16,
(a,b,c,d) = (.57,.19,.19,.05), seed 3, symmetrised / deduplicated / loop-free int32 CSR, with
per-vertex float32 weights uniform in (0,1] (seed 4); vertex-centric weighted Jaccard for
every stored edge.  Synthetic data of the named shape (there is no dataset).

A step is one call of the operator (``jx_jaccard_ws``) over the whole graph, resident in
HBM.  The graph (2.2 GB) is far larger than L2 (129 MB), so no L2 flush is needed between
steps.  Timing: W warm-up steps, then K steps between a barrier + synchronize on both sides,
CUDA events on the launching stream, max over ranks.  ``e2e`` times the host-buffer entry
point (``jx_jaccard_host``): pinned host arrays in, results out, copies inside the timed
region.  ``cpu_baseline`` times the reference's own kernels (through the host SYCL subset)
on a bounded, evenly spread sample of work-groups, on this machine's host cores.

``--impl reference`` runs only that CPU reference arm and prints its own line.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
METRIC = "edges scored/s"
UNIT = "edges/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def byte_model(V, E, sum_min, weighted):
    """Designated algorithmic bytes of one operator call (per-edge must-read model)."""
    b = 4 * (V + 1) + 16 * E + 4 * sum_min
    if weighted:
        b += 4 * (V + 1) + 8 * E + 4 * V + 4 * E
    return b


# DRAM bytes (read + write) of one operator call, summed over its kernels, from a one-pass ncu
# capture of the full-size call (profiles/traffic_rmat24_vc_weighted_unweighted.md).  Keyed by
# (workload, weighted, edge_centric); other configurations report null.
MEASURED_TRAFFIC = {
    ("rmat24w", True, False): 1254507681024,
    ("rmat24w", False, False): 1046260130560,
}


def l2_note(input_bytes):
    """How the timed steps relate to the 129 MB L2 (no flush between steps either way)."""
    if input_bytes > 129e6:
        return f"inputs ({input_bytes / 1e9:.2f} GB) larger than L2 (129 MB); no flush"
    return f"inputs ({input_bytes / 1e6:.1f} MB) fit in L2: warm-L2 numbers, no flush"


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_graph(name, threads):
    jx = importlib.import_module("sycl-jaccard_gb300")
    t = time.time()
    rp, col, w, desc = jx.graphgen.config_graph(name, threads=threads)
    st = jx.graphgen.stats(rp, col)
    log(f"graph {name}: V={st['V']} E={st['E']} max_deg={st['max_degree']} sum_min={st['sum_min']:.4g} "
        f"({time.time() - t:.1f}s)")
    return rp, col, w, desc, st


# ------------------------------------------------------------------ CPU reference arm

def sampled_rows(n, K, r):
    """Rows the reference's IS kernel processes when only work-groups g % K == r run.

    Jaccard_IsKernel::invoke (jaccard.cpp:414-418) uses groups of 8 rows and a grid of
    min(ceil(n/8), 65535) groups with a row grid-stride, so row x belongs to group
    ((x mod G0) // 8) with G0 = 8 * min(ceil(n/8), 65535).
    """
    G0 = 8 * min((n + 7) // 8, 65535)
    x = np.arange(n, dtype=np.int64)
    return ((x % G0) // 8) % K == r


def row_work(rp, col):
    """Per-row cost proxy of the reference's IS kernel: sum over the row's edges of
    min(d_u, d_v) * (1 + log2(max(d_u, d_v))) (binary searches of the shorter list)."""
    n = len(rp) - 1
    d = np.diff(rp.astype(np.int64))
    work = np.zeros(n, np.float64)
    step = 1 << 20
    for s in range(0, n, step):
        e0, e1 = int(rp[s]), int(rp[min(n, s + step)])
        du = np.repeat(d[s:min(n, s + step)], d[s:min(n, s + step)])
        dv = d[col[e0:e1]]
        c = np.minimum(du, dv) * (1.0 + np.log2(np.maximum(np.maximum(du, dv), 1)))
        rows = np.repeat(np.arange(s, min(n, s + step)), d[s:min(n, s + step)])
        work += np.bincount(rows, weights=c, minlength=n)
    return work


def cpu_reference(rp, col, w, target_s=20.0):
    """Time the reference (through the host SYCL subset) on a bounded work-group sample.

    Fixed per-call cost `a` (the reference allocates 12E + 4V bytes of temporaries per call,
    jaccard.cpp:931-934) is timed with a sample that runs no work-group.  Then every K-th
    work-group (residue K/2, evenly spread over the row range through the kernels' grid
    strides) runs; K is chosen for about target_s seconds.  The whole-graph call time is
    extrapolated by the sampled share of the IS kernel's work (row_work):
        T = a + (t_K - a) * W_total / W_sampled,   reported rate = E / T.
    """
    from oracle import oracle as O
    kind = "reference"
    try:
        L = O.ref_lib()
    except Exception as exc:  # build failure on this machine
        log(f"reference build unavailable: {exc}")
        L = None
    threads = os.cpu_count() or 1
    n, E = len(rp) - 1, len(col)
    work = row_work(rp, col)
    W = work.sum()

    def timed(K, r):
        t0 = time.perf_counter()
        if kind == "reference":
            O.ref_jaccard(rp, col, w, edge_centric=False, threads=threads, group_sample=K, group_residue=r)
        else:
            rows = (r, min(n, r + max(1, n // K)))
            O.jaccard(rp, col, w, rows=rows, threads=threads)
        return time.perf_counter() - t0

    if L is None:
        kind = "port"
    if kind == "reference":
        a = timed(1 << 40, (1 << 40) - 1)
        share = lambda K: work[sampled_rows(n, K, K // 2)].sum() / W
    else:
        a = 0.0
        share = lambda K: work[K // 2: min(n, K // 2 + max(1, n // K))].sum() / W
    K = 4096
    t_cal = timed(K, K // 2)
    full = max(t_cal - a, 1e-4) / max(share(K), 1e-12)
    K = 1
    while K < (1 << 20) and full * share(K * 2) >= target_s:
        K *= 2
    while K > 1 and full * share(K) < target_s / 2:
        K //= 2
    t = timed(K, K // 2)
    sh = share(K)
    T = a + max(t - a, 1e-6) / max(sh, 1e-12)
    if kind == "reference":
        sel = sampled_rows(n, K, K // 2)
        edges = int(np.diff(rp.astype(np.int64))[sel].sum())
        sample = (f"reference jaccard.cpp (VC{' weighted' if w is not None else ''}) via host SYCL "
                  f"subset, work-groups g % {K} == {K // 2} of each kernel ({edges} of {E} edges, "
                  f"{sh:.2e} of the IS work), {threads} threads; fixed per-call cost {a:.2f}s + "
                  f"sampled {t - a:.2f}s, extrapolated to the whole graph by work share")
    else:
        sample = f"C restatement (oracle port), a row range with {sh:.2e} of the work, {threads} threads"
    return {"value": E / T, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample,
            "seconds": round(a + t + t_cal, 3), "extrapolated_call_s": round(T, 2)}


# ------------------------------------------------------------------ batched workload

INT32_MAX = (1 << 31) - 1


def make_batch(threads):
    jx = importlib.import_module("sycl-jaccard_gb300")
    t = time.time()
    graphs = jx.graphgen.batch_graphs(2000, seed=5, threads=threads)
    st = [jx.graphgen.stats(rp, col) for rp, col, _ in graphs]
    log(f"batch: {len(graphs)} graphs V={sum(x['V'] for x in st)} E={sum(x['E'] for x in st)} "
        f"({time.time() - t:.1f}s)")
    return graphs, st


def super_batches(st):
    """Split the graph list, in order, into groups of at most 2^31 - 1 edges and vertices."""
    groups, cur, ce, cv = [], [], 0, 0
    for i, x in enumerate(st):
        if cur and (ce + x["E"] > INT32_MAX or cv + x["V"] + 1 >= INT32_MAX):
            groups.append(cur)
            cur, ce, cv = [], 0, 0
        cur.append(i)
        ce += x["E"]
        cv += x["V"]
    if cur:
        groups.append(cur)
    return groups


def cpu_reference_batch(graphs, st, target_s=20.0, weights=None, what="graphs of the batch"):
    """Reference on the host cores over a stratified sample of a list of graphs: 8 graphs
    evenly spaced in edge-count order, each timed with cpu_reference's work-group sampling; the
    rate is (sum of their edges) / (sum of their extrapolated call times).  weights: per-graph
    vertex weights (weighted VC) or None (unweighted VC)."""
    order = np.argsort([x["E"] for x in st], kind="stable")
    pick = [int(order[int(q)]) for q in np.linspace(0, len(order) - 1, 8)]
    E = T = 0.0
    threads, kind = None, None
    for i in pick:
        rp, col = graphs[i][0], graphs[i][1]
        cb = cpu_reference(rp, col, None if weights is None else weights[i], target_s / len(pick))
        E += st[i]["E"]
        T += cb["extrapolated_call_s"]
        threads, kind = cb["cores"], cb["kind"]
    return {"value": E / T, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"reference jaccard.cpp (VC{' weighted' if weights is not None else ''}) on 8 {what} "
                      f"evenly spaced in edge count "
                      f"({int(E)} edges), each on a work-group sample extrapolated to its whole call; "
                      f"rate = sum of edges / sum of call times",
            "extrapolated_call_s": round(T, 3)}


def run_gpu_batched(args, world, rank, local):
    import torch
    jx = importlib.import_module("sycl-jaccard_gb300")
    torch.cuda.set_device(local)
    threads = os.cpu_count() or 1
    graphs, st = make_batch(threads)
    groups = super_batches(st)
    V = sum(x["V"] for x in st)
    E = sum(x["E"] for x in st)
    stream = torch.cuda.current_stream()

    # batched form: one super-CSR per group, autotuned plan, captured CUDA graph
    t = time.time()
    batches = [jx.Batch([graphs[i][:2] for i in grp], tune=True) for grp in groups]
    infos = [b.info() for b in batches]
    log(f"batched: {len(batches)} super-CSRs built and tuned ({time.time() - t:.1f}s): "
        + "; ".join(i["plan"] for i in infos))

    def batched_step():
        for b in batches:
            b.run(stream)

    # plain form: the same graphs resident one by one, one operator call each
    plain_g = [jx.GraphCSRView.from_numpy(rp, col, device=f"cuda:{local}") for rp, col, _ in graphs]
    plain_out = torch.empty(E, dtype=torch.float32, device="cuda")
    eoff = np.concatenate([[0], np.cumsum([x["E"] for x in st])])
    ws = torch.empty(max(jx.workspace_size(g, False, False) for g in plain_g), dtype=torch.uint8, device="cuda")
    outs = [plain_out[int(eoff[i]):int(eoff[i + 1])] for i in range(len(graphs))]

    def plain_step():
        for g, o in zip(plain_g, outs):
            if o.numel():
                jx.jaccard(g, None, o, workspace=ws)

    def timed(step, steps, warmup, clocks=False):
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        jx.launch_count_reset()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            ev0.record(stream)
            for _ in range(steps):
                step()
            ev1.record(stream)
            torch.cuda.synchronize()
        launches = jx.launch_count()
        barrier(world)
        ms = max_over_ranks(ev0.elapsed_time(ev1) / steps, world)
        return ms, launches, clk.summary()

    ms, launches, clocks = timed(batched_step, args.steps, args.warmup)
    plain_ms, plain_launches, _ = timed(plain_step, max(1, args.steps // 2), 1)
    # identical results: every graph's slice of the batch equals its plain call, bit for bit
    plain_host = plain_out.cpu().numpy().view(np.uint32)
    for b, grp in zip(batches, groups):
        lo, hi = int(eoff[grp[0]]), int(eoff[grp[-1] + 1])
        if not np.array_equal(b.download(-1).view(np.uint32), plain_host[lo:hi]):
            raise AssertionError("batched results differ from the per-graph calls")

    # end to end through the public batch API: host CSRs (pinned) in, every result out
    e2e = None
    if not args.no_e2e:
        pinned = [(torch.from_numpy(rp).pin_memory().numpy(), torch.from_numpy(col).pin_memory().numpy())
                  for rp, col, _ in graphs]
        h_out = torch.empty(E, dtype=torch.float32).pin_memory().numpy()
        def e2e_step():
            for grp in groups:
                b = jx.Batch([pinned[i] for i in grp])
                b.run(stream)
                lo, hi = int(eoff[grp[0]]), int(eoff[grp[-1] + 1])
                b.download(-1, out=h_out[lo:hi], stream=stream)
                b.close()
        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, world)
        e2e = {"value": E * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 4 * (V + len(graphs)) + 4 * E,
               "d2h_bytes_per_step": 4 * E, "ms_per_step": round(e2e_s * 1e3, 3),
               "timing": "host wall clock: jx_batch_create (packing, no tuning) + run + download-all, per super-CSR"}
        if not np.array_equal(h_out.view(np.uint32), plain_host):
            raise AssertionError("end-to-end batch results differ from the per-graph calls")

    B = sum(byte_model(x["V"], x["E"], x["sum_min"], False) for x in st)
    peak, peak_kind = hbm_peak()
    achieved = B / (ms * 1e-3) / 1e9
    result = {
        "metric": METRIC, "value": E * world / (ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "batched: 2000 graphs seed 5, V log-uniform [256, 262144], half ER "
                               "(avg degree U[4,64]) half RMAT (ef U[8,32], .57/.19/.19), unit weights "
                               "(scored unweighted: identical values)",
                   "algorithm": "vertex_centric", "graphs": len(graphs), "super_csrs": len(groups),
                   "V": V, "E": E, "plans": [i["plan"] for i in infos],
                   "kernels_per_pass": sum(i["kernels_per_run"] for i in infos),
                   "l2": f"inputs ({(4 * (V + E)) / 1e9:.1f} GB) larger than L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches,
        "plain": {"value": E * world / (plain_ms * 1e-3), "unit": UNIT, "ms_per_step": round(plain_ms, 3),
                  "gpu_launches": plain_launches,
                  "what": "one jx_jaccard_ws call per graph, graphs resident, shared workspace"},
        "batched_over_plain": round(plain_ms / ms, 3),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "kernel": "one captured pass over every super-CSR", "algorithmic_bytes": B},
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            result["cpu_baseline"] = cpu_reference_batch(graphs, st, args.cpu_seconds)
        except Exception as exc:
            result["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
    for b in batches:
        b.close()
    return result


# ------------------------------------------------------------------ served workload

def make_served(threads):
    jx = importlib.import_module("sycl-jaccard_gb300")
    t = time.time()
    res, up = jx.graphgen.served_pools(seed=6, threads=threads)
    st_res = [jx.graphgen.stats(g[0], g[1]) for g in res]
    st_up = [jx.graphgen.stats(g[0], g[1]) for g in up]
    log(f"served pools: {len(res)} resident (E={sum(x['E'] for x in st_res)}), {len(up)} uploads "
        f"(E={sum(x['E'] for x in st_up)}) ({time.time() - t:.1f}s)")
    return res, up, st_res, st_up


def replay(jx, srv, trace_t, trace_g, targets, edges, alone, max_outstanding):
    """Submit the trace at its arrival times (scheduled time = arrival stamp) and verify every
    result against the request's graph scored alone.  At most max_outstanding requests hold a
    result buffer at once (submission blocks beyond that; latency still counts from the
    scheduled arrival).  Returns (mismatches, per-request latencies in ms)."""
    import queue as q
    done = q.Queue()
    tickets = q.Queue()
    sem = threading.Semaphore(max_outstanding)
    bad = []

    def collector():
        while True:
            item = tickets.get()
            if item is None:
                break
            t, key, out = item
            try:
                lat = srv.wait(t)
                if not np.array_equal(out.view(np.uint32), alone[key].view(np.uint32)):
                    bad.append(key)
                done.put(lat)
            except Exception as exc:  # a failed request is a mismatch
                bad.append((key, str(exc)))
            finally:
                sem.release()

    th = threading.Thread(target=collector, daemon=True)
    th.start()
    t0 = srv.clock_ns() + 2_000_000  # 2 ms to spare before the first arrival
    for at, key in zip(trace_t, trace_g):
        due = t0 + int(at * 1e9)
        while True:
            dt = (due - srv.clock_ns()) * 1e-9
            if dt <= 0:
                break
            time.sleep(dt - 50e-6 if dt > 100e-6 else 0)
        sem.acquire()
        out = np.empty(edges[key], np.float32)
        tickets.put((srv.submit(targets[key], out, weighted=True, arrival_ns=due), key, out))
    tickets.put(None)
    th.join()
    lats = []
    while not done.empty():
        lats.append(done.get())
    return bad, lats


def run_gpu_served(args, world, rank, local):
    import torch
    jx = importlib.import_module("sycl-jaccard_gb300")
    torch.cuda.set_device(local)
    threads = os.cpu_count() or 1
    res, up, st_res, st_up = make_served(threads)
    trace_t, trace_g = jx.graphgen.poisson_trace(args.requests, args.rate, len(res), len(up), seed=6)
    # pinned host copies of the upload pool (both arms upload from them)
    up_pinned = [tuple(torch.from_numpy(a).pin_memory().numpy() for a in g[:3]) for g in up]
    srv = jx.Server(memory_budget=60 << 30, slots=args.slots, fold_edges=args.fold_edges,
                    fold_max_edges=64 << 20)
    ids = [srv.add_graph(g[0], g[1], g[2]) for g in res]
    targets = {("resident", k): ids[k] for k in range(len(res))}
    targets.update({("upload", k): up_pinned[k] for k in range(len(up))})
    edges = {("resident", k): st_res[k]["E"] for k in range(len(res))}
    edges.update({("upload", k): st_up[k]["E"] for k in range(len(up))})
    stats = {("resident", k): st_res[k] for k in range(len(res))}
    stats.update({("upload", k): st_up[k] for k in range(len(up))})

    # alone: every graph of the pools scored by itself with the plain operator (the oracle of
    # "same result alone and in the mix"); the same plain calls time the serial baseline
    dev_res = [(jx.GraphCSRView.from_numpy(g[0], g[1], device=f"cuda:{local}"), torch.from_numpy(g[2]).cuda())
               for g in res]
    L = jx.lib()

    def plain(key, out):
        kind, k = key
        if kind == "resident":
            view, w = dev_res[k]
            r = jx.jaccard(view, w)
            torch.cuda.synchronize()
            out[:] = r.cpu().numpy()
        else:
            rp, col, w = up_pinned[k]
            rc = L.jx_jaccard_host(len(rp) - 1, len(col), rp.ctypes.data, col.ctypes.data, w.ctypes.data,
                                   out.ctypes.data, 0)
            assert rc == 0, rc

    alone = {}
    for key in edges:
        alone[key] = np.empty(edges[key], np.float32)
        plain(key, alone[key])

    # serial plain launches over the same request sequence, back to back
    torch.cuda.synchronize()
    svc = []
    scratch = {}
    tp0 = time.perf_counter()
    for key in trace_g:
        a = time.perf_counter()
        out = scratch.setdefault(key, np.empty(edges[key], np.float32))
        plain(key, out)
        svc.append(time.perf_counter() - a)
    plain_s = time.perf_counter() - tp0
    E_trace = sum(edges[k] for k in trace_g)
    # the serial server's latencies under the same arrivals (queue of one, measured service times)
    fin, plat = 0.0, []
    for at, sv in zip(trace_t, svc):
        fin = max(fin, at) + sv
        plat.append((fin - at) * 1e3)
    plat.sort()

    # warm-up requests, then the timed replay
    for i in range(args.warmup):
        key = trace_g[i % len(trace_g)]
        srv.wait(srv.submit(targets[key], np.empty(edges[key], np.float32), weighted=True))
    srv.reset_stats()
    with ClockSampler(local) as clk:
        bad, lats = replay(jx, srv, trace_t, trace_g, targets, edges, alone, args.max_outstanding)
    st = srv.stats()
    clocks = clk.summary()
    if bad or st["failed"]:
        raise AssertionError(f"served results differ from the graphs scored alone: {bad[:5]}")
    span = st["span_s"]
    value = st["edges"] / span

    # the same server at half the request rate it sustained above: latency when not overloaded
    light = None
    if args.light_requests > 0:
        rate = 0.5 * st["completed"] / span
        lt_t, lt_g = jx.graphgen.poisson_trace(args.light_requests, rate, len(res), len(up), seed=16)
        srv.reset_stats()
        bad_l, _ = replay(jx, srv, lt_t, lt_g, targets, edges, alone, args.max_outstanding)
        sl = srv.stats()
        if bad_l or sl["failed"]:
            raise AssertionError(f"served results differ from the graphs scored alone: {bad_l[:5]}")
        light = {"rate_per_s": round(rate, 2), "requests": args.light_requests,
                 "p50_ms": round(sl["p50_ms"], 3), "p99_ms": round(sl["p99_ms"], 3),
                 "mean_ms": round(sl["mean_ms"], 3), "edges_per_s": round(sl["edges"] / sl["span_s"], 1),
                 "passes": sl["passes"], "folded_requests": sl["folded_requests"],
                 "what": "Poisson arrivals (seed 16) at half the request rate sustained under overload"}

    B = sum(byte_model(stats[k]["V"], stats[k]["E"], stats[k]["sum_min"], True) for k in trace_g)
    peak, peak_kind = hbm_peak()
    achieved = B / span / 1e9
    h2d = sum(4 * (stats[k]["V"] + 1) + 4 * stats[k]["E"] + 4 * stats[k]["V"] for k in trace_g if k[0] == "upload")
    result = {
        "metric": METRIC, "value": value * world, "unit": UNIT, "n_gpus": world, "steps": 1,
        "warmup": args.warmup, "ms_per_step": round(span * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"served: {args.requests} requests, Poisson {args.rate:g}/s seed 6; 70% all edges "
                               f"of a resident graph (64 RMAT scale 14-20 ef 16), 30% uploads (32-graph pool, "
                               f"ER/RMAT 1e3-1e6 vertices); weighted VC, weights U(0,1]; budget 60 GB",
                   "slots": args.slots, "fold_edges": args.fold_edges, "E_trace": E_trace,
                   "l2": "graphs up to 1.3 GB; consecutive requests mostly touch different graphs; no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "served": {"p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                   "mean_ms": round(st["mean_ms"], 3), "max_ms": round(st["max_ms"], 3),
                   "completed": st["completed"], "passes": st["passes"],
                   "folded_requests": st["folded_requests"],
                   "peak_device_bytes": st["peak_reserved"], "span_s": round(span, 4),
                   "offered_edges_per_s": round(E_trace / max(trace_t[-1], 1e-9), 1),
                   "results": "every request bit-identical to its graph scored alone"},
        "plain": {"value": E_trace / plain_s, "unit": UNIT, "seconds": round(plain_s, 4),
                  "p50_ms": round(plat[len(plat) // 2], 3),
                  "p99_ms": round(plat[min(len(plat) - 1, int(np.ceil(0.99 * len(plat))) - 1)], 3),
                  "what": "the same requests one at a time: jx_jaccard + copy-out (resident), "
                          "jx_jaccard_host (uploads); latencies of a one-at-a-time server under the "
                          "same arrivals from the measured service times"},
        "served_over_plain": round(value / (E_trace / plain_s), 3),
        "served_light_load": light,
        "clocks": clocks,
        "e2e": {"value": value * world, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 4 * E_trace,
                "timing": "served path is end to end: host arrays in, host results out; step = the trace"},
        "gpu_launches": st["kernels"],
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "kernel": "served passes (algorithmic bytes of every request / span)",
                     "algorithmic_bytes": B},
    }
    srv.close()
    return result


# ------------------------------------------------------------------ GPU arm

def run_gpu(args, world, rank, local):
    import torch
    jx = importlib.import_module("sycl-jaccard_gb300")
    torch.cuda.set_device(local)
    threads = os.cpu_count() or 1
    rp, col, w, desc, st = make_graph(args.workload, threads)
    if args.unweighted:
        w, desc = None, desc + " (weights dropped: unweighted)"
    elif args.weighted and w is None:
        jx = importlib.import_module("sycl-jaccard_gb300")
        w = jx.graphgen.uniform_weights(st["V"], seed=4, threads=threads)
        desc += " + vertex weights U(0,1] seed 4"
    V, E = st["V"], st["E"]
    weighted = w is not None and not args.ec
    g = jx.GraphCSRView.from_numpy(rp, col, device=f"cuda:{local}")
    wd = torch.from_numpy(w).cuda() if weighted else None
    out = torch.empty(E, dtype=torch.float32, device="cuda")
    ws = torch.empty(jx.workspace_size(g, weighted, args.ec), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        jx.jaccard(g, wd, out, edge_centric=args.ec, workspace=ws)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    jx.launch_count_reset()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            jx.jaccard(g, wd, out, edge_centric=args.ec, workspace=ws)
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = jx.launch_count()
    barrier(world)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(ms, world)
    clocks = clk.summary()

    # per-launch breakdown of one extra (untimed) step
    jx.lib().jx_profile_begin()
    jx.jaccard(g, wd, out, edge_centric=args.ec, workspace=ws)
    buf = ctypes.create_string_buffer(4096)
    jx.lib().jx_profile_end(buf, 4096)
    kernels = {}
    for item in buf.value.decode().split(";"):
        if "=" in item:
            k, v = item.split("=")
            kernels[k] = round(float(v), 4)
    ksum = sum(kernels.values()) or 1.0
    dominant = max(kernels, key=kernels.get) if kernels else None

    # end-to-end through the host-buffer C-ABI entry point (pinned host memory)
    e2e = None
    if not args.no_e2e:
        h_rp = torch.from_numpy(rp).pin_memory()
        h_col = torch.from_numpy(col).pin_memory()
        h_w = torch.from_numpy(w).pin_memory() if weighted else None
        h_out = torch.empty(E, dtype=torch.float32).pin_memory()
        L = jx.lib()
        algo = 1 if args.ec else 0
        call = lambda: L.jx_jaccard_host(V, E, h_rp.data_ptr(), h_col.data_ptr(),
                                         h_w.data_ptr() if h_w is not None else None,
                                         h_out.data_ptr(), algo)
        for _ in range(min(2, args.warmup)):
            assert call() == 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            rc = call()
            assert rc == 0, rc
        t1 = time.perf_counter()
        e2e_s = (t1 - t0) / args.e2e_steps
        e2e_s = max_over_ranks(e2e_s, world)
        h2d = 4 * (V + 1) + 4 * E + (4 * V if weighted else 0)
        e2e = {"value": E * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 4 * E, "ms_per_step": round(e2e_s * 1e3, 3),
               "timing": "host wall clock around the synchronous call"}
        out_host = h_out.numpy()
        dev = out.cpu().numpy()
        if not np.array_equal(out_host.view(np.uint32), dev.view(np.uint32)):
            raise AssertionError("host-buffer entry point disagrees with the device path")

    B = byte_model(V, E, st["sum_min"], weighted)
    peak, peak_kind = hbm_peak()
    achieved = B / (ms * 1e-3) / 1e9
    traffic = MEASURED_TRAFFIC.get((args.workload, weighted, bool(args.ec)))
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "traffic_note": ("DRAM read+write bytes of one call, one-pass ncu capture of the full-size "
                                 "call; " + (f"{traffic / (ms * 1e-3) / 1e9:.0f} GB/s of DRAM at this call time"
                                            if traffic else "not captured for this configuration")),
                "kernel": "fused operator (one jx_jaccard_ws call = plan, rowsum, sentinel fill, "
                          "hub/CTA/warp row kernels, fix-up)",
                "algorithmic_bytes": B,
                "dominant_launch": dominant,
                "dominant_share": round(kernels.get(dominant, 0.0) / ksum, 4) if dominant else None}
    result = {
        "metric": METRIC, "value": E * world / (ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {desc}", "algorithm": "edge_centric" if args.ec else "vertex_centric",
                   "weighted": weighted, "V": V, "E": E, "sum_min": st["sum_min"],
                   "max_degree": st["max_degree"], "l2": l2_note(4 * (V + 1) + 4 * E + (4 * V if weighted else 0)),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
        "kernels_ms": kernels,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            result["cpu_baseline"] = cpu_reference(rp, col, w if weighted else None, args.cpu_seconds)
        except Exception as exc:
            result["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
    return result


def run_reference(args, world, rank):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    if args.workload == "served":
        jx = importlib.import_module("sycl-jaccard_gb300")
        res, up, st_res, st_up = make_served(threads)
        _, trace_g = jx.graphgen.poisson_trace(args.requests, args.rate, len(res), len(up), seed=6)
        pick = [(res if k == "resident" else up)[i] for k, i in trace_g]
        pst = [(st_res if k == "resident" else st_up)[i] for k, i in trace_g]
        vals, cb = [], None
        for i in range(args.warmup + args.steps):
            cb = cpu_reference_batch(pick, pst, args.cpu_seconds / max(1, args.steps),
                                     weights=[g[2] for g in pick], what="requests of the trace")
            if i >= args.warmup:
                vals.append(cb["value"])
        value = statistics.median(vals)
        cb["value"] = value
        return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": f"served: {args.requests} requests (see the jx arm), serial reference calls",
                           "algorithm": "vertex_centric", "weighted": True},
                "cpu_baseline": cb,
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.workload == "batched":
        graphs, st = make_batch(threads)
        vals, cb = [], None
        for i in range(args.warmup + args.steps):
            cb = cpu_reference_batch(graphs, st, args.cpu_seconds / max(1, args.steps))
            if i >= args.warmup:
                vals.append(cb["value"])
        value = statistics.median(vals)
        cb["value"] = value
        E = sum(x["E"] for x in st)
        return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(E / value * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": "batched: 2000 graphs seed 5 (see the jx arm)", "algorithm": "vertex_centric",
                           "graphs": len(graphs), "E": E},
                "cpu_baseline": cb,
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    rp, col, w, desc, st = make_graph(args.workload, threads)
    weighted = w is not None and not args.ec
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_reference(rp, col, w if weighted else None, args.cpu_seconds / max(1, args.steps))
        if i >= args.warmup:
            vals.append(cb["value"])
    value = statistics.median(vals)
    cb["value"] = value
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(st["E"] / value * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{args.workload}: {desc}", "algorithm": "vertex_centric",
                       "weighted": weighted, "V": st["V"], "E": st["E"], "sum_min": st["sum_min"]},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="jx", choices=["jx", "reference"])
    ap.add_argument("--workload", default="rmat24w", choices=["rmat24w", "rmat22w", "rmat20", "er4096", "batched", "served"])
    ap.add_argument("--requests", type=int, default=1000, help="served: requests in the trace")
    ap.add_argument("--rate", type=float, default=2000.0, help="served: Poisson arrival rate (1/s)")
    ap.add_argument("--slots", type=int, default=4, help="served: passes in flight")
    ap.add_argument("--fold-edges", type=int, default=1 << 21, help="served: fold requests up to this size")
    ap.add_argument("--max-outstanding", type=int, default=256, help="served: result buffers held at once")
    ap.add_argument("--light-requests", type=int, default=300,
                    help="served: requests of the second trace at half the sustained rate (0: skip)")
    ap.add_argument("--ec", action="store_true", help="edge-centric algorithm")
    ap.add_argument("--unweighted", action="store_true", help="drop the vertex weights")
    ap.add_argument("--weighted", action="store_true",
                    help="add U(0,1] vertex weights (seed 4) to a workload that has none")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "jx":
        log("warm-up raised to 3 steps")
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        res = run_reference(args, world, rank)
    elif args.workload == "batched":
        res = run_gpu_batched(args, world, rank, local)
    elif args.workload == "served":
        res = run_gpu_served(args, world, rank, local)
    else:
        res = run_gpu(args, world, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
