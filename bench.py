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
# capture (gpu__time_duration, dram__bytes_read/write) of the full-size call.  Keyed by
# (workload, weighted, edge_centric); each figure carries the fingerprint of the engine sources
# it was captured on (sources_fingerprint()) and is reported only while the sources match.
MEASURED_TRAFFIC = {  # median over 5 calls of one capture each
    ("rmat24w", True, False): (1322724323840, "9d9812efee9f5ec5"),
    ("rmat24w", False, False): (1025875655168, "9d9812efee9f5ec5"),
}


def sources_fingerprint():
    """sha256 (first 16 hex digits) over the engine's CUDA sources: csrc/*.cu, *.cuh, *.h,
    each as file name + code, in name order.  Comments and whitespace are left out, so that
    editing a comment keeps a measurement tied to the code it was taken on."""
    import glob
    import hashlib
    import re
    d = os.path.join(ROOT, "sycl-jaccard_gb300", "csrc")
    h = hashlib.sha256()
    for f in sorted(glob.glob(os.path.join(d, "*.cu")) + glob.glob(os.path.join(d, "*.cuh")) +
                    glob.glob(os.path.join(d, "*.h"))):
        h.update(os.path.basename(f).encode())
        with open(f, encoding="utf-8") as fh:
            code = fh.read()
        code = re.sub(r"/\*.*?\*/", " ", code, flags=re.S)
        code = re.sub(r"//[^\n]*", " ", code)
        h.update(" ".join(code.split()).encode())
    return h.hexdigest()[:16]


def measured_traffic(key, ms):
    """(traffic bytes or None, note) for this configuration and the current sources."""
    if key not in MEASURED_TRAFFIC:
        return None, "not captured for this configuration"
    b, fp = MEASURED_TRAFFIC[key]
    now = sources_fingerprint()
    if fp != now:
        return None, f"captured on engine sources {fp}; the sources are now {now}, so it no longer applies"
    return b, (f"DRAM read+write bytes of one call, one-pass ncu capture of the full-size call on these "
               f"sources ({fp}); {b / (ms * 1e-3) / 1e9:.0f} GB/s of DRAM at this call time")


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


def make_graph(name, threads, permute=0):
    jx = importlib.import_module("sycl-jaccard_gb300")
    t = time.time()
    rp, col, w, desc = jx.graphgen.config_graph(name, threads=threads, permute=permute)
    st = jx.graphgen.stats(rp, col)
    log(f"graph {name}: V={st['V']} E={st['E']} max_deg={st['max_degree']} sum_min={st['sum_min']:.4g} "
        f"({time.time() - t:.1f}s)")
    return rp, col, w, desc, st


# ------------------------------------------------------------------ CPU reference arm

def makespan(costs, threads):
    """Duration of one kernel launch of the host SYCL subset in cost units: the first group
    runs alone (it tells the subset whether the kernel needs fibers), the others are handed
    in id order to whichever of `threads` threads is free first (OpenMP dynamic schedule)."""
    import heapq
    if len(costs) == 0:
        return 0.0
    free = [0.0] * threads
    for c in costs[1:]:
        heapq.heappush(free, heapq.heappop(free) + float(c))
    return float(costs[0]) + max(free)


class RefSampler:
    """The reference's own kernels (jaccard.cpp through the host SYCL subset) on the host
    cores, timed on bounded samples of its work-groups and extrapolated to the whole call.

    The subset runs each work-group on one thread (its work-items as fibers or a loop), so a
    call's time is the makespan of its groups over the threads.  Each group's cost is
    estimated by a proxy (oracle group_work: min(d_u, d_v) * (1 + log2 max) per edge, the
    binary searches of the dominant kernel, Jaccard_IsKernel or Jaccard_ec_unweighted).  A
    sample runs, in every kernel of one call, the work-groups that are every K-th in order of
    cost (stratified: R-MAT degrees follow the bits of the vertex id, so a stride over group
    ids would pick groups of one cost level); with `a` the fixed per-call cost (a call that
    runs no group: the reference's per-call temporaries, jaccard.cpp:931-934) and t the
    sample's time, the seconds per cost unit are c = (t - a) / makespan(sample), and the whole
    call takes T = a + c * makespan(all groups).  A light calibration sample gives a first c;
    each step's sample then holds about one group per thread from the heaviest stratum whose
    predicted duration fits the target, at successive offsets, and gives its own c and T.  Without the reference build, the C
    restatement (kind "port") is timed on row ranges and extrapolated by work share."""

    def __init__(self, rp, col, w, edge_centric=False, threads=None):
        from oracle import oracle as O
        self.O = O
        self.rp, self.col, self.w, self.ec = rp, col, w, edge_centric
        self.n, self.E = len(rp) - 1, len(col)
        self.threads = threads or os.cpu_count() or 1
        try:
            self.L = O.ref_lib()
        except Exception as exc:  # build failure on this machine
            log(f"reference build unavailable: {exc}")
            self.L = None
        self.kind = "reference" if self.L is not None else "port"
        self.spent = 0.0
        self.calls = 0
        self.c = None
        if self.kind == "reference":
            self.gw = O.group_work(rp, col, edge_centric, self.threads)
            self.order = np.argsort(-self.gw, kind="stable")
            self.M_full = makespan(self.gw, self.threads)
            self.a = self._run(np.zeros(len(self.gw), np.uint8))
        else:
            self.rw = O.row_work(rp, col, self.threads)
            self.K_max = max(1, self.n // (8 * self.threads))
            self.W = float(self.rw.sum()) or 1.0
            self.a = 0.0

    def _ids(self, K, offset):
        return np.sort(self.order[offset % K::K])


    def _model(self, K, offset):
        """(what to run, cost units of the sample: its makespan, or its work share for a port)."""
        if self.kind == "reference":
            ids = self._ids(K, offset)
            mask = np.zeros(len(self.gw), np.uint8)
            mask[ids] = 1
            return mask, makespan(self.gw[ids], self.threads)
        size = max(1, self.n // K)
        lo = (offset * size) % max(1, self.n - size + 1)
        return (lo, min(self.n, lo + size)), float(self.rw[lo:lo + size].sum()) / self.W

    def _run(self, what):
        t0 = time.perf_counter()
        if self.kind == "reference":
            self.O.ref_jaccard(self.rp, self.col, self.w, edge_centric=self.ec, threads=self.threads,
                               group_mask=what)
        else:
            self.O.jaccard(self.rp, self.col, self.w, edge_centric=self.ec, rows=what, threads=self.threads)
        t = time.perf_counter() - t0
        self.spent += t
        return t

    def _full_units(self):
        return self.M_full if self.kind == "reference" else 1.0

    def _step_choice(self, target_s):
        """(K, offset) of a sample predicted to take about target_s seconds: one group per thread
        (K = groups / threads) from the heaviest offset that fits the target; denser samples
        when even offset 0 fits (small graphs)."""
        if self.kind != "reference":
            return int(min(self.n, max(1, round(1.0 / max(target_s / max(self.c, 1e-12), 1e-12))))), self.calls
        G = len(self.gw)
        pred = lambda K, off: self.a + self.c * self._model(K, off)[1]
        Ks = max(1, G // self.threads)
        if pred(Ks, 0) <= target_s:  # even the heaviest groups fit: make the sample denser
            lo, hi = 1, Ks
            while lo < hi:
                mid = (lo + hi) // 2
                if pred(mid, 0) <= target_s:
                    hi = mid
                else:
                    lo = mid + 1
            return lo, self.calls % lo
        lo, hi = 0, Ks - 1  # the lowest offset (heaviest groups) predicted to fit the target
        while lo < hi:
            mid = (lo + hi) // 2
            if pred(Ks, mid) <= target_s:
                hi = mid
            else:
                lo = mid + 1
        return Ks, (lo + self.calls) % Ks

    def sample(self, target_s):
        """One sample of about target_s seconds; returns (extrapolated whole-call seconds,
        details).  The first call also runs the calibration sample."""
        if self.c is None:  # calibration: a light sample, one group per thread
            K = self.K_max if self.kind != "reference" else max(1, len(self.gw) // self.threads)
            off = K - 1 if self.kind == "reference" else K // 2
            what, units = self._model(K, off)
            t = self._run(what)
            self.c = max(t - self.a, 1e-4) / max(units, 1e-12)
            self.calib = {"K": K, "offset": off, "sample_s": round(t, 3),
                          "call_s": round(self.a + self.c * self._full_units(), 2)}
        K, offset = self._step_choice(target_s)
        what, units = self._model(K, offset)
        t = self._run(what)
        self.calls += 1
        self.c = max(t - self.a, 1e-6) / max(units, 1e-12)
        T = self.a + self.c * self._full_units()
        info = {"K": K, "offset": offset, "sample_s": t, "units": units}
        if self.kind == "reference":
            ids = self._ids(K, offset)
            info["groups"] = len(ids)
            info["share"] = float(self.gw[ids].sum() / self.gw.sum())
            info["parallel_eff"] = float(self.gw[ids].sum() / self.threads / max(units, 1e-12))
        return T, info

    def describe(self, info, weighted):
        algo = "EC" if self.ec else f"VC{' weighted' if weighted else ''}"
        if self.kind == "reference":
            return (f"reference jaccard.cpp ({algo}) via host SYCL subset, {self.threads} threads: in every kernel "
                    f"of one call the work-groups that are every {info['K']}-th of the {len(self.gw)} in order of "
                    f"cost from offset {info['offset']} ({info['groups']} groups, {info['share']:.2e} of the "
                    f"{'EC' if self.ec else 'IS'} kernel's work, parallel efficiency {info['parallel_eff']:.2f}); "
                    f"fixed per-call cost {self.a:.2f}s + sampled {info['sample_s'] - self.a:.2f}s, extrapolated "
                    f"by the makespan of the groups' cost proxy over the threads (whole call: efficiency "
                    f"{self.gw.sum() / self.threads / self.M_full:.3f}); light calibration sample "
                    f"{self.calib['sample_s']}s, whole call {self.calib['call_s']}s")
        return f"C restatement (oracle port), a row range with {info['units']:.2e} of the work, {self.threads} threads"


def cpu_reference(rp, col, w, target_s=20.0, edge_centric=False):
    """The reference on this machine's host cores: one bounded sample of about target_s seconds
    (RefSampler), reported as edges per second of the extrapolated whole call."""
    s = RefSampler(rp, col, w, edge_centric)
    T, info = s.sample(target_s)
    return {"value": s.E / T, "unit": UNIT, "cores": s.threads, "kind": s.kind,
            "sample": s.describe(info, w is not None), "seconds": round(s.spent, 3),
            "extrapolated_call_s": round(T, 2)}


def oracle_parity(rp, col, w, edge_centric, got):
    """The engine's results checked against the oracle (the C restatement, pinned bit for bit to
    the reference) -- on the whole graph when it is small, else on the sampled row ranges of
    oracle.check_rows (largest hubs, a CTA-size row, a middle band, the tail)."""
    from oracle import oracle as O
    got = np.ascontiguousarray(got, np.float32).view(np.uint32)
    threads = os.cpu_count() or 1
    t0 = time.time()
    n, E = len(rp) - 1, len(col)
    if E <= 5_000_000:
        ranges = [("all", 0, n)]
    else:
        ranges = O.check_rows(rp)
    S = O.rowsum(rp, col, w, threads) if (w is not None and not edge_centric) else None
    bad, edges, names = 0, 0, []
    for name, r0, r1 in ranges:
        if S is not None:
            want = O.jaccard_rows_with_sums(rp, col, w, S, (r0, r1), threads)
        else:
            want = O.jaccard(rp, col, None, edge_centric=edge_centric, rows=(r0, r1), threads=threads)
        lo, hi = int(rp[r0]), int(rp[r1])
        bad += int((got[lo:hi] != want.view(np.uint32)).sum())
        edges += hi - lo
        names.append(name)
    return {"result": ("bit-exact" if bad == 0 else f"{bad} mismatches") + f" on {edges} edges",
            "mismatches": bad, "edges_checked": edges, "rows": names,
            "oracle": "C restatement of jaccard.cpp, pinned to the reference", "seconds": round(time.time() - t0, 2)}


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


class BatchRefSampler:
    """The reference on the host cores over a stratified sample of a list of graphs: 8 graphs
    evenly spaced in edge-count order, each with its own RefSampler.  A sample times every
    picked graph once (target_s split between them); the rate is (sum of their edges) / (sum
    of their extrapolated call times).  weights: per-graph vertex weights (weighted VC) or
    None (unweighted VC)."""

    def __init__(self, graphs, st, weights=None, what="graphs of the batch"):
        order = np.argsort([x["E"] for x in st], kind="stable")
        self.pick = [int(order[int(q)]) for q in np.linspace(0, len(order) - 1, 8)]
        self.samplers = [RefSampler(graphs[i][0], graphs[i][1], None if weights is None else weights[i])
                         for i in self.pick]
        self.E = float(sum(st[i]["E"] for i in self.pick))
        self.weighted = weights is not None
        self.what = what

    def sample(self, target_s):
        T = sum(s.sample(target_s / len(self.samplers))[0] for s in self.samplers)
        return T

    def result(self, T):
        s0 = self.samplers[0]
        return {"value": self.E / T, "unit": UNIT, "cores": s0.threads, "kind": s0.kind,
                "sample": f"reference jaccard.cpp (VC{' weighted' if self.weighted else ''}) on 8 {self.what} "
                          f"evenly spaced in edge count ({int(self.E)} edges), each on a work-group sample "
                          f"extrapolated to its whole call; rate = sum of edges / sum of call times",
                "seconds": round(sum(s.spent for s in self.samplers), 3), "extrapolated_call_s": round(T, 3)}


def cpu_reference_batch(graphs, st, target_s=20.0, weights=None, what="graphs of the batch"):
    b = BatchRefSampler(graphs, st, weights, what)
    return b.result(b.sample(target_s))


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
    batch_host = np.empty(E, np.uint32)
    for b, grp in zip(batches, groups):
        lo, hi = int(eoff[grp[0]]), int(eoff[grp[-1] + 1])
        batch_host[lo:hi] = b.download(-1).view(np.uint32)
    if not np.array_equal(batch_host, plain_host):
        raise AssertionError("batched results differ from the per-graph calls")
    for b in batches:
        b.close()

    # the weighted vertex-centric path on the same batch (unit weights: every sum is an exact
    # integer, so the values equal the unweighted ones bit for bit)
    weighted = None
    if not args.no_weighted_batch:
        t = time.time()
        ones = [np.ones(len(rp) - 1, np.float32) for rp, _, _ in graphs]
        wbatches = [jx.Batch([(graphs[i][0], graphs[i][1], ones[i]) for i in grp], weighted=True, tune=True)
                    for grp in groups]
        winfos = [b.info() for b in wbatches]
        log(f"weighted batch: built and tuned ({time.time() - t:.1f}s): " + "; ".join(i["plan"] for i in winfos))
        wms, wlaunches, wclocks = timed(lambda: [b.run(stream) for b in wbatches], args.steps, args.warmup)
        ones_d = [torch.from_numpy(o).cuda() for o in ones]
        ws_w = torch.empty(max(jx.workspace_size(g, True, False) for g in plain_g), dtype=torch.uint8, device="cuda")

        def plain_w_step():
            for g, o, wd in zip(plain_g, outs, ones_d):
                if o.numel():
                    jx.jaccard(g, wd, o, workspace=ws_w)
        wplain_ms, _, _ = timed(plain_w_step, max(1, args.steps // 2), 1)
        wb = np.empty(E, np.uint32)
        for b, grp in zip(wbatches, groups):
            lo, hi = int(eoff[grp[0]]), int(eoff[grp[-1] + 1])
            wb[lo:hi] = b.download(-1).view(np.uint32)
        if not (np.array_equal(wb, plain_host) and np.array_equal(plain_out.cpu().numpy().view(np.uint32), plain_host)):
            raise AssertionError("weighted batch (unit weights) differs from the unweighted results")
        Bw = sum(byte_model(x["V"], x["E"], x["sum_min"], True) for x in st)
        weighted = {"ms_per_step": round(wms, 4), "value": E * world / (wms * 1e-3), "unit": UNIT,
                    "plans": [i["plan"] for i in winfos], "kernels_per_pass": sum(i["kernels_per_run"] for i in winfos),
                    "gpu_launches": wlaunches, "clocks": wclocks,
                    "plain_ms_per_step": round(wplain_ms, 3), "batched_over_plain": round(wplain_ms / wms, 3),
                    "frac": round(Bw / (wms * 1e-3) / 1e9 / hbm_peak()[0], 4), "algorithmic_bytes": Bw,
                    "results": "bit-identical to the unweighted batch and to the per-graph calls"}
        for b in wbatches:
            b.close()

    # end to end through the public batch API: host CSRs (pinned) in, every result out
    e2e = None
    if not args.no_e2e:
        pinned = [(torch.from_numpy(rp).pin_memory().numpy(), torch.from_numpy(col).pin_memory().numpy())
                  for rp, col, _ in graphs]
        h_out = torch.empty(E, dtype=torch.float32).pin_memory().numpy()
        def e2e_step():
            for grp in groups:
                b = jx.Batch([pinned[i] for i in grp])  # default schedule: no tuning inside the timing
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
        "weighted": weighted,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "kernel": "one captured pass over every super-CSR", "algorithmic_bytes": B},
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            result["cpu_baseline"] = cpu_reference_batch(graphs, st, args.cpu_seconds)
        except Exception as exc:
            result["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
        try:  # the batch's results against the oracle on the graphs the CPU leg samples
            order = np.argsort([x["E"] for x in st], kind="stable")
            pick = [int(order[int(q)]) for q in np.linspace(0, len(order) - 1, 8)]
            checks = [oracle_parity(graphs[i][0], graphs[i][1], None, False,
                                    batch_host[int(eoff[i]):int(eoff[i + 1])].view(np.float32)) for i in pick]
            bad = sum(c["mismatches"] for c in checks)
            result["parity"] = {"result": ("bit-exact" if bad == 0 else f"{bad} mismatches") +
                                          f" on {sum(c['edges_checked'] for c in checks)} edges of 8 graphs",
                                "mismatches": bad, "graphs": pick,
                                "oracle": "C restatement of jaccard.cpp, pinned to the reference"}
        except Exception as exc:
            result["parity"] = {"result": None, "error": str(exc)[:200]}
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
    # passes run the persistent row kernel unless a schedule is given (measured: 2.05e9 edges/s
    # against 1.99e9 per-bin with 8 slots and folding up to 8M edges)
    sch = json.loads(args.schedule) if args.schedule else {"persistent": 1}
    srv = jx.Server(memory_budget=60 << 30, slots=args.slots, fold_edges=args.fold_edges,
                    fold_max_edges=64 << 20, schedule=sch)
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

    # the serial plain server, run for real: the same trace replayed at its arrival times, one
    # request at a time in arrival order (a request starts when it has arrived and the one
    # before it is done); latency = arrival -> results in host memory
    torch.cuda.synchronize()
    scratch = {}
    plat = []
    tp0 = time.perf_counter() + 0.002
    for at, key in zip(trace_t, trace_g):
        due = tp0 + float(at)
        now = time.perf_counter()
        if now < due:
            time.sleep(due - now)
        out = scratch.setdefault(key, np.empty(edges[key], np.float32))
        plain(key, out)
        plat.append((time.perf_counter() - due) * 1e3)
    plain_s = time.perf_counter() - tp0 - float(trace_t[0])
    E_trace = sum(edges[k] for k in trace_g)
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
                   "schedule": sch or "default",
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
                  "what": "the same trace replayed at its arrival times through a one-at-a-time server: "
                          "jx_jaccard + copy-out (resident), jx_jaccard_host (uploads); measured latencies"},
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

def time_calls(jx, world, local, stream, call, steps, warmup):
    """W untimed calls, then `steps` calls between barrier + synchronize, CUDA events on the
    launching stream; returns (ms per call, max over ranks), kernels launched, clock summary."""
    import torch
    for _ in range(warmup):
        call()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    jx.launch_count_reset()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(steps):
            call()
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = jx.launch_count()
    barrier(world)
    ms = max_over_ranks(ev0.elapsed_time(ev1) / steps, world)
    return ms, launches, clk.summary()


def copy_rates(V, E, weighted):
    """Host<->device copy rates of this machine for the e2e arrays (pinned host memory from
    jx_host_alloc, one copy per direction, CUDA events): GB/s for H2D of row_ptr + col (+ w) and
    D2H of J."""
    import torch
    jx = importlib.import_module("sycl-jaccard_gb300")
    ha = jx.HostArray((4 * (V + 1) + 4 * E + (4 * V if weighted else 0),), np.uint8)
    hb = jx.HostArray((4 * E,), np.uint8)
    h_in, h_out = torch.from_numpy(ha.array), torch.from_numpy(hb.array)
    d_in = torch.empty(h_in.numel(), dtype=torch.uint8, device="cuda")
    d_out = torch.empty(h_out.numel(), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    res = {}
    for name, dst, src in (("h2d", d_in, h_in), ("d2h", h_out, d_out)):
        dst.copy_(src, non_blocking=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record(s)
        torch.cuda.synchronize()
        res[name + "_gbs"] = round(3 * src.numel() / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
    del h_in, h_out, d_in, d_out
    ha.free()
    hb.free()
    return res


def e2e_worker(args):
    """The e2e leg in a process of its own: the same graph (regenerated: the generator is a pure
    function of its seeds), host arrays in the library's pinned memory, `e2e_steps` timed calls of
    jx_jaccard_host (copies in, operator, copy out) after 2 untimed ones, through ctypes and the C
    ABI only (no PyTorch in this process).  Prints one JSON line: ms per call, the split of one
    extra call and a digest of the results."""
    import hashlib
    jx = importlib.import_module("sycl-jaccard_gb300")
    threads = os.cpu_count() or 1
    rp, col, w, _ = jx.graphgen.config_graph(args.workload, threads=threads, permute=args.permute)
    if args.unweighted:
        w = None
    elif args.weighted and w is None:
        w = jx.graphgen.uniform_weights(len(rp) - 1, seed=4, threads=threads)
    weighted = w is not None and not args.ec
    V, E = len(rp) - 1, len(col)
    L = jx.lib()
    arrs = [jx.HostArray.copy_of(rp), jx.HostArray.copy_of(col), jx.HostArray.copy_of(w) if weighted else None,
            jx.HostArray((E,), np.float32)]
    ptr = [a.array.ctypes.data if a is not None else None for a in arrs]
    algo = 1 if args.ec else 0
    call = lambda: L.jx_jaccard_host(V, E, ptr[0], ptr[1], ptr[2], ptr[3], algo)
    for _ in range(2):
        assert call() == 0
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        assert call() == 0
    ms = (time.perf_counter() - t0) / args.e2e_steps * 1e3
    L.jx_profile_begin()
    assert call() == 0
    pbuf = ctypes.create_string_buffer(4096)
    L.jx_profile_end(pbuf, 4096)
    split = {k: round(float(v), 3) for k, v in (it.split("=") for it in pbuf.value.decode().split(";") if "=" in it)}
    digest = hashlib.sha256(arrs[3].array.view(np.uint8)).hexdigest()
    print(json.dumps({"ms_per_step": round(ms, 3), "split_ms": split, "digest": digest}), flush=True)


def e2e_in_worker(args, local):
    """Run e2e_worker in a child process on this rank's GPU; returns its JSON result."""
    env = dict(os.environ)
    vis = env.get("CUDA_VISIBLE_DEVICES")
    env["CUDA_VISIBLE_DEVICES"] = vis.split(",")[local] if vis else str(local)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--e2e-worker", "--workload", args.workload,
           "--e2e-steps", str(args.e2e_steps), "--permute", str(args.permute)]
    cmd += ["--unweighted"] if args.unweighted else []
    cmd += ["--weighted"] if args.weighted else []
    cmd += ["--ec"] if args.ec else []
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=900)
    if r.returncode != 0:
        raise RuntimeError("e2e worker failed: " + r.stderr[-500:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_gpu(args, world, rank, local):
    import torch
    jx = importlib.import_module("sycl-jaccard_gb300")
    torch.cuda.set_device(local)
    threads = os.cpu_count() or 1
    rp, col, w, desc, st = make_graph(args.workload, threads, args.permute)
    if args.unweighted:
        w, desc = None, desc + " (weights dropped: unweighted)"
    elif args.weighted and w is None:
        w = jx.graphgen.uniform_weights(st["V"], seed=4, threads=threads)
        desc += " + vertex weights U(0,1] seed 4"
    V, E = st["V"], st["E"]
    weighted = w is not None and not args.ec
    g = jx.GraphCSRView.from_numpy(rp, col, device=f"cuda:{local}")
    wd = torch.from_numpy(w).cuda() if weighted else None
    out = torch.empty(E, dtype=torch.float32, device="cuda")
    sch = json.loads(args.schedule) if args.schedule else None
    ws_bytes = max(jx.workspace_size(g, weighted, args.ec, sch), jx.workspace_size(g, False, False, sch))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    call = lambda: jx.jaccard(g, wd, out, edge_centric=args.ec, workspace=ws, schedule=sch)
    ms, launches, clocks = time_calls(jx, world, local, stream, call, args.steps, args.warmup)
    result_bits = out.cpu().numpy().copy()

    # per-launch breakdown of one extra (untimed) step
    jx.lib().jx_profile_begin()
    call()
    buf = ctypes.create_string_buffer(4096)
    jx.lib().jx_profile_end(buf, 4096)
    kernels = {}
    for item in buf.value.decode().split(";"):
        if "=" in item:
            k, v = item.split("=")
            kernels[k] = round(float(v), 4)
    dominant = max(kernels, key=kernels.get) if kernels else None

    # end-to-end through the host-buffer C-ABI entry point (pinned host memory)
    e2e = None
    if not args.no_e2e:
        # host arrays in pinned memory from the library's allocator (jx_host_alloc)
        h_rp = jx.HostArray.copy_of(rp)
        h_col = jx.HostArray.copy_of(col)
        h_w = jx.HostArray.copy_of(w) if weighted else None
        h_out = jx.HostArray((E,), np.float32)
        L = jx.lib()
        algo = 1 if args.ec else 0
        host_call = lambda: L.jx_jaccard_host(V, E, h_rp.array.ctypes.data, h_col.array.ctypes.data,
                                              h_w.array.ctypes.data if h_w is not None else None,
                                              h_out.array.ctypes.data, algo)
        for _ in range(min(2, args.warmup)):
            assert host_call() == 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            rc = host_call()
            assert rc == 0, rc
        t1 = time.perf_counter()
        in_process_s = (t1 - t0) / args.e2e_steps
        h2d = 4 * (V + 1) + 4 * E + (4 * V if weighted else 0)
        # the headline e2e: the same call in a process of its own (C ABI through ctypes, no
        # PyTorch), whose results must equal this run's bit for bit
        import hashlib
        wk = e2e_in_worker(args, local)
        if wk["digest"] != hashlib.sha256(result_bits.view(np.uint8)).hexdigest():
            raise AssertionError("the e2e worker's results differ from the device path")
        e2e_s = max_over_ranks(wk["ms_per_step"] * 1e-3, world)
        e2e = {"value": E * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 4 * E, "ms_per_step": round(e2e_s * 1e3, 3),
               "timing": "host wall clock around the synchronous jx_jaccard_host call, in a process of its own "
                         "(the same graph regenerated, ctypes + C ABI, no PyTorch); results checked bit for bit",
               "host_memory": "pinned, from jx_host_alloc", "split_ms": wk["split_ms"],
               "in_process": {"ms_per_step": round(max_over_ranks(in_process_s, world) * 1e3, 3),
                              "what": "the same call in this benchmark process (PyTorch loaded, the graph's "
                                      "arrays held): its copies run slower"}}
        # where one host call's time goes: stream events after its copies in, each kernel and
        # its copy out (event gaps include any wait of the device for the host)
        jx.lib().jx_profile_begin()
        t0 = time.perf_counter()
        assert host_call() == 0
        wall = time.perf_counter() - t0
        pbuf = ctypes.create_string_buffer(4096)
        jx.lib().jx_profile_end(pbuf, 4096)
        e2e["in_process"]["split_ms"] = {k: round(float(v), 3) for k, v in
                                         (item.split("=") for item in pbuf.value.decode().split(";") if "=" in item)}
        e2e["in_process"]["split_wall_ms"] = round(wall * 1e3, 3)
        e2e.update(copy_rates(V, E, weighted))
        e2e["copy_ms_at_these_rates"] = round(h2d / e2e["h2d_gbs"] / 1e6 + 4 * E / e2e["d2h_gbs"] / 1e6, 2)
        if not np.array_equal(h_out.array.view(np.uint32), result_bits.view(np.uint32)):
            raise AssertionError("host-buffer entry point disagrees with the device path")
        for h in (h_rp, h_col, h_w, h_out):
            if h is not None:
                h.free()

    B = byte_model(V, E, st["sum_min"], weighted)
    peak, peak_kind = hbm_peak()
    achieved = B / (ms * 1e-3) / 1e9
    traffic, traffic_note = measured_traffic((args.workload, weighted, bool(args.ec)), ms)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "traffic_source": traffic_note, "sources": sources_fingerprint(),
                "kernel": "fused operator (one jx_jaccard_ws call = plan, rowsum, sentinel fill, "
                          "hub/CTA/warp row kernels, fix-up)",
                "algorithmic_bytes": B,
                "dominant_launch": dominant,
                "dominant_share": round(kernels.get(dominant, 0.0) / ms, 4) if dominant else None,
                "dominant_share_of": "the step's event time"}
    result = {
        "metric": METRIC, "value": E * world / (ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {desc}", "algorithm": "edge_centric" if args.ec else "vertex_centric",
                   "weighted": weighted, "V": V, "E": E, "sum_min": st["sum_min"], "schedule": sch or "default",
                   "max_degree": st["max_degree"], "l2": l2_note(4 * (V + 1) + 4 * E + (4 * V if weighted else 0)),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
        "kernels_ms": kernels,
    }

    # the same graph unweighted (vertex-centric): a few more timed calls, reported beside
    unw_bits = None
    if weighted and not args.no_unweighted:
        call_u = lambda: jx.jaccard(g, None, out, edge_centric=False, workspace=ws, schedule=sch)
        ms_u, _, clk_u = time_calls(jx, world, local, stream, call_u, 5, 2)
        unw_bits = out.cpu().numpy()
        B_u = byte_model(V, E, st["sum_min"], False)
        result["unweighted"] = {"ms_per_step": round(ms_u, 4), "value": E * world / (ms_u * 1e-3), "unit": UNIT,
                                "steps": 5, "warmup": 2, "algorithmic_bytes": B_u,
                                "frac": round(B_u / (ms_u * 1e-3) / 1e9 / peak, 4), "clocks": clk_u}

    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            result["cpu_baseline"] = cpu_reference(rp, col, w if weighted else None, args.cpu_seconds, args.ec)
        except Exception as exc:
            result["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
        try:
            result["parity"] = oracle_parity(rp, col, w if weighted else None, args.ec, result_bits)
            if unw_bits is not None:
                result["unweighted"]["parity"] = oracle_parity(rp, col, None, False, unw_bits)
        except Exception as exc:
            result["parity"] = {"result": None, "error": str(exc)[:200]}
    return result


def run_reference(args, world, rank):
    """The reference arm: the reference's own kernels on this machine's host cores, all
    threads.  Set-up (graph, work model, calibration) happens once; then one untimed warm-up
    sample (when warmup > 0) and `steps` samples of about ref_seconds / steps seconds each,
    on successive work-group residues.  The value is E / the median extrapolated call time."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    per = max(0.5, args.ref_seconds / max(1, args.steps))
    common = {"metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
              "data": "synthetic", "impl": "reference"}
    if args.workload in ("served", "batched"):
        if args.workload == "served":
            jx = importlib.import_module("sycl-jaccard_gb300")
            res, up, st_res, st_up = make_served(threads)
            _, trace_g = jx.graphgen.poisson_trace(args.requests, args.rate, len(res), len(up), seed=6)
            pick = [(res if k == "resident" else up)[i] for k, i in trace_g]
            pst = [(st_res if k == "resident" else st_up)[i] for k, i in trace_g]
            bs = BatchRefSampler(pick, pst, weights=[g[2] for g in pick], what="requests of the trace")
            config = {"workload": f"served: {args.requests} requests (see the jx arm), serial reference calls",
                      "algorithm": "vertex_centric", "weighted": True}
        else:
            graphs, st = make_batch(threads)
            bs = BatchRefSampler(graphs, st)
            config = {"workload": "batched: 2000 graphs seed 5 (see the jx arm)", "algorithm": "vertex_centric",
                      "graphs": len(graphs), "E": sum(x["E"] for x in st)}
        if args.warmup > 0:
            bs.sample(per)
        Ts = [bs.sample(per) for _ in range(args.steps)]
        cb = bs.result(statistics.median(Ts))
        value = cb["value"]
        return dict(common, value=value, ms_per_step=round(bs.E / value * 1e3, 3), config=config,
                    cpu_baseline=cb,
                    e2e={"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    rp, col, w, desc, st = make_graph(args.workload, threads, args.permute)
    weighted = w is not None and not args.ec
    sm = RefSampler(rp, col, w if weighted else None, edge_centric=args.ec, threads=threads)
    if args.warmup > 0:
        sm.sample(per)
    runs = [sm.sample(per) for _ in range(args.steps)]
    Ts = [T for T, _ in runs]
    Tm = statistics.median(Ts)
    value = st["E"] / Tm
    info = runs[len(runs) // 2][1]
    cb = {"value": value, "unit": UNIT, "cores": sm.threads, "kind": sm.kind,
          "sample": sm.describe(info, weighted) + f"; median of {len(Ts)} samples at successive offsets",
          "seconds": round(sm.spent, 3), "extrapolated_call_s": round(Tm, 2),
          "extrapolated_call_s_range": [round(min(Ts), 2), round(max(Ts), 2)]}
    return dict(common, value=value, ms_per_step=round(Tm * 1e3, 3),
                config={"workload": f"{args.workload}: {desc}",
                        "algorithm": "edge_centric" if args.ec else "vertex_centric",
                        "weighted": weighted, "V": st["V"], "E": st["E"], "sum_min": st["sum_min"]},
                cpu_baseline=cb,
                e2e={"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="jx", choices=["jx", "reference"])
    ap.add_argument("--workload", default="rmat24w", choices=["rmat24w", "rmat22w", "rmat20", "er4096", "batched", "served"])
    ap.add_argument("--requests", type=int, default=1000, help="served: requests in the trace")
    ap.add_argument("--rate", type=float, default=2000.0, help="served: Poisson arrival rate (1/s)")
    ap.add_argument("--slots", type=int, default=8, help="served: passes in flight")
    ap.add_argument("--fold-edges", type=int, default=1 << 23, help="served: fold requests up to this size")
    ap.add_argument("--max-outstanding", type=int, default=256, help="served: result buffers held at once")
    ap.add_argument("--light-requests", type=int, default=300,
                    help="served: requests of the second trace at half the sustained rate (0: skip)")
    ap.add_argument("--ec", action="store_true", help="edge-centric algorithm")
    ap.add_argument("--schedule", default="",
                    help='launch schedule as JSON, e.g. \'{"persistent": 1}\' (jx_schedule fields; default: the library default)')
    ap.add_argument("--permute", type=int, default=0,
                    help="R-MAT workloads: relabel the vertex ids by a bijection with this seed (0: none)")
    ap.add_argument("--unweighted", action="store_true", help="drop the vertex weights")
    ap.add_argument("--weighted", action="store_true",
                    help="add U(0,1] vertex weights (seed 4) to a workload that has none")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--e2e-worker", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-weighted-batch", action="store_true", help="batched: skip the weighted batch")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU leg (reference sample, oracle parity)")
    ap.add_argument("--no-unweighted", action="store_true",
                    help="weighted workloads: skip the unweighted calls reported beside")
    ap.add_argument("--cpu-seconds", type=float, default=20.0,
                    help="jx arm: seconds of the reference sample behind cpu_baseline")
    ap.add_argument("--ref-seconds", type=float, default=150.0,
                    help="reference arm: seconds of reference samples over all timed steps")
    args = ap.parse_args()
    if args.e2e_worker:
        e2e_worker(args)
        return
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
