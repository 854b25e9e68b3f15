#!/usr/bin/env python
"""Benchmark: M edges/s to full k-core on one GB300.

Default workload (the largest single-graph configuration): R-MAT scale 25,
edge factor 16 (a, b, c, d = 0.57, 0.19, 0.19, 0.05) plus a planted
4,000-vertex subgraph at edge probability 0.6, de-duplicated and symmetrised
(33.5M vertices, ~1.06B directed CSR entries, k_max 2,308), generated on the
device from fixed seeds.  A step is one full decomposition of that graph,
from the device-resident CSR to the core-number array.

Printed JSON line (rank 0):
  value      undirected edges x steps x ranks / max-over-ranks device time
             (CUDA events on the launching stream), inputs resident in HBM;
  e2e        the same metric through the C ABI with host buffers: each step
             copies the CSR host->device (pinned), decomposes, copies the core
             array back and frees the graph; steps run from three host threads
             (independent graph handles), so one step's upload overlaps the
             previous steps' decompositions, and these graphs run the peel on
             one CTA per SM so that two decompositions share the GPU (a peel
             alone is latency-bound: 28.0 ms on half the CTAs against 22.7 ms
             on all, but two at once take 17.8 ms each); serial_value: one
             thread and the default grid;
             the same K steps as value, the pipeline's fill (the first upload,
             which overlaps nothing) inside the timed region;
  roofline   algorithmic bytes B = 10*nnz + 16*n + 8 per decomposition over the
             main kernel's average CUDA-event duration, against the measured
             HBM copy bandwidth;
  cpu_baseline  serial Batagelj-Zaversnik (the oracle) on the same graph, on
             one host core, median of 3 runs;
  rmat22 / batched / serving / inputs  R-MAT scale 22 (the reference-sized
             graph) timed the same way, the 4096-graph batched form against
             the plain form, the request server's latency, and the
             input/output paths (generation, edge files, MatrixMarket parse,
             snapshots, k-core extraction).
`--impl reference` times the reference's CPU path (serial Batagelj-Zaversnik,
the oracle port) on the host cores on the same graph, generated on the host:
each step is one full decomposition, and the steps run as independent serial
decompositions on all host threads (throughput of the host).
`--gpus N` (under torchrun) runs N independent replicas: the decomposition of
one graph does not shard, every rank decomposes its own copy.
"""
import argparse
import ctypes
import json
import os
import queue
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "M edges/s to full k-core on 1 GB300 (batched vs plain); p50/p99 req latency"

WORKLOADS = {
    "rmat22": dict(kind="rmat", scale=22, ef=16, seed=2,
                   desc="R-MAT scale 22, edge factor 16, a/b/c/d=0.57/0.19/0.19/0.05, seed 2, "
                        "self-loops dropped, de-duplicated, symmetrised; one graph per step"),
    "er65536": dict(kind="er", n=65536, m=1048576, seed=1,
                    desc="Erdos-Renyi G(n=65536, m=1048576) without replacement, seed 1; one graph per step"),
    "rmat25planted": dict(kind="rmat_planted", scale=25, ef=16, k=4000, p=0.6, seed=3,
                          desc="R-MAT scale 25, edge factor 16 plus a planted 4000-vertex subgraph at p=0.6, "
                               "seed 3, de-duplicated, symmetrised; one graph per step"),
    # the same construction at a quarter of the size: the case profiled with
    # many-pass counter sets (a few GB on the device)
    "rmat23planted": dict(kind="rmat_planted", scale=23, ef=16, k=4000, p=0.6, seed=3,
                          desc="R-MAT scale 23, edge factor 16 plus a planted 4000-vertex subgraph at p=0.6, "
                               "seed 3, de-duplicated, symmetrised; one graph per step"),
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(kernel, workload):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    e = d.get(kernel, {}).get(workload)
    return None if e is None else float(e["bytes_per_launch"])


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled while the GPU is loaded."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0, t1):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, line in self.samples:
            if ts < t0 or ts > t1:
                continue
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg_ = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg_ = dist
    return world, rank, local, pg_


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_graph(pg, wl, device):
    if wl["kind"] == "rmat":
        return pg.rmat_graph(wl["scale"], wl["ef"], wl["seed"], device=device)
    if wl["kind"] == "er":
        return pg.er_graph(wl["n"], wl["m"], wl["seed"], device=device)
    return pg.rmat_planted_graph(wl["scale"], wl["ef"], wl["k"], wl["p"], wl["seed"], device=device)


def host_graph(wl, threads=1):
    """The same graph built on the host only (numpy + the oracle), for the CPU arm."""
    import numpy as np

    import oracle
    from oracle import gen
    if wl["kind"] == "rmat":
        n = 1 << wl["scale"]
        s, d = gen.rmat(wl["scale"], wl["ef"] * n, wl["seed"], threads=threads)
    elif wl["kind"] == "er":
        n = wl["n"]
        s, d = gen.er(wl["n"], wl["m"], wl["seed"])
    else:
        n = 1 << wl["scale"]
        s1, d1 = gen.rmat(wl["scale"], wl["ef"] * n, wl["seed"], threads=threads)
        s2, d2 = gen.planted(n, wl["k"], wl["p"], wl["seed"] + 1)
        s, d = np.concatenate([s1, s2]), np.concatenate([d1, d2])
        del s1, d1
    return oracle.csr_dedup(n, s, d, threads=threads)


def cpu_bz(rowptr, col, reps):
    import oracle
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.bz(rowptr, col)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, wl, world, rank, dist):
    """The reference's CPU path (serial Batagelj-Zaversnik port) on host cores:
    every step is one full decomposition of the workload graph; the steps run
    as independent serial decompositions on all host threads (the oracle
    releases the interpreter lock), so the value is the host's throughput."""
    if rank != 0:
        return 0
    import oracle
    threads = max(1, os.cpu_count() or 1)
    t0 = time.perf_counter()
    rowptr, col = host_graph(wl, threads=threads)
    build_s = time.perf_counter() - t0
    n = rowptr.size - 1
    m = int(rowptr[-1]) // 2
    workers = max(1, min(threads, args.steps))

    def one(_i):
        oracle.bz(rowptr, col)

    with ThreadPoolExecutor(workers) as ex:
        list(ex.map(one, range(args.warmup)))
        t0 = time.perf_counter()
        list(ex.map(one, range(args.steps)))
        total = time.perf_counter() - t0
    value = m * args.steps / total / 1e6
    sample = ("full graph, %d decompositions as independent serial Batagelj-Zaversnik runs on %d host threads "
              "(%d warm-up runs first)" % (args.steps, workers, args.warmup))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "M edges/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": wl["desc"], "n": n, "m_undirected": m, "nnz": int(rowptr[-1]),
                   "method": "serial Batagelj-Zaversnik (oracle port), host", "l2": "n/a (host)"},
        "cpu_baseline": {"value": round(value, 3), "unit": "M edges/s", "cores": workers, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "M edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "host": {"nproc": os.cpu_count(), "cpu": _cpu_model(), "graph_build_s": round(build_s, 2)},
    }
    print(json.dumps(line), flush=True)
    return 0


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_engine(args, wl, world, rank, local, dist):
    import numpy as np
    import torch

    import pico_gb300 as pg
    device = local
    torch.cuda.set_device(device)
    g = make_graph(pg, wl, device)
    for name, val in args.param:
        g.set_param(name, val)
    n, nnz = g.n, g.nnz
    m = nnz // 2
    stream = torch.cuda.Stream(device=device)
    sptr = stream.cuda_stream
    method = args.method

    sampler = ClockSampler(device)
    sampler.start()
    t_load0 = time.time()
    for _ in range(args.warmup):
        g.decompose_device(method, stream=sptr)
    # keep the same load running until the clock sampler has seen it for a while
    while time.time() - t_load0 < args.clock_window:
        g.decompose_device(method, stream=sptr)
    kernel_ms = []
    barrier(dist)
    torch.cuda.synchronize(device)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        g.decompose_device(method, stream=sptr)
        kernel_ms.append(g.last_timing()[1])
    ev1.record(stream)
    torch.cuda.synchronize(device)
    barrier(dist)
    t_load1 = time.time()
    sampler.stop()
    local_ms = ev0.elapsed_time(ev1)
    total_ms = allmax(dist, local_ms)
    value = m * args.steps * world / (total_ms / 1e3) / 1e6

    # correctness of the timed configuration is covered by the gpu tests; the
    # bench still records the result summary
    st = g.decompose_device(method, stream=sptr, stats=True)

    bytes_alg = 10 * nnz + 16 * n + 8
    kavg = statistics.mean(kernel_ms)
    achieved = bytes_alg / (kavg / 1e3) / 1e9
    peak, peak_kind = load_peaks()
    kernel_name = "hindex_kernel" if pg.method_id(method) in (0, 1, 2) else "peel_kernel"
    # the recorded traffic belongs to the default tunables
    traffic = None if args.param else load_traffic(kernel_name, args.workload)

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "M edges/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded device generator)",
        "config": {"workload": wl["desc"], "n": n, "m_undirected": m, "nnz": nnz, "method": method,
                   "parallelism": "replicas x%d (graph does not shard)" % world,
                   "l2": "inputs larger than L2 (col array %.0f MB > 129 MB L2)" % (4 * nnz / 1e6),
                   "kmax": st.kmax, "levels": st.levels, "level_indices": st.iterations,
                   "build_ms": round(st.build_ms, 3), **({"params": dict(args.param)} if args.param else {})},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": kernel_name, "bytes_per_launch": bytes_alg,
                     "kernel_ms_avg": round(kavg, 4)},
        # kernels per decomposition: peel_ctl_reset + peel_init + peel_kernel
        # (+ gpp_zero_to_one for gppeel); hindex_init + hx_order_rows (the
        # degree-ordered copy of the long rows, unless hindex.order is 0) +
        # hindex_kernel
        "gpu_launches": args.steps * ((4 if pg.method_id(method) == 4 else 3) if kernel_name == "peel_kernel"
                                      else (2 if dict(args.param).get("hindex.order", 1) == 0 else 3)),
        "clocks": sampler.summary(t_load0, t_load1),
    }

    rowptr, col = g.csr()
    # end to end through the C ABI with pinned host buffers
    h_rp = pg.ctypes.c_void_p()
    h_col = pg.ctypes.c_void_p()
    h_core = pg.ctypes.c_void_p()
    pg.check(pg.lib().kc_host_alloc(pg.ctypes.byref(h_rp), 8 * (n + 1)))
    pg.check(pg.lib().kc_host_alloc(pg.ctypes.byref(h_col), 4 * max(nnz, 1)))
    pg.check(pg.lib().kc_host_alloc(pg.ctypes.byref(h_core), 4 * max(n, 1)))
    ctypes.memmove(h_rp.value, rowptr.ctypes.data, 8 * (n + 1))
    ctypes.memmove(h_col.value, col.ctypes.data, 4 * nnz)
    core_view = np.ctypeslib.as_array((ctypes.c_uint32 * max(n, 1)).from_address(h_core.value))
    e2e_steps = max(4, args.steps)
    mid = pg.method_id(method)
    depth = max(1, args.e2e_depth)
    h_cores = [h_core]
    for _ in range(depth - 1):
        extra = pg.ctypes.c_void_p()
        pg.check(pg.lib().kc_host_alloc(pg.ctypes.byref(extra), 4 * max(n, 1)))
        h_cores.append(extra)
    free_cores = queue.Queue()
    for c in h_cores:
        free_cores.put(c)

    phases = []  # (upload ms, decomposition ms) of each step, from the graph's CUDA events

    def e2e_step(_i=0, shared=True):
        # one step through the public C ABI: pinned host CSR -> device graph,
        # decomposition with the core array written to pinned host memory;
        # `shared`: the GPU runs other steps' decompositions beside this one
        out = free_cores.get()
        try:
            h = pg.Graph.from_csr_ptr(h_rp.value, h_col.value, n, device=device)
            if shared and args.e2e_ctas_per_sm:
                h.set_param("peel.ctas_per_sm", args.e2e_ctas_per_sm)
            for name, val in args.param:
                h.set_param(name, val)
            est = pg.kc_stats()
            pg.check(pg.lib().kc_decompose(h.handle, mid, pg.ctypes.c_void_p(out.value), 0, pg.ctypes.byref(est),
                                           None))
            phases.append((est.build_ms, est.ms))
            h.free()
        finally:
            free_cores.put(out)

    def timed(run):
        barrier(dist)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        run()
        torch.cuda.synchronize(device)
        t1 = time.perf_counter()
        barrier(dist)
        return allmax(dist, t1 - t0)

    e2e_step(shared=False)
    phases.clear()
    serial_s = timed(lambda: [e2e_step(shared=False) for _ in range(e2e_steps)])
    serial_up_ms = statistics.median(p[0] for p in phases) if phases else 0.0
    serial_dec_ms = statistics.median(p[1] for p in phases) if phases else 0.0
    # the same steps from `depth` host threads: graph handles are independent,
    # so one step's upload overlaps the previous step's decomposition
    with ThreadPoolExecutor(depth) as ex:
        list(ex.map(e2e_step, range(depth)))
        phases.clear()
        e2e_s = timed(lambda: list(ex.map(e2e_step, range(e2e_steps))))
    up_ms = statistics.median(p[0] for p in phases) if phases else 0.0
    dec_ms = statistics.median(p[1] for p in phases) if phases else 0.0
    _ = int(core_view[:n].max()) if n else 0
    line["e2e"] = {"value": round(m * e2e_steps * world / e2e_s / 1e6, 3), "unit": "M edges/s",
                   "h2d_bytes_per_step": 8 * (n + 1) + 4 * nnz, "d2h_bytes_per_step": 4 * n,
                   "steps": e2e_steps, "ms_per_step": round(1e3 * e2e_s / e2e_steps, 3),
                   "host_threads": depth, "peel_ctas_per_sm": args.e2e_ctas_per_sm or None,
                   "serial_value": round(m * e2e_steps * world / serial_s / 1e6, 3),
                   "serial_ms_per_step": round(1e3 * serial_s / e2e_steps, 3),
                   # per step, median: the upload's time and rate from its
                   # own CUDA events (with several steps in flight this
                   # includes waiting for the copy engine behind another
                   # step's upload; serial_upload_GB_per_s is the link's own
                   # rate, about 211 GB/s host to device) and the
                   # decomposition's device time
                   "upload_ms": round(up_ms, 3),
                   "upload_GB_per_s": round((8 * (n + 1) + 4 * nnz) / (up_ms * 1e6), 1) if up_ms else None,
                   "decompose_ms": round(dec_ms, 3),
                   "serial_upload_GB_per_s": round((8 * (n + 1) + 4 * nnz) / (serial_up_ms * 1e6), 1)
                   if serial_up_ms else None,
                   # one thread: a step's wall time = upload + decomposition +
                   # the rest (graph set-up and free, host calls, the read-back)
                   "serial_decompose_ms": round(serial_dec_ms, 3),
                   "serial_other_ms": round(1e3 * serial_s / e2e_steps - serial_up_ms - serial_dec_ms, 3)}
    for p in h_cores[1:]:
        pg.lib().kc_host_free(p)
    for p in (h_rp, h_col, h_core):
        pg.lib().kc_host_free(p)
    g.free()
    # the other sections are reported beside the headline; a failure there is
    # recorded in its section instead of losing the line.  The second
    # single-graph workload runs first, in the same state of the process as
    # the headline's timing.
    c2 = None
    if world == 1 and args.workload != "rmat22" and not args.no_c2:
        try:
            line["rmat22"], c2 = graph_section(pg, device, sptr, "rmat22", method, args.steps)
        except Exception as e:  # noqa: BLE001
            line["rmat22"] = {"error": "%s: %s" % (type(e).__name__, e)}
    # the CPU baseline runs after the device and end-to-end timings, which its
    # tens of seconds of host memory traffic would otherwise disturb
    if rank == 0 and world == 1 and not args.no_cpu:
        reps = 3
        t = cpu_bz(rowptr, col, reps)
        line["cpu_baseline"] = {"value": round(m / statistics.median(t) / 1e6, 3), "unit": "M edges/s",
                                "cores": 1, "kind": "port",
                                "sample": "full graph, serial Batagelj-Zaversnik, median of %d runs (%s s)"
                                          % (reps, ", ".join("%.2f" % x for x in t)),
                                "host": _cpu_model(), "nproc": os.cpu_count()}

    del rowptr, col
    if world == 1 and not args.no_batch:
        try:
            line["batched"] = batch_section(pg, device, sptr, args.steps, args.warmup, args.batch_graphs,
                                            not args.no_autotune)
        except Exception as e:  # noqa: BLE001
            line["batched"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if world == 1 and not args.no_serve:
        try:
            line["serving"] = serve_section(pg, device, args.serve_requests, args.serve_rate)
        except Exception as e:  # noqa: BLE001
            line["serving"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if world == 1 and not args.no_refgpu:
        try:
            line["reference_gpu"] = reference_gpu_section(pg, device, args.refgpu_graphs.split(","))
        except Exception as e:  # noqa: BLE001
            line["reference_gpu"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if world == 1 and not args.no_inputs:
        try:
            if c2 is None:
                gi = make_graph(pg, WORKLOADS["rmat22"], device)
                c2 = gi.csr() + (gi.decompose_device(method, stats=True).kmax,)
                gi.free()
            line["inputs"] = inputs_section(pg, device, WORKLOADS["rmat22"], *c2)
        except Exception as e:  # noqa: BLE001
            line["inputs"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


REFGPU_GRAPHS = {"er65536": ("Erdos-Renyi G(65536, 1048576), seed 1", "er65536"),
                 "rmat22": ("R-MAT scale 22, edge factor 16, seed 2", "rmat22")}


def reference_gpu_section(pg, device, graphs):
    """The reference's own GPU drivers (compiled for sm_103a from their
    sources, run as separate processes on a MatrixMarket file) beside this
    engine's decomposition of the same file with the same loader semantics:
    each driver's own printed time (index2core / peelone / gppeel: wall ms of
    the iteration loop; peel_dyn / peelone_dyn: integer ms of one call)
    against the CUDA-event time of this engine's decomposition (median of 5),
    and whether the core arrays are identical.  The peel/src drivers keep
    fixed per-block queues of 10^6 entries with a device assert on overflow,
    so they run only on graphs of fewer than 10^6 vertices."""
    import tempfile

    import numpy as np

    from oracle import ref_gpu
    if not ref_gpu.sources_present():
        return {"unavailable": "reference GPU driver sources not copied next to the tree"}
    t0 = time.perf_counter()
    ref_gpu.build()
    out = {"build_s": round(time.perf_counter() - t0, 1), "graphs": []}
    for name in graphs:
        desc, wl_name = REFGPU_GRAPHS[name]
        g = make_graph(pg, WORKLOADS[wl_name], device)
        rp, col = g.csr()
        g.free()
        n = rp.size - 1
        used = np.flatnonzero(np.diff(rp) > 0)
        n_file = int(used[-1]) + 1 if used.size else 0
        entry = {"graph": desc, "n": n_file, "m_undirected": int(rp[-1]) // 2, "drivers": []}
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, name + ".mtx")
            src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
            up = src < col
            e = np.stack([src[up] + 1, col[up].astype(np.int64) + 1], axis=1)
            with open(path, "w") as f:
                f.write("%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (n, n, e.shape[0]))
                np.savetxt(f, e, fmt="%d")
            del src, up, e
            drivers = list(ref_gpu.INDEX2CORE + ref_gpu.PEEL_VG)
            if n_file < 1000000:
                drivers += list(ref_gpu.DYN)
            engines = {}
            for d in drivers:
                mode = "csr" if d in ref_gpu.DYN else "coo"
                t1 = time.perf_counter()
                r = ref_gpu.run(d, path, n_file, timeout=1800)
                wall = time.perf_counter() - t1
                if mode not in engines:
                    engines[mode] = pg.Graph.from_mtx(path, mode, device=device)
                h = engines[mode]
                got, _ = h.decompose(d)
                ms = []
                for _ in range(5):
                    h.decompose_device(d)
                    ms.append(h.last_timing()[0])
                e_ms = statistics.median(ms)
                entry["drivers"].append({
                    "driver": d, "reference_ms": r.ms, "engine_ms": round(e_ms, 4),
                    "speedup": round(r.ms / e_ms, 1) if r.ms else None, "identical": bool(np.array_equal(got, r.core)),
                    "reference_iterations": r.iterations, "reference_process_s": round(wall, 1)})
            for h in engines.values():
                h.free()
        out["graphs"].append(entry)
    return out


def graph_section(pg, device, sptr, name, method, steps):
    """One more single-graph workload timed like the headline (CUDA events
    around `steps` decompositions after warm-up, the main kernel's own
    events for the roofline); returns the section and (rowptr, col, kmax)."""
    import torch
    wl = WORKLOADS[name]
    g = make_graph(pg, wl, device)
    n, nnz = g.n, g.nnz
    for _ in range(3):
        g.decompose_device(method, stream=sptr)
    stream = torch.cuda.ExternalStream(sptr, device=device)
    torch.cuda.synchronize(device)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kernel_ms = []
    ev0.record(stream)
    for _ in range(steps):
        g.decompose_device(method, stream=sptr)
        kernel_ms.append(g.last_timing()[1])
    ev1.record(stream)
    torch.cuda.synchronize(device)
    ms = ev0.elapsed_time(ev1) / steps
    st = g.decompose_device(method, stream=sptr, stats=True)
    kavg = statistics.mean(kernel_ms)
    bytes_alg = 10 * nnz + 16 * n + 8
    peak, peak_kind = load_peaks()
    kernel_name = "hindex_kernel" if pg.method_id(method) in (0, 1, 2) else "peel_kernel"
    out = {"workload": wl["desc"], "n": n, "nnz": nnz, "m_undirected": nnz // 2, "method": method,
           "steps": steps, "ms_per_step": round(ms, 4), "value": round((nnz // 2) / (ms / 1e3) / 1e6, 3),
           "unit": "M edges/s", "kmax": st.kmax, "levels": st.levels, "level_indices": st.iterations,
           "roofline": {"kernel": kernel_name, "kernel_ms_avg": round(kavg, 4), "bytes_per_launch": bytes_alg,
                        "achieved": round(bytes_alg / (kavg / 1e3) / 1e9, 1), "peak": peak, "peak_kind": peak_kind,
                        "frac": round(bytes_alg / (kavg / 1e3) / 1e9 / peak, 4),
                        "traffic": load_traffic(kernel_name, name)}}
    rowptr, col = g.csr()
    g.free()
    return out, (rowptr, col, st.kmax)


def inputs_section(pg, device, wl, rowptr, col, kmax):
    """The input and output paths around the decomposition, timed on the host
    clock (each call returns with its result on the device or host): device
    generation and CSR build of the workload graph, a binary edge file
    (mmap, upload, de-duplicating device build), a MatrixMarket text parse on
    a smaller R-MAT graph, snapshot save and load, a device build from host
    edge arrays, and induced k-core extraction.  Files are written first and
    read back while page-cached, so these are parse / upload / build rates,
    not disk rates."""
    import tempfile

    import numpy as np
    import torch

    out = {"workload": wl["desc"].split(";")[0]}

    def clock(fn):
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize(device)
        return r, 1e3 * (time.perf_counter() - t0)

    if wl["kind"] == "rmat":
        g, ms = clock(lambda: pg.rmat_graph(wl["scale"], wl["ef"], wl["seed"], device=device))
        out["generate_and_build_ms"] = round(ms, 2)
        g.free()
    n = rowptr.size - 1
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(rowptr))
    up = src < col  # each undirected edge once
    us, ud = src[up], col[up]
    m = int(us.size)
    with tempfile.TemporaryDirectory() as tmp:
        # binary edge file: little-endian uint32 (src, dst) pairs
        path = os.path.join(tmp, "edges.bin")
        np.stack([us, ud], axis=1).astype("<u4").tofile(path)
        nbytes = os.path.getsize(path)
        g, ms = clock(lambda: pg.Graph.from_edge_file(path, dedup=True, device=device))
        assert g.nnz == col.size
        out["edge_file"] = {"bytes": nbytes, "edges": m, "ms": round(ms, 2),
                            "GB_per_s": round(nbytes / ms / 1e6, 2)}
        g.free()
        os.remove(path)
        # host edge arrays -> device CSR with de-duplication
        g, ms = clock(lambda: pg.Graph.from_edges(us, ud, n, dedup=True, device=device))
        assert g.nnz == col.size
        out["from_host_edges_ms"] = round(ms, 2)
        # snapshot of the decomposed graph
        g.decompose_device("peelone_dyn")
        path = os.path.join(tmp, "graph.kcsnap")
        _, ms_save = clock(lambda: g.save(path))
        nbytes = os.path.getsize(path)
        h, ms_load = clock(lambda: pg.Graph.load(path, device=device))
        assert h.nnz == g.nnz
        h.free()
        os.remove(path)
        out["snapshot"] = {"bytes": nbytes, "save_ms": round(ms_save, 2), "load_ms": round(ms_load, 2),
                           "save_GB_per_s": round(nbytes / ms_save / 1e6, 2),
                           "load_GB_per_s": round(nbytes / ms_load / 1e6, 2)}
        # induced k-core of the decomposition
        k = max(1, kmax // 2)
        (sub, ids), ms = clock(lambda: g.kcore_subgraph(k))
        out["kcore_subgraph"] = {"k": k, "ms": round(ms, 2), "n_out": sub.n, "nnz_out": sub.nnz}
        sub.free()
        g.free()
        # MatrixMarket text (the reference's input format) of R-MAT scale 17
        g2 = pg.rmat_graph(17, 16, 9, device=device)
        rp2, col2 = g2.csr()
        g2.free()
        s2 = np.repeat(np.arange(rp2.size - 1, dtype=np.uint32), np.diff(rp2))
        up2 = s2 < col2
        e2 = np.stack([s2[up2] + 1, col2[up2] + 1], axis=1)
        path = os.path.join(tmp, "rmat17.mtx")
        with open(path, "w") as f:
            f.write("%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n"
                    % (rp2.size - 1, rp2.size - 1, e2.shape[0]))
            f.write("\n".join("%d %d" % (a, b) for a, b in e2.tolist()))
            f.write("\n")
        nbytes = os.path.getsize(path)
        (_, ps, _), ms_parse = clock(lambda: pg.parse_mtx(path, mode="coo"))
        assert ps.size == e2.shape[0]
        g3, ms_csr = clock(lambda: pg.Graph.from_mtx(path, mode="csr", device=device))
        assert g3.nnz == col2.size
        g3.free()
        out["mtx_text"] = {"graph": "R-MAT scale 17, edge factor 16, seed 9", "bytes": nbytes,
                           "edges": int(e2.shape[0]), "parse_ms": round(ms_parse, 2),
                           "parse_MB_per_s": round(nbytes / ms_parse / 1e3, 1),
                           "to_device_csr_ms": round(ms_csr, 2), "host_threads": os.cpu_count()}
    return out


BATCH_DESC = ("4096 graphs, n = floor(10^U(2,5)), generator uniform over Erdos-Renyi / R-MAT (a,b,c=.57,.19,.19) / "
              "Barabasi-Albert (m_BA in 1..32), average degree U[4,64], seed 4, packed as one segmented CSR")


def batch_section(pg, device, sptr, steps, warmup, num_graphs=4096, autotune=True):
    """Batched (one launch, CUDA graph, autotuned) against the plain form (one
    decomposition call per graph) over the same 4096 graphs; both results are
    compared graph by graph."""
    import numpy as np
    import torch

    from pico_gb300 import workloads
    t_gen = time.perf_counter()
    g, vbase, _ = workloads.batch_mix(num_graphs, seed=4, device=device)
    gen_s = time.perf_counter() - t_gen
    n, nnz = g.n, g.nnz
    m = nnz // 2
    b = pg.Batch(g, vbase)
    tuned_ms = b.autotune() if autotune else None
    for _ in range(warmup):
        b.decompose_device(stream=sptr)
    torch.cuda.synchronize(device)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.ExternalStream(sptr, device=device)
    ev0.record(stream)
    for _ in range(steps):
        b.decompose_device(stream=sptr)
    ev1.record(stream)
    torch.cuda.synchronize(device)
    batched_ms = ev0.elapsed_time(ev1) / steps
    core_b, _ = b.decompose(stream=sptr)

    G = vbase.size - 1
    segs = [g.segment(int(vbase[i]), int(vbase[i + 1])) for i in range(G)]
    for h in segs:
        h.decompose_device("peelone_dyn", stream=sptr)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    for h in segs:
        h.decompose_device("peelone_dyn", stream=sptr)
    torch.cuda.synchronize(device)
    plain_ms = 1e3 * (time.perf_counter() - t0)
    same = True
    for i, h in enumerate(segs):
        c, _ = h.decompose("peelone_dyn", stream=sptr)
        if not np.array_equal(c, core_b[int(vbase[i]):int(vbase[i + 1])]):
            same = False
        h.free()
    kb, kp = b.get_param("batch.small_n"), b.get_param("batch.small_threads")
    kc = b.get_param("batch.chunk")
    b.free()
    g.free()
    return {
        "workload": BATCH_DESC.replace("4096", str(G), 1), "graphs": G, "n_total": n, "m_undirected_total": m, "nnz_total": nnz,
        "value": round(m / (batched_ms / 1e3) / 1e6, 3), "unit": "M edges/s", "ms_per_step": round(batched_ms, 4),
        "steps": steps, "plain_value": round(m / (plain_ms / 1e3) / 1e6, 3), "plain_ms": round(plain_ms, 2),
        "plain_form": "one kc_decompose(KC_PEELONE_DYN) call per graph over the same device-resident graphs",
        "batched_over_plain": round(plain_ms / batched_ms, 2), "identical_results": same,
        "autotuned": {"batch.small_n": kb, "batch.small_threads": kp, "batch.chunk": kc,
                      "best_ms": round(tuned_ms, 4) if tuned_ms is not None else None},
        "generate_s": round(gen_s, 2),
    }


def serve_section(pg, device, requests, rate_hz, sweep_rates=(10.0, 50.0, 200.0)):
    """A Poisson stream of edge-update batches (against a resident R-MAT
    scale-22 graph) and decompositions of fresh batch-mix-style graphs,
    submitted at their arrival times to the continuous-batching server; then
    the same requests at the sweep's other arrival rates."""
    import numpy as np

    from pico_gb300 import workloads
    base = pg.rmat_graph(22, 16, 2, device=device)
    rp_base, col_base = base.csr()
    t_gen = time.perf_counter()
    reqs = workloads.serve_stream(rp_base, col_base, requests, seed=5, rate_hz=rate_hz, device=device)
    gen_s = time.perf_counter() - t_gen
    srv = pg.Server(base, decompose_slots=2, max_batch_graphs=64)
    t0 = time.perf_counter()
    res = workloads.run_stream(srv, reqs, realtime=True)
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    base.free()
    lat = np.array([r["latency_ms"] for r in res])
    # the same requests at other arrival rates (arrival times rescaled), each
    # against a fresh copy of the resident graph
    sweep = []
    for r_hz in sweep_rates:
        b2 = pg.rmat_graph(22, 16, 2, device=device)
        s2 = pg.Server(b2, decompose_slots=2, max_batch_graphs=64)
        scaled = [dict(q, t=q["t"] * rate_hz / r_hz) for q in reqs]
        t1 = time.perf_counter()
        res2 = workloads.run_stream(s2, scaled, realtime=True)
        w2 = time.perf_counter() - t1
        st2 = s2.stats()
        s2.close()
        b2.free()
        l2 = np.array([x["latency_ms"] for x in res2])
        sweep.append({"rate_req_s": r_hz, "p50_ms": round(float(np.percentile(l2, 50)), 3),
                      "p99_ms": round(float(np.percentile(l2, 99)), 3),
                      "throughput_req_s": round(len(res2) / w2, 2), "max_inflight": int(st2["max_inflight"]),
                      "failed": int(st2["failed"])})
    exact, checked = serve_exact(rp_base, col_base, reqs, res)
    del rp_base, col_base
    upd = [r for q, r in zip(reqs, res) if q["kind"] == "update"]
    dec = [r for q, r in zip(reqs, res) if q["kind"] == "decompose"]
    upd_edges = sum(q["ins"][0].size + q["dels"][0].size for q in reqs if q["kind"] == "update")
    dec_edges = sum(int(q["rowptr"][-1]) // 2 for q in reqs if q["kind"] == "decompose")

    def pct(x, p):
        return round(float(np.percentile(x, p)), 3) if len(x) else None

    return {
        "workload": ("resident R-MAT scale 22 ef 16 (seed 2); Poisson arrivals at %g req/s, seed 5; half edge-update "
                     "batches of floor(10^U(3,6)) edges (50/50 insert/delete), half decompositions of a fresh "
                     "batch-mix-style graph" % rate_hz),
        "requests": len(reqs), "updates": len(upd), "decompositions": len(dec),
        "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
        "p50_update_ms": pct([r["latency_ms"] for r in upd], 50),
        "p99_update_ms": pct([r["latency_ms"] for r in upd], 99),
        "p50_decompose_ms": pct([r["latency_ms"] for r in dec], 50),
        "p99_decompose_ms": pct([r["latency_ms"] for r in dec], 99),
        "throughput_req_s": round(len(reqs) / wall, 2),
        "throughput_m_edges_s": round((upd_edges + dec_edges) / wall / 1e6, 3),
        "failed": int(st["failed"]), "decompose_launches": int(st["decompose_launches"]),
        "max_inflight": int(st["max_inflight"]), "latency": "submission (arrival) to result on host",
        "exact": exact, "exact_checked": checked,
        "generate_s": round(gen_s, 2), "rate_sweep": sweep,
    }


def core_digest(core):
    """The request server's digest of a core array: sum of core[v] *
    splitmix64(v + 1), mod 2^64."""
    import numpy as np

    from oracle import gen
    v = np.arange(1, core.size + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return int((core.astype(np.uint64) * gen.mix64(v)).sum(dtype=np.uint64))


def serve_exact(base_rowptr, base_col, reqs, results):
    """Checks every served result against Batagelj-Zaversnik on the host,
    outside the timed latencies: decompositions on their own graphs, and each
    update on the resident graph as it stood after that update (the edge set
    replayed on the host: deletions, then insertions).  Compares the
    server's digests of the core arrays.  Returns (all equal, count)."""
    import numpy as np

    import oracle
    from pico_gb300 import workloads
    keys = workloads.edge_keys(base_rowptr, base_col)
    n = base_rowptr.size - 1
    jobs = []
    for q, r in zip(reqs, results):
        if q["kind"] == "decompose":
            jobs.append((q["rowptr"], q["col"], None, r["digest"]))
            continue
        (is_, id_), (ds_, dd_) = q["ins"], q["dels"]
        dk = np.minimum(ds_, dd_).astype(np.uint64) << np.uint64(32) | np.maximum(ds_, dd_).astype(np.uint64)
        ik = np.minimum(is_, id_).astype(np.uint64) << np.uint64(32) | np.maximum(is_, id_).astype(np.uint64)
        p = np.searchsorted(keys, dk)
        hit = (p < keys.size) & (keys[np.minimum(p, keys.size - 1)] == dk)
        keys = np.delete(keys, p[hit])
        ik = np.unique(ik[is_ != id_])
        p = np.searchsorted(keys, ik)
        ik = ik[~((p < keys.size) & (keys[np.minimum(p, keys.size - 1)] == ik))]
        keys = np.insert(keys, np.searchsorted(keys, ik), ik)
        jobs.append((None, None, keys, r["digest"]))

    def check(job):
        rp, col, k, want = job
        if k is not None:
            rp, col = oracle.csr_dedup(n, (k >> np.uint64(32)).astype(np.uint32),
                                       (k & np.uint64(0xffffffff)).astype(np.uint32), threads=2)
        core, _ = oracle.bz(rp, col)
        return core_digest(core) == want

    with ThreadPoolExecutor(max(1, min(8, (os.cpu_count() or 2) // 2))) as ex:
        ok = list(ex.map(check, jobs))
    return all(ok), len(ok)


def _param(text):
    name, sep, value = text.partition("=")
    if not sep or not name:
        raise argparse.ArgumentTypeError("expected NAME=VALUE, got %r" % text)
    return name, int(value, 0)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="rmat25planted")
    ap.add_argument("--method", default="peelone_dyn")
    ap.add_argument("--param", action="append", default=[], type=_param, metavar="NAME=VALUE",
                    help="a kc_graph_set_param tunable applied to the main graph (repeatable; the "
                         "roofline's traffic figure is then left out)")
    ap.add_argument("--clock-window", type=float, default=1.5,
                    help="seconds of identical load before the timed steps, so clocks are sampled under load")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-batch", action="store_true", help="skip the 4096-graph batched-vs-plain section")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving section")
    ap.add_argument("--no-inputs", action="store_true", help="skip the input/output path section")
    ap.add_argument("--no-c2", action="store_true", help="skip the R-MAT scale 22 section")
    ap.add_argument("--no-refgpu", action="store_true", help="skip the reference GPU driver section")
    ap.add_argument("--e2e-depth", type=int, default=3,
                    help="end-to-end steps in flight (host threads with their own graph handles)")
    ap.add_argument("--e2e-ctas-per-sm", type=int, default=1,
                    help="peel.ctas_per_sm of the end-to-end graphs (0: the library's default, all resident CTAs)")
    ap.add_argument("--refgpu-graphs", default="er65536,rmat22",
                    help="graphs of the reference GPU driver section (er65536, rmat22)")
    ap.add_argument("--batch-graphs", type=int, default=4096, help="graphs in the batched section")
    ap.add_argument("--no-autotune", action="store_true", help="batched section: keep the default configuration")
    ap.add_argument("--serve-requests", type=int, default=40)
    ap.add_argument("--serve-rate", type=float, default=20.0, help="Poisson arrival rate, requests/s")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    world, rank, local, dist = dist_setup()
    try:
        if args.impl == "reference":
            return run_reference(args, wl, world, rank, dist)
        return run_engine(args, wl, world, rank, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
