"""Benchmark of the pair-detection path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload NAME]

A step is one self-intersection query over the whole workload (count, scan,
scatter, pair test, compaction; the autotuner's choice is memoised after the
first query of a context). Default workload: 4,194,304 3-D boxes drawn from a
mixture of 64 Gaussians (sigma 0.02, means U[0.1,0.9]^3), lognormal sides
(median 0.002, log-sigma 0.5), fp32 quantised to the PBIG API's unsigned
coordinates (range 2^24); synthetic, seeded, generated on the host.

Reported: ``value`` = boxes/s with the boxes resident in HBM (CUDA events on
the query stream, L2 flushed between steps); ``e2e`` = the same through the
C ABI with pinned host buffers (H2D of the boxes and D2H of every pair inside
the timed region, host wall clock); ``roofline`` for the kernel with the
largest share of device time; ``cpu_baseline`` = the oracle (CPU restatement
of the reference pipeline, all host threads) on a bounded sample.

With --gpus N under torchrun every rank runs an independent replica on its
own GPU (the single-scene path does not shard); value = all ranks' boxes /
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "overlap pairs/s & boxes/s at 4M 3D boxes"
UNIT = "boxes/s"
BOX_BYTES = 28  # RectInfo, 3-D


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload(name: str):
    from pbig_gb300 import gen
    if name == "clustered4m":
        return gen.clustered3d(4194304, seed=0), gen.RANGE, "3D self-intersection, 4,194,304 boxes, 64-Gaussian mixture (sigma 0.02), lognormal sides (median 0.002, log-sigma 0.5), seed 0"
    if name == "clustered1m":
        return gen.clustered3d(1048576, seed=0), gen.RANGE, "3D self-intersection, 1,048,576 boxes, 64-Gaussian mixture (sigma 0.02), lognormal sides (median 0.002, log-sigma 0.5), seed 0 (profiling size)"
    if name == "plain2d":
        return gen.uniform2d(65536, seed=0), gen.RANGE, "2D self-intersection, 65,536 boxes, uniform corners, sides U[0.001,0.005], seed 0"
    if name == "bipartite4m":
        return ((gen.mixed3d(2097152, seed=0), gen.mixed3d(2097152, seed=1)), gen.RANGE,
                "3D bipartite red/blue, 2,097,152 red (seed 0) vs 2,097,152 blue (seed 1) boxes, uniform centres, "
                "sides U[0.001,0.004], 1% large with sides U[0.02,0.1]; red-blue pairs only")
    raise SystemExit(f"unknown workload {name}")


def nboxes(boxes) -> int:
    return sum(len(b) for b in boxes) if isinstance(boxes, tuple) else len(boxes)


def cpu_sample(boxes, m: int):
    """The first m boxes of a self-intersection workload; for a red/blue
    workload the union of the first m/2 red and m/2 blue boxes (blue rids
    renumbered after red): the reference has no red/blue mode, so its CPU
    path self-intersects the union."""
    if not isinstance(boxes, tuple):
        return boxes[:m]
    red, blue = boxes[0][:m // 2], boxes[1][:m - m // 2]
    u = np.concatenate([red, blue])
    u[len(red):, -1] += len(red)
    return np.ascontiguousarray(u)


class _Nvml:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml):
    SM clock, its maximum, power and the active clock-event reasons of one
    device. None when the library or the device cannot be opened."""

    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    @classmethod
    def open(cls, gpu: int):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = C.c_void_p()
            uuid = None
            try:
                import torch
                uuid = getattr(torch.cuda.get_device_properties(gpu), "uuid", None)
            except Exception:
                uuid = None
            rc = 1
            if uuid is not None:
                rc = lib.nvmlDeviceGetHandleByUUID(("GPU-" + str(uuid)).encode(), C.byref(h))
            if rc != 0:
                rc = lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(gpu), C.byref(h))
            if rc != 0:
                return None
            reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
            if reasons is None:
                reasons = lib.nvmlDeviceGetCurrentClocksThrottleReasons
            self = cls()
            self.C, self.lib, self.h, self.reasons = C, lib, h, reasons
            mx = C.c_uint()
            self.max_mhz = float(mx.value) if lib.nvmlDeviceGetMaxClockInfo(h, cls.SM, C.byref(mx)) == 0 else None
            return self
        except Exception:
            return None

    def sample(self):
        C = self.C
        clk, pw, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, C.byref(clk)) != 0:
            return None
        self.lib.nvmlDeviceGetPowerUsage(self.h, C.byref(pw))
        active = self.reasons(self.h, C.byref(rs)) == 0
        names = [nm for bit, nm in self.REASONS.items() if active and (rs.value & bit)]
        return float(clk.value), pw.value / 1000.0, names


class ClockSampler:
    """Clocks and throttle reasons sampled during the timed region: NVML
    queries every `period` seconds (read-only), else nvidia-smi every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int, period: float = 0.002):
        self.gpu = gpu
        self.period = period
        self.rows = []
        self.nvml_rows = []
        self._stop = threading.Event()
        self._t = None
        self._nvml = _Nvml.open(gpu)

    def _run(self):
        while not self._stop.is_set():
            if self._nvml is not None:
                try:
                    r = self._nvml.sample()
                    if r is not None:
                        self.nvml_rows.append(r)
                except Exception:
                    self._nvml = None
                self._stop.wait(self.period)
                continue
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(max(self.period, 0.2))

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if self.nvml_rows:
            sm = [r[0] for r in self.nvml_rows]
            reasons = sorted({nm for r in self.nvml_rows for nm in r[2]})
            return {"sm_mhz": float(np.median(sm)), "sm_min_mhz": min(sm), "sm_max_mhz": self._nvml_max(),
                    "reasons": reasons, "samples": len(self.nvml_rows), "source": f"nvml, {self.period * 1e3:g} ms"}
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows), "source": "nvidia-smi, 200 ms"}

    def _nvml_max(self):
        n = self._nvml
        return n.max_mhz if n is not None else None


def algorithmic_bytes(st: dict, n: int) -> dict:
    """Bytes each kernel must move at minimum (per launch): boxes are read
    whole (28 B), cells as one u32 count/start, entries as one u32, pairs as
    two u32; the pair test reads each entry and its box coordinates once."""
    C, E, P = st["cells"], st["entries"], st["pairs"]
    return {
        "count": n * BOX_BYTES + C * 4,
        "scan": 2 * C * 4,
        "scatter": n * BOX_BYTES + C * 4 + E * 4,
        "pairs": E * (4 + 24) + 8 * P,
    }


def cpu_baseline(boxes, range_, budget_s: float, threads: int):
    """Oracle (reference pipeline restated on the CPU, reference cell-size
    heuristic, all host threads) on the first n' boxes, n' sized so that one
    run takes about budget_s seconds."""
    from oracle import oracle as O
    n = nboxes(boxes)
    frac = 1 / 64
    m = max(1024, int(n * frac))
    t0 = time.perf_counter()
    O.grid_pairs(cpu_sample(boxes, m), range_, count_only=True, threads=threads)
    dt = time.perf_counter() - t0
    # the reference heuristic keeps the work per box roughly proportional to
    # the density, so time grows ~ n'^2 at fixed domain: scale conservatively
    while m < n and dt < budget_s / 4:
        m = min(n, m * 2)
        t0 = time.perf_counter()
        _, st = O.grid_pairs(cpu_sample(boxes, m), range_, count_only=True, threads=threads)
        dt = time.perf_counter() - t0
    smp = cpu_sample(boxes, m)
    _, st = O.grid_pairs(smp, range_, count_only=True, threads=threads)
    t0 = time.perf_counter()
    _, st = O.grid_pairs(smp, range_, count_only=True, threads=threads)
    dt = time.perf_counter() - t0
    what = "union of the first m/2 red and blue boxes, self-intersected" if isinstance(boxes, tuple) else "first boxes"
    return {"value": m / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{m} of {n} boxes ({what}; same generator), oracle grid pipeline with the reference cell-size heuristic (cs={st['cs']}), {st['pairs']} pairs, {dt:.2f} s",
            "pairs_per_s": st["pairs"] / dt}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        rank = int(os.environ["RANK"])
        local = int(os.environ.get("LOCAL_RANK", rank))
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return rank, local, ws
    return 0, 0, 1


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, ws):
    """Reference arm: the reference has no CPU implementation of its own, so
    its CPU path is the oracle's restatement of its pipeline (reference cell
    heuristic), timed on the host cores with all threads."""
    if rank != 0:
        return
    from oracle import oracle as O
    if args.workload in ("serving", "update4m"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving mode or resident scenes "
                          "(one pbig_check at a time, from scratch, on a process-global state)"}), flush=True)
        return
    if args.workload == "batched":
        return run_reference_batched(args)
    boxes, rng, desc = workload(args.workload)
    threads = os.cpu_count() or 1
    total_budget = 150.0
    per_step = total_budget / max(1, args.steps + args.warmup)
    n = nboxes(boxes)
    m = max(1024, n // 64)
    while m < n:
        t0 = time.perf_counter()
        O.grid_pairs(cpu_sample(boxes, m), rng, count_only=True, threads=threads)
        if time.perf_counter() - t0 > per_step / 3:
            break
        m = min(n, m * 2)
    sample = cpu_sample(boxes, m)
    for _ in range(args.warmup):
        O.grid_pairs(sample, rng, count_only=True, threads=threads)
    ts = []
    st = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, st = O.grid_pairs(sample, rng, count_only=True, threads=threads)
        ts.append(time.perf_counter() - t0)
    t = float(np.mean(ts))
    val = m / t
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": desc, "sample_boxes": m, "parallelism": "cpu threads"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{m} of {n} boxes per step ({'red/blue union' if isinstance(boxes, tuple) else 'first boxes'}); oracle restatement of the reference grid pipeline with its cell-size heuristic (cs={st['cs']}); {st['pairs']} pairs per step"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "pairs_per_s": st["pairs"] / t}
    print(json.dumps(line), flush=True)


def run_reference_batched(args):
    """Batched workload on the CPU reference: one grid query per scene (as the
    reference runs one pbig_check per scene), the scenes in order until the
    step's time budget is spent; boxes/s over the scenes done."""
    from oracle import oracle as O
    from pbig_gb300 import gen
    threads = os.cpu_count() or 1
    sizes = gen.scene_sizes(args.scenes, 0, 256, 262144)
    per_step = 150.0 / max(1, args.steps + args.warmup)

    def step():
        t_start = time.perf_counter()
        nb = npairs = k = 0
        busy = 0.0
        while k < len(sizes) and time.perf_counter() - t_start < per_step:
            b = gen.scene3d(int(sizes[k]), k)  # scene k of the batched workload (seed 1000003*0 + k)
            t1 = time.perf_counter()
            _, st = O.grid_pairs(b, gen.RANGE, count_only=True, threads=threads)
            busy += time.perf_counter() - t1
            nb += len(b)
            npairs += st["pairs"]
            k += 1
        return nb, npairs, k, busy

    for _ in range(args.warmup):
        step()
    res = [step() for _ in range(args.steps)]
    nb, npairs, k, dt = res[-1]
    val = nb / dt
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"{args.scenes} independent 3D scenes (the batched workload), one query per scene",
                       "parallelism": "cpu threads"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"the first {k} of {args.scenes} scenes per step ({nb} boxes), one oracle grid "
                                       f"query per scene with the reference cell-size heuristic; scene generation "
                                       f"not timed"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "pairs_per_s": npairs / dt, "scenes_per_s": k / dt}
    print(json.dumps(line), flush=True)


def stream_of_queries(eng, query, host, P, n, args, local, ws):
    """End to end for a stream of queries: two contexts (each with its own
    stream and page-locked pair buffer) on two host threads, the same host
    boxes in and host pairs out as the single-query figure, so that one
    query's box upload overlaps the other's pair download on the
    full-duplex host link. Every result is checked for its pair count and
    its place in its context's buffer."""
    import threading
    import torch
    from pbig_gb300 import Engine
    engs = [eng, Engine(local)]
    outs = [torch.empty((P + 64, 2), dtype=torch.int32).pin_memory() for _ in engs]
    streams = [torch.cuda.Stream(device=f"cuda:{local}") for _ in engs]
    nq = max(4, args.steps)
    ok = [True, True]
    try:
        for e, o, st in zip(engs, outs, streams):
            e.set_pair_output(o)
            for _ in range(2):  # warm-up: buffers and the tuner's memo of the second context
                query(host, e, st)
        torch.cuda.synchronize()

        def worker(k):
            for _ in range(nq):
                if query(host, engs[k], streams[k]) != P or not engs[k].result_in(outs[k]):
                    ok[k] = False

        barrier(ws)
        th = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
        t0 = time.perf_counter()
        for t in th:
            t.start()
        for t in th:
            t.join()
        dt = allmax(time.perf_counter() - t0, ws)
    finally:
        for e in engs:
            e.set_pair_output(None)
        engs[1].close()
    assert all(ok)
    per_q = dt / (2 * nq)
    return {"value": n * ws / per_q, "unit": UNIT, "ms_per_query": per_q * 1e3, "contexts": 2, "host_threads": 2,
            "queries": 2 * nq, "h2d_bytes_per_query": n * BOX_BYTES, "d2h_bytes_per_query": P * 8,
            "pairs_per_s": P * ws / per_q}


def run_gb300(args, rank, local, ws):
    import torch
    from pbig_gb300 import Engine

    torch.cuda.set_device(local)
    boxes, rng, desc = workload(args.workload)
    n = nboxes(boxes)
    parts = boxes if isinstance(boxes, tuple) else (boxes,)
    dev = [torch.from_numpy(b.view(np.int32)).to(f"cuda:{local}") for b in parts]
    host = [torch.from_numpy(b.view(np.int32)).pin_memory() for b in parts]
    # one stream for the L2 flush, the timing events and the queries, so
    # that each timed query starts after the flush and the events bracket it
    stream = torch.cuda.Stream(device=f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")  # > L2 (129 MB)
    torch.cuda.synchronize()
    eng = Engine(local)

    def query(src, e=None, st=None):
        e = e or eng
        st = st or stream
        if len(src) == 2:
            return e.bipartite_intersect(src[0], src[1], rng, stream=st)
        return e.self_intersect(src[0], rng, stream=st)

    for _ in range(args.warmup):
        query(dev)
        torch.cuda.synchronize()
    P = eng.result_count()
    out_host = torch.empty((P, 2), dtype=torch.int32).pin_memory()

    # device-resident timing
    step_ms, phase_acc, kernels, dev_acc = [], {}, 0, 0.0
    stats = None
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            np_ = query(dev)
            b.record(stream)
            b.synchronize()
            step_ms.append(a.elapsed_time(b))
            stats = eng.stats()
            kernels += stats["kernels"]
            dev_acc += stats["device_ms"]
            for k, v in stats["phase_ms"].items():
                phase_acc[k] = phase_acc.get(k, 0.0) + v
            assert np_ == P
        torch.cuda.synchronize()
    barrier(ws)
    t_step = allmax(float(np.sum(step_ms)) / 1e3, ws)
    value = n * args.steps * ws / t_step
    phase = {k: v / args.steps for k, v in phase_acc.items()}

    # end to end through the C ABI with page-locked host buffers: boxes go up
    # each step, and the pair kernels store the pairs straight into the host
    # buffer (pbig2_set_pair_output) while they run
    eng.set_pair_output(out_host)
    e2e_t = []
    for i in range(max(2, args.steps // 2) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        np_ = query(host)
        eng.sync(stream)
        t1 = time.perf_counter()
        assert np_ == P and eng.result_in(out_host)
        if i > 0:
            e2e_t.append(t1 - t0)
    eng.set_pair_output(None)
    e2e_step = allmax(float(np.mean(e2e_t)), ws)
    e2e = {"value": n * ws / e2e_step, "unit": UNIT, "h2d_bytes_per_step": n * BOX_BYTES,
           "d2h_bytes_per_step": P * 8, "ms_per_step": e2e_step * 1e3, "pairs_per_s": P * ws / e2e_step,
           "output": "pair kernels store into the page-locked host buffer (no separate copy)"}
    e2e["stream_of_queries"] = stream_of_queries(eng, query, host, P, n, args, local, ws)
    # parity spot check of the e2e copy (canonical pairs)
    got = out_host.numpy().view(np.uint32)
    if len(parts) == 1:
        assert (got[:, 0] < got[:, 1]).all()
    else:
        assert (got[:, 0] < len(parts[0])).all() and (got[:, 1] < len(parts[1])).all()

    # roofline of the dominant kernel; a query that ran as one launch (small
    # scenes) has one kernel doing every phase: its time on its own clock,
    # the phases' algorithmic bytes summed
    peak, peak_kind = peaks()
    algo = algorithmic_bytes(stats, n)
    one_launch = stats["kernels"] == 1
    if one_launch:
        algo = {"one_launch": sum(algo.values())}
        phase = {"one_launch": dev_acc / args.steps}
    share = {k: phase.get(k, 0.0) for k in algo}
    top = max(share, key=lambda k: share[k])
    ms = phase[top]
    achieved = algo[top] / (ms * 1e-3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tf):
        try:
            with open(tf) as f:
                traffic = json.load(f).get(args.workload, {}).get(top)
        except Exception:
            traffic = None
    kern = {k: {"ms": phase[k], "algorithmic_bytes": algo[k],
                "achieved_gbs": algo[k] / (phase[k] * 1e-3) / 1e9 if phase[k] > 0 else None,
                "frac_of_" + peak_kind: (algo[k] / (phase[k] * 1e-3) / 1e9) / peak if phase[k] > 0 else None}
            for k in algo}
    if one_launch:
        kern["one_launch"]["pair_tests_per_s"] = stats["pair_tests"] / (phase["one_launch"] * 1e-3)
    else:
        kern["pairs"]["pair_tests_per_s"] = stats["pair_tests"] / (phase["pairs"] * 1e-3)
        kern["pairs"]["split_ms"] = {k: phase.get("pairs_" + k, 0.0) for k in ("small", "med", "block")}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": desc, "boxes": n, "pairs": P, "range": rng, "cell_shift": stats["cell_shift"],
                   "entries": stats["entries"], "cells": stats["cells"], "pair_tests": stats["pair_tests"],
                   "class_map": hex(stats["class_map"]),
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "flushed between steps (256 MiB write)"},
        "pairs_per_s": P * args.steps * ws / t_step,
        "e2e": e2e,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": algo[top]},
        "kernels": kern,
        "gpu_launches": kernels,
        "clocks": clk.summary(),
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(boxes, rng, args.cpu_budget, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()


def _pair_keys(t):
    """[P,2] int32 device pairs (a, b) -> sorted int64 keys a << 32 | b."""
    import torch
    k = (t[:, 0].to(torch.int64) << 32) | t[:, 1].to(torch.int64)
    return torch.sort(k).values


def run_batched(args, rank, local, ws):
    """Batched scenes: one launch sequence for all scenes, pairs grouped by
    scene. Timed twice: with every scene's cell size chosen inside the call
    (the headline: the tuner's sample and choices are part of each step) and
    with per-scene cell sizes computed beforehand (the engine's tuner on a
    512-box sample of each scene, host side). The plain loop runs one
    single-scene query per scene with those precomputed sizes. After the
    timing every scene's batched pair list is compared with its plain-path
    list (both sorted on the device): the outputs are identical scene by
    scene, not only in total."""
    import torch
    from pbig_gb300 import Engine, gen, tune_shift

    torch.cuda.set_device(local)
    count = args.scenes
    boxes, offs = gen.scene_batch(count, seed=0)
    n = boxes.shape[0]
    shifts = np.array([tune_shift(boxes[int(offs[i]):int(offs[i + 1])], gen.RANGE, 512) for i in range(count)],
                      dtype=np.uint32)
    dev = torch.from_numpy(boxes.view(np.int32)).to(f"cuda:{local}")
    stream = torch.cuda.current_stream()
    eng = Engine(local)

    def timed(cell_shifts):
        for _ in range(args.warmup):
            eng.batch_intersect(dev, offs, gen.RANGE, cell_shifts=cell_shifts, stream=stream)
        P = eng.result_count()
        ts, kern = [], 0
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            assert eng.batch_intersect(dev, offs, gen.RANGE, cell_shifts=cell_shifts, stream=stream) == P
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
            kern += eng.stats()["kernels"]
        return P, allmax(float(np.mean(ts)), ws), kern, eng.stats()

    with ClockSampler(local) as clk:
        P0, t_pre, _, _ = timed(shifts)
        P, t_b, kern, st = timed(None)
    assert P == P0
    # the tuned batch's result, grouped by scene, kept on the device
    res = torch.empty((P, 2), dtype=torch.int32, device=f"cuda:{local}")
    eng.pairs_into(res, stream=stream)
    so = eng.scene_offsets()
    torch.cuda.synchronize()
    # plain loop: one query per scene (precomputed cell sizes), pairs left on the device
    plain_pairs = 0
    for i in range(min(count, 64)):  # warm-up
        eng.self_intersect(dev[int(offs[i]):int(offs[i + 1])], gen.RANGE, cell_shift=int(shifts[i]), stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(count):
        plain_pairs += eng.self_intersect(dev[int(offs[i]):int(offs[i + 1])], gen.RANGE, cell_shift=int(shifts[i]),
                                          stream=stream)
    torch.cuda.synchronize()
    t_p = allmax(time.perf_counter() - t0, ws)
    # scene-by-scene equality (outside the timed regions)
    mismatched = 0
    for i in range(count):
        k = eng.self_intersect(dev[int(offs[i]):int(offs[i + 1])], gen.RANGE, cell_shift=int(shifts[i]),
                               stream=stream)
        mine = res[int(so[i]):int(so[i + 1])]
        if k != mine.shape[0]:
            mismatched += 1
            continue
        if k == 0:
            continue
        plain = torch.empty((k, 2), dtype=torch.int32, device=f"cuda:{local}")
        eng.pairs_into(plain, stream=stream)
        if not torch.equal(_pair_keys(mine), _pair_keys(plain)):
            mismatched += 1
    torch.cuda.synchronize()
    assert plain_pairs == P and mismatched == 0, (plain_pairs, P, mismatched)
    line = {
        "metric": METRIC + " (batched scenes)", "value": n * ws / t_b, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_b * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"{count} independent 3D scenes, sizes log-uniform in [256, 262144] (total {n} boxes), uniform centres, sides U[0.5,2]*n^(-1/3)*0.5, seed 0; every scene's cell size tuned inside the call",
                   "scenes": count, "boxes": n, "pairs": P, "class_map": hex(st["class_map"]),
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "inputs (4.3 GB) far larger than L2"},
        "pairs_per_s": P * ws / t_b,
        "scenes_per_s": count * ws / t_b,
        "precomputed_cell_sizes": {"value": n * ws / t_pre, "unit": UNIT, "ms": t_pre * 1e3},
        "plain_loop": {"value": n * ws / t_p, "unit": UNIT, "ms": t_p * 1e3, "scenes_per_s": count * ws / t_p,
                       "cell_sizes": "precomputed (512-box sample per scene), not timed"},
        "batched_over_plain": t_p / t_b,
        "parity": {"scenes_compared": count, "scenes_mismatched": mismatched,
                   "how": "each scene's batched pair list (cell sizes tuned in the call) equals its plain-path "
                          "list, sorted on the device"},
        "phase_ms": st["phase_ms"],
        "gpu_launches": kern,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()


def run_update(args, rank, local, ws):
    """Incremental updates of a resident scene (pbig2_scene_*): the clustered
    4M-box scene stays on the device, every step moves 1% of its boxes by
    N(0, 0.001) and asks for the pairs they had and have (copied to the host)
    and the updated full pair list (kept on the device). The same boxes are
    also queried from scratch for comparison."""
    import torch
    from pbig_gb300 import Engine, Scene, gen
    from pbig_gb300.serve import move_indices

    torch.cuda.set_device(local)
    boxes = gen.clustered3d(4194304, seed=0)
    n = len(boxes)
    eng = Engine(local)
    sc = Scene(eng, boxes, gen.RANGE, keep_pairs=not args.delta_only)
    cur = boxes.copy()
    steps = []

    def pinned(a):  # page-locked copy of a host array
        t = torch.empty(a.shape, dtype=torch.int32).pin_memory()
        v = t.numpy().view(np.uint32)
        v[...] = a
        return v

    for i in range(args.warmup + args.steps):  # the moves, made before the timing (page-locked inputs)
        idx = move_indices(n, 0.01, 7000 + i)
        gen.move3d(cur, idx, 7000 + i, sigma=0.001)
        steps.append((pinned(idx), pinned(cur[idx])))
    out_rem = pinned(np.zeros((4 << 20, 2), dtype=np.uint32))
    out_add = pinned(np.zeros((4 << 20, 2), dtype=np.uint32))
    for idx, nb in steps[:args.warmup]:
        sc.move(idx, nb)
        sc.delta(out_rem, out_add)
    ts, moved, delta_pairs = [], 0, 0
    with ClockSampler(local) as clk:
        for idx, nb in steps[args.warmup:]:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            nr, na = sc.move(idx, nb)
            rem, add = sc.delta(out_rem, out_add)
            ts.append(time.perf_counter() - t0)
            moved += len(idx)
            delta_pairs += nr + na
    t_up = allmax(float(np.mean(ts)), ws)
    P = len(sc.pairs()) if not args.delta_only else None
    # the same final boxes from scratch, device-resident
    dev = torch.from_numpy(cur.view(np.int32)).to(f"cuda:{local}")
    for _ in range(2):
        eng.self_intersect(dev, gen.RANGE)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        P2 = eng.self_intersect(dev, gen.RANGE)
        assert P is None or P2 == P
    P = P2
    torch.cuda.synchronize()
    t_full = (time.perf_counter() - t0) / reps
    line = {
        "metric": METRIC, "value": n * ws / t_up, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_up * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "incremental updates of a resident scene: 4,194,304 clustered 3D boxes (seed 0), "
                               "each step moves 1% of them (41,943 boxes) by N(0,0.001); value = scene boxes / update time"
                               + ("; delta only (no full pair list kept)" if args.delta_only else
                                  "; the full pair list is kept current on the device"),
                   "pairs": P, "parallelism": "replicas" if ws > 1 else "single GPU"},
        "moved_per_step": moved // max(1, args.steps), "delta_pairs_per_step": delta_pairs // max(1, args.steps),
        "full_query_ms": t_full * 1e3, "speedup_vs_full_query": t_full / t_up,
        "e2e": {"value": n * ws / t_up, "unit": UNIT, "h2d_bytes_per_step": int(moved // max(1, args.steps) * 32),
                "d2h_bytes_per_step": int(delta_pairs // max(1, args.steps) * 8),
                "note": "moved rows go up from the host and both pair lists come back inside the timed step"},
        "gpu_launches": 9 * args.steps,  # per move: check, mark, query, remove, write, insert, query, filter, unmark
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    sc.close()
    eng.close()


def run_serving(args, rank, local, ws):
    """Serving loop: Poisson arrivals of scene queries (sizes log-uniform in
    [1024, 1048576], the batched scenes' generator) and updates (30 %: 1 % of
    a resident scene's boxes moved by N(0, 0.001)), continuous batching over
    two engine slots, 40 GB device budget. Latency = completion - arrival,
    including the host->device copy of new scenes and the device->host copy
    of every pair."""
    import torch
    from pbig_gb300 import serve

    torch.cuda.set_device(local)
    reqs = serve.make_requests(args.duration, rate=args.rate, seed=0)
    # warm-up: a short stream of small scenes through a separate server
    warm = serve.make_requests(0.02, rate=args.rate, seed=99, lo=1024, hi=65536)
    srv = serve.Server(device=local)
    th = serve.feed(srv, warm)
    srv.serve(len(warm))
    th.join()
    srv.close()
    # pairs are delivered into each slot's page-locked host buffer (the
    # device->host copy is timed; no second host copy)
    srv = serve.Server(device=local, budget_bytes=40 << 30, copy_pairs=False, reserve_boxes=4 << 20)
    with ClockSampler(local, period=0.05) as clk:  # (the serving loop runs in Python threads)
        th = serve.feed(srv, reqs)
        srv.serve(len(reqs))
        th.join()
    s = serve.latency_summary(reqs)
    sizes = [r.nboxes for r in reqs]
    line = {
        "metric": METRIC + " (serving p50/p99)", "value": s["p99_ms"], "unit": "ms (p99 latency)", "n_gpus": ws,
        "steps": len(reqs), "warmup": len(warm), "ms_per_step": s["mean_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"serving: Poisson arrivals at {args.rate:.0f} req/s for {args.duration} s, 30% updates moving 1% of a resident scene's boxes by N(0,0.001), new scenes log-uniform in [1024, 1048576] boxes, 40 GB device budget, 2 slots, capacity for 4,194,304-box batches reserved at start",
                   "requests": len(reqs), "updates": sum(r.kind == "update" for r in reqs),
                   "mean_scene_boxes": float(np.mean(sizes)), "parallelism": "single GPU"},
        "latency_ms": {"p50": s["p50_ms"], "p99": s["p99_ms"], "mean": s["mean_ms"], "max": s["max_ms"]},
        "pairs_per_s": s["pairs_per_s"], "boxes_per_s": s["boxes_per_s"],
        "batches": srv.batches, "mean_batch_requests": len(reqs) / max(1, srv.batches),
        "gpu_slot_busy_fraction": srv.busy_time / max(1e-9, s["span_s"]) / len(srv.engines),
        "evictions": srv.evictions, "refused": srv.refused,
        "host_ms_per_batch": {k: v * 1e3 / max(1, srv.batches) for k, v in srv.phase_s.items()},
        "slowest_batches": [{"start_s": round(b[0], 4), "boxes": b[1], "requests": b[2],
                             "phase_ms": [round(x, 3) for x in b[3:7]],
                             "prepare_split_ms": [round(x, 3) for x in b[7:]]}
                            for b in sorted(srv.batch_log, key=lambda b: -sum(b[3:7]))[:5]],
        "clocks": clk.summary(),
    }
    srv.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_legacy(args, rank, local, ws):
    """The drop-in path: a client of the unchanged pbig.h API in the style of
    the reference's example program (pbig_init once, pbig_check per step with
    a counting report object, pbig_finalize), built against this library and
    run on the clustered 4M-box scene read from a file into pageable memory.
    A step is one pbig_check: upload, query and one report callback per pair,
    timed by the client around the call (wall clock)."""
    import re
    import tempfile
    from pbig_gb300 import build, gen
    if rank != 0:
        return
    boxes, rng, desc = workload("clustered4m")
    n = len(boxes)
    clients = os.path.join(ROOT, "tests", "clients")
    with tempfile.TemporaryDirectory() as tmp:
        exe = build.compile_client([os.path.join(clients, "legacy_client.cc"),
                                    os.path.join(clients, "counting", "report.cc")],
                                   os.path.join(tmp, "client"), include_first=[os.path.join(clients, "counting")])
        f = os.path.join(tmp, "boxes.bin")
        boxes.tofile(f)
        steps = args.warmup + args.steps
        r = subprocess.run([exe, f, str(n), str(rng), str(steps)], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise SystemExit("legacy client failed: " + r.stdout[-2000:] + r.stderr[-2000:])
    us = [int(x) for x in re.findall(r"step\d+,(\d+) us", r.stdout)]
    counts = [int(x) for x in re.findall(r"Number of pairs = (\d+)", r.stdout)]
    assert len(us) == steps and len(set(counts)) == 1
    P = counts[0]
    t = float(np.mean(us[args.warmup:])) * 1e-6
    line = {
        "metric": METRIC + " (pbig.h drop-in, counting report)", "value": n / t, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": desc + "; through pbig_init/pbig_check/pbig_finalize with a counting report",
                   "boxes": n, "pairs": P, "range": rng, "parallelism": "single GPU"},
        "pairs_per_s": P / t,
        "e2e": {"value": n / t, "unit": UNIT, "h2d_bytes_per_step": n * BOX_BYTES, "d2h_bytes_per_step": P * 8,
                "ms_per_step": t * 1e3,
                "note": "boxes from pageable memory; one report callback per pair on the calling thread"},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="clustered4m")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--scenes", type=int, default=4096, help="scenes of the batched workload")
    ap.add_argument("--duration", type=float, default=1.0, help="seconds of arrivals (serving workload)")
    ap.add_argument("--rate", type=float, default=2000.0, help="arrivals per second (serving workload)")
    ap.add_argument("--delta-only", action="store_true", help="update workload: keep no full pair list")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, local, ws = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, ws)
    elif args.workload == "batched":
        run_batched(args, rank, local, ws)
    elif args.workload == "serving":
        run_serving(args, rank, local, ws)
    elif args.workload == "update4m":
        run_update(args, rank, local, ws)
    elif args.workload == "legacy4m":
        run_legacy(args, rank, local, ws)
    else:
        run_gb300(args, rank, local, ws)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
