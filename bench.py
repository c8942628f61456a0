#!/usr/bin/env python3
"""Benchmark of the GB300 pairwise-alignment path.

Workload (one "step"): 100,000 protein pairs of uneven length (log-normal,
median 350, sigma 0.5, clipped 50..2,000; partner at 30..90 % identity with
5 % indels; seed 2), BLOSUM62, gap open 11 / extend 1, global, score only --
about 2.0e10 DP cells.  Metric: GCUPS (giga cell updates per second).

  value  batched form: the planned, length-bucketed persistent launches of a
         device-resident batch replayed as a CUDA graph, inputs already in
         HBM; CUDA events on the batch's own stream around each step; L2
         flushed (256 MB memset on that stream) between timed steps.
  e2e    the same metric through the C ABI entry point tsq_align_batch with
         host buffers: pinned host residues and pair table copied in, results
         copied back, every step.
  plain  one tsq_align_pair call (one launch sequence) per pair over a
         sample of the same pairs: the per-pair GPU path batching is
         measured against.

``--impl reference`` times the CPU implementation of the path (the oracle,
all host cores) on a bounded sample of the same workload.

Multi-GPU: pairs are independent, so N GPUs run N replicas of the workload
(weak scaling) with no data-path collective; rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes
import datetime
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("uneven_pairs_100k: 100,000 protein pairs, lengths log-normal (median 350, sigma 0.5, clipped 50-2000), "
            "partner 30-90% identity with 5% indels, seed 2; BLOSUM62, gap 11/1, global, score only")
METRIC = "GCUPS (batched, 100k uneven protein pairs, score-only, bit-exact); served p50/p99 in 'serving'"
CPU_SAMPLE_PAIRS = 20000


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--plain-pairs", type=int, default=2000)
    ap.add_argument("--e2e-steps", type=int, default=0, help="0 = same as --steps")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile", type=int, default=0, metavar="PAIRS",
                    help="profiling case: only the batched leg over the first PAIRS pairs, no graph")
    ap.add_argument("--serve-requests", type=int, default=120, help="requests in the serving leg (0 = skip)")
    ap.add_argument("--serve-only", action="store_true", help="run only the serving leg and print it")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations")
    ap.add_argument("--configs-only", action="store_true", help="run only the other configurations")
    ap.add_argument("--msa-only", action="store_true", help="run only the consensus and guide-tree legs")
    ap.add_argument("--profile-lane", choices=["auto", "i16", "i32"], default="auto",
                    help="lane type of the --profile-case batch")
    ap.add_argument("--profile-case", choices=["long_dna", "identity", "consensus", "uniform", "traceback", "plain"],
                    default=None,
                    help="small profiling case of another kernel (for ncu)")
    return ap.parse_args()


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []  # (sample wall-clock time, fields)
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "20", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        # nvidia-smi's output reaches the pipe in bursts, so each sample is
        # placed by its own timestamp, not by when it arrives.
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except (ValueError, IndexError):
                continue
            self.lines.append((ts, f[1:]))

    def wait_started(self, timeout_s=5.0):
        """Blocks until nvidia-smi has printed its first sample (it takes a
        while to start), so the samples cover the region timed next."""
        t_end = time.perf_counter() + timeout_s
        while self.proc and not self.lines and time.perf_counter() < t_end:
            time.sleep(0.01)

    def mark(self, t0, t1):
        """The timed region (wall-clock seconds): only samples taken in it
        (give or take one sampling period) are summarised."""
        self.window = (t0 - 0.025, t1 + 0.025)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.window:
            inside = [x for x in lines if self.window[0] <= x[0] <= self.window[1]]
            # A region shorter than the sampling period: the sample nearest it.
            lines = inside or sorted(lines, key=lambda x: abs(x[0] - self.window[0]))[:1]
        for _, f in lines:
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxs.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sms)), "sm_max_mhz": float(max(maxs)), "reasons": sorted(reasons),
                "samples": len(sms)}


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) and where it came from."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            return float(json.load(open(path))["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
        except (OSError, ValueError, KeyError):
            pass
    return 6800.0, "fallback 6.8 TB/s (no measured peak on this box)"


_DPX = {}


def dpx_cell_peak(packed):
    """Roofline peak of a fill in Gcell/s: the measured DPX-class instruction
    rate (tsq_probe_dpx) x lanes per instruction / 4 instructions per cell."""
    from tweakseq_gb300 import aligner as A
    if packed not in _DPX:
        _DPX[packed] = A.probe_dpx(packed=packed)
    return _DPX[packed] * (2.0 if packed else 1.0) / 4.0 / 1e9


def traffic_record(name):
    """The ncu record committed as profiles/<name>.json (or None)."""
    path = os.path.join(ROOT, "profiles", name + ".json")
    try:
        return json.load(open(path))
    except (OSError, ValueError):
        return None


def traffic_from_profile(name="fill_uneven_pairs_100k"):
    """DRAM bytes (read + write) per launch of a kernel, from the ncu record
    committed as profiles/<name>.json (or None when there is none)."""
    path = os.path.join(ROOT, "profiles", name + ".json")
    try:
        rec = json.load(open(path))
    except (OSError, ValueError):
        return None
    v = rec.get("dram_bytes_per_launch")
    return float(v) if v is not None else None


def cpu_leg(ps, sample_pairs, steps=1, warmup=0):
    """The oracle (CPU restatement of the path) on all host cores over a
    bounded, seeded sample of the workload."""
    from oracle import oracle as O
    O.build()
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(len(ps), size=min(sample_pairs, len(ps)), replace=False))
    sub = ps.subset(idx)
    cores = O.num_cores()
    times, out = [], None
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        out = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, ps.matrix, ps.gap_open, ps.gap_extend,
                      False, O.MODE_SCORE, cores)
        dt = time.perf_counter() - t0
        if k >= warmup:
            times.append(dt)
    gcups = sub.cells / float(np.mean(times)) / 1e9
    return {"value": gcups, "unit": "GCUPS", "cores": cores, "kind": "port",
            "sample": f"{len(idx)} of the 100,000 pairs (seeded subset, {sub.cells:.3e} cells), all host cores",
            "seconds_per_sample": float(np.mean(times))}, idx, out


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from tweakseq_gb300 import workloads as W
    ps = W.uneven_pairs()
    base, _, _ = cpu_leg(ps, CPU_SAMPLE_PAIRS, steps=args.steps, warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["seconds_per_sample"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator; no public dataset is named for this path)",
        "config": {"workload": WORKLOAD, "sample_pairs": CPU_SAMPLE_PAIRS},
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": base["value"], "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (groundstate/tweakseq) has no in-tree pairwise DP; its CPU path for this arm is "
                "the project's CPU restatement (oracle/), run on every host core",
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist

    from tweakseq_gb300 import aligner as A
    from tweakseq_gb300 import build as B
    from tweakseq_gb300 import workloads as W

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    B.build()
    ps = W.uneven_pairs()
    cells = ps.cells

    # ---- value: device-resident batch, graph replay --------------------------
    batch = A.Batch(ps, output="score", use_graph=True)
    ext = torch.cuda.ExternalStream(batch.stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        batch.run()
    st = batch.stats()
    launches_per_step = int(st["launches"])

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    step_ms, fill_ms = [], []
    barrier()
    with ClockSampler(local) as clk:
        clk.wait_started()
        barrier()
        t_region = time.time()
        for _ in range(args.steps):
            with torch.cuda.stream(ext):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            batch.run_async()
            e1.record(ext)
            batch.sync()
            step_ms.append(e0.elapsed_time(e1))
            fill_ms.append(batch.stats()["fill_ms"])
        barrier()
        clk.mark(t_region, time.time())
    from tweakseq_gb300.multi import max_over_ranks
    total_ms = max_over_ranks(float(np.sum(step_ms)))  # the job's time is its slowest rank's
    value = world * cells * args.steps / (total_ms * 1e-3) / 1e9
    res_dev = batch.results()

    # ---- e2e: C ABI with host buffers --------------------------------------
    e2e_steps = args.e2e_steps or args.steps
    pinned = torch.empty(len(ps.seqs), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = ps.seqs
    # The caller's buffers, as a C or C++ caller of tsq_align_batch holds them:
    # pinned residues, the pair table and the result array (tsq_result per
    # pair), all on the host; every call copies in, runs and copies out.
    from tweakseq_gb300 import _native as N
    tab = A.pair_table(ps.a_off, ps.a_len, ps.b_off, ps.b_len)
    raw = np.zeros(len(tab), dtype=N.RESULT_DTYPE)
    params, keep_params = N.make_params(output="score")
    opts = A._opts()
    L = N.lib()

    def c_call():
        rc = L.tsq_align_batch(pinned.data_ptr(), len(ps.seqs), tab.ctypes.data, len(tab), ctypes.byref(params),
                               ctypes.byref(opts), raw.ctypes.data)
        N.check(rc, "tsq_align_batch")

    c_call()  # warm the cached engine
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        c_call()
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_s = max_over_ranks(e2e_s)
    e2e_value = world * cells * e2e_steps / e2e_s / 1e9
    h2d = int(len(ps.seqs) + 24 * len(ps))
    d2h = int(32 * len(ps))
    assert np.array_equal(raw["score"], res_dev.table["score"])

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # ---- plain per-pair path over a sample ------------------------------------
    P = min(args.plain_pairs, len(ps))
    plain_cells = int(np.dot(ps.a_len[:P].astype(np.int64), ps.b_len[:P].astype(np.int64)))
    a0, b0 = ps.pair(0)
    A.align_pair(a0, b0, output="score")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_scores = np.empty(P, dtype=np.int64)
    for k in range(P):
        a, b = ps.pair(k)
        plain_scores[k] = A.align_pair(a, b, output="score").score
    plain_s = time.perf_counter() - t0
    plain_gcups = plain_cells / plain_s / 1e9
    assert np.array_equal(plain_scores, res_dev.table["score"][:P])
    # The same calls at the C ABI, as a C caller makes them: residue pointers
    # into the input buffer, one parameter block and one tsq_result reused.
    from tweakseq_gb300 import _native as N
    L = N.lib()
    c_params, keep_c_params = N.make_params(output="score")
    c_res = N.Result()
    base = ps.seqs.ctypes.data
    args_c = [(base + int(ps.a_off[k]), int(ps.a_len[k]), base + int(ps.b_off[k]), int(ps.b_len[k]))
              for k in range(P)]
    c_scores = np.empty(P, dtype=np.int64)
    pref, rref = ctypes.byref(c_params), ctypes.byref(c_res)
    t0 = time.perf_counter()
    for k, (pa, la, pb, lb) in enumerate(args_c):
        if L.tsq_align_pair(pa, la, pb, lb, pref, rref):
            raise RuntimeError("tsq_align_pair failed")
        c_scores[k] = c_res.score
    plain_c_s = time.perf_counter() - t0
    assert np.array_equal(c_scores, res_dev.table["score"][:P])

    # ---- roofline of the fill ---------------------------------------------
    # Roofline denominator: the measured int16x2 DPX instruction rate, two
    # cells per instruction, 4 DPX-class instructions per cell (E add-max, F
    # add-max, diagonal add, three-way max).
    peak_gcups = dpx_cell_peak(True)
    fill_avg_ms = float(np.mean(fill_ms))
    achieved = cells / (fill_avg_ms * 1e-3) / 1e9
    roofline = {"bound": "int", "achieved": achieved, "peak": peak_gcups, "unit": "Gcell/s",
                "frac": achieved / peak_gcups, "traffic": traffic_from_profile(),
                "peak_source": "measured live: tsq_probe_dpx int16x2 rate x 2 cells / 4 DPX instructions per cell",
                "kernel": "fill_i16_kernel (score, global; int32 re-run on overflow)", "fill_ms_avg": fill_avg_ms,
                "rerun_pairs": int(st["rerun_pairs"])}

    # ---- CPU baseline (the oracle on this host) ----------------------------
    cpu = None
    bitexact = None
    if not args.no_cpu:
        cpu, idx, want = cpu_leg(ps, CPU_SAMPLE_PAIRS)
        mism = int(np.count_nonzero(res_dev.table["score"][idx] != want["score"]))
        bitexact = {"pairs_checked": int(len(idx)), "mismatches": mism}
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}

    serving = serve_leg(args.serve_requests) if args.serve_requests > 0 else None
    configs = configs_leg() if not args.no_configs else None
    msa_steps = msa_leg() if not args.no_configs else None

    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16x2",
        "data": "synthetic (seeded generator with the workload's shapes and distributions; no public dataset)",
        "config": {"workload": WORKLOAD, "pairs": len(ps), "cells": cells, "parallelism": f"replicas x{world}",
                   "l2": "flushed between timed steps (256 MB memset on the launch stream)",
                   "launch": "device-resident batch, CUDA graph replay"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "GCUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "api": "tsq_align_batch (pinned host residues in, host results out)"},
        "plain": {"gcups": plain_gcups, "pairs": P, "ms_per_pair": plain_s / P * 1e3,
                  "api": "tsq_align_pair through the Python API (aligner.align_pair), one pair per call",
                  "c_abi_gcups": plain_cells / plain_c_s / 1e9, "c_abi_ms_per_pair": plain_c_s / P * 1e3},
        "batched_over_plain": value / plain_gcups,
        "bitexact": bitexact,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "serving": serving,
        "configs": configs,
        "msa": msa_steps,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def serve_leg(n_requests=120, loads=(0.25, 0.5, 0.9), seed=5, plain_pairs=600):
    """Served form on the serving workload: Poisson arrivals of requests of
    1-2,000 pairs (log-uniform), protein (BLOSUM62 11/1) or DNA (+2/-3, 5/2),
    lengths 50-5,000 (log-uniform), traceback on half of the requests.

    Capacity is measured closed-loop (every request submitted at once); the
    offered loads are fractions of it.  Latency is submit-to-completion of
    each request (server statistics).  The plain per-pair path runs the
    same pairs one tsq_align_pair call at a time on a sample."""
    from tweakseq_gb300 import aligner as A
    from tweakseq_gb300 import workloads as W

    reqs = W.serving_stream(n_requests, 1.0, seed=seed)

    def kw(r):
        base = dict(matrix="dna", gap_open=5, gap_extend=2) if r.pairs.matrix == W.DNA else {}
        return dict(base, output="alignment" if r.traceback else "score")

    cells = np.array([r.pairs.cells for r in reqs], dtype=np.float64)
    total = float(cells.sum())
    # Warm the server path before measuring: one closed-loop pass of the
    # same requests (first launches, the page-locked result blocks and the
    # device memory pool a long-running server already holds).
    with A.Server(slots=4) as srv:
        for rid in [srv.submit(r.pairs, **kw(r)) for r in reqs]:
            srv.poll(rid)
    with A.Server(slots=4) as srv:
        t0 = time.perf_counter()
        ids = [srv.submit(r.pairs, **kw(r)) for r in reqs]
        for rid in ids:
            srv.poll(rid)
        closed_s = time.perf_counter() - t0
        st = srv.stats()
    capacity = total / closed_s  # cells per second
    out = {"workload": f"{n_requests} requests, {int(sum(len(r.pairs) for r in reqs))} pairs, {total:.3e} cells, "
                       "1-2000 pairs per request (log-uniform), protein or DNA, lengths 50-5000, traceback on half",
           "capacity_gcups": capacity / 1e9, "closed_loop": {"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                                                              "ticks": st["ticks"]}, "loads": []}
    rng = np.random.default_rng(seed + 1)
    for load in loads:
        lam = load * capacity / float(cells.mean())  # requests per second
        arrivals = np.cumsum(rng.exponential(1.0 / lam, size=len(reqs)))
        with A.Server(slots=4) as srv:
            t0 = time.perf_counter()
            ids = []
            for r, t_arr in zip(reqs, arrivals):
                delay = t0 + t_arr - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                ids.append(srv.submit(r.pairs, **kw(r)))
            for rid in ids:
                srv.poll(rid)
            st = srv.stats()
        out["loads"].append({"offered": load, "offered_gcups": load * capacity / 1e9,
                             "achieved_gcups": total / st["span_s"] / 1e9, "p50_ms": st["p50_ms"],
                             "p99_ms": st["p99_ms"], "max_ms": st["max_ms"], "ticks": st["ticks"],
                             "peak_hbm_gb": st["peak_reserved_bytes"] / 1e9})
    # Plain per-pair path on a sample of the same pairs (score and
    # traceback as each request asks).
    sample_cells, t_plain, done = 0, 0.0, 0
    for r in reqs:
        if done >= plain_pairs:
            break
        for k in range(min(len(r.pairs), plain_pairs - done)):
            a, b = r.pairs.pair(k)
            t0 = time.perf_counter()
            A.align_pair(a, b, **kw(r))
            t_plain += time.perf_counter() - t0
            sample_cells += len(a) * len(b)
            done += 1
    out["plain_gcups"] = sample_cells / t_plain / 1e9
    out["plain_pairs_sampled"] = done
    out["served_over_plain"] = out["capacity_gcups"] / out["plain_gcups"]

    # The same workload with the device-resident request loop on (it takes
    # the score requests whose pairs are all at most 2,048 residues long).
    res = {}
    with A.Server(slots=4, resident=True) as srv:
        t0 = time.perf_counter()
        ids = [srv.submit(r.pairs, **kw(r)) for r in reqs]
        for rid in ids:
            srv.poll(rid)
        closed_s = time.perf_counter() - t0
        st = srv.stats()
    res["capacity_gcups"] = total / closed_s / 1e9
    res["resident_requests"] = st["resident_requests"]
    res["loads"] = []
    rng = np.random.default_rng(seed + 1)
    for load in loads:
        lam = load * capacity / float(cells.mean())
        arrivals = np.cumsum(rng.exponential(1.0 / lam, size=len(reqs)))
        st = _served_run(A, reqs, kw, arrivals, dict(slots=4, resident=True))
        res["loads"].append({"offered": load, "achieved_gcups": total / st["span_s"] / 1e9, "p50_ms": st["p50_ms"],
                             "p99_ms": st["p99_ms"], "max_ms": st["max_ms"]})
    out["resident"] = res

    # Editor-sized traffic: many small score and identity requests (1-64
    # pairs, proteins or DNA of 50-1,000 residues) at 1,000 requests per
    # second, through ticks and through the device-resident loop.
    small = W.serving_stream(300, 1000.0, max_pairs=64, lo=50, hi=1000, seed=seed + 2)

    def kw_small(r):
        base = dict(matrix="dna", gap_open=5, gap_extend=2) if r.pairs.matrix == W.DNA else {}
        return dict(base, output="identity" if r.traceback else "score")

    arrivals = np.array([r.arrival_s for r in small])
    small_cells = float(sum(r.pairs.cells for r in small))
    sm = {"workload": f"{len(small)} requests, {sum(len(r.pairs) for r in small)} pairs, {small_cells:.3e} cells, "
                      "1-64 pairs (log-uniform), protein or DNA, lengths 50-1000, score or identity, "
                      "Poisson arrivals at 1,000 requests/s"}
    for name, skw in (("ticks", dict(slots=4)), ("resident", dict(slots=4, resident=True))):
        _served_run(A, small, kw_small, arrivals, skw)  # warm
        st = _served_run(A, small, kw_small, arrivals, skw)
        sm[name] = {"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                    "achieved_gcups": small_cells / st["span_s"] / 1e9, "ticks": st["ticks"],
                    "resident_requests": st["resident_requests"], "resident_launches": st["resident_launches"]}
    out["small_requests"] = sm
    return out


def _served_run(A, reqs, kw, arrivals, server_kw):
    """Submits the requests at their arrival times (seconds from the start)
    and polls them all; returns the server's statistics."""
    with A.Server(**server_kw) as srv:
        t0 = time.perf_counter()
        ids = []
        for r, t_arr in zip(reqs, arrivals):
            delay = t0 + t_arr - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(r.pairs, **kw(r)))
        for rid in ids:
            srv.poll(rid)
        return srv.stats()


def configs_leg(c3_pairs=12):
    """The other workloads (not the headline): the all-vs-all of 64 proteins
    with traceback (batched vs plain), 1,000 long DNA pairs with traceback
    end to end, and the 4,000-sequence guide-tree all-vs-all (7,998,000
    pairs, score + identity).  Each is checked against the oracle."""
    from oracle import oracle as O
    from tweakseq_gb300 import aligner as A
    from tweakseq_gb300 import workloads as W

    out = {}
    cores = O.num_cores()
    # All-vs-all of 64 proteins, alignment output.
    ps = W.all_vs_all_proteins()
    with A.Batch(ps, output="alignment", use_graph=True) as b:
        for _ in range(3):
            b.run()
        ms = []
        for _ in range(5):
            b.run()
            ms.append(b.stats()["device_ms"])
        res = b.results()
    t0 = time.perf_counter()
    A.align_batch(ps, output="alignment")
    e2e_s = time.perf_counter() - t0
    # The same call at the C ABI, as a C or C++ caller makes it: pinned
    # residues, host pair table and tsq_result array, the strings freed
    # after each call; the median of 5 calls after a warm-up.
    import torch

    from tweakseq_gb300 import _native as N
    pinned = torch.empty(len(ps.seqs), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = ps.seqs
    tab = A.pair_table(ps.a_off, ps.a_len, ps.b_off, ps.b_len)
    raw = np.zeros(len(tab), dtype=N.RESULT_DTYPE)
    params, keep_params = N.make_params(output="alignment")
    opts = A._opts()
    L = N.lib()
    c_times = []
    for it in range(6):
        t0 = time.perf_counter()
        rc = L.tsq_align_batch(pinned.data_ptr(), len(ps.seqs), tab.ctypes.data, len(tab), ctypes.byref(params),
                               ctypes.byref(opts), raw.ctypes.data)
        c_s = time.perf_counter() - t0
        N.check(rc, "tsq_align_batch")
        L.tsq_results_free(raw.ctypes.data, len(raw))
        if it > 0:
            c_times.append(c_s)
    c_abi_s = float(np.median(c_times))
    t0 = time.perf_counter()
    for k in range(len(ps)):
        a, bb = ps.pair(k)
        A.align_pair(a, bb, output="alignment")
    plain_s = time.perf_counter() - t0
    want, sa, sb = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_ALIGN, strings=True,
                           nthreads=cores)
    mism = int(sum((res.table[f] != want[f]).sum() for f in ("score", "n_ident", "n_cols")))
    mism += sum(x != y for x, y in zip(res.aln_a, sa)) + sum(x != y for x, y in zip(res.aln_b, sb))
    out["all_vs_all_64_proteins"] = {
        "pairs": len(ps), "cells": ps.cells, "output": "alignment (global, BLOSUM62 11/1)",
        "batched_gcups": ps.cells / (float(np.median(ms)) * 1e-3) / 1e9, "e2e_gcups": ps.cells / e2e_s / 1e9,
        "e2e_c_abi_gcups": ps.cells / c_abi_s / 1e9, "e2e_c_abi_ms": c_abi_s * 1e3,
        "e2e_note": "e2e_gcups: through the Python API (Python string objects included); e2e_c_abi: "
                    "tsq_align_batch with host buffers, strings freed per call",
        "plain_gcups": ps.cells / plain_s / 1e9, "mismatches_vs_oracle": mism}
    # Full traceback on the headline's 100,000 uneven pairs: the int16x2
    # traceback fill (planes in HBM) and the walker, device-resident, next
    # to the same batch on int32 lanes; strings of a seeded sample against
    # the oracle.
    out["traceback_uneven_pairs_100k"] = traceback_uneven(O, A, W, cores)
    # All 1,000 long DNA pairs with traceback through tsq_align_batch,
    # which runs them in waves sized to the free HBM (their planes need about
    # 500 GB), checked against the oracle on a seeded sample of pairs.
    ps = W.long_dna_pairs(1000)
    # Kernel rooflines first, before the call below leaves its traceback
    # planes cached in the calling thread's engine.
    kernels = long_pair_kernels(ps)
    t0 = time.perf_counter()
    res = A.align_batch(ps, matrix="dna", gap_open=5, gap_extend=2, output="alignment")
    c3_s = time.perf_counter() - t0
    # The same call with int32 lanes throughout (the int32 CTA fill for the
    # long pairs); every result must equal the default run's.
    t0 = time.perf_counter()
    res32 = A.align_batch(ps, matrix="dna", gap_open=5, gap_extend=2, output="alignment", lane="i32")
    c3_i32_s = time.perf_counter() - t0
    same32 = bool(all(np.array_equal(res32.table[f], res.table[f]) for f in ("score", "n_ident", "n_cols"))
                  and res32.aln_a == res.aln_a and res32.aln_b == res.aln_b)
    del res32
    # The longest pair of the workload plus a seeded sample, compared with
    # the oracle byte for byte (its direction matrix takes a byte per cell,
    # so its threads are bounded by the host's free memory).
    all_cells = ps.a_len.astype(np.int64) * ps.b_len.astype(np.int64)
    longest = int(np.argmax(all_cells))
    rest = np.random.default_rng(3).choice(np.delete(np.arange(len(ps)), longest), c3_pairs - 1, replace=False)
    idx = np.concatenate([[longest], np.sort(rest)])
    sub = ps.subset(idx)
    nthr = O.threads_for_traceback(int(all_cells[idx].max()), cap=8)
    t0 = time.perf_counter()
    want, sa, sb = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, O.DNA, 5, 2, False, O.MODE_ALIGN,
                           nthr, True)
    oracle_s = time.perf_counter() - t0
    fields = ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols")
    mism = int(sum((res.table[f][idx] != want[f]).sum() for f in fields))
    mism += sum(res.aln_a[k] != sa[j] or res.aln_b[k] != sb[j] for j, k in enumerate(idx))
    # The plain per-pair path on the shortest pairs of the sample.
    plain_idx = idx[np.argsort(all_cells[idx])[:3]]
    t0 = time.perf_counter()
    for k in plain_idx:
        a, bb = ps.pair(int(k))
        A.align_pair(a, bb, matrix="dna", gap_open=5, gap_extend=2, output="alignment")
    plain_s = time.perf_counter() - t0
    out["long_dna_pairs_1000"] = {
        "pairs": len(ps), "cells": ps.cells, "output": "alignment (global, +2/-3, gap 5/2)",
        "e2e_gcups": ps.cells / c3_s / 1e9, "seconds": c3_s,
        "e2e_gcups_int32_lanes": ps.cells / c3_i32_s / 1e9, "int32_lanes_equal": same32,
        "lanes": "e2e_gcups: the long-pair fill in int16x2 lanes whose values each warp keeps relative to a "
                 "moving int32 base (exact: the int32 recurrence's integers, proven in range); "
                 "e2e_gcups_int32_lanes: the same call on int32 lanes (lane i32), every result compared",
        "api": "tsq_align_batch, host buffers; waves sized to free HBM, largest pairs first",
        "plain_gcups": float(all_cells[plain_idx].sum()) / plain_s / 1e9,
        "plain_pairs": len(plain_idx),
        "mismatches_vs_oracle": mism,
        "checked": f"strings: {c3_pairs} pairs (the longest, {int(ps.a_len[longest])} x {int(ps.b_len[longest])}, "
                   f"and {c3_pairs - 1} seeded) byte for byte: score, coordinates, identity, both gapped strings",
        "oracle": {"threads": nthr, "seconds": oracle_s}}
    del res
    out["long_dna_pairs_1000"]["kernels"] = kernels
    # The guide-tree all-vs-all in full, with autotuned length buckets (a
    # quick tuning pass on this GPU first) and, for comparison, without.
    ps = W.guide_tree_families()
    import tempfile
    tune_path = os.path.join(tempfile.mkdtemp(), "tune.json")
    t0 = time.perf_counter()
    A.tune(tune_path, quick=True)
    tune_s = time.perf_counter() - t0
    A.load_tuning(tune_path)
    tuned_entries = [e for e in json.load(open(tune_path))["entries"] if e["out"] == "identity"]
    with A.Batch(ps, output="identity", use_graph=True) as b:
        b.run()
        b.run()
        st_untuned = b.stats()
    with A.Batch(ps, output="identity", use_graph=True, autotune=True) as b:
        b.run()
        b.run()
        st = b.stats()
        res = b.results()
    idx = np.random.default_rng(4).choice(len(ps), 4000, replace=False)
    sub = ps.subset(idx)
    want = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, mode=O.MODE_IDENT, nthreads=cores)
    mism = int(sum((res.table[f][idx] != want[f]).sum() for f in ("score", "n_ident", "n_cols")))
    # The same batch on int32 lanes only (the int32 identity fill), for
    # comparison with the int16x2 identity fill the planner picks.
    with A.Batch(ps, output="identity", use_graph=True, lane="i32") as b:
        b.run()
        b.run()
        st_i32 = b.stats()
    fill_gcups = ps.cells / (st["fill_ms"] * 1e-3) / 1e9
    peak = dpx_cell_peak(True)
    rec = traffic_record("fill_i16_identity_guide_tree_200k")
    traffic = rec["dram_bytes_per_launch"] * len(ps) / rec["pairs"] if rec else None
    # The plain per-pair path on a sample of the same pairs.
    plain_idx = np.random.default_rng(6).choice(len(ps), 300, replace=False)
    t0 = time.perf_counter()
    for k in plain_idx:
        a, bb = ps.pair(int(k))
        A.align_pair(a, bb, output="identity")
    plain_s = time.perf_counter() - t0
    plain_cells = float(np.dot(ps.a_len[plain_idx].astype(np.int64), ps.b_len[plain_idx].astype(np.int64)))
    out["guide_tree_all_vs_all"] = {
        "pairs": len(ps), "cells": ps.cells, "output": "score + identity (global, BLOSUM62 11/1)",
        "batched_gcups": ps.cells / (st["device_ms"] * 1e-3) / 1e9, "fill_gcups": fill_gcups,
        "plain_gcups": plain_cells / plain_s / 1e9, "plain_pairs": len(plain_idx),
        "autotune": {"tune_s": tune_s, "identity_buckets": tuned_entries,
                     "untuned_fill_gcups": ps.cells / (st_untuned["fill_ms"] * 1e-3) / 1e9},
        "int32_lanes_fill_gcups": ps.cells / (st_i32["fill_ms"] * 1e-3) / 1e9,
        "roofline": {"bound": "int", "kernel": "fill_i16_kernel (identity, global)", "achieved": fill_gcups,
                     "peak": peak, "unit": "Gcell/s", "frac": fill_gcups / peak, "traffic": traffic,
                     "traffic_source": "ncu DRAM bytes of a 200,000-pair launch, scaled by pairs",
                     "peak_source": "measured live: tsq_probe_dpx int16x2 rate x 2 cells / 4 DPX instructions "
                                    "per cell (the recurrence's four maxima; the identity fill also issues the "
                                    "path-count decisions and selects)"},
        "mismatches_vs_oracle": mism, "checked": "4,000 seeded pairs"}
    return out


def traceback_uneven(O, A, W, cores, sample=2000):
    ps = W.uneven_pairs()
    runs = {}
    for lane in ("auto", "i32"):
        fills, devs = [], []
        with A.Batch(ps, output="alignment", use_graph=True, lane=lane) as b:
            b.run()
            for _ in range(3):
                b.run()
                st = b.stats()
                fills.append(st["fill_ms"])
                devs.append(st["device_ms"])
            res = b.results() if lane == "auto" else None
        runs[lane] = (float(np.median(fills)), float(np.median(devs)), res)
    fill_ms, dev_ms, res = runs["auto"]
    idx = np.sort(np.random.default_rng(8).choice(len(ps), sample, replace=False))
    sub = ps.subset(idx)
    want, sa, sb = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, mode=O.MODE_ALIGN, strings=True,
                           nthreads=cores)
    fields = ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols")
    mism = int(sum((res.table[f][idx] != want[f]).sum() for f in fields))
    mism += sum(res.aln_a[k] != sa[j] or res.aln_b[k] != sb[j] for j, k in enumerate(idx))
    gc = ps.cells / (fill_ms * 1e-3) / 1e9
    peak = dpx_cell_peak(True)
    hbm, hbm_src = hbm_peak()
    plane_gbs = 0.5 * ps.cells / (fill_ms * 1e-3) / 1e9
    rec = traffic_record("fill_i16_traceback_uneven_20k")
    traffic = rec["dram_bytes_per_launch"] * ps.cells / rec["cells"] if rec else None
    return {
        "pairs": len(ps), "cells": ps.cells, "output": "alignment (global, BLOSUM62 11/1)",
        "fill_gcups": gc, "device_gcups": ps.cells / (dev_ms * 1e-3) / 1e9,
        "int32_lanes_fill_gcups": ps.cells / (runs["i32"][0] * 1e-3) / 1e9,
        "int32_lanes_device_gcups": ps.cells / (runs["i32"][1] * 1e-3) / 1e9,
        "roofline": {"bound": "int", "kernel": "fill_i16_kernel (traceback, global)", "achieved": gc, "peak": peak,
                     "unit": "Gcell/s", "frac": gc / peak, "traffic": traffic,
                     "traffic_source": "ncu DRAM bytes of a 20,000-pair launch, scaled by cells",
                     "peak_source": "measured live: tsq_probe_dpx int16x2 rate x 2 cells / 4 DPX instructions "
                                    "per cell (the recurrence's four maxima; the traceback fill also issues the "
                                    "decision bits)"},
        "plane_writes": {"bound": "hbm", "achieved": plane_gbs, "peak": hbm, "unit": "GB/s", "frac": plane_gbs / hbm,
                         "bytes_per_cell": 0.5, "peak_source": hbm_src},
        "mismatches_vs_oracle": mism,
        "checked": f"{sample} seeded pairs byte for byte: score, coordinates, identity, both gapped strings"}


def long_pair_kernels(ps, per_sm=2):
    """Rooflines of the long-pair kernels: a device-resident batch of the
    first long DNA pairs, per_sm of them per SM (one 16-warp CTA is resident
    per SM; the second pair per SM evens out the first pairs' uneven
    lengths) as far as their traceback planes fit in 40 % of the free HBM
    (at most 120 GB): the CTA traceback fill in int16x2 lanes, then one
    walker warp per pair, timed by the batch's own events."""
    import torch

    from tweakseq_gb300 import aligner as A
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    free = torch.cuda.mem_get_info()[0]
    budget = min(120e9, 0.4 * free)
    cells = np.cumsum(ps.a_len.astype(np.float64) * ps.b_len.astype(np.float64))
    n_pairs = int(min(per_sm * sms, max(1, np.searchsorted(cells * 0.5, budget))))
    sub = ps.subset(np.arange(n_pairs))
    fills, rest = [], []
    with A.Batch(sub, matrix="dna", gap_open=5, gap_extend=2, output="alignment", use_graph=False) as b:
        b.run()
        for _ in range(3):
            b.run()
            st = b.stats()
            fills.append(st["fill_ms"])
            rest.append(st["device_ms"] - st["fill_ms"])
        res = b.results()
    fill_s = float(np.median(fills)) * 1e-3
    walk_s = float(np.median(rest)) * 1e-3
    gc = sub.cells / fill_s / 1e9
    peak = dpx_cell_peak(True)
    hbm, hbm_src = hbm_peak()
    rec = traffic_record("fill_cta16_long_dna_32")
    traffic = rec["dram_bytes_per_launch"] * sub.cells / rec["cells"] if rec else None
    plane_gbs = 0.5 * sub.cells / fill_s / 1e9
    # Walker bytes: the nibble of each walked cell, both gapped rows written
    # and the residues read.
    cols = res.table["n_cols"].astype(np.float64)
    walk_bytes = float((0.5 * cols + 2 * cols).sum() + sub.a_len.sum() + sub.b_len.sum())
    return {
        "pairs": n_pairs, "cells": sub.cells,
        "fill_cta16_kernel": {
            "fill_ms": fill_s * 1e3,
            "roofline": {"bound": "int", "achieved": gc, "peak": peak, "unit": "Gcell/s", "frac": gc / peak,
                         "traffic": traffic, "traffic_source": "ncu DRAM bytes of a 32-pair launch, scaled by cells",
                         "peak_source": "measured live: tsq_probe_dpx int16x2 rate x 2 cells / 4 DPX instructions "
                                        "per cell",
                         "note": f"{n_pairs} pairs, one 16-warp CTA each, one CTA resident per SM"},
            "plane_writes": {"bound": "hbm", "achieved": plane_gbs, "peak": hbm, "unit": "GB/s",
                             "frac": plane_gbs / hbm, "bytes_per_cell": 0.5, "peak_source": hbm_src}},
        "walk_warp_kernel": {
            "ms": walk_s * 1e3, "note": "device time after the fill: the walker and the result copies",
            "roofline": {"bound": "latency", "achieved": walk_bytes / walk_s / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": walk_bytes / walk_s / 1e9 / hbm, "bytes": walk_bytes,
                         "bytes_note": "0.5 B per walked cell + 2 B of gapped rows per column + the residues",
                         "peak_source": hbm_src}}}


def msa_leg(cpu_cols=40, cpu_tree_leaves=1000):
    """The steps either side of the pairwise path: the consensus line of a
    4,000 x 1,000 and a 100,000 x 2,000 alignment (HBM-bound count pass),
    and UPGMA / NJ guide trees of the 4,000-sequence guide-tree workload
    built from its device-resident all-vs-all identities."""
    import torch

    from oracle import oracle as O
    from tweakseq_gb300 import _native as N
    from tweakseq_gb300 import aligner as A
    from tweakseq_gb300 import msa
    from tweakseq_gb300 import workloads as W

    out = {}
    L = N.lib()
    peak, _ = hbm_peak()
    for nseq, ncols in ((4000, 1000), (100_000, 2000)):
        rng = np.random.default_rng(nseq)
        # Columns with a favourite residue (kept in 60 % of rows), 15 % gaps.
        fav = W.random_protein(rng, ncols)
        rows = W.AA_LETTERS[rng.integers(0, 20, size=(nseq, ncols), dtype=np.uint8)]
        u = rng.integers(0, 100, size=(nseq, ncols), dtype=np.uint8)
        rows = np.where(u < 60, fav[None, :], rows)
        rows[u >= 85] = ord("-")
        rows = np.ascontiguousarray(rows, dtype=np.uint8)
        d_rows = torch.from_numpy(rows).cuda()
        d_out = torch.zeros(ncols, dtype=torch.uint8, device="cuda")
        nb = L.tsq_consensus_scratch_bytes(ncols)
        scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        st = torch.cuda.current_stream()
        ms = []
        for it in range(13):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            rc = L.tsq_consensus_device(d_rows.data_ptr(), nseq, ncols, ncols, -1.0, d_out.data_ptr(), None, None,
                                        scratch.data_ptr(), nb, st.cuda_stream)
            e1.record(st)
            assert rc == 0
            st.synchronize()
            if it >= 3:
                ms.append(e0.elapsed_time(e1))
        dev_ms = float(np.median(ms))
        t0 = time.perf_counter()
        got = msa.consensus(rows)
        host_ms = (time.perf_counter() - t0) * 1e3
        # The reference's algorithm (O(nseq^2) per column) on a column sample.
        cols = np.random.default_rng(1).choice(ncols, min(cpu_cols, ncols), replace=False)
        sub = np.ascontiguousarray(rows[:, cols]) if nseq <= 4000 else np.ascontiguousarray(rows[:4000, cols])
        t0 = time.perf_counter()
        want = O.consensus(sub)
        cpu_s = time.perf_counter() - t0
        ok = bytes(got.sequence[c] for c in cols) == want[0] if nseq <= 4000 else None
        pair_ops = float(sub.shape[0]) ** 2 * sub.shape[1]
        bytes_ = nseq * ncols
        out[f"consensus_{nseq}x{ncols}"] = {
            "device_ms": dev_ms, "host_api_ms": host_ms, "gbs": bytes_ / (dev_ms * 1e-3) / 1e9,
            "roofline": {"bound": "hbm", "achieved": bytes_ / (dev_ms * 1e-3) / 1e9, "peak": peak,
                         "frac": bytes_ / (dev_ms * 1e-3) / 1e9 / peak, "unit": "GB/s",
                         "bytes_per_launch": bytes_},
            "cpu_reference_algorithm": {"columns_per_s": sub.shape[1] / cpu_s,
                                        "row_pairs_per_s": pair_ops / cpu_s, "cores": O.num_cores(),
                                        "sample": f"{sub.shape[1]} columns x {sub.shape[0]} rows"},
            "cpu_extrapolated_s": cpu_s * (float(nseq) ** 2 * ncols) / pair_ops,
            "bitexact_sample": ok}
        del d_rows, scratch, flush
    # Guide trees of the 4,000-sequence all-vs-all.
    ps = W.guide_tree_families()
    n = int(ps.meta["n_seqs"])
    with A.Batch(ps, output="identity") as b:
        b.run()
        res = b.results()
        for method in ("upgma", "nj"):
            msa.guide_tree_from_batch(b, n, method)  # warm
            t0 = time.perf_counter()
            tree = msa.guide_tree_from_batch(b, n, method)
            tree_ms = (time.perf_counter() - t0) * 1e3
            D = O.identity_distances(n, res.table["n_ident"], res.table["n_cols"])
            want = O.guide_tree(D, N.TREE[method])
            same = all(np.array_equal(tree.nodes[f], want[f]) for f in N.TREE_NODE_DTYPE.names)
            k = cpu_tree_leaves
            t0 = time.perf_counter()
            O.guide_tree(np.ascontiguousarray(D[:k, :k]), N.TREE[method])
            cpu_s = time.perf_counter() - t0
            out[f"guide_tree_{method}_{n}"] = {
                "ms": tree_ms, "joins": n - 1, "bitexact_vs_oracle": bool(same),
                "what": "from the batch's device-resident identities: distances, n-1 join launches, joins to host",
                "cpu_oracle_s_at_1000_leaves": cpu_s,
                "cpu_oracle_s_extrapolated": cpu_s * (n / k) ** 3}
    return out


def run_profile_case(args):
    """Small cases for ncu of the kernels behind the other measurements:
    long_dna (32 DNA pairs of 10-12 kb with traceback: the CTA fill and the
    walker),
    identity (200,000 pairs of the guide-tree all-vs-all: the identity
    fill), traceback (20,000 of the uneven pairs with traceback: the
    traceback fill and the walker), consensus (100,000 x 2,000 alignment:
    the class-count kernel),
    uniform (20,000 protein pairs of 320 x 2,000: the int16x2 score fill with
    interior steps only, for instruction counts per step),
    plain (tsq_align_pair at the C ABI on the first 200 uneven pairs, score
    then alignment: the one-pair path's kernels per call).
    Device-resident, no graph, warm-up then timed runs."""
    import torch

    from tweakseq_gb300 import _native as N
    from tweakseq_gb300 import aligner as A
    from tweakseq_gb300 import build as B
    from tweakseq_gb300 import workloads as W

    B.build()
    case = args.profile_case
    if case in ("long_dna", "identity", "uniform", "traceback"):
        if case == "long_dna":
            ps = W.long_dna_pairs(32, lo=10_000, hi=12_000)
            kw = dict(matrix="dna", gap_open=5, gap_extend=2, output="alignment")
        elif case == "uniform":
            # Equal shapes, so nearly every step of the int16x2 fill is an
            # interior step: instruction counts per step read off directly.
            rng = np.random.default_rng(1)
            seqs, pairs = [], []
            for k in range(20000):
                seqs += [W.random_protein(rng, 320).tobytes(), W.random_protein(rng, 2000).tobytes()]
                pairs.append((2 * k, 2 * k + 1))
            ps = W._pairset_from_lists(seqs, pairs)
            kw = dict(output="score")
        elif case == "traceback":
            ps = W.uneven_pairs().subset(np.arange(20_000))
            kw = dict(output="alignment")
        else:
            ps = W.guide_tree_families()
            ps = ps.subset(np.arange(200_000))
            kw = dict(output="identity")
        kw["lane"] = args.profile_lane
        with A.Batch(ps, use_graph=False, **kw) as b:
            for _ in range(args.warmup + args.steps):
                b.run()
            st = b.stats()
        print(json.dumps({"profile_case": case, "pairs": len(ps), "cells": ps.cells, "fill_ms": st["fill_ms"],
                          "device_ms": st["device_ms"], "fill_gcups": ps.cells / (st["fill_ms"] * 1e-3) / 1e9}))
        return
    if case == "plain":
        ps = W.uneven_pairs().subset(np.arange(200))
        L = N.lib()
        base = ps.seqs.ctypes.data
        res = N.Result()
        out = {"profile_case": case, "pairs": len(ps), "cells": ps.cells}
        for output in ("score", "alignment"):
            params, keep = N.make_params(output=output)
            times = []
            for it in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                for k in range(len(ps)):
                    rc = L.tsq_align_pair(base + int(ps.a_off[k]), int(ps.a_len[k]), base + int(ps.b_off[k]),
                                          int(ps.b_len[k]), ctypes.byref(params), ctypes.byref(res))
                    assert rc == 0
                    L.tsq_result_free(ctypes.byref(res))
                times.append(time.perf_counter() - t0)
            t = float(np.median(times[args.warmup:])) if args.steps > 0 else float(times[-1])
            out[output] = {"ms_per_pair": t / len(ps) * 1e3, "gcups": ps.cells / t / 1e9}
        print(json.dumps(out))
        return
    if case == "consensus":
        nseq, ncols = 100_000, 2000
        rng = np.random.default_rng(nseq)
        fav = W.random_protein(rng, ncols)
        rows = W.AA_LETTERS[rng.integers(0, 20, size=(nseq, ncols), dtype=np.uint8)]
        u = rng.integers(0, 100, size=(nseq, ncols), dtype=np.uint8)
        rows = np.ascontiguousarray(np.where(u < 60, fav[None, :], rows), dtype=np.uint8)
        rows[u >= 85] = ord("-")
        L = N.lib()
        d_rows = torch.from_numpy(rows).cuda()
        d_out = torch.zeros(ncols, dtype=torch.uint8, device="cuda")
        nb = L.tsq_consensus_scratch_bytes(ncols)
        scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
        st = torch.cuda.current_stream()
        for _ in range(args.warmup + args.steps):
            rc = L.tsq_consensus_device(d_rows.data_ptr(), nseq, ncols, ncols, -1.0, d_out.data_ptr(), None, None,
                                        scratch.data_ptr(), nb, st.cuda_stream)
            assert rc == 0
        st.synchronize()
        print(json.dumps({"profile_case": case, "rows": nseq, "cols": ncols, "bytes": nseq * ncols}))
        return
    raise SystemExit(f"unknown profile case {case}")


def run_profile(args):
    """Small case for ncu: the device-resident batch over a prefix of the
    workload, launched without a graph so each kernel is a separate launch."""
    import torch

    from tweakseq_gb300 import aligner as A
    from tweakseq_gb300 import build as B
    from tweakseq_gb300 import workloads as W

    B.build()
    ps = W.uneven_pairs()
    sub = ps.subset(np.arange(min(args.profile, len(ps))))
    batch = A.Batch(sub, output="score", use_graph=False)
    for _ in range(args.warmup + args.steps):
        batch.run()
    torch.cuda.synchronize()
    st = batch.stats()
    print(json.dumps({"profile_pairs": len(sub), "cells": sub.cells, "fill_ms": st["fill_ms"],
                      "gcups": sub.cells / (st["fill_ms"] * 1e-3) / 1e9, "launches_per_run": st["launches"]}))


def main():
    args = parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.profile_case:
        run_profile_case(args)
        return
    if args.configs_only:
        from tweakseq_gb300 import build as B
        B.build()
        print(json.dumps({"configs": configs_leg()}), flush=True)
        return
    if args.msa_only:
        from tweakseq_gb300 import build as B
        B.build()
        print(json.dumps({"msa": msa_leg()}), flush=True)
        return
    if args.serve_only:
        from tweakseq_gb300 import build as B
        B.build()
        print(json.dumps({"serving": serve_leg(args.serve_requests)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
