#!/usr/bin/env python3
"""Benchmark of the GB300 multiple-FFT library (one JSON line on stdout).

Default workload (cfg3): vsip_ccfftmop_f on 65536 rows x 4096 points, complex
float32, VSIP_ROW, forward, scale 1, iid N(0,1) -- the large plain batch the
fftm hot path is quoted on.  A step is one vsip_ccfftmop_f call over the whole
matrix.

  value        GB/s of algorithmic bytes (16 per point, read + write), blocks
               admitted (device resident), CUDA events on the library stream
               over exactly --steps calls; inputs (2 GiB/buffer) exceed L2.
  e2e          the same metric through the same C call on pinned host user
               blocks that are not admitted: each call stages 2 GiB in and
               2 GiB out.
  roofline     achieved GB/s of the row kernel against the measured HBM copy
               bandwidth; traffic from the committed ncu summary.
  cpu_baseline the CPU oracle (the reference's algorithm, restated in C; the
               reference's own sources do not exist on the GPU host) on all
               host threads over a bounded sample of the same rows; this leg
               also checks sampled GPU rows against the FP64 oracle.
  forms        (one GPU) the precision form (cfg4) and the batching form (cfg5)
               against the plain kernel, each from its own bench.py run.

Other configurations (--workload): cfg1 (64x1024), cfg2col (1000-point
columns x 4096), cfg2rc / cfg2cr (4096 x 1536 real <-> 4096 x 769), cfg3d
(16384 x 4096 c128), cfg4 (32768 x 1024, rows scaled by 10^U(-3,3)), cfg5
(batching: uneven lengths and row counts in one launch vs a loop of per-plan
calls), vec / vecd / vecrc (one single FFT of --points points: c64, c128,
real f32 -> c64), cols / rows (2^24 c64 points as --points-point transforms
down the columns / along the rows of a matrix), komega (the k-omega power
estimate of the reference's kw example on --kw-sensors x --kw-samples real
data through jvsip_komega_f), split (2^24 c64 points as --points-point rows
of split-complex blocks, real and imaginary parts in separate arrays),
measured the same way.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

--impl reference times the reference algorithm (CPU oracle port) on the host
cores for the same metric and workload, each step a bounded sample of rows;
under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched FFT GB/s (% HBM peak): split-TC & batched vs plain FP32 at ≤1e-6 rel err"
FALLBACK_HBM = 6800.0
WORKLOADS = ["cfg3", "cfg1", "cfg2col", "cfg2rc", "cfg2cr", "cfg3d", "cfg4", "cfg5", "vec", "vecd", "vecrc", "veccr",
             "cols", "rows", "komega", "split", "primes"]


def args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg3", choices=WORKLOADS)
    ap.add_argument("--rows", type=int, default=65536, help="rows of cfg3 (smaller cases for profiling)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU-baseline sample (wall seconds)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-forms", action="store_true",
                    help="default workload: skip the precision-form and batching-form summaries")
    ap.add_argument("--no-autotune", action="store_true",
                    help="cfg5: use the cached or heuristic tiling (profiling runs: no tuner launches)")
    ap.add_argument("--batch-gb", type=float, default=2.0, help="cfg5: bytes per buffer of the instance sequence (0: the literal 20000 instances)")
    ap.add_argument("--kw-sensors", type=int, default=4096, help="komega: sensors (rows of the data)")
    ap.add_argument("--kw-samples", type=int, default=4096, help="komega: samples per sensor (even)")
    ap.add_argument("--points", type=int, default=1 << 24,
                    help="vec / vecd / vecrc: single-FFT length; cols / rows: transform length (2^24 points in all)")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


# ---------------------------------------------------------------- clocks
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx, self.proc, self.lines = gpu_index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                pw.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s, p in zip(sm, pw) if p > 0.3 * max(pw)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(pw)}


# ---------------------------------------------------------------- CPU baseline leg (the only oracle user)
def cpu_leg(x, N, rows_total, gpu_out=None, target_s=10.0, threads=None):
    """Time the CPU oracle (reference algorithm, one plan per thread on disjoint
    row slabs) on a bounded sample of the workload's rows x[rows, 2N] (float32,
    dense, forward, scale 1) and, when gpu_out is given, check sampled GPU rows
    against the FP64 oracle.  Returns the cpu_baseline object."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    threads = threads or (os.cpu_count() or 1)
    X = x.reshape(-1, 2 * N)
    r0 = min(rows_total, 16 * threads)
    t0 = time.perf_counter()
    O.ccfftm_rows_mt(np.ascontiguousarray(X[:r0]), -1, 1.0, threads)
    t0 = time.perf_counter() - t0
    rows = int(min(rows_total, max(r0, r0 * target_s / max(t0, 1e-4))))
    xs = np.ascontiguousarray(X[:rows])
    t = time.perf_counter()
    ys = O.ccfftm_rows_mt(xs, -1, 1.0, threads)
    t = time.perf_counter() - t
    out = {"value": round(rows * N * 16 / t / 1e9, 4), "unit": "GB/s", "cores": threads, "kind": "port",
           "sample": f"{rows} of {rows_total} rows x {N} points in {t:.2f} s (oracle/fftm_oracle.c, the reference "
                     "algorithm restated bit for bit; the reference sources are absent on this host)"}
    out["one_thread"] = one_thread_rate(X, N, rows_total, min(target_s / 2, 5.0), O)
    if gpu_out is not None:
        outs = gpu_out if isinstance(gpu_out, dict) else {"": gpu_out}
        sample = sorted({0, 1, rows_total // 3, rows_total // 2, rows_total - 1})
        ref = {}
        for r in sample:
            yo = O.CView(np.zeros(2 * N), 0, N, 1, 1, N)
            O.Plan(O.CCOP, 1, N, 1.0, O.FWD, O.ROW, np.float64).ccfftmop(
                O.CView(X[r].astype(np.float64), 0, N, 1, 1, N), yo)
            ref[r] = yo.buf
        for name, arr in outs.items():
            G = arr.reshape(-1, 2 * N)
            errs_d = [float(np.linalg.norm(G[r].astype(np.float64) - ref[r]) / np.linalg.norm(ref[r])) for r in sample]
            errs_f = [float(np.linalg.norm(G[r].astype(np.float64) - ys[r]) / np.linalg.norm(ys[r]))
                      for r in sample if r < rows]
            sfx = ("_" + name) if name else ""
            out["gpu_rel_l2_vs_fp64_oracle" + sfx] = max(errs_d)
            out["gpu_rel_l2_vs_reference_f32" + sfx] = max(errs_f) if errs_f else None
    return out


def one_thread_rate(X, N, rows_total, target_s, O):
    """The reference algorithm on one thread (the reference library is
    single-threaded): GB/s over a bounded sample of the rows of X[rows, 2N]."""
    import numpy as np
    r0 = min(rows_total, 8)
    t0 = time.perf_counter()
    O.ccfftm_rows_mt(np.ascontiguousarray(X[:r0]), -1, 1.0, 1)
    t0 = time.perf_counter() - t0
    rows = int(min(rows_total, max(r0, r0 * target_s / max(t0, 1e-4))))
    xs = np.ascontiguousarray(X[:rows])
    t = time.perf_counter()
    O.ccfftm_rows_mt(xs, -1, 1.0, 1)
    t = time.perf_counter() - t
    return {"value": round(rows * N * 16 / t / 1e9, 4), "unit": "GB/s", "cores": 1, "kind": "port",
            "sample": f"{rows} of {rows_total} rows x {N} points in {t:.2f} s on one thread"}


def reference_arm(a):
    """--impl reference: the CPU oracle port on the host cores, same metric."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from jvsip_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    threads = os.cpu_count() or 1
    N, total_rows = 4096, 65536
    probe = synth.fill(2 * 16 * threads * N, 4, 1).reshape(-1, 2 * N)
    t0 = time.perf_counter()
    O.ccfftm_rows_mt(probe, -1, 1.0, threads)
    t0 = time.perf_counter() - t0
    per_step = max(0.05, 150.0 / max(1, a.steps + a.warmup))
    rows = int(min(total_rows, max(threads, 16 * threads * per_step / max(t0, 1e-4))))
    x = synth.fill(2 * rows * N, 4, 1).reshape(rows, 2 * N)
    for _ in range(a.warmup):
        O.ccfftm_rows_mt(x, -1, 1.0, threads)
    ts = []
    for _ in range(a.steps):
        t = time.perf_counter()
        O.ccfftm_rows_mt(x, -1, 1.0, threads)
        ts.append(time.perf_counter() - t)
    tot = sum(ts)
    value = rows * N * 16 * len(ts) / tot / 1e9
    line = {"metric": METRIC, "value": round(value, 4), "unit": "GB/s", "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(1000 * tot / len(ts), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic iid N(0,1), seeded SplitMix64 stream",
            "config": {"workload": "vsip_ccfftmop_f 65536x4096 c64 VSIP_ROW forward scale 1",
                       "sample_rows_per_step": rows},
            "cpu_baseline": {"value": round(value, 4), "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": f"{rows} of {total_rows} rows per step",
                             "one_thread": one_thread_rate(x, N, total_rows, 3.0, O)},
            "e2e": {"value": round(value, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- shared GPU helpers
def gpu_init():
    import torch
    import jvsip_gb300 as J
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    L = J.lib()
    L.vsip_init(None)
    return torch, J, L, torch.cuda.ExternalStream(L.jvsip_gpu_stream())


def timed_calls(torch, ext, call, steps, flush=None):
    """Per-call CUDA-event times (ms) on the library stream; L2 flushed between calls
    (outside the events) when `flush` is a buffer larger than L2."""
    per = []
    for _ in range(steps):
        if flush is not None:
            with torch.cuda.stream(ext):
                flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        call()
        e1.record(ext)
        e1.synchronize()
        per.append(e0.elapsed_time(e1))
    return per


def max_over_ranks(torch, dist, ms, device="cuda"):
    """The largest per-rank time (ms) over all ranks (the job's time); the
    rank's own time without a process group."""
    if dist is None:
        return ms
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gbs(bytes_per_rank, world, ms):
    """Whole-job GB/s: every rank moves bytes_per_rank in ms (replicas, weak scaling)."""
    return bytes_per_rank * world / (ms / 1e3) / 1e9


def link_time(torch, hin, hout, reps=3):
    """ms to copy hin host->device and, at the same time, a device buffer of
    hout's size device->host (pinned memory, two streams): the host-link bound
    of a call that moves those bytes each way."""
    din = torch.empty_like(hin, device="cuda")
    dout = torch.zeros_like(hout, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def both():
        with torch.cuda.stream(s1):
            din.copy_(hin, non_blocking=True)
        with torch.cuda.stream(s2):
            hout.copy_(dout, non_blocking=True)

    both()
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        both()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3
        best = ms if best is None else min(best, ms)
    del din, dout
    return best


def line_for(a, value, ms, nbytes, dtype, launches, extra):
    peak, kind = peaks()
    d = {"metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": 1, "steps": a.steps,
         "warmup": a.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)",
         "hbm_frac": round(value / peak, 4), "gpu_launches": int(launches),
         "roofline": {"bound": "hbm", "achieved": round(value, 1), "peak": peak, "unit": "GB/s",
                      "frac": round(value / peak, 4), "peak_kind": kind, "traffic": None}}
    d.update(extra)
    return d


# ---------------------------------------------------------------- other configurations
def other_workload(a):
    import numpy as np
    from jvsip_gb300 import synth
    torch, J, L, ext = gpu_init()
    w, f32 = a.workload, np.float32
    if w == "cfg5":
        return batching_workload(a, torch, J, L, ext)
    if w == "komega":
        return komega_workload(a, torch, J, L, ext)
    x = y = None
    if w in ("cfg1", "cfg2col", "cfg4"):
        M, N = (64, 1024) if w == "cfg1" else (1000, 4096) if w == "cfg2col" else (32768, 1024)
        x = synth.fill(2 * M * N, 1 if w == "cfg1" else 3 if w == "cfg2col" else 5, 0 if w == "cfg1" else 1)
        if w == "cfg4":
            u = synth.unit(55, M) * 6.0 - 3.0
            x = (x.reshape(M, 2 * N) * (10.0 ** u).astype(f32)[:, None]).reshape(-1)
        y = np.zeros_like(x)
        major = J.VSIP_COL if w == "cfg2col" else J.VSIP_ROW
        plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, major)
        bx, by = J.CBlock(x), J.CBlock(y)
        vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        call = lambda: L.vsip_ccfftmop_f(plan.h, vx.h, vy.h)
        nbytes, dt = 16 * M * N, "f32"
        desc = {"cfg1": "vsip_ccfftmop_f 64x1024 c64 VSIP_ROW forward, U[-1,1)",
                "cfg2col": "vsip_ccfftmop_f M=1000 x N=4096 c64 VSIP_COL (1000-point columns), N(0,1)",
                "cfg4": "vsip_ccfftmop_f 32768x1024 c64 VSIP_ROW, rows N(0,1)*10^U(-3,3)"}[w]
    elif w in ("cfg2rc", "cfg2cr"):
        M, N, H = 4096, 1536, 769
        xr = synth.fill(M * N, 2, 1)
        z = synth.fill(2 * M * H, 22, 1)
        if w == "cfg2rc":
            plan = J.FFTM(J.KIND_RCOP, M, N, 1.0, -1, J.VSIP_ROW)
            bx, by = J.RBlock(xr), J.CBlock(z)
            vx, vy = bx.view(0, N, M, 1, N), by.view(0, H, M, 1, H)
            call = lambda: L.vsip_rcfftmop_f(plan.h, vx.h, vy.h)
            desc = "vsip_rcfftmop_f 4096x1536 f32 -> 4096x769 c64 VSIP_ROW, N(0,1)"
        else:
            plan = J.FFTM(J.KIND_CROP, M, N, 1.0 / N, 1, J.VSIP_ROW)
            bx, by = J.CBlock(z), J.RBlock(xr)
            vx, vy = bx.view(0, H, M, 1, H), by.view(0, N, M, 1, N)
            call = lambda: L.vsip_crfftmop_f(plan.h, vx.h, vy.h)
            desc = "vsip_crfftmop_f 4096x769 c64 -> 4096x1536 f32 VSIP_ROW, scale 1/1536"
        nbytes, dt = M * (4 * N + 8 * H), "f32"
    elif w in ("cols", "rows"):
        # 2^24 points as n-point transforms down the columns / along the rows
        n, tot = a.points, 1 << 24
        other = tot // n
        x = synth.fill(2 * tot, 9, 1)
        y = np.zeros_like(x)
        if w == "cols":
            M, N = n, other
            plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_COL)
        else:
            M, N = other, n
            plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_ROW)
        bx, by = J.CBlock(x), J.CBlock(y)
        vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        call = lambda: L.vsip_ccfftmop_f(plan.h, vx.h, vy.h)
        nbytes, dt = 16 * tot, "f32"
        desc = f"vsip_ccfftmop_f {M}x{N} c64 {'VSIP_COL' if w == 'cols' else 'VSIP_ROW'} ({n}-point transforms), N(0,1)"
    elif w == "split":
        # 2^24 points as n-point rows of split complex blocks (cstride 1)
        n, tot = a.points, 1 << 24
        M, N = tot // n, n
        xr, xi = synth.fill(tot, 12, 1), synth.fill(tot, 13, 1)
        x = np.concatenate([xr, xi])
        y = np.zeros(2 * tot, np.float32)
        plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_ROW)
        bx, by = J.CBlock(xr, xi), J.CBlock(y[:tot], y[tot:])
        vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        call = lambda: L.vsip_ccfftmop_f(plan.h, vx.h, vy.h)
        nbytes, dt = 16 * tot, "f32"
        desc = f"vsip_ccfftmop_f {M}x{N} c64 VSIP_ROW, split complex blocks (cstride 1), N(0,1)"
    elif w == "primes":
        # a length with a prime factor above 7: 4096 rows of 5632 = 8 x 8 x 8 x 11 points
        # (the multi-pass global path, the radix-11 pass a direct sum)
        M, N = 4096, 5632
        x = synth.fill(2 * M * N, 14, 1)
        y = np.zeros_like(x)
        plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_ROW, ntimes=1)
        bx, by = J.CBlock(x), J.CBlock(y)
        vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        call = lambda: L.vsip_ccfftmop_f(plan.h, vx.h, vy.h)
        nbytes, dt = 16 * M * N, "f32"
        desc = "vsip_ccfftmop_f 4096x5632 (8*8*8*11) c64 VSIP_ROW forward, N(0,1)"
    elif w in ("vec", "vecd", "vecrc", "veccr"):
        # one single FFT of --points points (vsip_ccfftop / vsip_rcfftop / vsip_crfftop)
        N = M = a.points
        if w == "veccr":
            # C2R of N/2+1 bins into a real vector of stride 2 (the final store
            # goes through the unpack kernel)
            x = synth.fill(2 * (N // 2 + 1), 15, 1)
            y = np.zeros(2 * N, np.float32)
            plan = J.FFT(J.KIND_CROP, N, 1.0 / N)
            bx, by = J.CBlock(x), J.RBlock(y)
            vx, vy = bx.vview(0, 1, N // 2 + 1), by.vview(0, 2, N)
            call = lambda: L.vsip_crfftop_f(plan.h, vx.h, vy.h)
            nbytes, dt = 4 * N + 8 * (N // 2 + 1), "f32"
            desc = f"vsip_crfftop_f {N // 2 + 1} c64 -> {N} f32 (real vector of stride 2), scale 1/{N}"
        elif w == "vecrc":
            x = synth.fill(N, 8, 1)
            y = np.zeros(2 * (N // 2 + 1), np.float32)
            plan = J.FFT(J.KIND_RCOP, N, 1.0)
            bx, by = J.RBlock(x), J.CBlock(y)
            vx, vy = bx.vview(0, 1, N), by.vview(0, 1, N // 2 + 1)
            call = lambda: L.vsip_rcfftop_f(plan.h, vx.h, vy.h)
            nbytes, dt = 4 * N + 8 * (N // 2 + 1), "f32"
            desc = f"vsip_rcfftop_f {N} f32 -> {N // 2 + 1} c64, N(0,1)"
        else:
            dtype = np.float32 if w == "vec" else np.float64
            x = synth.fill(2 * N, 7, 1, dtype)
            y = np.zeros_like(x)
            plan = J.FFT(J.KIND_CCOP, N, 1.0, -1, dtype)
            bx, by = J.CBlock(x), J.CBlock(y)
            vx, vy = bx.vview(0, 1, N), by.vview(0, 1, N)
            fn = L.vsip_ccfftop_f if w == "vec" else L.vsip_ccfftop_d
            call = lambda: fn(plan.h, vx.h, vy.h)
            nbytes, dt = (16 if w == "vec" else 32) * N, ("f32" if w == "vec" else "f64")
            desc = f"vsip_ccfftop_{'f' if w == 'vec' else 'd'} {N} points {'c64' if w == 'vec' else 'c128'} forward, N(0,1)"
    else:  # cfg3d
        M, N = 16384, 4096
        g = torch.Generator(device="cuda").manual_seed(4)
        x = torch.randn(2 * M * N, device="cuda", dtype=torch.float64, generator=g).cpu().numpy()
        y = np.zeros_like(x)
        plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_ROW, dtype=np.float64)
        bx, by = J.CBlock(x), J.CBlock(y)
        vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        call = lambda: L.vsip_ccfftmop_d(plan.h, vx.h, vy.h)
        nbytes, dt = 32 * M * N, "f64"
        desc = "vsip_ccfftmop_d 16384x4096 c128 VSIP_ROW forward, N(0,1)"
    bx.admit(True)
    by.admit(False)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if nbytes < (512 << 20) else None
    for _ in range(a.warmup):
        call()
    J.check("warm-up")
    L.jvsip_gpu_synchronize()
    n0 = L.jvsip_gpu_kernel_launches()
    per = timed_calls(torch, ext, call, a.steps, flush)
    launches = L.jvsip_gpu_kernel_launches() - n0
    J.check("timed loop")
    by.sync()
    ms = statistics.mean(per)
    extra = {"config": {"workload": desc, "bytes_per_step": nbytes,
                        "l2": "flushed between calls" if flush is not None else "inputs larger than L2"}}
    outs = {"": y.copy() if w in ("cfg4", "cfg3d") else y}
    if w in ("cfg4", "cfg3d"):
        # the precision forms on the same plan and data: tensor-core DFT products
        # (cfg4), double-float arithmetic on the FP32 pipes (cfg3d)
        forms = {}
        flist = ((("split_fp16", J.JVSIP_FORM_SPLIT_FP16), ("split_bf16", J.JVSIP_FORM_SPLIT_BF16)) if w == "cfg4"
                 else (("df64", J.JVSIP_FORM_DF64),))
        for name, form in flist:
            plan.setform(form)
            for _ in range(a.warmup):
                call()
            k0 = L.jvsip_gpu_kernel_launches()
            per_f = timed_calls(torch, ext, call, a.steps, flush)
            kl = L.jvsip_gpu_kernel_launches() - k0
            assert L.jvsip_gpu_synchronize() == 0, J.last_error()
            by.sync()
            outs[name] = y.copy()
            msf = statistics.mean(per_f)
            forms[name] = {"value": round(nbytes / (msf / 1e3) / 1e9, 2), "unit": "GB/s", "ms_per_step": round(msf, 4),
                           "gpu_launches": int(kl)}
            if w == "cfg3d":
                ref = outs[""]
                forms[name]["rel_l2_vs_plain_fp64"] = float(np.linalg.norm(y - ref) / np.linalg.norm(ref))
        plan.setform(J.JVSIP_FORM_PLAIN)
        extra["forms"] = forms
        y = outs[""]
    if not a.no_cpu and w in ("cfg2col", "cfg2rc", "cfg2cr"):
        host_in = x if w == "cfg2col" else (xr if w == "cfg2rc" else z)
        host_out = y if w == "cfg2col" else (z if w == "cfg2rc" else xr)
        extra.update(cfg2_oracle_check(w, host_in, host_out))
    if not a.no_cpu and w in ("cfg1", "cfg4"):
        extra["cpu_baseline"] = cpu_leg(x, N, M, gpu_out=outs, target_s=min(a.cpu_seconds, 3.0))
        extra["rel_l2_vs_fp64_oracle"] = extra["cpu_baseline"]["gpu_rel_l2_vs_fp64_oracle"]
        for name in extra.get("forms", {}):
            extra["forms"][name]["rel_l2_vs_fp64_oracle"] = extra["cpu_baseline"]["gpu_rel_l2_vs_fp64_oracle_" + name]
    print(json.dumps(line_for(a, nbytes / (ms / 1e3) / 1e9, ms, nbytes, dt, launches, extra)), flush=True)


def cfg2_oracle_check(w, xin, yout):
    """Mixed-radix configurations: sampled transforms of the GPU output against
    the FP64 oracle on the same inputs (rel-L2, worst sample), and the
    reference algorithm (the f32 oracle) timed over the whole call on one
    thread."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    f64, f32 = np.float64, np.float32
    errs = []
    if w == "cfg2col":   # 4096 columns of 1000 points, row-major 1000 x 4096
        M, N = 1000, 4096
        X, Y = xin.reshape(M, N, 2), yout.reshape(M, N, 2)
        for j in (0, 1, 1234, 2047, N - 1):
            col = np.ascontiguousarray(X[:, j]).reshape(-1).astype(f64)
            ref = O.CView(np.zeros(2 * M), 0, M, 1, 1, M)
            O.Plan(O.CCOP, 1, M, 1.0, O.FWD, O.ROW, f64).ccfftmop(O.CView(col, 0, M, 1, 1, M), ref)
            got = np.ascontiguousarray(Y[:, j]).reshape(-1).astype(f64)
            errs.append(float(np.linalg.norm(got - ref.buf) / np.linalg.norm(ref.buf)))
        t = time.perf_counter()
        O.Plan(O.CCOP, M, N, 1.0, O.FWD, O.COL, f32).ccfftmop(
            O.CView(xin.copy(), 0, N, M, 1, N), O.CView(np.zeros_like(xin), 0, N, M, 1, N))
        t = time.perf_counter() - t
        nbytes = 16 * M * N
    else:
        M, N, H = 4096, 1536, 769
        rows = (0, 1, 1000, 2048, M - 1)
        for r in rows:
            if w == "cfg2rc":
                xr = xin.reshape(M, N)[r].astype(f64)
                ref = O.CView(np.zeros(2 * H), 0, H, 1, 1, H)
                O.Plan(O.RCOP, 1, N, 1.0, O.FWD, O.ROW, f64).rcfftmop(O.RView(xr, 0, N, 1, 1, N), ref)
                got = yout.reshape(M, 2 * H)[r].astype(f64)
            else:
                zr = xin.reshape(M, 2 * H)[r].astype(f64)
                ref = O.RView(np.zeros(N), 0, N, 1, 1, N)
                O.Plan(O.CROP, 1, N, 1.0 / N, O.INV, O.ROW, f64).crfftmop(O.CView(zr, 0, H, 1, 1, H), ref)
                got = yout.reshape(M, N)[r].astype(f64)
            errs.append(float(np.linalg.norm(got - ref.buf) / np.linalg.norm(ref.buf)))
        t = time.perf_counter()
        if w == "cfg2rc":
            O.Plan(O.RCOP, M, N, 1.0, O.FWD, O.ROW, f32).rcfftmop(
                O.RView(xin.copy(), 0, N, M, 1, N), O.CView(np.zeros(2 * M * H, f32), 0, H, M, 1, H))
        else:
            O.Plan(O.CROP, M, N, 1.0 / N, O.INV, O.ROW, f32).crfftmop(
                O.CView(xin.copy(), 0, H, M, 1, H), O.RView(np.zeros(M * N, f32), 0, N, M, 1, N))
        t = time.perf_counter() - t
        nbytes = M * (4 * N + 8 * H)
    return {"rel_l2_vs_fp64_oracle": max(errs), "sampled_transforms": len(errs),
            "cpu_baseline": {"value": round(nbytes / t / 1e9, 4), "unit": "GB/s", "cores": 1, "kind": "port",
                             "sample": f"the whole call once on one thread in {t:.2f} s (oracle/fftm_oracle.c)"}}


def komega_workload(a, torch, J, L, ext):
    """The k-omega power estimate (kw.c komega(): tapers, R2C rows, c2c
    columns, |.|^2, scale, accumulate) on Nsens x Nts real data through
    jvsip_komega_f (two launches), blocks admitted.  Algorithmic bytes: the
    data read and written back (8 B/sample), the spectrum written once and the
    gram read and written (8 + 8 B/bin); the spectrum's round trip between the
    two launches is not counted."""
    import numpy as np
    from jvsip_gb300 import synth
    Ns, Nt = a.kw_sensors, a.kw_samples
    Nf = Nt // 2 + 1
    x = synth.fill(Ns * Nt, 11, 1)
    x0 = x.copy()
    f = np.zeros(2 * Ns * Nf, np.float32)
    g = np.zeros(Ns * Nf, np.float32)
    n = np.arange(1, Nt + 1, dtype=np.float64)
    ts = (0.5 * (1 - np.cos(2 * np.pi * n / (Nt + 1)))).astype(np.float32)
    m = np.arange(1, Ns + 1, dtype=np.float64)
    arr = (0.5 * (1 - np.cos(2 * np.pi * m / (Ns + 1)))).astype(np.float32)
    bx, bf, bg, bt, ba = J.RBlock(x), J.CBlock(f), J.RBlock(g), J.RBlock(ts), J.RBlock(arr)
    for b in (bx, bf, bg, bt, ba):
        b.admit(True)
    vx, vf, vg = bx.view(0, Nt, Ns, 1, Nt), bf.view(0, 1, Ns, Ns, Nf), bg.view(0, 1, Ns, Ns, Nf)
    vt, va = bt.vview(0, 1, Nt), ba.vview(0, 1, Ns)
    rc = J.FFTM(J.KIND_RCOP, Ns, Nt, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=1)
    cc = J.FFTM(J.KIND_CCIP, Ns, Nf, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, ntimes=1)
    scale = 1.0 / 16

    def call():
        if L.jvsip_komega_f(rc.h, cc.h, vt.h, va.h, vx.h, vf.h, scale, vg.h):
            raise RuntimeError("jvsip_komega_f: %s" % (J.last_error(),))

    nbytes = 8 * Ns * Nt + 16 * Ns * Nf + 8 * Ns * Nf
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if nbytes < (512 << 20) else None
    for _ in range(a.warmup):
        call()
    L.jvsip_gpu_synchronize()
    n0 = L.jvsip_gpu_kernel_launches()
    per = timed_calls(torch, ext, call, a.steps, flush)
    launches = L.jvsip_gpu_kernel_launches() - n0
    J.check("komega")
    ms = statistics.mean(per)
    extra = {"config": {"workload": f"jvsip_komega_f {Ns} sensors x {Nt} samples f32 (kw.c komega: tapers, "
                                    f"rcfftmop ROW, ccfftmip COL, |.|^2, scale, accumulate), freq and gram "
                                    f"column-major as kw.c creates them", "bytes_per_step": nbytes,
                        "l2": "flushed between calls" if flush is not None else "inputs larger than L2"}}
    # one call from the original data, checked against the oracle on the host
    bx.release(False)
    bg.release(False)
    x[:] = x0
    g[:] = 0
    bx.admit(True)
    bg.admit(True)
    call()
    for b in (bx, bf, bg):
        b.release(True)
    if not a.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as O
        d = O.RView(x0.copy(), 0, Nt, Ns, 1, Nt)
        fo = O.CView(np.zeros_like(f), 0, 1, Ns, Ns, Nf)
        go = O.RView(np.zeros_like(g), 0, 1, Ns, Ns, Nf)
        t0 = time.perf_counter()
        O.komega_f(ts, arr, d, fo, go, np.float32(scale))
        cpu_s = time.perf_counter() - t0
        extra["cpu_baseline"] = {"value": round(nbytes / cpu_s / 1e9, 3), "unit": "GB/s", "cores": 1,
                                 "kind": "port", "sample": "the whole call once (the oracle's kw.c sequence)"}
        extra["data_bit_exact_vs_oracle"] = bool(np.array_equal(x, d.buf))
        ref = go.buf.astype(np.float64)
        extra["gram_rel_l2_vs_oracle"] = float(np.linalg.norm(g - ref) / np.linalg.norm(ref))
    for v in (vx, vf, vg, vt, va):
        v.destroy()
    for b in (bx, bf, bg, bt, ba):
        b.destroy()
    print(json.dumps(line_for(a, nbytes / (ms / 1e3) / 1e9, ms, nbytes, "f32", launches, extra)), flush=True)


def batching_workload(a, torch, J, L, ext):
    """cfg5: the batching configuration's instance sequence (truncated at
    --batch-gb per buffer) as one batch launch (graph replay) against a loop of
    per-plan vsip_ccfftmop_f calls on the same views."""
    import ctypes as C
    import numpy as np
    from jvsip_gb300 import synth
    seq = synth.batch_sequence(20000, seed=6, max_bytes=(a.batch_gb * 1e9 if a.batch_gb > 0 else None))
    lit = synth.batch_sequence(20000, seed=6)
    total = sum(N * r for N, r, _, _ in seq)
    x = torch.randn(2 * total, device="cuda", generator=torch.Generator(device="cuda").manual_seed(6)).cpu().numpy()
    torch.cuda.empty_cache()
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    plans, vin, vout = [], [], []
    off = 0
    for N, r, d, major in seq:
        scale = 1.0 if d == -1 else 1.0 / N
        if major == 0:   # r rows of N points
            p = J.FFTM(J.KIND_CCOP, r, N, scale, d, J.VSIP_ROW)
            vi, vo = bx.view(off, N, r, 1, N), by.view(off, N, r, 1, N)
        else:            # N x r matrix whose r columns are the transforms
            p = J.FFTM(J.KIND_CCOP, N, r, scale, d, J.VSIP_COL)
            vi, vo = bx.view(off, r, N, 1, r), by.view(off, r, N, 1, r)
        plans.append(p)
        vin.append(vi)
        vout.append(vo)
        off += N * r
    n = len(plans)
    P = (C.c_void_p * n)(*[p.h for p in plans])
    VI = (C.c_void_p * n)(*[v.h for v in vin])
    VO = (C.c_void_p * n)(*[v.h for v in vout])
    nbytes = 16 * total
    lens = sorted({N for N, _, _, _ in seq})
    arr = (C.c_ulong * len(lens))(*lens)
    tune_t = time.perf_counter()
    if not a.no_autotune:
        L.jvsip_fftm_autotune_f(len(lens), arr, 0)
        L.jvsip_fftm_autotune_f(len(lens), arr, 1)
    tune_t = time.perf_counter() - tune_t
    J.check("autotune")
    bp = L.jvsip_fftm_batch_create_f(n, P, VI, VO)
    if not bp:
        J.check("batch create")
    run = lambda: L.jvsip_fftm_batch_run_f(bp)

    def loop():
        # the per-plan loop from C (the library's jvsip_fftm_loop_f): one
        # vsip_ccfftmop_f call per instance, no Python between the calls
        if L.jvsip_fftm_loop_f(n, P, VI, VO):
            raise RuntimeError("jvsip_fftm_loop_f: %s" % (J.last_error(),))

    for _ in range(a.warmup):
        run()
    loop()
    J.check("warm-up")
    L.jvsip_gpu_synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if nbytes < (512 << 20) else None
    n0 = L.jvsip_gpu_kernel_launches()
    per = timed_calls(torch, ext, run, a.steps, flush)
    launches = L.jvsip_gpu_kernel_launches() - n0
    ms = statistics.mean(per)
    by.sync()
    # sampled instances: the batch's outputs (kept), then the loop's, then numpy's FP64 FFT
    offs = np.cumsum([0] + [N * r for N, r, _, _ in seq])
    sample = sorted({0, 1, n // 4, n // 2, (3 * n) // 4, n - 2, n - 1} & set(range(n)))
    ysave = {k: y[2 * offs[k]:2 * offs[k + 1]].copy() for k in sample}
    lsteps = max(1, min(a.steps, 20))
    per_loop = timed_calls(torch, ext, loop, lsteps, flush)
    ms_loop = statistics.mean(per_loop)
    by.sync()
    same = max(float(np.abs(ysave[k] - y[2 * offs[k]:2 * offs[k + 1]]).max()) for k in sample)
    errs = []
    for k in sample:
        N, r, d, major = seq[k]
        xi = x[2 * offs[k]:2 * offs[k + 1]].reshape(-1, 2)
        yi = ysave[k].reshape(-1, 2)
        xc = (xi[:, 0] + 1j * xi[:, 1]).astype(np.complex128)
        yc = (yi[:, 0] + 1j * yi[:, 1]).astype(np.complex128)
        A = xc.reshape(r, N) if major == 0 else xc.reshape(N, r).T
        B = yc.reshape(r, N) if major == 0 else yc.reshape(N, r).T
        ref = np.fft.fft(A, axis=1) if d == -1 else np.fft.ifft(A, axis=1)
        errs.append(float(np.linalg.norm(B - ref) / np.linalg.norm(ref)))
    L.jvsip_fftm_batch_destroy_f(bp)
    value = nbytes / (ms / 1e3) / 1e9
    loop_gbs = nbytes / (ms_loop / 1e3) / 1e9
    desc = (f"batching: {n} instances (seed 6, N log-uniform over the 175 2^a3^b5^c lengths in [64,16384], "
            f"rows U{{1..256}}, 50/50 fwd/inv and ROW/COL) "
            + (f"truncated at {a.batch_gb} GB per buffer; " if a.batch_gb > 0 else "the literal draw, untruncated; ")
            + f"the literal 20000 instances are {sum(8 * N * r for N, r, _, _ in lit) / 1e9:.1f} GB per buffer")
    extra = {"config": {"workload": desc, "bytes_per_step": nbytes, "instances": n,
                        "l2": "flushed between calls" if flush is not None else "inputs larger than L2"},
             "plain_loop": {"value": round(loop_gbs, 2), "unit": "GB/s", "ms_per_step": round(ms_loop, 4),
                            "calls_per_step": n, "how": "jvsip_fftm_loop_f: vsip_ccfftmop_f per instance from C"},
             "batched_over_loop": round(value / loop_gbs, 2),
             "batch_vs_loop_max_abs_diff_sampled": same, "rel_l2_vs_fp64_numpy_sampled": max(errs),
             "sampled_instances": len(sample),
             "autotune_s": round(tune_t, 2), "autotune_entries": int(L.jvsip_fftm_autotune_entries())}
    print(json.dumps(line_for(a, value, ms, nbytes, "f32", launches, extra)), flush=True)


# ---------------------------------------------------------------- default workload
def cfg3_variants(a, torch, J, L, ext, bx, by, vx, vy, M, N, x_np):
    """The rest of the large plain batch on the same admitted 65536 x 4096
    blocks: vsip_ccfftmop_f inverse (scale 1/4096, x -> y) and
    vsip_ccfftmip_f in place on y, forward and inverse calls alternating (so
    the data stays bounded).  Each with CUDA-event times on the library stream
    and a check: sampled inverse rows against the FP64 oracle, the first
    in-place forward call (applied to the inverse of x) against x itself, and
    the in-place round trips against the data they started from."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    nbytes = 16 * M * N
    inv_op = J.FFTM(J.KIND_CCOP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW)
    fwd_ip = J.FFTM(J.KIND_CCIP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW)
    inv_ip = J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW)
    steps = max(2, a.steps)
    out = {"workload": f"{M}x{N} c64 VSIP_ROW, the default line's admitted blocks", "unit": "GB/s"}
    call_inv = lambda: L.vsip_ccfftmop_f(inv_op.h, vx.h, vy.h)
    for _ in range(min(3, a.warmup)):
        call_inv()
    per = timed_calls(torch, ext, call_inv, steps)
    J.check("ccfftmop inverse")
    by.sync()
    y_np = by.re
    X, Y = x_np.reshape(M, 2 * N), y_np.reshape(M, 2 * N)
    errs = []
    for r in sorted({0, 1, M // 3, M // 2, M - 1}):
        ref = O.CView(np.zeros(2 * N), 0, N, 1, 1, N)
        O.Plan(O.CCOP, 1, N, 1.0 / N, O.INV, O.ROW, np.float64).ccfftmop(
            O.CView(X[r].astype(np.float64), 0, N, 1, 1, N), ref)
        errs.append(float(np.linalg.norm(Y[r].astype(np.float64) - ref.buf) / np.linalg.norm(ref.buf)))
    ms = statistics.mean(per)
    out["ccfftmop_f_inverse"] = {"value": round(nbytes / (ms / 1e3) / 1e9, 2), "ms_per_step": round(ms, 4),
                                 "scale": 1.0 / N, "rel_l2_vs_fp64_oracle": max(errs), "sampled_rows": len(errs)}
    y0 = Y[:64].copy()
    # in place on y: the first forward call gives back x
    L.vsip_ccfftmip_f(fwd_ip.h, vy.h)
    J.check("ccfftmip forward")
    by.sync()
    e_first = float(np.linalg.norm(Y[:64].astype(np.float64) - X[:64]) / np.linalg.norm(X[:64].astype(np.float64)))
    L.vsip_ccfftmip_f(inv_ip.h, vy.h)
    pf, pi = [], []
    for _ in range(steps):
        pf += timed_calls(torch, ext, lambda: L.vsip_ccfftmip_f(fwd_ip.h, vy.h), 1)
        pi += timed_calls(torch, ext, lambda: L.vsip_ccfftmip_f(inv_ip.h, vy.h), 1)
    J.check("ccfftmip loop")
    by.sync()
    e_rt = float(np.linalg.norm(Y[:64].astype(np.float64) - y0) / np.linalg.norm(y0.astype(np.float64)))
    mf, mi = statistics.mean(pf), statistics.mean(pi)
    out["ccfftmip_f_forward"] = {"value": round(nbytes / (mf / 1e3) / 1e9, 2), "ms_per_step": round(mf, 4),
                                 "rel_l2_first_call_vs_input_x": e_first}
    out["ccfftmip_f_inverse"] = {"value": round(nbytes / (mi / 1e3) / 1e9, 2), "ms_per_step": round(mi, 4),
                                 "scale": 1.0 / N,
                                 f"rel_l2_after_{steps + 1}_round_trips": e_rt}
    for p in (inv_op, fwd_ip, inv_ip):
        p.destroy()
    return out


def forms_summary(a):
    """The precision form (cfg4: plain against split FP16 / BF16 on 32768x1024,
    rows scaled by 10^U(-3,3)) and the batching form (cfg5: the 2 GB instance
    sequence, one graph replay against a loop of per-plan calls), each measured
    by its own bench.py run on the same GPU, summarised for the default line."""
    out = {}
    runs = (("cfg4", ["--cpu-seconds", "2"]), ("cfg5", ["--no-cpu"]), ("cfg1", ["--cpu-seconds", "2"]),
            ("cfg2rc", []), ("cfg2cr", []), ("cfg2col", []))
    for wl, extra in runs:
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", wl, "--steps", "20", "--warmup", "5"]
        try:
            r = subprocess.run(cmd + extra, capture_output=True, text=True, timeout=900)
            d = json.loads(r.stdout.strip().splitlines()[-1])
        except Exception as e:  # reported, never fatal for the main line
            out[wl] = {"error": str(e)[-300:]}
            continue
        if wl == "cfg4":
            f = d.get("forms", {})
            out["precision_form"] = {
                "workload": d["config"]["workload"], "unit": "GB/s",
                "plain": {"value": d["value"], "rel_l2_vs_fp64_oracle": d.get("rel_l2_vs_fp64_oracle")},
                "split_fp16": f.get("split_fp16"), "split_bf16": f.get("split_bf16"),
                "hbm_frac_plain": d.get("hbm_frac")}
        elif wl != "cfg5":
            out[wl] = {"workload": d["config"]["workload"], "value": d["value"], "unit": "GB/s",
                       "ms_per_step": d["ms_per_step"], "hbm_frac": d.get("hbm_frac"),
                       "gpu_launches": d.get("gpu_launches"),
                       "rel_l2_vs_fp64_oracle": d.get("rel_l2_vs_fp64_oracle"),
                       "cpu_baseline": d.get("cpu_baseline")}
            if wl == "cfg1" and isinstance(out[wl]["cpu_baseline"], dict):
                out[wl]["cpu_baseline"] = {k: v for k, v in out[wl]["cpu_baseline"].items()
                                           if not k.startswith("gpu_rel")}
        else:
            out["batching_form"] = {
                "workload": d["config"]["workload"], "unit": "GB/s",
                "batched": {"value": d["value"], "ms_per_step": d["ms_per_step"], "gpu_launches": d.get("gpu_launches")},
                "plain_loop": d.get("plain_loop"), "batched_over_loop": d.get("batched_over_loop"),
                "rel_l2_vs_fp64_numpy_sampled": d.get("rel_l2_vs_fp64_numpy_sampled"), "hbm_frac": d.get("hbm_frac")}
    return out


def main():
    a = args()
    if a.impl == "reference":
        reference_arm(a)
        return
    if a.workload != "cfg3":
        other_workload(a)
        return
    import numpy as np
    torch, J, L, ext = gpu_init()
    M, N = a.rows, 4096
    nbytes = M * N * 16
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    # synthetic N(0,1) input generated on the device from a seed, in pinned host memory
    n2 = 2 * M * N
    g = torch.Generator(device="cuda").manual_seed(4 + rank)
    xh = torch.empty(n2, dtype=torch.float32, pin_memory=True)
    xh.copy_(torch.randn(n2, device="cuda", generator=g))
    yh = torch.empty(n2, dtype=torch.float32, pin_memory=True)
    x_np, y_np = xh.numpy(), yh.numpy()

    plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW)
    bx, by = J.CBlock(x_np), J.CBlock(y_np)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)

    def step():
        L.vsip_ccfftmop_f(plan.h, vx.h, vy.h)

    for _ in range(a.warmup):
        step()
    J.check("warm-up")
    L.jvsip_gpu_synchronize()
    torch.cuda.synchronize()

    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    L.jvsip_gpu_synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps + 1)]
    n0 = L.jvsip_gpu_kernel_launches()
    ev[0].record(ext)
    for i in range(a.steps):
        step()
        ev[i + 1].record(ext)
    L.jvsip_gpu_synchronize()
    torch.cuda.synchronize()
    launches = L.jvsip_gpu_kernel_launches() - n0
    J.check("timed loop")
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(a.steps)]
    total_ms = max_over_ranks(torch, dist, ev[0].elapsed_time(ev[a.steps]))
    ms_per_step = total_ms / a.steps
    value = job_gbs(nbytes, world, ms_per_step)
    by.sync()

    # end to end: the same call on pinned host user blocks that are not admitted
    e2e = None
    if not a.no_e2e:
        xe = torch.empty(n2, dtype=torch.float32, pin_memory=True)
        xe.copy_(xh)
        ye = torch.empty(n2, dtype=torch.float32, pin_memory=True)
        bxe, bye = J.CBlock(xe.numpy()), J.CBlock(ye.numpy())
        vxe, vye = bxe.view(0, N, M, 1, N), bye.view(0, N, M, 1, N)
        for _ in range(min(3, a.warmup)):
            L.vsip_ccfftmop_f(plan.h, vxe.h, vye.h)
        J.check("e2e warm-up")
        if dist:
            dist.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        e0.record(ext)
        for _ in range(a.steps):
            L.vsip_ccfftmop_f(plan.h, vxe.h, vye.h)
        e1.record(ext)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        J.check("e2e loop")
        ems = max_over_ranks(torch, dist, max(e0.elapsed_time(e1) / a.steps, 1000 * wall / a.steps))
        ye_np = ye.numpy()
        k = 2 * N * min(64, M)
        diff = float(np.abs(ye_np[:k] - y_np[:k]).max())
        link_ms = link_time(torch, xe, ye)  # overwrites ye
        e2e = {"value": round(job_gbs(nbytes, world, ems), 2), "unit": "GB/s",
               "h2d_bytes_per_step": n2 * 4, "d2h_bytes_per_step": n2 * 4, "ms_per_step": round(ems, 3),
               "path": "vsip_ccfftmop_f on pinned, non-admitted user blocks (staged inside the call)",
               "max_abs_diff_vs_resident": diff,
               "link": {"ms_both_directions": round(link_ms, 3),
                        "gbs_each_way": round(n2 * 4 / (link_ms / 1e3) / 1e9, 1),
                        "roofline_value": round(nbytes / (link_ms / 1e3) / 1e9, 2),
                        "frac": round(link_ms / ems, 4),
                        "how": "the same bytes copied host->device and device->host at once on two streams "
                               "(pinned memory), no transform: the host link bounds the e2e path"}}
        for v in (vxe, vye):
            v.destroy()
        for b in (bxe, bye):
            b.destroy()
    clk = clocks.stop()
    cpu = None if (a.no_cpu or rank != 0) else cpu_leg(x_np, N, M, gpu_out=y_np, target_s=a.cpu_seconds)
    variants = None
    if not a.no_forms:
        variants = cfg3_variants(a, torch, J, L, ext, bx, by, vx, vy, M, N, x_np)

    for v in (vx, vy):
        v.destroy()
    bx.release(False)
    by.release(False)
    for b in (bx, by):
        b.destroy()
    if rank != 0:
        return
    peak, peak_kind = peaks()
    kern_ms = statistics.mean(per)
    achieved = nbytes / (kern_ms / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "k_fast_c64_4096_rows.md")
    if os.path.exists(tf):
        for ln in open(tf):
            if ln.startswith("traffic_bytes_per_launch_65536_rows:"):
                traffic = int(int(ln.split(":")[1]) * M / 65536)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic iid N(0,1) (seeded torch generator), 2 GiB per buffer",
        "config": {"workload": f"vsip_ccfftmop_f {M}x{N} c64 VSIP_ROW forward scale 1, admitted blocks",
                   "rows": M, "points": N, "bytes_per_step": nbytes,
                   "l2": "inputs larger than L2 (2 GiB per buffer vs 129 MB)", "parallelism": f"replicas x{world}"},
        "hbm_frac": round(value / world / peak, 4),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": traffic,
                     "traffic_how": "dram__bytes_read.sum + dram__bytes_write.sum of one k_fast launch in steady state "
                                    "(ncu --cache-control none, 8192 rows, scaled by rows): "
                                    "profiles/k_fast_c64_4096_rows.md",
                     "kernel_ms": round(kern_ms, 4), "algorithmic_bytes_per_launch": nbytes},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if line["cpu_baseline"]:
        line["rel_l2_vs_fp64_oracle"] = line["cpu_baseline"].get("gpu_rel_l2_vs_fp64_oracle")
    if variants:
        line["cfg3_variants"] = variants
    if not a.no_forms and world == 1:
        line["forms"] = forms_summary(a)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
