#!/usr/bin/env python
"""Benchmark: aggregation + breakage RHS evaluations per second at n = 16384, FP64.

Workload (single instance, one GPU): n = 16384 pivots x_i = 1e-21 * 2^(i/512) m^3,
lognormal N (median bin 2048, sigma_ln = 1, total 1e14 m^-3), Brownian+shear
aggregation (beta_br = 6.73e-18, beta_sh = 4 G / 3, G = 50 1/s) plus threshold
breakage (S0 = 1e-3 1/s, v_min = x_8192) with the symmetric-binary daughter
written as n_quad = 16 coincident quadrature entries. Synthetic inputs.

One step = zero rhs + aggregation RHS + breakage RHS (the source term an ODE
integrator asks for once per stage).

  value : steps/s with N, x, tables resident in HBM; each step timed with CUDA
          events on the launching stream; L2 (126 MiB) is flushed by writing a
          512 MiB buffer before every timed step (outside the events).
  e2e   : the same step through the C ABI from pinned HOST buffers: H2D copy of
          N, the RHS, D2H copy of rhs, all inside the timed events.

  roofline: the pair kernel (agg_main_kernel) timed alone with CUDA events;
          bound = the FP64 pipe, in FP64 instructions per second against the
          DFMA-chain probe's rate (one pipe slot per instruction). The
          reference-formula flop rate (22 flops per pair) is reported beside
          it as reference_equivalent_*: it exceeds the peak because the
          kernel executes about 4.5 FP64 instructions per pair.
  cpu_baseline: the oracle port on this host, all threads and one thread.

--impl reference times the reference's path on the machine's host cores. The
reference implements the path only in CUDA (no CPU implementation), so the arm
runs the oracle port (oracle/pbe_oracle.cpp: the reference's pair and fragment
loops restated serially, aggregation rows spread over all host threads) on
the same workload and config; each step is one full n = 16384 RHS
evaluation, with --steps and --warmup honoured unless the steps would take
more than about four minutes.

The JSON line ends with `summary`: the headline figures of the other sections
(the reference's CUDA kernels built unmodified from its sources into
oracle/_ref and timed on the same GPU, the other accumulation mode, the VJP,
batched cells, the adjoint tape, size classes). The sections themselves go to
--sections-out (default bench_sections.json) and to stderr.

Multi-GPU: the single-instance RHS does not shard; with torchrun each rank runs
an independent replica on its own GPU ("replicas only"), value = total steps/s.
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
for _p in (os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N_BINS = 16384
N_QUAD = 16
PAIRS = N_BINS * (N_BINS + 1) // 2
FRAGMENTS = N_BINS * N_QUAD
FLOPS_PER_PAIR = 22      # algorithmic FP64 flops per pair interaction
FLOPS_PER_FRAGMENT = 8   # per breakage fragment
# FP64 instructions of the Brownian+shear pair kernel per pair evaluation:
# lags with lo > k: rate (DMUL, DFMA, DMUL) + R += rate (DADD) + TH (DFMA) = 5;
# lags with lo = k: q (DMUL, DFMA) + R (DADD) + TH (DFMA) = 4. The weight
# numerator runs on the integer pipe. fp64_instr_per_launch() counts the
# evaluations of both kinds the kernel performs on a given grid (each pair
# once: tiles hand the w-part of their top slot to the tile above), plus 4 per
# clipped pair (the clip tasks). On this workload the count is within 3 % of
# ncu's FP64 instruction counters (dadd + dfma + dmul) for one launch.
FP64_PHASE1, FP64_PHASE2 = 5, 4


def fp64_instr_per_launch(x) -> int:
    n = len(x)
    v = x[0] + x
    L = np.searchsorted(x, v, side="right") - 1          # bracket of x_0 + x_d
    L = np.where(v >= x[-1], 1 << 30, L)
    # clipped pairs (summed by the clip tasks): rate (3) + accumulation (1)
    d_all = np.arange(n)
    jlo = np.where(L >= (1 << 30), 0, np.maximum(0, n - 1 - L))
    clipped = int(np.maximum(0, (n - 1 - d_all) - jlo + 1).sum())
    e0 = np.flatnonzero(L == np.arange(n))
    D0 = int(e0[0]) if len(e0) else n
    # pair (j, j + d) lands on slot j + L[d] <= n - 2
    cnt = np.where(L <= n - 2, np.maximum(0, n - 1 - L), 0)
    return (FP64_PHASE1 * int(cnt[d_all < D0].sum()) + FP64_PHASE2 * int(cnt[d_all >= D0].sum())
            + 4 * clipped)
# Lane-block pair kernel (agg_lane_kernel, geometric grids): one slot per lane,
# blocks of 32 bins, lag chunks of max(256, n/16 rounded up to 64) lags split
# evenly over 8 warps. Per non-clipped pair 4 FP64 instructions for
# Brownian + shear (q = B N_j + S x_j N_j: DMUL + DFMA; its sum: DADD; its
# weighted sum: DFMA); every run of lags with one bracket offset, in every
# warp's share, costs 2 DFMA per lane when it is folded in; 4 per clipped pair.
LANE_BINS, LANE_WARPS, LANE_MIN_CHUNK, LAG_CLIP = 32, 8, 256, 0x3fffffff


def vjp_lane_fp64_instr(x) -> int:
    """FP64 instructions of the lane-block aggregation VJP (Brownian + shear)
    on a geometric grid: 7 per pair j < k (P, P Bf, P Sf, two sums of row j,
    two FMAs into the sum of row k), 6 when the pair is clipped at x[n-1]
    (P = lambda_{n-1}, no FMA)."""
    n = len(x)
    v = x[0] + x
    L = np.searchsorted(x, v, side="right") - 1
    L = np.where(v >= x[-1], LAG_CLIP, L)[1:]
    d = np.arange(1, n)
    nj = n - d                                            # rows j = 0 .. n-1-d
    jclip = np.where(L >= LAG_CLIP, 0, np.maximum(0, n - 1 - L))
    clipped = int(np.maximum(0, nj - jclip).sum())
    return 7 * int(nj.sum()) - clipped


def lane_fp64_instr_per_launch(x) -> int:
    n = len(x)
    v = x[0] + x
    L = np.searchsorted(x, v, side="right") - 1          # bracket of x_0 + x_d
    L = np.where(v >= x[-1], LAG_CLIP, L)
    d_all = np.arange(n)
    jlo = np.where(L >= LAG_CLIP, 0, np.maximum(0, n - 1 - L))
    clipped = int(np.maximum(0, (n - 1 - d_all) - jlo + 1).sum())
    pairs = int(np.where(L <= n - 2, np.maximum(0, n - 1 - L), 0).sum())
    e = L - d_all
    chg = np.concatenate([[0], np.cumsum(e[1:] != e[:-1])])   # run starts at d >= 1
    C = max(LANE_MIN_CHUNK, ((n + 15) // 16 + 63) // 64 * 64)
    nblk = (n + LANE_BINS - 1) // LANE_BINS
    ts, cs = [], []
    c = 0
    while True:
        if c == 0:
            cnt = nblk
        elif c * C > n - 2:
            cnt = 0
        else:
            cnt = min(nblk, (n - 1 - c * C) // LANE_BINS + 1)
        if cnt == 0:
            break
        ts.append(np.arange(cnt))
        cs.append(np.full(cnt, c))
        c += 1
    t = np.concatenate(ts)
    c = np.concatenate(cs)
    smax = np.minimum(n - LANE_BINS * t - 1, n - 2)
    dA = c * C
    dB = np.minimum(dA + C, smax + 1)
    Lc = np.where(L >= LAG_CLIP, np.iinfo(np.int64).max, L)
    dB = np.clip(np.searchsorted(Lc, smax, side="right"), dA, np.maximum(dA, dB))
    per = (dB - dA + LANE_WARPS - 1) // LANE_WARPS
    runs = 0
    for w in range(LANE_WARPS):
        d0 = dA + w * per
        d1 = np.minimum(dB, d0 + per)
        ok = d1 > d0
        runs += int((1 + chg[np.maximum(d1 - 1, 0)] - chg[np.minimum(d0, n - 1)])[ok].sum())
    return 4 * pairs + 2 * 32 * runs + 4 * clipped


# dram__bytes_read.sum + dram__bytes_write.sum of one agg_main_kernel launch on
# this workload, read from an ncu capture of that launch (L2 flushed before it,
# as in the timed loop); not measured by this script.
MAIN_KERNEL_DRAM_BYTES = 1343488
# algorithmic bytes of one aggregation RHS: N and x read, rhs read and written
ALGO_BYTES_PER_LAUNCH = 24 * N_BINS
L2_FLUSH_BYTES = 512 << 20


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


WORKLOAD = ("single-instance agg+brk RHS, n=16384, x_i=1e-21*2^(i/512), BrownianShear + "
            "threshold breakage, n_quad=16")


def run_config() -> dict:
    """The `config` of both arms' JSON lines (identical on purpose)."""
    return {"workload": WORKLOAD, "n": N_BINS, "n_quad": N_QUAD, "pairs_per_eval": PAIRS,
            "fragments_per_eval": FRAGMENTS,
            "l2": "GPU arm: flushed before every timed step (512 MiB write)",
            "parallelism": "single instance per GPU (replicas only)"}


def cpu_model() -> str:
    """CPU model name of this host (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                             text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def workload():
    import pbe_gb300 as pg

    c = pg.grids.config_n16384()
    x, N = c["x"], c["N"]
    ap = pg.AggregationParams(n=N_BINS, kernel_type=pg.AGG_BROWNIAN_SHEAR, beta0=0.0,
                              beta_br=c["beta_br"], beta_sh=c["beta_sh"])
    ap.log_x0, ap.inv_log_r = pg.grids.geometric_params(x)
    t_q, bw_q = pg.quadrature.symmetric_binary_split(N_QUAD)
    bp = pg.BreakageParams(n=N_BINS, n_quad=N_QUAD, selection=pg.SEL_THRESHOLD, S0=c["S0"],
                           v_min=c["v_min"])
    return x, N, t_q, bw_q, ap, bp


def fp64_peak_tflops(stream) -> float | None:
    import ctypes

    import pbe_gb300 as pg

    path = os.path.join(os.path.dirname(pg.LIB_PATH), "libpbe_probe.so")
    if not os.path.isfile(path):
        return None
    lib = ctypes.CDLL(path)
    lib.pbe_probe_dfma_tflops.restype = ctypes.c_double
    lib.pbe_probe_dfma_tflops.argtypes = [ctypes.c_int, ctypes.c_void_p]
    v = lib.pbe_probe_dfma_tflops(5, stream.cuda_stream)
    return v if v > 0 else None


def cpu_baseline(x, N, t_q, bw_q, ap, bp, seconds=3.0, serial_evals=3):
    """Oracle port (the reference's pair and fragment loops restated as serial
    C++, g++ -O3 -ffp-contract=off) on this host's cores, full n = 16384 RHS
    evaluations: `value` with aggregation rows spread over every host thread
    (OpenMP, repeated for `seconds`), `serial` on one thread (`serial_evals`
    evaluations)."""
    import pyoracle

    threads = os.cpu_count() or 1

    def run(nthreads, min_s, min_evals):
        t0 = time.perf_counter()
        evals = 0
        while True:
            pyoracle.aggregation_rhs_mt(N, x, ap.kernel_type, ap.beta0, ap.beta_br, ap.beta_sh,
                                        ap.log_x0, ap.inv_log_r, nthreads=nthreads)
            pyoracle.breakage_rhs(N, x, t_q, bw_q, bp.selection, bp.S0, bp.v_ref, bp.alpha,
                                  bp.v_min)
            evals += 1
            el = time.perf_counter() - t0
            if el >= min_s and evals >= min_evals:
                return evals, el

    evals, el = run(threads, seconds, 1)
    s_evals, s_el = run(1, 0.0, serial_evals)
    model = cpu_model()
    return {"value": evals / el, "unit": "evals/s", "cores": threads, "kind": "port",
            "sample": "%d full n=16384 agg+brk RHS evaluations (%.1f s wall, OpenMP over "
                      "aggregation rows, breakage serial)" % (evals, el),
            "cpu_model": model,
            "serial": {"value": s_evals / s_el, "unit": "evals/s", "cores": 1,
                       "sample": "%d full n=16384 agg+brk RHS evaluations on one thread (%.1f s)"
                                 % (s_evals, s_el)},
            "build": "g++ -O3 -ffp-contract=off (portable flags: the same oracle binary "
                     "semantics on x86_64 and aarch64, no -march=native)"}


def fp64_instr_tiles(x, n_cell=None) -> int:
    """FP64 instructions of the tile kernel for a cell with the first n_cell
    pivots of x (same counting as fp64_instr_per_launch)."""
    x = x[:n_cell] if n_cell else x
    return fp64_instr_per_launch(x)


def batched_section(dev, stream):
    """Batched cells: 4096 cells with n in {64..3840}, q in {4,8,16,32}
    (pbe_gb300.grids.config_batched_cells, seed 2026), Brownian+shear with a
    per-cell shear rate, power-law selection, uniform daughter (GL 8); 100 RK4
    steps of dt = 0.5 s as one CUDA graph, against the per-cell launch loop
    (single-instance calls per cell and stage) over one step."""
    import torch

    import pbe_gb300 as pg

    cfg = pg.grids.config_batched_cells()
    t0 = time.perf_counter()
    plan = pg.BatchPlan(cfg["grids"], cfg["cell_n"], cfg["cell_grid"], pg.AGG_BROWNIAN_SHEAR,
                        pg.SEL_POWERLAW, cfg["t_q"], cfg["bw_q"], tune=True, stream=stream)
    plan_s = time.perf_counter() - t0
    f64 = dict(dtype=torch.float64, device=dev)
    dN = torch.tensor(cfg["N"], **f64)
    P = torch.tensor(cfg["params"], **f64)
    out = torch.zeros(plan.total, **f64)
    n_cells = len(cfg["cell_n"])
    cn = cfg["cell_n"].astype(np.float64)
    pairs = float((cn * (cn + 1) / 2).sum())
    frags = float(cn.sum() * len(cfg["t_q"]))
    steps, dt = 100, 0.5
    with torch.cuda.stream(stream):
        for _ in range(3):
            pg.check(plan.rhs(dN, out, P, stream=stream), "batch rhs")
        reps = 5
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            pg.check(plan.rhs(dN, out, P, stream=stream), "batch rhs")
        b.record(stream)
        torch.cuda.synchronize()
        rhs_ms = a.elapsed_time(b) / reps
        # 100 steps in one graph (captured and uploaded before the timing)
        Y = dN.clone()
        pg.check(plan.rk4_prepare(Y, P, dt, steps), "rk4 prepare")
        torch.cuda.synchronize()
        a.record(stream)
        pg.check(plan.rk4(Y, P, dt, steps, stream=stream), "rk4")
        b.record(stream)
        torch.cuda.synchronize()
        graph_ms = a.elapsed_time(b)
        fin = torch.isfinite(Y).cpu().numpy()
        off = np.r_[0, np.cumsum(cfg["cell_n"])]
        bad_cells = int(sum(not fin[off[c]:off[c + 1]].all() for c in range(n_cells)))
        finite = bad_cells == 0
        # per-cell launch loop, one step
        Z = dN.clone()
        pg.check(plan.rk4_percell(Z, P, dt, 1, stream=stream), "percell warm-up")
        Z = dN.clone()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        a.record(stream)
        pg.check(plan.rk4_percell(Z, P, dt, 1, stream=stream), "percell")
        b.record(stream)
        torch.cuda.synchronize()
        loop_ms = a.elapsed_time(b)
        loop_wall = time.perf_counter() - w0
        Y1 = dN.clone()
        pg.check(plan.rk4(Y1, P, dt, 1, stream=stream), "rk4 one step")
        torch.cuda.synchronize()
        agree = float((Y1 - Z).abs().max() / dN.abs().max())
    gs, nb = plan.schedule()
    plan.close()
    # FP64 instructions of one batched RHS (tile evaluations, per cell)
    instr = 0
    memo = {}
    for g, n in zip(cfg["cell_grid"], cfg["cell_n"]):
        key = (int(g), int(n))
        if key not in memo:
            memo[key] = fp64_instr_tiles(cfg["grids"][g], int(n))
        instr += memo[key]
    peak = fp64_peak_tflops(stream)
    cell_steps = n_cells * steps / (graph_ms / 1e3)
    loop_cell_steps = n_cells / (loop_ms / 1e3)
    achieved = (FLOPS_PER_PAIR * pairs + FLOPS_PER_FRAGMENT * frags) / (rhs_ms / 1e3) / 1e12
    return {
        "workload": "4096 cells, n ~ U{64..3840}, x_i = 1e-21*2^(i/q), q ~ U{4,8,16,32}, "
                    "Brownian+shear (per-cell G log-uniform [10,200]) + power-law selection "
                    "(S0=1e-3, a ~ U[0.5,1.5], x_ref = middle pivot) + uniform daughter GL8, "
                    "lognormal N; seed 2026; 100 RK4 steps dt=0.5 s in one CUDA graph",
        "cell_steps_per_s": round(cell_steps, 1),
        "graph_ms": round(graph_ms, 2),
        "steps": steps,
        "percell_loop_cell_steps_per_s": round(loop_cell_steps, 1),
        "percell_loop_ms_per_step": round(loop_ms, 2),
        "percell_loop_wall_s": round(loop_wall, 3),
        "speedup_vs_percell_loop": round(cell_steps / loop_cell_steps, 3),
        "graph_vs_loop_max_rel_diff_1step": agree,
        "finite_after_100_steps": finite,
        "cells_not_finite": bad_cells,
        "rhs_ms": round(rhs_ms, 3),
        "pair_interactions_per_s": round(pairs / (rhs_ms / 1e3), 1),
        "pairs_per_rhs": pairs,
        "roofline": {"bound": "fp64", "kernel": "batch_main_kernel<5> + batch_prep_kernel<5>",
                     "achieved": round(instr / (rhs_ms / 1e3) / 1e12, 4),
                     "peak": round(peak / 2.0, 4) if peak else None,
                     "unit": "T FP64 instr/s",
                     "frac": round(instr / (rhs_ms / 1e3) / (peak * 1e12 / 2.0), 4) if peak else None,
                     "fp64_instr_per_rhs": instr,
                     "fp64_instr_source": "instruction model of the tile kernel on the cells' grids",
                     "reference_equivalent_tflops": round(achieved, 4),
                     "reference_equivalent_unit": "22 FP64 flops per pair + 8 per fragment per s"},
        "schedule": {"group_size_by_log2n": gs, "bundles": nb, "tuned": True,
                     "plan_create_s": round(plan_s, 3)},
        "l2": "not flushed: one RHS touches > 300 MB of stage arrays (L2 126 MiB)",
    }


def adjoint_section(dev, stream):
    """Two-stage flocculation adjoint (pbe_gb300.grids.config_flocculation_adjoint):
    n = 3840, 200 RK4 steps dt = 0.5 s, G 100 -> 20 at step 100, checkpoints
    every 20 steps; gradient of L = sum x^(2/3) N(T) w.r.t. N(0) and the
    coefficients of both stages."""
    import torch

    import pbe_gb300 as pg

    cfg = pg.grids.config_flocculation_adjoint()
    f64 = dict(dtype=torch.float64, device=dev)
    n = len(cfg["x"])
    dx, dtq, dbw = (torch.tensor(cfg[k], **f64) for k in ("x", "t_q", "bw_q"))
    lam = torch.tensor(cfg["lam_T"], **f64)
    gN0 = torch.zeros(n, **f64)
    ga, gb = torch.zeros(6, **f64), torch.zeros(8, **f64)
    tape = pg.Rk4Tape(cfg["n_steps"], cfg["dt"], 20, cfg["agg_sets"], cfg["brk_sets"],
                      cfg["step_set"])
    a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    with torch.cuda.stream(stream):
        for _ in range(2):
            N = torch.tensor(cfg["N0"], **f64)
            pg.check(tape.forward(N, dx, dtq, dbw, stream=stream), "tape forward")
            pg.check(tape.backward(lam, gN0, ga, gb, stream=stream), "tape backward")
        N = torch.tensor(cfg["N0"], **f64)
        torch.cuda.synchronize()
        a.record(stream)
        pg.check(tape.forward(N, dx, dtq, dbw, stream=stream), "tape forward")
        b.record(stream)
        pg.check(tape.backward(lam, gN0, ga, gb, stream=stream), "tape backward")
        c.record(stream)
        torch.cuda.synchronize()
        fwd_ms, bwd_ms = a.elapsed_time(b), b.elapsed_time(c)
        # one RHS and one VJP at N(0), n = 3840
        N0 = torch.tensor(cfg["N0"], **f64)
        rhs = torch.zeros(n, **f64)
        ap, bp = cfg["agg_sets"][0], cfg["brk_sets"][0]

        def rhs_call():
            rhs.zero_()
            pg.check(pg.aggregation_rhs(N0, dx, rhs, ap, stream=stream), "agg")
            pg.check(pg.breakage_rhs(N0, dx, dtq, dbw, rhs, bp, stream=stream), "brk")

        def vjp_call():
            gN0.zero_()
            pg.check(pg.aggregation_rhs_vjp(N0, dx, lam, gN0, ga, ap, stream=stream), "agg vjp")
            pg.check(pg.breakage_rhs_vjp(N0, dx, dtq, dbw, lam, gN0, gb, bp, stream=stream), "brk vjp")
        times = {}
        for name, fn in (("rhs", rhs_call), ("vjp", vjp_call)):
            for _ in range(3):
                fn()
            a.record(stream)
            for _ in range(20):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            times[name] = a.elapsed_time(b) / 20
    tape.close()
    g = gN0.cpu().numpy()
    return {
        "workload": "n=3840, x_i=1e-21*2^(i/128), Brownian+shear G=100 -> 20 at step 100, "
                    "power-law selection S0=5e-4 a=1 v_ref=1e-18, power-law daughter p=2 (8 pts), "
                    "200 RK4 steps dt=0.5 s, checkpoints every 20, L = sum x^(2/3) N(T)",
        "forward_ms": round(fwd_ms, 3),
        "backward_ms": round(bwd_ms, 3),
        "backward_forward_ratio": round(bwd_ms / fwd_ms, 4),
        "gradient_cost_ratio": round((fwd_ms + bwd_ms) / fwd_ms, 4),
        "rhs_ms_n3840": round(times["rhs"], 4),
        "vjp_ms_n3840": round(times["vjp"], 4),
        "vjp_rhs_ratio_n3840": round(times["vjp"] / times["rhs"], 4),
        "gradient_finite": bool(np.all(np.isfinite(g))),
    }


def probe_tflops(stream, name) -> float | None:
    import ctypes

    import pbe_gb300 as pg

    path = os.path.join(os.path.dirname(pg.LIB_PATH), "libpbe_probe.so")
    if not os.path.isfile(path):
        return None
    lib = ctypes.CDLL(path)
    fn = getattr(lib, name)
    fn.restype = ctypes.c_double
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p]
    v = fn(5, stream.cuda_stream)
    return v if v > 0 else None


def classes_section(dev, stream):
    """Cells sharing grids by size class (pbe_gb300.grids.config_batched_classes):
    512 cells, n ~ U[256, 2048], class width 256, per-cell lognormal
    coefficients. 100 RK4 steps as one graph; the aggregation death term by the
    per-cell moment form and by the FP64 tensor-core GEMM (mma.sync f64)."""
    import torch

    import pbe_gb300 as pg

    cfg = pg.grids.config_batched_classes()
    plan = pg.BatchPlan(cfg["grids"], cfg["cell_n"], cfg["cell_grid"], pg.AGG_BROWNIAN_SHEAR,
                        pg.SEL_POWERLAW, cfg["t_q"], cfg["bw_q"], tune=True, stream=stream)
    f64 = dict(dtype=torch.float64, device=dev)
    dN, P = torch.tensor(cfg["N"], **f64), torch.tensor(cfg["params"], **f64)
    out = {m: torch.zeros(plan.total, **f64) for m in (pg.DEATH_MOMENTS, pg.DEATH_DMMA)}
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = {}
    with torch.cuda.stream(stream):
        for m in (pg.DEATH_MOMENTS, pg.DEATH_DMMA):
            for _ in range(3):
                pg.check(plan.death(dN, out[m], P, m, stream=stream), "death")
            a.record(stream)
            for _ in range(10):
                pg.check(plan.death(dN, out[m], P, m, stream=stream), "death")
            b.record(stream)
            torch.cuda.synchronize()
            times[m] = a.elapsed_time(b) / 10
        ref = out[pg.DEATH_MOMENTS]
        diff = float(((out[pg.DEATH_DMMA] - ref).abs() / ref.abs().clamp_min(1e-300)).max())
        steps = 100
        Y = dN.clone()
        pg.check(plan.rk4_prepare(Y, P, 0.5, steps), "rk4 prepare")
        torch.cuda.synchronize()
        a.record(stream)
        pg.check(plan.rk4(Y, P, 0.5, steps, stream=stream), "rk4")
        b.record(stream)
        torch.cuda.synchronize()
        graph_ms = a.elapsed_time(b)
        finite = bool(torch.isfinite(Y).all())
        # adjoint: L = 1/2 |N(T) - N*(T)|^2, N* from coefficients perturbed by 5 %
        Pstar = P.clone()
        Pstar[:, 1] *= 1.05
        Pstar[:, 2] *= 0.95
        Nstar = dN.clone()
        pg.check(plan.rk4(Nstar, Pstar, 0.5, steps, stream=stream), "target run")
        gN0 = torch.zeros(plan.total, **f64)
        gP = torch.zeros((len(cfg["cell_n"]), 8), **f64)
        NT = dN.clone()
        pg.check(plan.tape_forward(NT, P, 0.5, steps, 20, stream=stream), "tape forward warm-up")
        pg.check(plan.tape_backward(NT - Nstar, gN0, gP, stream=stream), "tape backward warm-up")
        NT = dN.clone()
        c_ = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        pg.check(plan.tape_forward(NT, P, 0.5, steps, 20, stream=stream), "tape forward")
        b.record(stream)
        lamT = NT - Nstar
        pg.check(plan.tape_backward(lamT, gN0, gP, stream=stream), "tape backward")
        c_.record(stream)
        torch.cuda.synchronize()
        tape_fwd_ms, tape_bwd_ms = a.elapsed_time(b), b.elapsed_time(c_)
        grad_finite = bool(torch.isfinite(gN0).all()) and bool(torch.isfinite(gP).all())
        # Jacobian-vector product against the RHS, and the linearly implicit ROS2 step
        rhs = torch.zeros(plan.total, **f64)
        vv = dN.flip(0).contiguous()
        jv = torch.zeros(plan.total, **f64)
        t_call = {}
        for name, call in (("rhs", lambda: plan.rhs(dN, rhs, P, stream=stream)),
                           ("jvp", lambda: plan.jvp(dN, vv, jv, P, stream=stream))):
            for _ in range(3):
                pg.check(call(), name)
            a.record(stream)
            for _ in range(10):
                pg.check(call(), name)
            b.record(stream)
            torch.cuda.synchronize()
            t_call[name] = a.elapsed_time(b) / 10
        m_kry, ros_steps = 8, 3
        resid = torch.zeros(len(cfg["cell_n"]), **f64)
        Yr = dN.clone()
        pg.check(plan.ros2(Yr, P, 0.5, 1, m_kry, resid, stream=stream), "ros2 warm-up")
        Yr = dN.clone()
        torch.cuda.synchronize()
        a.record(stream)
        pg.check(plan.ros2(Yr, P, 0.5, ros_steps, m_kry, resid, stream=stream), "ros2")
        b.record(stream)
        torch.cuda.synchronize()
        ros_ms = a.elapsed_time(b) / ros_steps
        ros_finite = bool(torch.isfinite(Yr).all())
        ros_resid = float(resid.max())
        # the same steps with solves that end at a relative residual of 1e-6
        kry_tol = 1e-6
        pg.check(plan.set_krylov_tol(kry_tol), "krylov tol")
        resid_t = torch.zeros_like(resid)
        Yt = dN.clone()
        pg.check(plan.ros2(Yt, P, 0.5, 1, m_kry, resid_t, stream=stream), "ros2 warm-up")
        Yt = dN.clone()
        resid_t.zero_()
        torch.cuda.synchronize()
        a.record(stream)
        pg.check(plan.ros2(Yt, P, 0.5, ros_steps, m_kry, resid_t, stream=stream), "ros2 tol")
        b.record(stream)
        torch.cuda.synchronize()
        pg.check(plan.set_krylov_tol(0.0), "krylov tol")
        ros_tol_ms = a.elapsed_time(b) / ros_steps
        ros_tol_diff = float(((Yt - Yr).abs().max() / Yr.abs().max().clamp_min(1e-300)))
    plan.close()
    cn = cfg["cell_n"].astype(np.float64)
    gemm_flops = float((2.0 * cn * cn).sum() * 2)          # two separable components
    dmma_peak = probe_tflops(stream, "pbe_probe_dmma_tflops")
    dmma_tf = gemm_flops / (times[pg.DEATH_DMMA] / 1e3) / 1e12
    return {
        "workload": "512 cells, n ~ U[256,2048], grids shared by size class (width 256), "
                    "x_i = 1e-21*2^(i/128); Brownian+shear + power-law selection, per-cell "
                    "coefficients lognormal(0.5) around beta_br=6.73e-18, G=50, S0=1e-3; seed 2026",
        "cell_steps_per_s": round(len(cn) * steps / (graph_ms / 1e3), 1),
        "graph_ms_100_steps": round(graph_ms, 2),
        "finite_after_100_steps": finite,
        "adjoint": {"what": "L = 1/2 |N(T) - N*(T)|^2 after 100 RK4 steps, N* from beta_br x 1.05 "
                            "and beta_sh x 0.95; batched checkpointed tape (every 20 steps): "
                            "dL/dN(0) and dL/d(7 coefficients) of all 512 cells",
                    "forward_ms": round(tape_fwd_ms, 2), "backward_ms": round(tape_bwd_ms, 2),
                    "backward_forward_ratio": round(tape_bwd_ms / tape_fwd_ms, 4),
                    "gradient_finite": grad_finite},
        "rhs_ms": round(t_call["rhs"], 4),
        "jvp_ms": round(t_call["jvp"], 4),
        "jvp_rhs_ratio": round(t_call["jvp"] / t_call["rhs"], 4),
        "ros2": {"what": "linearly implicit ROS2 steps of dt = 0.5 s, every stage solved by "
                         "GMRES(8) with Jacobian-vector products (2 RHS + 16 JVP per step)",
                 "krylov_dim": m_kry, "ms_per_step": round(ros_ms, 3),
                 "rhs_equivalents_per_step": round(ros_ms / t_call["rhs"], 2),
                 "cell_steps_per_s": round(len(cn) / (ros_ms / 1e3), 1),
                 "max_relative_residual": ros_resid, "finite": ros_finite,
                 "with_krylov_tol": {"tol": kry_tol, "ms_per_step": round(ros_tol_ms, 3),
                                     "rhs_equivalents_per_step": round(ros_tol_ms / t_call["rhs"], 2),
                                     "max_relative_residual": float(resid_t.max()),
                                     "max_diff_vs_full_solves": ros_tol_diff}},
        "death_moments_ms": round(times[pg.DEATH_MOMENTS], 4),
        "death_dmma_ms": round(times[pg.DEATH_DMMA], 4),
        "dmma_over_moments_time": round(times[pg.DEATH_DMMA] / times[pg.DEATH_MOMENTS], 2),
        "death_max_rel_diff": diff,
        "dmma_roofline": {"bound": "fp64 tensor (mma.sync f64)", "achieved": round(dmma_tf, 4),
                          "peak": round(dmma_peak, 4) if dmma_peak else None, "unit": "TFLOP/s",
                          "frac": round(dmma_tf / dmma_peak, 4) if dmma_peak else None,
                          "flops_per_call": gemm_flops,
                          "algorithmic_unit": "2 n^2 flops per cell and separable component "
                                              "(Brownian, shear)",
                          "peak_source": "mma.sync m8n8k4 f64 chain probe timed in this run "
                                         "(libpbe_probe.so), of measured"},
    }


def summarize(sections: dict, value: float) -> dict:
    """Headline figures of each section, for the one JSON line."""
    out = {}
    rk = sections.get("reference_kernels_sm103a", {})
    if "evals_per_s" in rk:
        out["reference_kernels_sm103a"] = {"evals_per_s": rk["evals_per_s"],
                                           "speedup_of_value": round(value / rk["evals_per_s"], 2)}
    elif rk:
        out["reference_kernels_sm103a"] = rk
    if "vjp" in sections:
        out["vjp_rhs_ratio_n16384"] = sections["vjp"]["vjp_rhs_ratio"]
        if "roofline" in sections["vjp"]:
            out["vjp_roofline_frac"] = sections["vjp"]["roofline"].get("frac")
    if "other_mode" in sections:
        om = sections["other_mode"]
        out["other_mode"] = {"mode": om["mode"], "evals_per_s": om["evals_per_s"]}
    b = sections.get("batched")
    if b:
        out["batched_config3"] = {k: b[k] for k in ("cell_steps_per_s", "percell_loop_cell_steps_per_s",
                                                    "speedup_vs_percell_loop", "finite_after_100_steps")}
        out["batched_config3"]["roofline_frac"] = b.get("roofline", {}).get("frac")
    a = sections.get("adjoint")
    if a:
        out["adjoint_config4"] = {k: a[k] for k in ("forward_ms", "backward_ms", "gradient_cost_ratio",
                                                    "rhs_ms_n3840", "vjp_rhs_ratio_n3840")}
    c = sections.get("classes")
    if c:
        out["classes_config5"] = {"cell_steps_per_s": c["cell_steps_per_s"],
                                  "adjoint_backward_forward": c["adjoint"]["backward_forward_ratio"],
                                  "jvp_rhs_ratio": c["jvp_rhs_ratio"],
                                  "death_dmma_over_moments_time": c["dmma_over_moments_time"]}
    return out


def profile_case(name: str) -> None:
    """A few launches of one kernel family on a mid-size case, for ncu:
      batched : 1024 cells of the batched workload (seed 2026), 4 batched RHS
      batched_small: one cell of n = 3840 (x_i = 1e-21 2^(i/128), the
                form of the batched workload) through the batched plan, 4 RHS
      death   : the 512-cell size-class workload, 3 DMMA and 3 moment death calls
      vjp     : the n = 16384 workload, 3 aggregation + breakage VJPs
      breakage: the n = 16384 workload, 3 breakage RHS calls in each mode
      lane    : the n = 16384 workload, 4 aggregation RHS calls (gather mode)
      adjoint : the n = 3840 flocculation tape, 10 steps forward + backward"""
    import torch

    import pbe_gb300 as pg

    dev = torch.device("cuda", 0)
    f64 = dict(dtype=torch.float64, device=dev)
    if name == "batched":
        cfg = pg.grids.config_batched_cells(n_cells=1024)
        with pg.BatchPlan(cfg["grids"], cfg["cell_n"], cfg["cell_grid"], pg.AGG_BROWNIAN_SHEAR,
                          pg.SEL_POWERLAW, cfg["t_q"], cfg["bw_q"]) as plan:
            dN, P = torch.tensor(cfg["N"], **f64), torch.tensor(cfg["params"], **f64)
            out = torch.zeros(plan.total, **f64)
            for _ in range(4):
                pg.check(plan.rhs(dN, out, P), "batch rhs")
    elif name == "batched_small":
        cfg = pg.grids.config_batched_cells(n_cells=1)
        x = pg.grids.geometric_pow2(3840, 1e-21, 128.0)
        N = pg.grids.lognormal_ic(x, 1280, 1.0, 1e13, cut=5.0)
        with pg.BatchPlan([x], [3840], [0], pg.AGG_BROWNIAN_SHEAR, pg.SEL_POWERLAW,
                          cfg["t_q"], cfg["bw_q"]) as plan:
            prm = pg.batch.cell_params(1, beta0=0.0, beta_br=6.73e-18, beta_sh=4 * 50 / 3,
                                       S0=1e-3, v_ref=float(x[1920]), alpha=1.0)
            dN, P = torch.tensor(N, **f64), torch.tensor(prm, **f64)
            out = torch.zeros(plan.total, **f64)
            for _ in range(4):
                pg.check(plan.rhs(dN, out, P), "batch rhs")
    elif name == "death":
        cfg = pg.grids.config_batched_classes()
        with pg.BatchPlan(cfg["grids"], cfg["cell_n"], cfg["cell_grid"], pg.AGG_BROWNIAN_SHEAR,
                          pg.SEL_POWERLAW, cfg["t_q"], cfg["bw_q"]) as plan:
            dN, P = torch.tensor(cfg["N"], **f64), torch.tensor(cfg["params"], **f64)
            out = torch.zeros(plan.total, **f64)
            for m in (pg.DEATH_DMMA, pg.DEATH_MOMENTS) * 3:
                pg.check(plan.death(dN, out, P, m), "death")
    elif name == "vjp":
        x, N, t_q, bw_q, ap, bp = workload()
        dN, dx = torch.tensor(N, **f64), torch.tensor(x, **f64)
        dt, db = torch.tensor(t_q, **f64), torch.tensor(bw_q, **f64)
        lam = torch.randn(N_BINS, dtype=torch.float64, device=dev,
                          generator=torch.Generator(device=dev).manual_seed(7))
        gN = torch.zeros(N_BINS, **f64)
        ga, gb = torch.zeros(3, **f64), torch.zeros(4, **f64)
        for _ in range(3):
            pg.check(pg.aggregation_rhs_vjp(dN, dx, lam, gN, ga, ap), "agg vjp")
            pg.check(pg.breakage_rhs_vjp(dN, dx, dt, db, lam, gN, gb, bp), "brk vjp")
    elif name == "lane":
        x, N, t_q, bw_q, ap, bp = workload()
        dN, dx = torch.tensor(N, **f64), torch.tensor(x, **f64)
        rhs = torch.zeros(N_BINS, **f64)
        for _ in range(4):
            pg.check(pg.aggregation_rhs(dN, dx, rhs, ap, mode=pg.MODE_GATHER), "agg")
    elif name == "breakage":
        x, N, t_q, bw_q, ap, bp = workload()
        dN, dx = torch.tensor(N, **f64), torch.tensor(x, **f64)
        dt, db = torch.tensor(t_q, **f64), torch.tensor(bw_q, **f64)
        rhs = torch.zeros(N_BINS, **f64)
        for mode in (pg.MODE_GATHER,) * 3 + (pg.MODE_SCATTER,) * 3:
            pg.check(pg.breakage_rhs(dN, dx, dt, db, rhs, bp, mode=mode), "brk")
    elif name == "adjoint":
        cfg = pg.grids.config_flocculation_adjoint(n_steps=10, switch_step=5)
        dx, dtq, dbw = (torch.tensor(cfg[k], **f64) for k in ("x", "t_q", "bw_q"))
        with pg.Rk4Tape(10, cfg["dt"], 5, cfg["agg_sets"], cfg["brk_sets"], cfg["step_set"]) as tape:
            N = torch.tensor(cfg["N0"], **f64)
            pg.check(tape.forward(N, dx, dtq, dbw), "tape forward")
            g = torch.zeros_like(N)
            ga, gb = torch.zeros(6, **f64), torch.zeros(8, **f64)
            pg.check(tape.backward(torch.tensor(cfg["lam_T"], **f64), g, ga, gb), "tape backward")
    else:
        raise SystemExit("unknown profile case %r" % name)
    torch.cuda.synchronize()


def reference_arm(args) -> None:
    """The reference's path on the host cores (oracle port, all threads)."""
    import pyoracle

    world = int(os.environ.get("WORLD_SIZE", "1"))
    if int(os.environ.get("RANK", "0")) != 0:
        return  # rank 0 alone runs the reference arm
    x, N, t_q, bw_q, ap, bp = workload()
    threads = os.cpu_count() or 1

    def step():
        pyoracle.aggregation_rhs_mt(N, x, ap.kernel_type, ap.beta0, ap.beta_br, ap.beta_sh,
                                    ap.log_x0, ap.inv_log_r, nthreads=threads)
        pyoracle.breakage_rhs(N, x, t_q, bw_q, bp.selection, bp.S0, bp.v_ref, bp.alpha, bp.v_min)

    warmup = max(args.warmup, 0)
    w0 = time.perf_counter()
    for _ in range(max(warmup, 1)):
        step()
    per = (time.perf_counter() - w0) / max(warmup, 1)
    # every requested step unless that would take more than about four minutes
    steps = int(min(args.steps, max(3, 240.0 / max(per, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    el = time.perf_counter() - t0
    value = steps / el
    sample = ("%d full n=16384 agg+brk RHS evaluations (%.1f s), oracle port with aggregation "
              "rows over %d host threads, breakage serial" % (steps, el, threads))
    out = {
        "metric": "Agg+br RHS evals/s at N=16384 FP64",
        "value": round(value, 4),
        "unit": "evals/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": max(warmup, 1),
        "ms_per_step": round(el / steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded lognormal N on the stated grid)",
        "config": run_config(),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "evals/s", "cores": threads,
                         "kind": "port", "sample": sample, "cpu_model": cpu_model()},
        "e2e": {"value": round(value, 4), "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_note": "the reference implements this path only in CUDA; the oracle port "
                          "restates its loops on the CPU (oracle/pbe_oracle.cpp)",
    }
    if steps != args.steps:
        out["steps_requested"] = args.steps
    print(json.dumps(out))


def reference_kernels_section(dev, stream, dN, dx, dt, db, rhs, ap, bp, flush, steps=20):
    """The reference's CUDA kernels (built unmodified from its sources into
    oracle/_ref, launched with its launch geometry) on the same GPU, step and
    timing as the main value (L2 flushed before each timed step)."""
    import torch

    import pbe_gb300 as pg
    import pyoracle

    try:
        ref = pyoracle.RefRunner()
    except (FileNotFoundError, OSError, RuntimeError) as exc:
        return {"unavailable": str(exc)}

    def step():
        rhs.zero_()
        pg.check(ref.aggregation_rhs(dN, dx, rhs, ap, stream), "reference aggregation")
        pg.check(ref.breakage_rhs(dN, dx, dt, db, rhs, bp, stream), "reference breakage")

    with torch.cuda.stream(stream):
        for _ in range(3):
            step()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    return {"evals_per_s": round(1e3 / ms, 3), "ms_per_eval": round(ms, 3), "steps": steps,
            "what": "acuoci/pbe-fixed-pivot-cuda src/aggregation.cu + src/breakage.cu, unmodified, "
                    "nvcc -O3 for sm_103a (oracle/build_ref.sh), its launch geometry, same GPU"}


def main():
    ap_ = argparse.ArgumentParser()
    ap_.add_argument("--profile-case", choices=["batched", "batched_small", "death", "adjoint",
                                                "vjp", "breakage", "lane"],
                     help="run a few launches of one kernel family (for ncu) and exit")
    ap_.add_argument("--gpus", type=int, default=1)
    ap_.add_argument("--steps", type=int, default=200)
    ap_.add_argument("--warmup", type=int, default=5)
    ap_.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap_.add_argument("--mode", choices=["gather", "scatter"], default="gather")
    ap_.add_argument("--no-cpu-baseline", action="store_true")
    ap_.add_argument("--no-extras", action="store_true",
                     help="skip the batched-cell and adjoint sections")
    ap_.add_argument("--sections-out", default="bench_sections.json",
                     help="file for the full per-section results (a summary stays in the line)")
    args = ap_.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.impl == "reference":
        reference_arm(args)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import pbe_gb300 as pg

    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    x, N, t_q, bw_q, ap, bp = workload()
    f64 = dict(dtype=torch.float64, device=dev)
    dN, dx = torch.tensor(N, **f64), torch.tensor(x, **f64)
    dt, db = torch.tensor(t_q, **f64), torch.tensor(bw_q, **f64)
    rhs = torch.zeros(N_BINS, **f64)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    hN = torch.tensor(N, dtype=torch.float64).pin_memory()
    hR = torch.empty(N_BINS, dtype=torch.float64).pin_memory()

    mode = pg.MODE_GATHER if args.mode == "gather" else pg.MODE_SCATTER

    def step(n_dev):
        rhs.zero_()
        pg.check(pg.aggregation_rhs(n_dev, dx, rhs, ap, stream=stream, mode=mode), "aggregation")
        pg.check(pg.breakage_rhs(n_dev, dx, dt, db, rhs, bp, stream=stream, mode=mode), "breakage")
    # our kernels per step: aggregation prep + pair kernel; breakage prep +
    # gather (gather mode) or one scatter kernel. (The aggregation call also
    # enqueues one 32-byte cudaMemsetAsync of its counters, not counted.)
    launches_per_step = 2 + (2 if mode == pg.MODE_GATHER else 1)

    clocks = ClockSampler(local)
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step(dN)
        stream.synchronize()
        clocks.start()
        time.sleep(0.3)

        # ---- value: device-resident inputs, L2 flushed before each step ----
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        main_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                    for _ in range(args.steps)]
        for a, b in main_evs:   # torch creates the CUDA events on first record
            a.record(stream)
            b.record(stream)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            pg.load().pbe_set_profile_events(main_evs[k][0].cuda_event, main_evs[k][1].cuda_event)
            evs[k][0].record(stream)
            step(dN)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        pg.load().pbe_set_profile_events(None, None)
        step_ms = [a.elapsed_time(b) for a, b in evs]
        total_ms = sum(step_ms)
        main_ms = [a.elapsed_time(b) for a, b in main_evs]

        # ---- e2e: host buffers through the C ABI, copies inside the timing ----
        e2e_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(args.steps)]
        dN2 = torch.empty_like(dN)
        for k in range(args.steps):
            flush.zero_()
            e2e_evs[k][0].record(stream)
            dN2.copy_(hN, non_blocking=True)
            step(dN2)
            hR.copy_(rhs, non_blocking=True)
            e2e_evs[k][1].record(stream)
        torch.cuda.synchronize()
        e2e_ms = sum(a.elapsed_time(b) for a, b in e2e_evs)

        # ---- adjoint: aggregation + breakage VJP of the same step ----------
        vjp_ms = None
        lam = torch.randn(N_BINS, dtype=torch.float64, device=dev,
                          generator=torch.Generator(device=dev).manual_seed(7))
        gN = torch.zeros(N_BINS, **f64)
        ga = torch.zeros(3, **f64)
        gb = torch.zeros(4, **f64)

        def vjp_step():
            gN.zero_()
            pg.check(pg.aggregation_rhs_vjp(dN, dx, lam, gN, ga, ap, stream=stream), "agg vjp")
            pg.check(pg.breakage_rhs_vjp(dN, dx, dt, db, lam, gN, gb, bp, stream=stream), "brk vjp")
        for _ in range(3):
            vjp_step()
        v_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(max(args.steps // 4, 5))]
        for a_, b_ in v_evs:
            flush.zero_()
            a_.record(stream)
            vjp_step()
            b_.record(stream)
        torch.cuda.synchronize()
        vjp_ms = sum(a_.elapsed_time(b_) for a_, b_ in v_evs) / len(v_evs)

        # ---- the other accumulation mode on the same step ------------------
        other = pg.MODE_SCATTER if mode == pg.MODE_GATHER else pg.MODE_GATHER

        def other_step():
            rhs.zero_()
            pg.check(pg.aggregation_rhs(dN, dx, rhs, ap, stream=stream, mode=other), "aggregation")
            pg.check(pg.breakage_rhs(dN, dx, dt, db, rhs, bp, stream=stream, mode=other), "breakage")
        for _ in range(3):
            other_step()
        o_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(max(args.steps // 4, 5))]
        for a_, b_ in o_evs:
            flush.zero_()
            a_.record(stream)
            other_step()
            b_.record(stream)
        torch.cuda.synchronize()
        other_ms = sum(a_.elapsed_time(b_) for a_, b_ in o_evs) / len(o_evs)
        time.sleep(0.2)
        clk = clocks.stop()

    if dist is not None:
        t = torch.tensor([total_ms, e2e_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_ms = float(t[0]), float(t[1])
    n_gpus = world if dist is not None else 1
    value = n_gpus * args.steps / (total_ms / 1e3)
    e2e_value = n_gpus * args.steps / (e2e_ms / 1e3)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    peak = fp64_peak_tflops(stream)
    mk = statistics.mean(main_ms) * 1e-3 if main_ms else None
    instr = lane_fp64_instr_per_launch(x)
    # FP64 pipe: every FP64 instruction (DFMA, DMUL, DADD) takes one issue slot
    # of the pipe per thread; the DFMA-chain probe runs it at peak/2 slots per
    # second (2 flops per DFMA).
    slots_peak = peak / 2.0 if peak else None                # T FP64 instructions/s
    achieved = instr / mk / 1e12 if mk else None
    ref_equiv = FLOPS_PER_PAIR * PAIRS / mk / 1e12 if mk else None
    roofline = {
        "bound": "fp64",
        "kernel": "agg_lane_kernel<5> (+ agg_main_kernel<5>, which returns at once on this grid)",
        "achieved": round(achieved, 4) if achieved else None,
        "peak": round(slots_peak, 4) if slots_peak else None,
        "unit": "T FP64 instr/s",
        "frac": round(achieved / slots_peak, 4) if (achieved and slots_peak) else None,
        "traffic": MAIN_KERNEL_DRAM_BYTES,
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of "
                          "this workload after an L2 flush, captured apart from this run",
        "algo_bytes": ALGO_BYTES_PER_LAUNCH,
        "kernel_ms": round(mk * 1e3, 5) if mk else None,
        "fp64_instr_per_launch": instr,
        "fp64_instr_source": "instruction model of the lane-block kernel on this grid",
        "peak_source": "DFMA-chain probe timed in this run (libpbe_probe.so), of measured; "
                       "MEASURED_PEAKS.json has no FP64 entry",
        "reference_equivalent_tflops": round(ref_equiv, 4) if ref_equiv else None,
        "reference_equivalent_frac": round(ref_equiv / peak, 4) if (ref_equiv and peak) else None,
        "reference_equivalent_unit": "22 FP64 flops per pair interaction (the reference's "
                                     "formula) per s, over the DFMA peak in TFLOP/s",
    }
    out = {
        "metric": "Agg+br RHS evals/s at N=16384 FP64",
        "value": round(value, 3),
        "unit": "evals/s",
        "n_gpus": n_gpus,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": round(total_ms / args.steps, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded lognormal N on the stated grid)",
        "config": run_config(),
        "mode": args.mode,
        "e2e": {"value": round(e2e_value, 3), "unit": "evals/s",
                "h2d_bytes_per_step": N_BINS * 8, "d2h_bytes_per_step": N_BINS * 8},
        "gpu_launches": launches_per_step * args.steps,
        "memsets_per_step": 1,
        "clocks": clk,
        "roofline": roofline,
        "pair_interactions_per_s": round(value * PAIRS, 1),
        "fragments_per_s": round(value * N_BINS * N_QUAD, 1),
        "wall_s_timed_loop": round(wall, 4),
    }
    sections = {}
    if vjp_ms is not None:
        sections["other_mode"] = {"mode": "scatter" if other == pg.MODE_SCATTER else "gather",
                                  "evals_per_s": round(1e3 / other_ms, 3),
                                  "ms_per_step": round(other_ms, 5),
                                  "what": "the same step in the other accumulation mode, "
                                          "device-resident, L2 flushed"}
        vjp_instr = vjp_lane_fp64_instr(x)
        vjp_ach = vjp_instr / (vjp_ms * 1e-3) / 1e12
        vjp_frac = round(vjp_ach / slots_peak, 4) if slots_peak else None
        sections["vjp"] = {"ms_per_eval": round(vjp_ms, 5),
                           "vjp_rhs_ratio": round(vjp_ms / (total_ms / args.steps), 4),
                           "roofline": {"bound": "fp64", "kernel": "vjp_lane_kernel<5>",
                                        "achieved": round(vjp_ach, 4),
                                        "peak": round(slots_peak, 4) if slots_peak else None,
                                        "unit": "T FP64 instr/s",
                                        "frac": vjp_frac,
                                        "fp64_instr_per_eval": vjp_instr,
                                        "time": "the whole aggregation + breakage VJP step "
                                                "(the pair kernel is ~93 % of it)"},
                           "what": "aggregation + breakage VJP (dL/dN and parameter gradients) "
                                   "of the same n=16384 step, device-resident, L2 flushed"}
    if n_gpus == 1 and not args.no_extras:
        rk = reference_kernels_section(dev, stream, dN, dx, dt, db, rhs, ap, bp, flush)
        if "evals_per_s" in rk:
            rk["speedup_of_value"] = round(value / rk["evals_per_s"], 2)
        sections["reference_kernels_sm103a"] = rk
        sections["batched"] = batched_section(dev, stream)
        sections["adjoint"] = adjoint_section(dev, stream)
        sections["classes"] = classes_section(dev, stream)
    if n_gpus == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(x, N, t_q, bw_q, ap, bp)
    # the full sections go to a file (and stderr); the JSON line keeps a short
    # summary of each so the headline figures stay in the line's tail
    if sections:
        path = args.sections_out
        try:
            with open(path, "w") as f:
                json.dump(sections, f, indent=1)
            out["sections_file"] = path
        except OSError as exc:
            out["sections_file"] = "not written: %s" % exc
        print(json.dumps({"bench_sections": sections}), file=sys.stderr)
        out["summary"] = summarize(sections, value)
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
