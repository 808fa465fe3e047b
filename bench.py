#!/usr/bin/env python3
"""Benchmark of the GB300 Ewald-split boundary-integral matvec.

Metric: Ewald matvec targets/s.  One step = one full matvec of AddIntOnRbcs
(real-space Stokeslet + stresslet pair sums with the same-cell mask, FP64
self and near-singular polar-patch corrections, linear term) plus
PME_Distrib_Source / PME_Transform / PME_Add_Interp_Vel, evaluated at every
cell surface point (c1 = c2 = 1/(4 pi), as CalcVelocityField), on the
256-cell periodic workload: L = 40, 25x50 surface grid per cell (320,000
targets), alpha = 1.5757 (rc = 3), PME mesh 128^3, B-spline order 6,
viscosity ratio 5.  Inputs are seeded synthetic cells (biconcave shape,
random placement and rotation, SH densities), generated identically for the
GPU and the CPU oracle.

  value  -- FP32-compensated matvec with every input resident in HBM.
  e2e    -- the same matvec through the C ABI with host buffers: upload of
            geometry, densities and spline tables from pinned memory, and the
            download of the velocities, inside the timed region.

`python bench.py --impl reference` times the CPU oracle (FP64 restatement
of the reference path, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

if int(os.environ.get("WORLD_SIZE", "1")) > 1 and "LOCAL_RANK" in os.environ:
    # one process per GPU: each rank sees only its own device
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

# Algorithmic flops per unit of work (plain arithmetic of the reference
# formulas; add/sub/mul/div/sqrt = 1 flop, FMA = 2 flops):
FLOP_PAIR_SL = 39   # EwaldCoeff_SL lerp + Stokeslet term, ModIntOnRbcs.F90:91-97
FLOP_PAIR_DL = 27   # EwaldCoeff_DL lerp + stresslet term, ModIntOnRbcs.F90:99-106
FLOP_SELFQ_SL = 294  # one RBC_SingInt patch point, SL: 2 bicubic 3-var interps + kernel
FLOP_SELFQ_SLDL = 550  # one patch point, SL+DL: 4 bicubic 3-var interps + both kernels

WORKLOAD = {
    "workload": "Ewald-split SL+DL matvec, 256 biconcave cells, 25x50 grid (320000 targets), "
                "periodic L=40, rc=3 (alpha=1.5757), PME 128^3 P=6, viscRat=5",
    "config": "C2",
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.p = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for i, n in enumerate(names):
                    if r[5 + i].strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def make_inputs(seed, ncell=None):
    from rbc3d_gb300 import geometry as G
    prm, cells, _ = G.config("C2", seed=seed, ncell=ncell)
    if ncell:  # same cell density as the 256-cell box (profiling runs)
        prm["Lb"] = [40.0 * (ncell / 256.0) ** (1 / 3)] * 3
        prm, cells, _ = G.config("C2", seed=seed, ncell=ncell, L=prm["Lb"][0])
    return prm, cells


def oracle_lib():
    from rbc3d_gb300.abi import Library
    path = os.path.join(HERE, "oracle", "liboracle_rbc3d.so")
    if not os.path.exists(path):
        subprocess.run(["make", "-C", os.path.join(HERE, "oracle"), "-s"], check=True)
    return Library(path, "rbc3d_oracle_")


def time_oracle(prm, cells, steps, threads=None):
    """Full FP64 CPU matvec (oracle) on the host cores; returns (s per step, cores)."""
    import ctypes
    from rbc3d_gb300.abi import Context, TLIST_RBC, TERM_ALL
    L = oracle_lib()
    cores = os.cpu_count() or 1
    setn = getattr(L.lib, "rbc3d_oracle_set_threads")
    setn.restype = ctypes.c_int
    setn.argtypes = [ctypes.c_int]
    used = setn(threads or cores)
    ctx = Context(L, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    c = 1.0 / (4 * math.pi)
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ctx.matvec(TLIST_RBC, c, c, TERM_ALL)
        ts.append(time.perf_counter() - t0)
    ctx.close()
    return ts, used


def run_reference(args, dist):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    prm, cells = make_inputs(args.seed)
    N = cells.x.shape[1]
    ts, cores = time_oracle(prm, cells, args.warmup + args.steps)
    t = sum(ts[args.warmup:]) / max(args.steps, 1)
    val = N / t
    line = {"impl": "reference", "metric": "Ewald matvec targets/s", "value": val, "unit": "targets/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": WORKLOAD,
            "cpu_baseline": {"value": val, "unit": "targets/s", "cores": cores, "kind": "port",
                             "sample": f"full matvec, {N} targets, {args.steps} timed steps"},
            "e2e": {"value": val, "unit": "targets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    ap.add_argument("--cells", type=int, default=None, help="smaller workload (profiling)")
    ap.add_argument("--quick", action="store_true", help="one mode's matvec timing only (profiling)")
    ap.add_argument("--quick-prec", choices=("fp32c", "fp32m", "fp32d"), default="fp32d",
                    help="the mode --quick times (profiling)")
    ap.add_argument("--no-wall", action="store_true", help="skip the learned-guess wall GMRES comparison")
    ap.add_argument("--no-scaleup", action="store_true", help="skip the 2048-cell (PME 256^3) scale-up line")
    ap.add_argument("--no-cellsolve", action="store_true", help="skip the cell velocity GMRES line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist = dist_init()
    if args.impl == "reference":
        return run_reference(args, dist)

    rank = int(os.environ.get("RANK", "0"))
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    from rbc3d_gb300 import build as B
    B.build()
    from rbc3d_gb300 import library
    from rbc3d_gb300.abi import (FP32C, FP32D, FP32M, FP64, STAGES, TERM_ALL, TERM_CORR, TERM_LINEAR, TERM_PME, TERM_REAL,
                                 TLIST_RBC, Context)

    t0 = time.perf_counter()
    prm, cells = make_inputs(args.seed + rank, args.cells)
    log(f"inputs generated in {time.perf_counter() - t0:.1f}s")
    N = cells.x.shape[1]
    lib = library()
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    c = 1.0 / (4 * math.pi)

    def step(prec):
        ctx.matvec(TLIST_RBC, c, c, TERM_ALL, prec, device_only=True)

    # ---- FP32-compensated matvec, inputs resident in HBM
    head = {"fp32m": FP32M, "fp32c": FP32C}.get(args.quick_prec, FP32D) if args.quick else FP32D
    for _ in range(args.warmup):
        step(head)
    counts = ctx.counts()
    l0 = counts["kernel_launches"]
    clk = Clocks()
    barrier(dist)
    clk.start()
    ctx.set_profiling(1)
    ctx.timer_start()
    for _ in range(args.steps):
        step(head)
    ms = ctx.timer_stop()
    clocks = clk.stop()
    stages = ctx.stage_times()
    ctx.set_profiling(0)
    counts = ctx.counts()
    launches = counts["kernel_launches"] - l0
    ms = dist_max(dist, ms)
    ms_step = ms / args.steps
    value = ws * N / (ms_step * 1e-3)

    if args.quick:
        if rank == 0:
            print(json.dumps({"quick": True, "mode": args.quick_prec, "ms_per_step": ms_step, "targets": N, "value": value,
                              "stages_ms_per_step": {k: v[0] / args.steps for k, v in stages.items()},
                              "gpu_launches": launches}), flush=True)
        ctx.close()
        return 0

    # ---- FP64 plain form (same algorithm, everything FP64)
    for _ in range(2):
        step(FP64)
    k64 = max(2, args.steps // 3)
    ctx.set_profiling(1)
    ctx.timer_start()
    for _ in range(k64):
        step(FP64)
    ms64 = dist_max(dist, ctx.timer_stop()) / k64
    st64 = {k: v[0] / k64 for k, v in ctx.stage_times().items()}
    ctx.set_profiling(0)

    # ---- FP32M: FP32C with the own-cell polar patch in FP32 + hi/lo geometry
    for _ in range(2):
        step(FP32M)
    ctx.set_profiling(1)
    ctx.timer_start()
    for _ in range(args.steps):
        step(FP32M)
    msm = dist_max(dist, ctx.timer_stop()) / args.steps
    stm = {k: v[0] / args.steps for k, v in ctx.stage_times().items()}
    ctx.set_profiling(0)
    fp32m_value = ws * N / (msm * 1e-3)

    # ---- FP32C: the own-cell polar patch on the FP64 pipe
    for _ in range(2):
        step(FP32C)
    ctx.set_profiling(1)
    ctx.timer_start()
    for _ in range(args.steps):
        step(FP32C)
    msc = dist_max(dist, ctx.timer_stop()) / args.steps
    stc = {k: v[0] / args.steps for k, v in ctx.stage_times().items()}
    ctx.set_profiling(0)
    fp32c_value = ws * N / (msc * 1e-3)
    # the patch corrections alone (self + near-singular; the near pass is the
    # same FP64 code in both modes): float-float patch against the FP64 patch
    corr_c = ctx.matvec(TLIST_RBC, c, c, TERM_CORR, FP32C)
    corr_d = ctx.matvec(TLIST_RBC, c, c, TERM_CORR, FP32D)
    self_ff_vs_fp64 = float(np.linalg.norm(corr_d - corr_c) / np.linalg.norm(corr_c))

    # ---- relative L2 error of the FP32 modes against the FP64 plain form
    v64 = ctx.matvec(TLIST_RBC, c, c, TERM_ALL, FP64)
    err32c = float(np.linalg.norm(ctx.matvec(TLIST_RBC, c, c, TERM_ALL, FP32C) - v64) / np.linalg.norm(v64))
    err32m = float(np.linalg.norm(ctx.matvec(TLIST_RBC, c, c, TERM_ALL, FP32M) - v64) / np.linalg.norm(v64))
    err32d = float(np.linalg.norm(ctx.matvec(TLIST_RBC, c, c, TERM_ALL, FP32D) - v64) / np.linalg.norm(v64))
    fp64_value = ws * N / (ms64 * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers
    pin = {}
    for k in ("x", "a3", "detJ", "area", "meshSize", "spl_x", "spl_a3", "spl_detJ", "f", "g", "spl_F", "spl_G"):
        a = np.ascontiguousarray(getattr(cells, k), dtype=np.float64)
        p = lib.pinned(a.shape)
        p[...] = a
        pin[k] = p
    vout = lib.pinned((3, N))

    class PinnedCells:
        pass

    pc = PinnedCells()
    for k in ("nlat", "nlon", "th", "phi", "w", "ncell", "celltype"):
        setattr(pc, k, getattr(cells, k))
    for k, p in pin.items():
        setattr(pc, k, p)
    # the caller's accumulator goes up and down (v += result on the device)
    h2d = sum(p.nbytes for p in pin.values()) + vout.nbytes
    d2h = vout.nbytes

    e2e_parts = {"set_cells": 0.0, "set_cell_density": 0.0, "matvec_with_download": 0.0}

    def e2e_step():
        t0 = time.perf_counter()
        ctx.set_cells(pc)
        t1 = time.perf_counter()
        ctx.set_cell_density(f=pc.f, g=pc.g, spl_F=pc.spl_F, spl_G=pc.spl_G)
        t2 = time.perf_counter()
        vout[...] = 0.0
        ctx.matvec(TLIST_RBC, c, c, TERM_ALL, FP32D, v=vout)
        t3 = time.perf_counter()
        e2e_parts["set_cells"] += t1 - t0
        e2e_parts["set_cell_density"] += t2 - t1
        e2e_parts["matvec_with_download"] += t3 - t2

    for _ in range(2):
        e2e_step()
    for k in e2e_parts:
        e2e_parts[k] = 0.0
    barrier(dist)
    te = time.perf_counter()
    ke = max(3, args.steps // 2)
    for _ in range(ke):
        e2e_step()
    te = dist_max(dist, (time.perf_counter() - te) / ke)
    e2e_value = ws * N / te
    e2e_parts = {k: v / ke * 1e3 for k, v in e2e_parts.items()}
    h2d_gbs = lib.h2d_bandwidth(h2d)  # one pinned copy of the step's upload volume

    # ---- roofline of the dominant stage (device time measured above)
    nq = 200  # RBC_SingInt points per target on the 25x50 grid (nrad 10 x nazm 20)
    peak32 = lib.fma_peak(FP32C)
    peak64 = lib.fma_peak(FP64)
    st_ms = {k: v[0] / args.steps for k, v in stages.items()}
    pairs = counts["pairs_within_rc"]
    # k_self_ff loads per patch point 4 stencil nodes x 4 slots x 6 float4
    # quads of hi/lo values and 9 weight words (136 B); the L1 load peak is
    # 128 B/clk/SM (nominal; no measured L1 figure exists)
    l1_bytes = counts["self_items"] * nq * (4 * 4 * 6 * 16 + 136)
    l1_peak = 128.0 * 152 * ((clocks or {}).get("sm_mhz") or 2070.0) * 1e6 / 1e9
    # ---- per-kernel rooflines with the stages timed alone on one stream
    # (REAL|CORR|LINEAR without PME keeps the matvec on the main stream)
    def alone(prec, terms, reps=3):
        ctx.matvec(TLIST_RBC, c, c, terms, prec, device_only=True)
        ctx.set_profiling(1)
        for _ in range(reps):
            ctx.matvec(TLIST_RBC, c, c, terms, prec, device_only=True)
        st = ctx.stage_times()
        ctx.set_profiling(0)
        return {k: v[0] / reps for k, v in st.items()}

    hbm_peak, hbm_src = 6800.0, "fallback"
    try:
        mp = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
        hbm_peak, hbm_src = float(mp["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except Exception:
        pass
    s_c = alone(FP32C, TERM_REAL | TERM_CORR | TERM_LINEAR)
    s_m = alone(FP32M, TERM_REAL | TERM_CORR | TERM_LINEAR)
    s_d = alone(FP32D, TERM_REAL | TERM_CORR | TERM_LINEAR)
    s_p = alone(FP32C, TERM_PME)
    G3 = 1
    for d in prm["Nb"]:
        G3 *= d
    pme_ms = s_p["pme_spread"] + s_p["pme_fft_infl"] + s_p["pme_gather"]
    pme_bytes = 4.0 * G3 * (12 + 12 + 12 + 12 + 3 + 3 + 3 + 3) + 4.0 * N * (3 + 3 + 3 + 1) + 4.0 * N * (3 + 3)
    pair_fl = pairs * (FLOP_PAIR_SL + FLOP_PAIR_DL)
    self_fl = counts["self_items"] * nq * FLOP_SELFQ_SLDL
    rooflines = {
        "k_pair32": {"bound": "fp32", "ms": s_c["pair"], "achieved": pair_fl / (s_c["pair"] * 1e-3) / 1e12,
                     "peak": peak32, "unit": "TFLOP/s", "frac": pair_fl / (s_c["pair"] * 1e-3) / 1e12 / peak32,
                     "work": f"{pairs} pairs within rc x {FLOP_PAIR_SL + FLOP_PAIR_DL} flops"},
        "k_self": {"bound": "fp64", "ms": s_c["self"], "achieved": self_fl / (s_c["self"] * 1e-3) / 1e12,
                   "peak": peak64, "unit": "TFLOP/s", "frac": self_fl / (s_c["self"] * 1e-3) / 1e12 / peak64,
                   "work": f"{counts['self_items']} targets x {nq} patch points x {FLOP_SELFQ_SLDL} flops"},
        "k_self_mix": {"bound": "l1 (ncu: L1 91% of peak)", "ms": s_m["self"],
                       "achieved": self_fl / (s_m["self"] * 1e-3) / 1e12, "peak": peak32, "unit": "TFLOP/s",
                       "frac": self_fl / (s_m["self"] * 1e-3) / 1e12 / peak32,
                       "work": "the k_self patch work in FP32 with hi/lo geometry"},
        "k_self_ff": {"bound": "l1", "ms": s_d["self"], "achieved": l1_bytes / (s_d["self"] * 1e-3) / 1e9,
                      "peak": l1_peak, "unit": "GB/s", "frac": l1_bytes / (s_d["self"] * 1e-3) / 1e9 / l1_peak,
                      "flops_achieved_tflops": self_fl / (s_d["self"] * 1e-3) / 1e12,
                      "work": "L1 bytes requested by the lanes (the k_self patch work in float-float arithmetic)"},
        "pme": {"bound": "hbm", "ms": pme_ms, "achieved": pme_bytes / (pme_ms * 1e-3) / 1e9, "peak": hbm_peak,
                "unit": "GB/s", "frac": pme_bytes / (pme_ms * 1e-3) / 1e9 / hbm_peak, "peak_source": hbm_src,
                "work": "algorithmic bytes 4 G (12+12+12+12+3+3+3+3) + 4 N (3+3+3+1) + 4 N (3+3), FP32 grids "
                        "(a 128^3 grid set stays largely in the 129 MB L2)"},
        "note": "stages timed alone on one stream (the matvec itself runs them on two streams)",
    }
    # ---- the dominant kernel of the headline mode, from the stages timed alone
    # (the matvec's stage spans overlap across the two streams)
    if s_d["self"] >= s_d["pair"]:
        roof = {"kernel": "k_self_ff (RBC_SingInt, float-float)", **rooflines["k_self_ff"],
                "peak_source": "nominal L1 load bandwidth 128 B/clk/SM x 152 SMs x the sampled SM clock "
                               "(ncu: L1 data pipe 78% of its wavefront peak, FMA pipe 65%)"}
    else:
        roof = {"kernel": "k_pair32 (AddIntOnRbcs pair sums, FP32)", **rooflines["k_pair32"],
                "peak_source": "measured FP32 FMA chain (rbc3d_fma_peak), same GPU, same run"}
    roof["traffic"] = None
    tpath = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            tr = json.load(open(tpath))
            roof["traffic"] = tr.get(roof["kernel"].split()[0])
        except Exception:
            pass

    # ---- scale-up: 2048 cells, L = 80, PME 256^3 (2.56 M targets), all three modes
    scale = None
    if not args.quick and not args.no_scaleup:
        from rbc3d_gb300 import geometry as G
        t1 = time.perf_counter()
        prm5, cells5, _ = G.config("C5", seed=args.seed + rank)
        N5 = cells5.x.shape[1]
        ctx5 = Context(lib, prm5)
        ctx5.set_cells(cells5)
        ctx5.set_cell_density(f=cells5.f, g=cells5.g, spl_F=cells5.spl_F, spl_G=cells5.spl_G)

        def timed(prec, warm, steps):
            for _ in range(warm):
                ctx5.matvec(TLIST_RBC, c, c, TERM_ALL, prec, device_only=True)
            ctx5.timer_start()
            for _ in range(steps):
                ctx5.matvec(TLIST_RBC, c, c, TERM_ALL, prec, device_only=True)
            return dist_max(dist, ctx5.timer_stop()) / steps

        m32c = timed(FP32C, 2, 3)
        m32m = timed(FP32M, 2, 3)
        m32d = timed(FP32D, 2, 3)
        m64 = timed(FP64, 1, 1)
        v64 = ctx5.matvec(TLIST_RBC, c, c, TERM_ALL, FP64)
        e32c = float(np.linalg.norm(ctx5.matvec(TLIST_RBC, c, c, TERM_ALL, FP32C) - v64) / np.linalg.norm(v64))
        e32m = float(np.linalg.norm(ctx5.matvec(TLIST_RBC, c, c, TERM_ALL, FP32M) - v64) / np.linalg.norm(v64))
        e32d = float(np.linalg.norm(ctx5.matvec(TLIST_RBC, c, c, TERM_ALL, FP32D) - v64) / np.linalg.norm(v64))
        cnt5 = ctx5.counts()
        ctx5.close()
        log(f"scale-up in {time.perf_counter() - t1:.1f}s")
        scale = {"workload": "2048 biconcave cells, 25x50 grid (2,560,000 targets), periodic L=80, rc=3, "
                             "PME 256^3 P=6, SL+DL, viscRat=5 (C5)",
                 "targets": N5,
                 "fp32c": {"ms_per_step": m32c, "value": ws * N5 / (m32c * 1e-3), "rel_l2_vs_fp64_plain": e32c},
                 "fp32m": {"ms_per_step": m32m, "value": ws * N5 / (m32m * 1e-3), "rel_l2_vs_fp64_plain": e32m},
                 "fp32d": {"ms_per_step": m32d, "value": ws * N5 / (m32d * 1e-3), "rel_l2_vs_fp64_plain": e32d},
                 "fp64_plain": {"ms_per_step": m64, "value": ws * N5 / (m64 * 1e-3)},
                 "fp32c_over_fp64": m64 / m32c, "fp32m_over_fp64": m64 / m32m, "fp32d_over_fp64": m64 / m32d,
                 "pairs_within_rc": cnt5["pairs_within_rc"], "nearsing_items": cnt5["nearsing_items"],
                 "steps": "fp32c, fp32m, fp32d: 2 warm-up + 3 timed; fp64: 1 + 1"}

    # ---- wall no-slip GMRES on the tube workload: plain vs history vs learned guess
    wall = None
    if not args.quick and not args.no_wall:
        from rbc3d_gb300.learned_run import run as wall_run
        t1 = time.perf_counter()
        w = wall_run(ncell=64, warm_steps=25, test_steps=3, rtol=1e-8, restart=300, max_it=900, train_iters=30,
                     history=48, seed=args.seed + rank, dynamics="skalak", dt=1e-3)
        log(f"wall GMRES comparison in {time.perf_counter() - t1:.1f}s")
        wall = {"workload": "C3 tube (R=8, L=48, 64 cells) under RK2 membrane dynamics (Skalak ES 1, ED 50, "
                            "bending 5.4e-3, intra-cell repulsion 0.81, dt 1e-3), NoSlipWall after each RK2 "
                            "stage; FP64 matvec + FP64 Arnoldi, ||r|| < 1e-8 ||b||",
                **{k: w[k] for k in ("wall_dof", "restart", "history", "plain", "history_only", "learned",
                                     "speedup_learned", "speedup_history_only", "train_ms_per_step",
                                     "speedup_learned_incl_training", "mlp")},
                "steps": "25 warm-up RK2 steps (50 plain solves: history + online training), then 3 steps "
                         "(6 solves) each solved plain, from the history guess and from the learned guess"}
        # the same run with mixed-precision solves (FP32M operator inside FP64 refinement, FP64 residual)
        t1 = time.perf_counter()
        wm = wall_run(ncell=64, warm_steps=25, test_steps=3, rtol=1e-8, restart=300, max_it=900, train_iters=30,
                      history=48, seed=args.seed + rank, prec=FP32M, dynamics="skalak", dt=1e-3)
        log(f"mixed-precision wall GMRES comparison in {time.perf_counter() - t1:.1f}s")
        wall["mixed_fp32m"] = {k: wm[k] for k in ("plain", "history_only", "learned", "speedup_learned",
                                                  "speedup_history_only", "speedup_learned_incl_training")}
        wall["mixed_fp32m"]["learned_over_fp64_plain"] = w["plain"]["ms"] / wm["learned"]["ms"]

    # ---- cell velocity GMRES (Solve_RBC_Vel, degree 12, rtol 1e-11 as the reference
    # sets it) on the same 256 cells: FP64 solve vs the mixed-precision solves
    cellsolve = None
    if not args.quick and not args.no_cellsolve:
        t1 = time.perf_counter()
        arms = {}
        for name, p in (("fp64", FP64), ("fp32d", FP32D), ("fp32m", FP32M), ("fp32c", FP32C)):
            sol, v, st, code = ctx.solve_rbc_vel(12, rtol=1e-11, max_it=300, restart=30, prec=p, check=False)
            arms[name] = (sol, v, st, code)
        s64, v64 = arms["fp64"][0], arms["fp64"][1]
        cellsolve = {"workload": "Solve_RBC_Vel on the 256-cell workload (viscRat 5, SH degree 12, "
                                 f"{3 * 144 * 256} unknowns), restart 30, ||r|| < 1e-11 ||b|| (FP64 residual)"}
        for name, (sol, v, st, code) in arms.items():
            cellsolve[name] = {"ms": st.ms, "iterations": st.iterations, "matvecs": st.matvecs,
                               "refinements": st.refinements, "status": code,
                               "final_rel_residual": st.rnorm / st.bnorm if st.bnorm > 0 else 0.0,
                               "rel_l2_vs_fp64_solution": float(np.linalg.norm(sol - s64) / np.linalg.norm(s64)),
                               "rel_l2_vs_fp64_velocity": float(np.linalg.norm(v - v64) / np.linalg.norm(v64))}
        for name in ("fp32d", "fp32m", "fp32c"):
            cellsolve[name]["speedup_vs_fp64"] = arms["fp64"][2].ms / arms[name][2].ms
        log(f"cell solve comparison in {time.perf_counter() - t1:.1f}s")

    # ---- CPU baseline (rank 0, N = 1 only): oracle, all host threads
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        try:
            ts, cores = time_oracle(prm, cells, 1)
            cpu = {"value": N / ts[0], "unit": "targets/s", "cores": cores, "kind": "port",
                   "sample": f"one full FP64 matvec of the same workload ({N} targets), {ts[0]:.1f}s"}
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": "targets/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"unavailable: {e}"}

    if rank == 0:
        line = {
            "metric": "Ewald matvec targets/s", "value": value, "unit": "targets/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+ff48-patch+f64-near",
            "data": "synthetic (seeded biconcave cells, SH densities)",
            "config": dict(WORKLOAD, targets=N, l2="working set (spline tables 307 MB, PME grids) > 129 MB L2"),
            "mode": "FP32D: pair sums, PME in FP32 with compensated accumulation; own-cell polar patch in "
                    "float-float arithmetic (48-bit significands, 2e-12 from the FP64 patch); near-singular "
                    "correction in FP64",
            "rel_l2_vs_fp64_plain": err32d,
            "patch_corrections_rel_l2_vs_fp64_patch": self_ff_vs_fp64,
            "fp64_plain": {"value": fp64_value, "unit": "targets/s", "ms_per_step": ms64,
                           "fp32d_over_fp64": value / fp64_value, "stages_ms_per_step": st64},
            "fp32c": {"value": fp32c_value, "unit": "targets/s", "ms_per_step": msc,
                      "over_fp64": fp32c_value / fp64_value, "rel_l2_vs_fp64_plain": err32c,
                      "stages_ms_per_step": stc,
                      "note": "own-cell polar patch on the FP64 pipe"},
            "fp32m": {"value": fp32m_value, "unit": "targets/s", "ms_per_step": msm,
                      "over_fp64": fp32m_value / fp64_value, "rel_l2_vs_fp64_plain": err32m,
                      "stages_ms_per_step": stm,
                      "note": "own-cell polar patch in FP32 with FP64-accurate (hi/lo) geometry"},
            "e2e": {"value": e2e_value, "unit": "targets/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": te * 1e3, "host_ms_per_step": e2e_parts,
                    "h2d_gbs_measured": h2d_gbs,
                    "floor_ms": ms_step + h2d / (h2d_gbs * 1e9) * 1e3,
                    "floor": "device matvec + the step's uploads at the measured pinned copy bandwidth"},
            "stages_ms_per_step": st_ms,
            "counts": {k: counts[k] for k in ("pairs_within_rc", "nbr_items", "nearsing_items", "self_items",
                                              "screen_misses", "near_replays", "near_projections")},
            "roofline": roof,
            "rooflines": rooflines,
            "fp32_over_fp64_plain": {"fp32d": value / fp64_value, "fp32c": fp32c_value / fp64_value,
                                     "fp32m": fp32m_value / fp64_value, "target": 20.0,
                                     "note": "fp32d: self patch in float-float on the FP32 pipe (GB300 FP64 is "
                                             "1/74 of FP32); fp32c: on the FP64 pipe; fp32m: in FP32 with hi/lo "
                                             "geometry"},
            "scaleup_c5": scale,
            "wall_gmres": wall,
            "cell_gmres": cellsolve,
            "fma_peaks_tflops": {"fp32": peak32, "fp64": peak64},
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
