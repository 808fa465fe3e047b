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

WORKLOADS = {
    "C2": {"workload": "Ewald-split SL+DL matvec, 256 biconcave cells, 25x50 grid (320000 targets), "
                       "periodic L=40, rc=3 (alpha=1.5757), PME 128^3 P=6, viscRat=5",
           "config": "C2", "targets": 320000,
           "l2": "inputs larger than L2: spline tables 307 MB + PME grids, > 129 MB L2"},
    "C5": {"workload": "Ewald-split SL+DL matvec, 2048 biconcave cells, 25x50 grid (2560000 targets), "
                       "periodic L=80, rc=3 (alpha=1.5757), PME 256^3 P=6, viscRat=5",
           "config": "C5", "targets": 2560000,
           "l2": "inputs larger than L2: spline tables 2.5 GB + PME grids, > 129 MB L2"},
}
WORKLOAD = WORKLOADS["C2"]
NQ = 200  # RBC_SingInt points per target on the 25x50 grid (nrad 10 x nazm 20)


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


def make_inputs(seed, ncell=None, name="C2"):
    from rbc3d_gb300 import geometry as G
    prm, cells, _ = G.config(name, seed=seed, ncell=ncell)
    if ncell:  # same cell density as the 256-cell box (profiling runs)
        prm["Lb"] = [40.0 * (ncell / 256.0) ** (1 / 3)] * 3
        prm, cells, _ = G.config(name, seed=seed, ncell=ncell, L=prm["Lb"][0])
    return prm, cells


def oracle_lib():
    from rbc3d_gb300.abi import Library
    path = os.path.join(HERE, "oracle", "liboracle_rbc3d.so")
    if not os.path.exists(path):
        subprocess.run(["make", "-C", os.path.join(HERE, "oracle"), "-s"], check=True)
    return Library(path, "rbc3d_oracle_")


def time_oracle(prm, cells, steps, threads=None):
    """Full FP64 CPU matvec (oracle) on the host cores: (seconds per step,
    cores used, the velocity vector of the last step)."""
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
    ts, v = [], None
    for _ in range(steps):
        t0 = time.perf_counter()
        v = ctx.matvec(TLIST_RBC, c, c, TERM_ALL)
        ts.append(time.perf_counter() - t0)
    ctx.close()
    return ts, used, v


def run_reference(args, dist):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    prm, cells = make_inputs(args.seed)
    N = cells.x.shape[1]
    ts, cores, _ = time_oracle(prm, cells, args.warmup + args.steps)
    t = sum(ts[args.warmup:]) / max(args.steps, 1)
    val = N / t
    line = {"impl": "reference", "metric": "Ewald matvec targets/s", "value": val, "unit": "targets/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded biconcave cells, SH densities)", "config": WORKLOAD,
            "cpu_baseline": {"value": val, "unit": "targets/s", "cores": cores, "kind": "port",
                             "sample": f"full matvec, {N} targets, {args.steps} timed steps"},
            "e2e": {"value": val, "unit": "targets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


class Bench:
    """Timings of one workload on one context (all modes share the context)."""

    def __init__(self, lib, prm, cells, dist, ws):
        from rbc3d_gb300.abi import Context
        self.lib, self.prm, self.cells, self.dist, self.ws = lib, prm, cells, dist, ws
        self.N = cells.x.shape[1]
        self.ctx = Context(lib, prm)
        self.ctx.set_cells(cells)
        self.ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
        self.c = 1.0 / (4 * math.pi)

    def step(self, prec, terms=None):
        from rbc3d_gb300.abi import TERM_ALL, TLIST_RBC
        self.ctx.matvec(TLIST_RBC, self.c, self.c, TERM_ALL if terms is None else terms, prec, device_only=True)

    def timed(self, prec, warm, steps, clocks=None):
        """(ms per step, max over ranks; stage ms per step; kernel launches; clocks)."""
        for _ in range(warm):
            self.step(prec)
        l0 = self.ctx.counts()["kernel_launches"]
        barrier(self.dist)
        if clocks:
            clocks.start()
        self.ctx.set_profiling(1)
        self.ctx.timer_start()
        for _ in range(steps):
            self.step(prec)
        ms = self.ctx.timer_stop()
        clk = clocks.stop() if clocks else None
        st = {k: v[0] / steps for k, v in self.ctx.stage_times().items()}
        self.ctx.set_profiling(0)
        launches = self.ctx.counts()["kernel_launches"] - l0
        return dist_max(self.dist, ms) / steps, st, launches, clk

    def vector(self, prec, terms=None):
        from rbc3d_gb300.abi import TERM_ALL, TLIST_RBC
        return self.ctx.matvec(TLIST_RBC, self.c, self.c, TERM_ALL if terms is None else terms, prec)

    def alone(self, prec, terms, reps=3):
        """Stage times with the stages run alone on the main stream (no PME in
        the call keeps the matvec on one stream)."""
        self.step(prec, terms)
        self.ctx.set_profiling(1)
        for _ in range(reps):
            self.step(prec, terms)
        st = self.ctx.stage_times()
        self.ctx.set_profiling(0)
        return {k: v[0] / reps for k, v in st.items()}

    def e2e(self, prec, steps, raw=True, nlat0=12):
        """The matvec through the C ABI from pinned host buffers, the caller's
        velocity accumulator up and the velocities down every step.  raw: the
        caller holds positions and raw densities only, as RBC3D's time
        integrator does (rbc3d_set_cells_x / rbc3d_set_cell_density_x derive
        the geometry and the spline tables on the device, degree < nlat0);
        else positions, geometry, densities and all spline tables go up."""
        from rbc3d_gb300.abi import TERM_ALL, TLIST_RBC
        cells, lib, ctx, c = self.cells, self.lib, self.ctx, self.c
        resident = self.vector(prec) if raw else None
        pin = {}
        keys = ("x", "f", "g") if raw else ("x", "a3", "detJ", "area", "meshSize", "spl_x", "spl_a3", "spl_detJ",
                                            "f", "g", "spl_F", "spl_G")
        for k in keys:
            a = np.ascontiguousarray(getattr(cells, k), dtype=np.float64)
            p = lib.pinned(a.shape)
            p[...] = a
            pin[k] = p
        vout = lib.pinned((3, self.N))

        class PinnedCells:
            pass

        pc = PinnedCells()
        for k in ("nlat", "nlon", "th", "phi", "w", "ncell", "celltype"):
            setattr(pc, k, getattr(cells, k))
        for k, p in pin.items():
            setattr(pc, k, p)
        h2d = sum(p.nbytes for p in pin.values()) + vout.nbytes
        d2h = vout.nbytes
        parts = {"set_cells": 0.0, "set_cell_density": 0.0, "matvec_with_download": 0.0}

        def one():
            t0 = time.perf_counter()
            if raw:
                ctx.set_cells_x(pc, nlat0)
            else:
                ctx.set_cells(pc)
            t1 = time.perf_counter()
            if raw:
                ctx.set_cell_density_x(nlat0, f=pc.f, g=pc.g)
            else:
                ctx.set_cell_density(f=pc.f, g=pc.g, spl_F=pc.spl_F, spl_G=pc.spl_G)
            t2 = time.perf_counter()
            vout[...] = 0.0
            ctx.matvec(TLIST_RBC, c, c, TERM_ALL, prec, v=vout)
            t3 = time.perf_counter()
            parts["set_cells"] += t1 - t0
            parts["set_cell_density"] += t2 - t1
            parts["matvec_with_download"] += t3 - t2

        for _ in range(2):
            one()
        for k in parts:
            parts[k] = 0.0
        barrier(self.dist)
        te = time.perf_counter()
        for _ in range(steps):
            one()
        te = dist_max(self.dist, (time.perf_counter() - te) / steps)
        out = {"value": self.ws * self.N / te, "unit": "targets/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": te * 1e3,
               "host_ms_per_step": {k: v / steps * 1e3 for k, v in parts.items()},
               "h2d_gbs_measured": lib.h2d_bandwidth(h2d),
               "inputs": ("positions and raw densities (geometry and spline tables derived on the device, degree "
                          f"< {nlat0})") if raw else "positions, geometry, densities and spline tables"}
        if raw:
            # the synthetic workload's resident tables are analytic samples; the
            # derived ones filter a3 and detJ as the reference does
            out["rel_l2_vs_resident_tables"] = rel(np.array(vout), resident)
            ctx.set_cells(cells)  # back to the resident inputs
            ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
        return out

    def close(self):
        self.ctx.close()


def rooflines_of(b, counts, peak32, peak64, hbm_peak, hbm_src, sm_mhz):
    """Per-kernel rooflines from algorithmic work, each stage timed alone."""
    from rbc3d_gb300.abi import FP32C, FP32D, FP32M, TERM_CORR, TERM_LINEAR, TERM_PME, TERM_REAL
    s_c = b.alone(FP32C, TERM_REAL | TERM_CORR | TERM_LINEAR)
    s_m = b.alone(FP32M, TERM_REAL | TERM_CORR | TERM_LINEAR)
    s_d = b.alone(FP32D, TERM_REAL | TERM_CORR | TERM_LINEAR)
    s_p = b.alone(FP32C, TERM_PME)
    G3 = 1
    for d in b.prm["Nb"]:
        G3 *= d
    N = b.N
    pme_ms = s_p["pme_spread"] + s_p["pme_fft_infl"] + s_p["pme_gather"]
    pme_bytes = 4.0 * G3 * (12 + 12 + 12 + 12 + 3 + 3 + 3 + 3) + 4.0 * N * (3 + 3 + 3 + 1) + 4.0 * N * (3 + 3)
    pairs = counts["pairs_within_rc"]
    pair_fl = pairs * (FLOP_PAIR_SL + FLOP_PAIR_DL)
    self_fl = counts["self_items"] * NQ * FLOP_SELFQ_SLDL
    # requested L1 load bytes of k_self_ff per patch point: 4 stencil nodes x
    # 4 slots x 3 quads x 32 B (hi and lo) + 136 B of weights
    l1_bytes = counts["self_items"] * NQ * (4 * 4 * 3 * 32 + 136)
    l1_peak = 128.0 * 152 * sm_mhz * 1e6 / 1e9

    def fl(name, ms, flops, peak, bound, work):
        a = flops / (ms * 1e-3) / 1e12
        return {"kernel": name, "bound": bound, "ms": ms, "achieved": a, "peak": peak, "unit": "TFLOP/s",
                "frac": a / peak, "work": work}

    r = {
        "k_pair32": fl("k_pair32 + k_pair_own32 (the pair-sum stage)", s_c["pair"], pair_fl, peak32, "fp32",
                       f"{pairs} pairs within rc x {FLOP_PAIR_SL + FLOP_PAIR_DL} flops"),
        "k_self_ff": fl("k_self_ff", s_d["self"], self_fl, peak32, "fp32",
                        f"{counts['self_items']} targets x {NQ} patch points x {FLOP_SELFQ_SLDL} flops of the FP64 "
                        "formula, evaluated in float-float on the FP32 pipe"),
        "k_self": fl("k_self", s_c["self"], self_fl, peak64, "fp64",
                     f"{counts['self_items']} targets x {NQ} x {FLOP_SELFQ_SLDL} flops"),
        "k_self_mix": fl("k_self_mix", s_m["self"], self_fl, peak32, "fp32", "the k_self work in FP32"),
        "pme": {"kernel": "k_spread_tile + cuFFT + k_influence + k_gather", "bound": "hbm", "ms": pme_ms,
                "achieved": pme_bytes / (pme_ms * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": pme_bytes / (pme_ms * 1e-3) / 1e9 / hbm_peak, "peak_source": hbm_src,
                "work": "algorithmic bytes 4 G (12+12+12+12+3+3+3+3) + 4 N (3+3+3+1) + 4 N (3+3), FP32 grids"},
        "near_ms_fp32d": s_d["near"],
        "note": "stages timed alone on one stream (the matvec runs them on two); FP32 peak = measured FMA chain "
                "(rbc3d_fma_peak), FP64 likewise",
    }
    r["k_self_ff"]["l1_request_gbs"] = l1_bytes / (s_d["self"] * 1e-3) / 1e9
    r["k_self_ff"]["l1_request_frac_of_nominal"] = r["k_self_ff"]["l1_request_gbs"] / l1_peak
    return r, s_d


def headline_roofline(r, s_d, targets):
    """The dominant kernel of the FP32D matvec (longest stage timed alone);
    traffic = the ncu bytes per target of that kernel x this launch's targets."""
    key = "k_self_ff" if s_d["self"] >= s_d["pair"] else "k_pair32"
    roof = dict(r[key])
    roof["peak_source"] = "measured FP32 FMA chain over all SMs (rbc3d_fma_peak), same GPU, same run"
    roof["traffic"] = None
    tpath = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            rec = json.load(open(tpath))[key]
            roof["traffic"] = rec["bytes_per_target"] * targets
            if "ncu_pipes" in rec:
                roof["ncu_pipes"] = rec["ncu_pipes"]
        except Exception:
            pass
    return roof


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
    ap.add_argument("--quick-prec", choices=("fp32c", "fp32m", "fp32d", "fp64"), default="fp32d",
                    help="the mode --quick times (profiling)")
    ap.add_argument("--quick-e2e", action="store_true",
                    help="only the end-to-end FP32D step from positions and raw densities (profiling)")
    ap.add_argument("--no-wall", action="store_true", help="skip the learned-guess wall GMRES comparison")
    ap.add_argument("--no-scaleup", action="store_true", help="skip the 2048-cell (PME 256^3) workload")
    ap.add_argument("--no-cellsolve", action="store_true", help="skip the cell velocity GMRES line")
    ap.add_argument("--wall-steps", type=int, nargs=2, default=(100, 10), metavar=("TRAIN", "TEST"),
                    help="RK2 steps of the learned-guess comparison: training steps, compared steps")
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
    from rbc3d_gb300.abi import FP32C, FP32D, FP32M, FP64, TERM_CORR

    t0 = time.perf_counter()
    prm, cells = make_inputs(args.seed + rank, args.cells)
    log(f"inputs generated in {time.perf_counter() - t0:.1f}s")
    lib = library()
    b = Bench(lib, prm, cells, dist, ws)
    N = b.N
    cpu_on = rank == 0 and ws == 1 and not args.no_cpu

    if args.quick_e2e:
        e = b.e2e(FP32D, args.steps)
        if rank == 0:
            print(json.dumps({"quick_e2e": True, **{k: v for k, v in e.items() if k != "inputs"}}), flush=True)
        b.close()
        return 0

    # ---- headline: FP32D matvec with every input resident in HBM
    head = {"fp32m": FP32M, "fp32c": FP32C, "fp64": FP64}.get(args.quick_prec, FP32D) if args.quick else FP32D
    clk = Clocks()
    ms_step, stages, launches, clocks = b.timed(head, args.warmup, args.steps, clk)
    value = ws * N / (ms_step * 1e-3)
    counts = b.ctx.counts()
    if args.quick:
        if rank == 0:
            print(json.dumps({"quick": True, "mode": args.quick_prec, "ms_per_step": ms_step, "targets": N,
                              "value": value, "stages_ms_per_step": stages, "gpu_launches": launches}), flush=True)
        b.close()
        return 0

    # ---- the other modes on the same context
    ms64, st64, _, _ = b.timed(FP64, 2, max(3, args.steps // 3))
    msm, stm, _, _ = b.timed(FP32M, 2, args.steps)
    msc, stc, _, _ = b.timed(FP32C, 2, args.steps)
    fp64_value, fp32m_value, fp32c_value = (ws * N / (m * 1e-3) for m in (ms64, msm, msc))
    # the patch corrections alone (self + near-singular; the near pass is the same
    # FP64 code in both modes): float-float patch against the FP64 patch
    self_ff_vs_fp64 = rel(b.vector(FP32D, TERM_CORR), b.vector(FP32C, TERM_CORR))
    vec = {name: b.vector(p) for name, p in (("fp64", FP64), ("fp32c", FP32C), ("fp32m", FP32M), ("fp32d", FP32D))}
    err_fp64 = {k: rel(v, vec["fp64"]) for k, v in vec.items() if k != "fp64"}

    e2e = b.e2e(FP32D, max(3, args.steps // 2), raw=True)
    e2e["floor_ms"] = ms_step + e2e["h2d_bytes_per_step"] / (e2e["h2d_gbs_measured"] * 1e9) * 1e3
    e2e["floor"] = "device matvec + the step's uploads at the measured pinned copy bandwidth"
    e2e_tables = b.e2e(FP32D, max(3, args.steps // 2), raw=False)

    peak32 = lib.fma_peak(FP32C)
    peak64 = lib.fma_peak(FP64)
    hbm_peak, hbm_src = 6800.0, "fallback"
    try:
        mp = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
        hbm_peak, hbm_src = float(mp["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except Exception:
        pass
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    rooflines, s_d = rooflines_of(b, counts, peak32, peak64, hbm_peak, hbm_src, sm_mhz)
    roof = headline_roofline(rooflines, s_d, N)

    # ---- CPU baseline on the same inputs (rank 0, N = 1): the oracle on all
    # host threads; its vector gives the error of every mode against the oracle
    cpu, err_oracle = None, None
    if cpu_on:
        try:
            ts, cores, vo = time_oracle(prm, cells, 1)
            cpu = {"value": N / ts[0], "unit": "targets/s", "cores": cores, "kind": "port",
                   "sample": f"one full FP64 matvec of the same workload ({N} targets), {ts[0]:.1f}s"}
            err_oracle = {k: rel(v, vo) for k, v in vec.items()}
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": "targets/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"unavailable: {e}"}
    b.close()
    del vec

    # ---- 2048 cells, L = 80, PME 256^3 (2.56 M targets): the same fields
    c5 = None
    if not args.no_scaleup and not args.cells:
        t1 = time.perf_counter()
        prm5, cells5 = make_inputs(args.seed + rank, name="C5")
        b5 = Bench(lib, prm5, cells5, dist, ws)
        N5 = b5.N
        k5 = max(10, args.steps // 2)
        m5d, st5d, l5, _ = b5.timed(FP32D, 3, k5)
        m5m, _, _, _ = b5.timed(FP32M, 2, k5)
        m5c, _, _, _ = b5.timed(FP32C, 1, 3)
        m564, _, _, _ = b5.timed(FP64, 1, 3)
        cnt5 = b5.ctx.counts()
        vec5 = {n: b5.vector(p) for n, p in (("fp64", FP64), ("fp32c", FP32C), ("fp32m", FP32M), ("fp32d", FP32D))}
        e5 = b5.e2e(FP32D, 5, raw=True)
        e5["floor_ms"] = m5d + e5["h2d_bytes_per_step"] / (e5["h2d_gbs_measured"] * 1e9) * 1e3
        r5, s5d = rooflines_of(b5, cnt5, peak32, peak64, hbm_peak, hbm_src, sm_mhz)
        b5.close()
        c5 = {"config": WORKLOADS["C5"], "value": ws * N5 / (m5d * 1e-3), "unit": "targets/s",
              "ms_per_step": m5d, "steps": k5, "warmup": 3, "stages_ms_per_step": st5d, "gpu_launches": l5,
              "fp64_plain": {"value": ws * N5 / (m564 * 1e-3), "ms_per_step": m564, "steps": 3},
              "fp32c": {"value": ws * N5 / (m5c * 1e-3), "ms_per_step": m5c, "steps": 3},
              "fp32m": {"value": ws * N5 / (m5m * 1e-3), "ms_per_step": m5m, "steps": k5},
              "fp32_over_fp64_plain": {"fp32d": m564 / m5d, "fp32c": m564 / m5c, "fp32m": m564 / m5m},
              "rel_l2_vs_fp64_plain": {k: rel(v, vec5["fp64"]) for k, v in vec5.items() if k != "fp64"},
              "e2e": e5, "roofline": headline_roofline(r5, s5d, N5), "rooflines": r5,
              "counts": {k: cnt5[k] for k in ("pairs_within_rc", "nbr_items", "nearsing_items", "self_items")}}
        if cpu_on:
            try:
                ts5, cores5, vo5 = time_oracle(prm5, cells5, 1)
                c5["cpu_baseline"] = {"value": N5 / ts5[0], "unit": "targets/s", "cores": cores5, "kind": "port",
                                      "sample": f"one full FP64 matvec of the same workload ({N5} targets), "
                                                f"{ts5[0]:.1f}s"}
                c5["rel_l2_vs_oracle"] = {k: rel(v, vo5) for k, v in vec5.items()}
                del vo5
            except Exception as e:
                c5["cpu_baseline"] = {"value": None, "sample": f"unavailable: {e}"}
        del vec5
        log(f"2048-cell workload in {time.perf_counter() - t1:.1f}s")

    # ---- wall no-slip GMRES on the tube workload: plain vs history vs learned guess
    wall = None
    if not args.no_wall and not args.cells:
        from rbc3d_gb300.learned_run import run as wall_run
        keys = ("wall_dof", "restart", "history", "plain", "history_only", "spectral_only", "learned",
                "spectral_preconditioned", "speedup_learned", "speedup_history_only", "speedup_spectral_only",
                "speedup_spectral_preconditioned", "learned_over_history_its",
                "train_ms_per_step", "speedup_learned_incl_training", "spectral", "mlp")
        t1 = time.perf_counter()
        warm, test = args.wall_steps
        w = wall_run(ncell=64, warm_steps=warm, test_steps=test, rtol=1e-8, restart=300, max_it=900, train_iters=30,
                     history=48, seed=args.seed + rank, dynamics="skalak", dt=1e-3)
        log(f"wall GMRES comparison in {time.perf_counter() - t1:.1f}s")
        wall = {"workload": "C3 tube (R=8, L=48, 64 cells) under RK2 membrane dynamics (Skalak ES 1, ED 50, "
                            "bending 5.4e-3, intra-cell repulsion 0.81, dt 1e-3), NoSlipWall after each RK2 "
                            "stage; FP64 matvec + FP64 Arnoldi, ||r|| < 1e-8 ||b||",
                **{k: w[k] for k in keys},
                "steps": f"{warm} RK2 steps ({2 * warm} plain solves: the pairs that train the spectral operator "
                         f"and the MLP online), then {test} steps ({2 * test} solves) each solved plain, from the "
                         "history projection, from the spectral operator alone, from the learned guess "
                         "(spectral operator + MLP) and with the spectral operator as the right preconditioner "
                         "(guess mode 5); each compared step's pair is learned only after every arm has solved it "
                         "(held out)"}
        t1 = time.perf_counter()
        # as many training steps as the FP64 run, so that the spectral bases
        # complete and the preconditioner acts on every mode; half the compared steps
        wm_warm, wm_test = warm, max(3, test // 2)
        wm = wall_run(ncell=64, warm_steps=wm_warm, test_steps=wm_test, rtol=1e-8, restart=300, max_it=900,
                      train_iters=30, history=48, seed=args.seed + rank, prec=FP32M, dynamics="skalak", dt=1e-3)
        log(f"mixed-precision wall GMRES comparison in {time.perf_counter() - t1:.1f}s")
        wall["mixed_fp32m"] = {k: wm[k] for k in ("plain", "history_only", "spectral_only", "learned",
                                                  "spectral_preconditioned", "speedup_spectral_preconditioned",
                                                  "speedup_learned", "speedup_history_only", "speedup_spectral_only",
                                                  "speedup_learned_incl_training")}
        wall["mixed_fp32m"]["learned_over_fp64_plain"] = w["plain"]["ms"] / wm["learned"]["ms"]
        wall["mixed_fp32m"]["steps"] = f"{wm_warm} training + {wm_test} compared RK2 steps"

    # ---- cell velocity GMRES (Solve_RBC_Vel, degree 12, rtol 1e-11 as the reference
    # sets it) on the 256 cells: FP64 solve vs the mixed-precision solves
    cellsolve = None
    if not args.no_cellsolve and not args.cells:
        from rbc3d_gb300.abi import Context
        t1 = time.perf_counter()
        ctx = Context(lib, prm)
        ctx.set_cells(cells)
        ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
        arms = {}
        for name, p in (("fp64", FP64), ("fp32d", FP32D), ("fp32m", FP32M), ("fp32c", FP32C)):
            sol, v, st, code = ctx.solve_rbc_vel(12, rtol=1e-11, max_it=300, restart=30, prec=p, check=False)
            arms[name] = (sol, v, st, code)
        ctx.close()
        s64, v64 = arms["fp64"][0], arms["fp64"][1]
        cellsolve = {"workload": "Solve_RBC_Vel on the 256-cell workload (viscRat 5, SH degree 12, "
                                 f"{3 * 144 * 256} unknowns), restart 30, ||r|| < 1e-11 ||b|| (FP64 residual)"}
        for name, (sol, v, st, code) in arms.items():
            cellsolve[name] = {"ms": st.ms, "iterations": st.iterations, "matvecs": st.matvecs,
                               "refinements": st.refinements, "status": code,
                               "final_rel_residual": st.rnorm / st.bnorm if st.bnorm > 0 else 0.0,
                               "rel_l2_vs_fp64_solution": rel(sol, s64) if name != "fp64" else 0.0,
                               "rel_l2_vs_fp64_velocity": rel(v, v64) if name != "fp64" else 0.0}
        for name in ("fp32d", "fp32m", "fp32c"):
            cellsolve[name]["speedup_vs_fp64"] = arms["fp64"][2].ms / arms[name][2].ms
        log(f"cell solve comparison in {time.perf_counter() - t1:.1f}s")

    if rank == 0:
        config = dict(WORKLOAD) if not args.cells else {"workload": f"{args.cells} cells (profiling)",
                                                        "targets": N}
        line = {
            "metric": "Ewald matvec targets/s", "value": value, "unit": "targets/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+ff48-patch+f64-near",
            "data": "synthetic (seeded biconcave cells, SH densities)",
            "config": config,
            "mode": "FP32D: pair sums, PME in FP32 with compensated accumulation; own-cell polar patch in "
                    "float-float arithmetic (48-bit significands, 2e-12 from the FP64 patch); near-singular "
                    "correction in FP64",
            "rel_l2_vs_oracle": err_oracle,
            "rel_l2_vs_fp64_plain": err_fp64["fp32d"],
            "patch_corrections_rel_l2_vs_fp64_patch": self_ff_vs_fp64,
            "fp64_plain": {"value": fp64_value, "unit": "targets/s", "ms_per_step": ms64,
                           "fp32d_over_fp64": value / fp64_value, "stages_ms_per_step": st64},
            "fp32c": {"value": fp32c_value, "unit": "targets/s", "ms_per_step": msc,
                      "over_fp64": fp32c_value / fp64_value, "rel_l2_vs_fp64_plain": err_fp64["fp32c"],
                      "stages_ms_per_step": stc, "note": "own-cell polar patch on the FP64 pipe"},
            "fp32m": {"value": fp32m_value, "unit": "targets/s", "ms_per_step": msm,
                      "over_fp64": fp32m_value / fp64_value, "rel_l2_vs_fp64_plain": err_fp64["fp32m"],
                      "stages_ms_per_step": stm,
                      "note": "own-cell polar patch in FP32 with FP64-accurate (hi/lo) geometry"},
            "e2e": e2e,
            "e2e_host_tables": e2e_tables,
            "stages_ms_per_step": stages,
            "counts": {k: counts[k] for k in ("pairs_within_rc", "nbr_items", "nearsing_items", "self_items",
                                              "screen_misses", "near_replays", "near_projections")},
            "roofline": roof,
            "rooflines": rooflines,
            "fp32_over_fp64_plain": {"fp32d": value / fp64_value, "fp32c": fp32c_value / fp64_value,
                                     "fp32m": fp32m_value / fp64_value, "target": 20.0,
                                     "tolerance_vs_oracle": 1e-6,
                                     "modes_meeting_target": [k for k, r in (("fp32d", value / fp64_value),
                                                                             ("fp32c", fp32c_value / fp64_value),
                                                                             ("fp32m", fp32m_value / fp64_value))
                                                              if r >= 20.0 and (err_oracle or {}).get(k, 1.0) <= 1e-6],
                                     "note": "fp32d: self patch in float-float on the FP32 pipe (GB300 FP64 is "
                                             "1/74 of FP32); fp32c: on the FP64 pipe; fp32m: in FP32 with hi/lo "
                                             "geometry"},
            "c5": c5,
            "wall_gmres": wall,
            "cell_gmres": cellsolve,
            "fma_peaks_tflops": {"fp32": peak32, "fp64": peak64},
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
