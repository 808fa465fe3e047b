"""Learned vs plain wall GMRES along a run of the tube workload.

Two ways to move the cells: "skalak" integrates the membrane dynamics with
TimeInt_RK2 (ModTimeInt.F90:183-271): Compute_Rbc_Vel with the Skalak and
bending residual force (rbc3d_shell_res_force), the cell velocity solve, and
NoSlipWall after each stage; "kinematic" advects the cells rigidly with a
Poiseuille profile and rotates them with its shear (one wall solve per step).
Every wall no-slip solve runs to ||r|| < rtol ||b|| with GMRES.  The first
`warm_steps` steps are plain solves (zero increment, i.e. warm start from the
previous density as NoSlipWall) that fill the history and train the network
online; afterwards every solve is done from the same state plain, from the
history projection, from the learned spectral operator's prediction, from
that prediction with the network's correction, and with the spectral
operator as the right preconditioner, and iterations, times and final
residuals are compared.  The plain solution continues the run and
is recorded for the guess, so all arms see the same states.

    python -m rbc3d_gb300.learned_run --cells 64 --warm 50 --test 10 --dynamics skalak
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import geometry as G
from . import library
from .abi import FP32C, FP32D, FP32M, FP64, Context
from .dynamics import CellDynamics
from .learned import WallGuess, ring_count

# Shell_ElasStrs / Shell_Bend moduli of the tube run: shear 1, area dilation
# 50 (ED / ES), bending 5.4e-3 (the EB / ES ratio of the reference's example
# cells, examples/cutout/ctube.F90:112-114)
SKALAK_MODULI = (1.0, 50.0, 5.4e-3)
# ForceCoef of AddIntraCellRepulsionForce at the reference example's ratio to
# the shear modulus (ForceCoef 10 in examples/case/Input/tube.in for cells
# with ES 12.4)
FORCE_COEF = 10.0 * SKALAK_MODULI[0] / 12.4


def _unique_increment(wall, f1, f0):
    un = np.zeros((wall.ndof // 3, 3))
    un[wall.glb - 1] = (f1 - f0).T
    return un.reshape(-1)


def run(ncell=64, warm_steps=30, test_steps=10, rtol=1e-8, restart=100, max_it=800, dt=5e-3, umax=8.0,
        train_iters=10, width=512, depth=4, history=48, seed=20261203, prec=FP64, log=None, dynamics="kinematic",
        moduli=SKALAK_MODULI, force_coef=FORCE_COEF):
    prm, cells, wall = G.config("C3", seed=seed, ncell=ncell)
    lib = library()
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
    ctx.set_walls(wall)
    ctx.prepare_sing_int_on_wall()
    guess = WallGuess(lib, ctx, wall, width=width, depth=depth, seed=seed, history=history)
    axis = (prm["Lb"][0] / 2, prm["Lb"][1] / 2)
    rng = np.random.default_rng(seed)
    dyn = None
    if dynamics == "skalak":
        # membrane mechanics: reference cell = the undeformed biconcave shape
        xr, _, _ = G.biconcave_surface(cells.th, cells.phi, np.eye(3), np.zeros(3))
        dyn = CellDynamics(ctx, cells, G._to_points(xr[None]), moduli, force_coef=force_coef)
        dyn.compute_rbc_vel(dyn.x)  # tractions and g of the initial state
    elif dynamics != "kinematic":
        raise ValueError(dynamics)
    ctx.no_slip_wall(rtol, max_it, restart, prec, check=False)  # initial density
    arms = {"plain": [], "history": [], "spectral": [], "learned": [], "preconditioned": []}
    guess_arms = ("history", "spectral", "learned", "preconditioned")
    losses, train_ms = [], []
    state = {"step": 0}

    def wall_step(stage=0):
        """NoSlipWall at the current cell state: the guess arms (test steps) from
        the same state, then the plain solve that continues the run."""
        step = state["step"]
        f0 = ctx.get_wall_density(wall.nvert)
        testing = step >= warm_steps
        if testing:
            for mode in guess_arms:
                st, ok, ms, _ = guess.solve(ctx, wall, rtol, max_it, restart, prec, mode=mode)
                arms[mode].append(dict(its=st.iterations, ms=ms, rel=st.rnorm / st.bnorm, accepted=ok,
                                       r0=st.rnorm0 / st.bnorm))
                ctx.set_wall_density(f0)
        b = guess.rhs(ctx, prec)
        t0 = time.perf_counter()
        st, code = ctx.no_slip_wall(rtol, max_it, restart, prec, check=False)
        ms = (time.perf_counter() - t0) * 1e3
        arms["plain"].append(dict(its=st.iterations, ms=ms, rel=st.rnorm / st.bnorm, accepted=True, r0=1.0))
        guess.record(b, _unique_increment(wall, ctx.get_wall_density(wall.nvert), f0))
        t1 = time.perf_counter()
        loss = guess.train(iters=train_iters, rng=rng)
        train_ms.append((time.perf_counter() - t1) * 1e3)
        if loss is not None:
            losses.append(loss)
        if log:
            msg = f"step {step}.{stage} plain its {st.iterations} ms {ms:.0f}"
            if testing:
                for mode in guess_arms:
                    a = arms[mode][-1]
                    msg += f" | {mode} its {a['its']} ms {a['ms']:.0f} r0 {a['r0']:.2e}"
            elif loss is not None:
                msg += f" loss {loss:.3e}"
            if dyn is not None:
                msg += f" | force rms {dyn.last['force_rms']:.3e}"
            log(msg)

    for step in range(warm_steps + test_steps):
        state["step"] = step
        if dyn is not None:
            dyn.rk2(dt, after_stage=wall_step)  # TimeInt_RK2: NoSlipWall after each Compute_Rbc_Vel
        else:
            cells = G.poiseuille_step(cells, axis, 8.0, umax, dt)
            ctx.set_cells(cells)
            ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
            wall_step()
    per_step = 2 if dyn is not None else 1

    def summary(mode):
        a = arms[mode][-test_steps * per_step:]
        return {"its": float(np.mean([x["its"] for x in a])), "ms": float(np.mean([x["ms"] for x in a])),
                "initial_rel_residual": float(np.mean([x["r0"] for x in a])),
                "accepted": int(sum(x["accepted"] for x in a)),
                "max_final_rel_residual": float(max(x["rel"] for x in a))}

    res = {"cells": ncell, "wall_dof": int(wall.ndof), "warm_steps": warm_steps, "test_steps": test_steps,
           "rtol": rtol, "restart": restart, "history": history, "dynamics": dynamics, "dt": dt,
           "solves_per_step": per_step,
           "plain": summary("plain"), "history_only": summary("history"), "spectral_only": summary("spectral"),
           "learned": summary("learned"), "spectral_preconditioned": summary("preconditioned")}
    res["speedup_learned"] = res["plain"]["ms"] / res["learned"]["ms"]
    res["speedup_history_only"] = res["plain"]["ms"] / res["history_only"]["ms"]
    res["speedup_spectral_only"] = res["plain"]["ms"] / res["spectral_only"]["ms"]
    res["speedup_spectral_preconditioned"] = res["plain"]["ms"] / res["spectral_preconditioned"]["ms"]
    res["learned_over_history_its"] = res["learned"]["its"] / res["history_only"]["its"]
    nb, npairs = guess.basis_sizes()
    res["spectral"] = {"modes": int(nb.size), "pairs": int(npairs), "basis_min": int(nb.min()),
                       "basis_median": float(np.median(nb)), "basis_max": int(nb.max()),
                       "block": wall.ndof // ring_count(wall)}
    res["train_ms_per_step"] = float(np.mean(train_ms))
    res["speedup_learned_incl_training"] = res["plain"]["ms"] / (res["learned"]["ms"] + res["train_ms_per_step"])
    res["final_loss"] = float(losses[-1]) if losses else None
    res["mlp"] = {"layers": f"{guess.mlp.dims[0]} -> {width} x {depth} (SiLU) -> 3", "weights": "bf16 (tcgen05.mma kind::f16)",
                  "accumulation": "fp32", "params": int(guess.mlp.nparam)}
    guess.mlp.close()
    ctx.close()
    return res


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--warm", type=int, default=50)
    ap.add_argument("--test", type=int, default=10)
    ap.add_argument("--restart", type=int, default=300)
    ap.add_argument("--train-iters", type=int, default=30)
    ap.add_argument("--history", type=int, default=48)
    ap.add_argument("--dynamics", choices=("kinematic", "skalak"), default="skalak",
                    help="cell motion: RK2 membrane dynamics (Compute_Rbc_Vel) or rigid Poiseuille advection")
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--prec", choices=("fp64", "fp32c", "fp32m", "fp32d"), default="fp64",
                    help="operator arithmetic of every arm (FP32 modes: mixed-precision solves)")
    a = ap.parse_args()
    prec = {"fp64": FP64, "fp32c": FP32C, "fp32m": FP32M, "fp32d": FP32D}[a.prec]
    dt = a.dt if a.dt is not None else (1e-3 if a.dynamics == "skalak" else 5e-3)
    print(json.dumps(run(a.cells, a.warm, a.test, restart=a.restart, train_iters=a.train_iters, history=a.history,
                         prec=prec, dynamics=a.dynamics, dt=dt, log=print)))
