"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Bar: relative L2 velocity error <= 1e-6 for the FP32 matvec modes (FP32C,
FP32D, FP32M); the FP64 plain form agrees with the oracle to rounding (1e-10).  Counts of
pairs within rc, neighbour-cell items and near-singular corrections must be
identical."""
import math
import os

import numpy as np
import pytest

from rbc3d_gb300 import RBC3DError
from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import (Context, FP32C, FP32D, FP32M, FP64, TERM_ALL, TERM_CORR, TERM_LINEAR, TERM_PME, TERM_REAL,
                             TLIST_RAW, TLIST_RBC, TLIST_WALL)

pytestmark = pytest.mark.gpu
C = 1 / (4 * math.pi)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def setup(lib, prm, cells, dl):
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g if dl else None, spl_F=cells.spl_F, spl_G=cells.spl_G if dl else None)
    return ctx


@pytest.fixture(scope="module")
def c1_case():
    prm, cells, _ = G.config("C1")
    return prm, cells


@pytest.fixture(scope="module")
def sldl_case():
    prm, cells, _ = G.config("C2", ncell=24)
    prm["Lb"] = [20.0] * 3
    return prm, cells


@pytest.mark.parametrize("prec,tol", [(FP64, 1e-12), (FP32C, 1e-6), (FP32M, 1e-6), (FP32D, 1e-6)])
def test_c1_single_layer(gpu, oracle, c1_case, prec, tol):
    prm, cells = c1_case
    o = setup(oracle, prm, cells, False)
    g = setup(gpu, prm, cells, False)
    vo = o.add_int_on_rbcs(TLIST_RBC, C, 0.0)
    vg = g.add_int_on_rbcs(TLIST_RBC, C, 0.0, prec=prec)
    assert rel(vg, vo) < tol
    co, cg = o.counts(), g.counts()
    assert cg["pairs_within_rc"] == co["pairs_within_rc"]
    assert cg["nbr_items"] == co["nbr_items"] and cg["self_items"] == co["self_items"]
    po = o.pme(TLIST_RBC, C, 0.0)
    pg = g.pme(TLIST_RBC, C, 0.0, prec=prec)
    assert rel(pg, po) < max(tol, 1e-6 if prec != FP64 else 1e-12)
    assert rel(vg + pg, vo + po) < tol


@pytest.mark.parametrize("prec,tol", [(FP64, 1e-10), (FP32C, 1e-6), (FP32M, 1e-6), (FP32D, 1e-6)])
def test_sldl_with_near_singular(gpu, oracle, sldl_case, prec, tol):
    prm, cells = sldl_case
    o = setup(oracle, prm, cells, True)
    g = setup(gpu, prm, cells, True)
    vo = o.matvec(TLIST_RBC, C, C, TERM_ALL)
    vg = g.matvec(TLIST_RBC, C, C, TERM_ALL, prec)
    assert rel(vg, vo) < tol
    co, cg = o.counts(), g.counts()
    assert cg["nearsing_items"] == co["nearsing_items"] > 0
    assert cg["nbr_items"] == co["nbr_items"]


def test_near_screen_agrees_with_fp64(gpu, sldl_case, monkeypatch):
    """FP32C screens the projections; with RBC3D_VERIFY_SCREEN=1 every
    screened item is also decided in FP64: no disagreement allowed."""
    monkeypatch.setenv("RBC3D_VERIFY_SCREEN", "1")
    prm, cells = sldl_case
    g = setup(gpu, prm, cells, True)
    g.matvec(TLIST_RBC, C, C, TERM_ALL, FP32C)
    cnt = g.counts()
    assert cnt["screen_misses"] == 0 and cnt["nearsing_items"] > 0


@pytest.mark.parametrize("cap", ["0", "7"])
def test_near_stage_capacity(gpu, sldl_case, monkeypatch, cap):
    """The FP32 modes' FP64 pass over their short list runs staged
    (projections, one warp per quadrature, combination) up to a capacity and
    through the one-warp-per-item kernel past it.  With the capacity cut to 0
    or 7 entries (RBC3D_NEAR_STAGE_CAP) every entry is still taken once: the
    same projection and correction counts, and per target the same
    corrections up to the order of the accumulation."""
    prm, cells = sldl_case
    g = setup(gpu, prm, cells, True)
    ref = g.matvec(TLIST_RBC, C, C, TERM_CORR, FP32D)
    cref = g.counts()
    g.close()
    monkeypatch.setenv("RBC3D_NEAR_STAGE_CAP", cap)
    h = setup(gpu, prm, cells, True)
    v = h.matvec(TLIST_RBC, C, C, TERM_CORR, FP32D)
    cnt = h.counts()
    h.close()
    assert cref["near_projections"] > 7 and cref["nearsing_items"] > 0
    assert cnt["near_projections"] == cref["near_projections"]
    assert cnt["nearsing_items"] == cref["nearsing_items"]
    assert np.abs(v - ref).max() <= 1e-12 * np.abs(ref).max()


def test_l2_entry_points_compose(gpu, sldl_case):
    """AddIntOnRbcs + PME_* called separately equal the composite matvec."""
    prm, cells = sldl_case
    g = setup(gpu, prm, cells, True)
    v1 = g.add_int_on_rbcs(TLIST_RBC, C, C, prec=FP64)
    v1 = g.pme(TLIST_RBC, C, C, prec=FP64, v=v1)
    v2 = g.matvec(TLIST_RBC, C, C, TERM_REAL | TERM_CORR | TERM_LINEAR | TERM_PME, FP64)
    assert rel(v1, v2) < 1e-13


def test_raw_targets_near_surfaces(gpu, oracle, sldl_case):
    prm, cells = sldl_case
    rng = np.random.default_rng(9)
    pick = rng.choice(cells.x.shape[1], 64, replace=False)
    raw = np.concatenate([cells.x[:, pick] + d * cells.a3[:, pick] for d in (0.002, -0.002, 0.1, -0.3)], axis=1)
    raw = np.ascontiguousarray(np.concatenate([raw, rng.uniform(0, 20, (3, 64))], axis=1))
    out = {}
    for lab, lib in (("o", oracle), ("g", gpu)):
        ctx = setup(lib, prm, cells, True)
        ctx.set_raw_targets(raw)
        out[lab] = (ctx.calc_velocity_field(TLIST_RAW, FP64), ctx.counts())
    assert rel(out["g"][0], out["o"][0]) < 1e-10
    assert out["g"][1]["nearsing_items"] == out["o"][1]["nearsing_items"] > 0


def test_fp32c_vs_fp64_full_size_c2(gpu):
    """Full 256-cell SL+DL workload: FP32C within 1e-6 of the FP64 plain form
    (which matches the oracle at the sizes above)."""
    prm, cells, _ = G.config("C2")
    g = setup(gpu, prm, cells, True)
    v64 = g.matvec(TLIST_RBC, C, C, TERM_ALL, FP64)
    v32 = g.matvec(TLIST_RBC, C, C, TERM_ALL, FP32C)
    assert rel(v32, v64) < 1e-6
    v32m = g.matvec(TLIST_RBC, C, C, TERM_ALL, FP32M)
    assert rel(v32m, v64) < 1e-6
    v32d = g.matvec(TLIST_RBC, C, C, TERM_ALL, FP32D)
    assert rel(v32d, v64) < 1e-6
    # the float-float patch agrees with the FP64 patch far below the FP32 error
    cc = g.matvec(TLIST_RBC, C, C, TERM_CORR, FP32C)
    cd = g.matvec(TLIST_RBC, C, C, TERM_CORR, FP32D)
    assert rel(cd, cc) < 1e-11


@pytest.mark.parametrize("c1,c2", [(C, C), (C, 0.0), (0.0, C)])
def test_fp32d_patch_matches_fp64_patch(gpu, sldl_case, c1, c2):
    """RBC_SingInt in float-float arithmetic (FP32D) against the FP64 kernel
    (FP32C): the patch corrections alone (self + near-singular, the latter the
    same FP64 pass in both modes) agree to 1e-11 relative for SL+DL, SL and DL."""
    prm, cells = sldl_case
    g = setup(gpu, prm, cells, True)
    cc = g.matvec(TLIST_RBC, c1, c2, TERM_CORR, FP32C)
    cd = g.matvec(TLIST_RBC, c1, c2, TERM_CORR, FP32D)
    assert np.linalg.norm(cc) > 0
    assert rel(cd, cc) < 1e-11
    # records are rebuilt after the density changes
    g.set_cell_density(f=2 * cells.f, g=-cells.g, spl_F=2 * cells.spl_F, spl_G=-cells.spl_G)
    cc2 = g.matvec(TLIST_RBC, c1, c2, TERM_CORR, FP32C)
    cd2 = g.matvec(TLIST_RBC, c1, c2, TERM_CORR, FP32D)
    assert rel(cd2, cc2) < 1e-11


def test_linearity_in_density(gpu, sldl_case):
    prm, cells = sldl_case
    g = setup(gpu, prm, cells, True)
    a = g.matvec(TLIST_RBC, C, C, TERM_ALL, FP64)
    g.set_cell_density(f=2 * cells.f, g=-cells.g, spl_F=2 * cells.spl_F, spl_G=-cells.spl_G)
    b = g.matvec(TLIST_RBC, C, 0.0, TERM_ALL, FP64)
    c = g.matvec(TLIST_RBC, 0.0, C, TERM_ALL, FP64)
    g.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    s = g.matvec(TLIST_RBC, C, 0.0, TERM_ALL, FP64)
    d = g.matvec(TLIST_RBC, 0.0, C, TERM_ALL, FP64)
    assert rel(b, 2 * s) < 1e-12 and rel(c, -d) < 1e-12 and rel(s + d, a) < 1e-12


def _tube_case():
    rng = np.random.default_rng(5)
    L = [9.0, 9.0, 12.0]
    prm = dict(Lb=L, alpha=G.alpha_for_cutoff(2.9, 1e-6), rc=2.9, eps=1e-6, Nb=[48, 48, 64], P=6, nlat=25,
               nlon=50, ncelltypes=1, viscRat=[1.0], vBkg=[0, 0, 8.0])
    wall = G.make_tube(4.0, 12.0, 24, 48, (4.5, 4.5))
    cells = G.make_cells(rng, 4, L, 3.0, inside=lambda c: (c[0] - 4.5) ** 2 + (c[1] - 4.5) ** 2 < 1.5 ** 2)
    return prm, cells, wall


def test_walls_and_no_slip_solve(gpu, oracle):
    prm, cells, wall = _tube_case()
    res = {}
    fw = np.ascontiguousarray(np.sin(wall.x))
    u = np.ascontiguousarray(np.cos(np.arange(wall.ndof) * 0.37))
    for lab, lib in (("o", oracle), ("g", gpu)):
        ctx = setup(lib, prm, cells, False)
        ctx.set_walls(wall)
        ctx.set_wall_density(fw)
        ctx.prepare_sing_int_on_wall()
        vq = ctx.add_int_on_walls(TLIST_RBC, C)
        vs = ctx.add_int_on_walls(TLIST_WALL, C)
        y = ctx.wall_matmult(u)
        r = ctx.compute_wall_residual_vel()
        ctx.set_wall_density(np.zeros((3, wall.nvert)))
        st, code = ctx.no_slip_wall(1e-8, 200)
        res[lab] = (vq, vs, y, r, ctx.get_wall_density(wall.nvert), st, code, ctx.counts())
    o, g = res["o"], res["g"]
    for i in range(4):
        assert rel(g[i], o[i]) < 1e-12, i
    assert g[6] == 0 and o[6] == 0 and g[5].converged == 1
    assert abs(g[5].iterations - o[5].iterations) <= 1
    assert g[5].rnorm / g[5].bnorm <= 1.01e-8
    assert rel(g[4], o[4]) < 1e-8
    assert g[7]["wall_pairs"] == o[7]["wall_pairs"]


@pytest.mark.parametrize("prec", [FP32C, FP32M])
def test_mixed_precision_wall_solve(gpu, prec):
    # FP32 operator inside FP64 refinement: the FP64 residual meets the FP64 solve's tolerance
    prm, cells, wall = _tube_case()
    out = {}
    for p in (FP64, prec):
        ctx = setup(gpu, prm, cells, False)
        ctx.set_walls(wall)
        ctx.prepare_sing_int_on_wall()
        ctx.set_wall_density(np.zeros((3, wall.nvert)))
        st, code = ctx.no_slip_wall(1e-8, 300, 100, prec=p)
        out[p] = (st, code, ctx.get_wall_density(wall.nvert))
        ctx.close()
    (st, code, f), (st64, code64, f64) = out[prec], out[FP64]
    assert code == 0 and code64 == 0 and st.converged == 1
    assert st.refinements >= 1 and st64.refinements == 0
    assert st.rnorm / st.bnorm <= 1e-8
    assert abs(st.bnorm - st64.bnorm) <= 1e-12 * st64.bnorm  # the same FP64 right-hand side
    assert rel(f, f64) < 1e-4


def test_error_paths(gpu, c1_case):
    prm, cells = c1_case
    g = setup(gpu, prm, cells, False)
    with pytest.raises(RBC3DError) as e:
        g.matvec(7, C, 0.0)
    assert e.value.code == 1
    import ctypes
    g2 = Context(gpu, prm)
    dummy = np.zeros(3)
    code = g2.L.fn["pme_add_interp_vel"](g2.h, TLIST_RBC, dummy.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert code == 6  # PME_Transform not called yet
    # empty raw target list is a no-op
    g.set_raw_targets(np.zeros((3, 0)))
    assert g.matvec(TLIST_RAW, C, 0.0).shape == (3, 0)


def test_wall_solve_error_codes(gpu):
    prm, cells, wall = _tube_case()
    ctx = setup(gpu, prm, cells, False)
    ctx.set_walls(wall)
    st, code = ctx.no_slip_wall(1e-8, 10, check=False)
    assert code == 6  # PrepareSingIntOnWall not called
    ctx.prepare_sing_int_on_wall()
    st, code = ctx.no_slip_wall(1e-12, 2, check=False)
    assert code == 4 and st.iterations == 2 and st.converged == 0  # NOCONV, bounded


@pytest.mark.gpu
def test_fp32_modes_vs_fp64_full_size_c5(gpu):
    # the 2048-cell, PME 256^3 workload (2.56 M targets): both FP32 modes
    # within 1e-6 of the FP64 plain form, identical pair counts
    prm, cells, _ = G.config("C5")
    ctx = Context(gpu, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    c = 1 / (4 * np.pi)
    v64 = ctx.matvec(TLIST_RBC, c, c, TERM_ALL, FP64)
    n64 = ctx.counts()["pairs_within_rc"]
    for prec in (FP32C, FP32M):
        v = ctx.matvec(TLIST_RBC, c, c, TERM_ALL, prec)
        assert np.linalg.norm(v - v64) <= 1e-6 * np.linalg.norm(v64)
        assert abs(ctx.counts()["pairs_within_rc"] - n64) <= 1e-6 * n64  # only pairs at r = rc may differ
    ctx.close()


@pytest.mark.parametrize("P", [4, 8])
def test_pme_spline_orders(gpu, oracle, c1_case, P):
    # the tiled spread is instantiated per spline order; each order against the
    # oracle (even orders: with an odd order the SPME factor b(k) of the
    # reference's PME_Init is singular at the Nyquist frequency)
    prm, cells = c1_case
    prm = dict(prm, P=P)
    out = {}
    for name, lib in (("o", oracle), ("g", gpu)):
        ctx = setup(lib, prm, cells, dl=False)
        out[name] = [ctx.matvec(TLIST_RBC, C, 0.0, TERM_PME, prec) for prec in ((FP64,) if name == "o" else (FP64, FP32C))]
        ctx.close()
    assert rel(out["g"][0], out["o"][0]) < 1e-12
    assert rel(out["g"][1], out["o"][0]) < 1e-6
