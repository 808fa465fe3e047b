"""Parity at the full benchmark sizes: the GPU's output vectors against the
FP64 oracle's on the same seeded inputs.

* 256 cells, L = 40, PME 128^3, SL+DL (320,000 targets): every precision
  mode against the oracle's matvec (FP64 <= 1e-10, FP32C / FP32M / FP32D
  <= 1e-6 relative L2), pair, neighbour-cell and near-singular counts.
* 2048 cells, L = 80, PME 256^3 (2,560,000 targets): the same.
* The near-singular screen of the FP32 modes, verified in FP64 at both
  sizes (RBC3D_VERIFY_SCREEN=1: every screened item is also decided in FP64;
  no disagreement allowed).
* The 64-cell tube (wall of radius 8, length 48, 9,216 unique vertices,
  27,648 unknowns, PME 96x96x256): wall quadrature at the cell points,
  Compute_Wall_Residual_Vel and MyMatMult against the oracle (1e-12), and the
  GPU's NoSlipWall solutions (FP64 and mixed precision) checked with the
  oracle's own operator: the true residual of the GPU density, evaluated by
  the oracle, is below the solve tolerance 1e-8 ||b||.

The oracle is the FP64 restatement of the reference path; the reference
itself cannot be compiled here, so these errors are against that
restatement."""
import math

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import Context, FP32C, FP32D, FP32M, FP64, TERM_ALL, TLIST_RBC, TLIST_WALL

pytestmark = pytest.mark.gpu
C = 1 / (4 * math.pi)
MODES = [("fp64", FP64, 1e-10), ("fp32c", FP32C, 1e-6), ("fp32m", FP32M, 1e-6), ("fp32d", FP32D, 1e-6)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def setup(lib, prm, cells):
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    return ctx


def oracle_case(oracle, name):
    prm, cells, _ = G.config(name)
    o = setup(oracle, prm, cells)
    v = o.matvec(TLIST_RBC, C, C, TERM_ALL)
    cnt = o.counts()
    o.close()
    return prm, cells, v, cnt


@pytest.fixture(scope="module")
def c2(oracle):
    return oracle_case(oracle, "C2")


@pytest.fixture(scope="module")
def c5(oracle):
    return oracle_case(oracle, "C5")


def check_modes(gpu, case, label):
    prm, cells, vo, co = case
    g = setup(gpu, prm, cells)
    errs = {}
    for name, prec, tol in MODES:
        v = g.matvec(TLIST_RBC, C, C, TERM_ALL, prec)
        cg = g.counts()
        errs[name] = rel(v, vo)
        assert errs[name] < tol, (label, name, errs[name])
        assert cg["nearsing_items"] == co["nearsing_items"] > 0, (label, name)
        assert cg["self_items"] == co["self_items"]
        if prec == FP64:
            assert cg["pairs_within_rc"] == co["pairs_within_rc"]
            assert cg["nbr_items"] == co["nbr_items"]
        else:
            # an FP32 distance may put a pair at r = rc on the other side of the cutoff
            assert abs(cg["pairs_within_rc"] - co["pairs_within_rc"]) <= 1e-6 * co["pairs_within_rc"]
            assert abs(cg["nbr_items"] - co["nbr_items"]) <= 1e-4 * co["nbr_items"]
    g.close()
    print(f"{label} rel L2 vs oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))


def check_screen(gpu, case, monkeypatch):
    monkeypatch.setenv("RBC3D_VERIFY_SCREEN", "1")
    prm, cells, vo, co = case
    g = setup(gpu, prm, cells)
    for prec in (FP32D, FP32M):
        v = g.matvec(TLIST_RBC, C, C, TERM_ALL, prec)
        cnt = g.counts()
        assert cnt["screen_misses"] == 0
        assert cnt["nearsing_items"] == co["nearsing_items"]
        assert rel(v, vo) < 1e-6
    g.close()


def test_c2_all_modes_vs_oracle(gpu, c2):
    check_modes(gpu, c2, "C2 (256 cells)")


def test_c2_near_screen_verified_in_fp64(gpu, c2, monkeypatch):
    check_screen(gpu, c2, monkeypatch)


def test_c5_all_modes_vs_oracle(gpu, c5):
    check_modes(gpu, c5, "C5 (2048 cells)")


def test_c5_near_screen_verified_in_fp64(gpu, c5, monkeypatch):
    check_screen(gpu, c5, monkeypatch)


def assemble(r, wall):
    """AddArray of Compute_Wall_Residual_Vel onto the unique wall unknowns
    (ModNoSlip.F90:361-384: later vertices overwrite earlier duplicates)."""
    out = np.zeros(wall.ndof)
    for iv in range(wall.nvert):
        g = wall.glb[iv] - 1
        out[3 * g:3 * g + 3] = r[:, iv]
    return out


def test_c3_wall_operators_and_solves_vs_oracle(gpu, oracle):
    prm, cells, wall = G.config("C3")
    u = np.ascontiguousarray(np.cos(np.arange(wall.ndof) * 0.37))
    fw = np.ascontiguousarray(0.1 * np.sin(wall.x))
    res = {}
    for lab, lib in (("o", oracle), ("g", gpu)):
        ctx = Context(lib, prm)
        ctx.set_cells(cells)
        ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
        ctx.set_walls(wall)
        ctx.prepare_sing_int_on_wall()
        ctx.set_wall_density(fw)
        vq = ctx.add_int_on_walls(TLIST_RBC, C)
        y = ctx.wall_matmult(u)
        r = ctx.compute_wall_residual_vel()
        res[lab] = (vq, y, r, ctx.counts()["wall_pairs"])
        if lab == "o":
            orc = ctx
        else:
            gctx = ctx
    for i, what in enumerate(("AddIntOnWalls at cell points", "MyMatMult", "Compute_Wall_Residual_Vel")):
        assert rel(res["g"][i], res["o"][i]) < 1e-12, what
    assert res["g"][3] == res["o"][3] > 0

    # NoSlipWall from a zero density on the GPU (FP64, and mixed precision with
    # the FP32D and FP32M operators); the oracle evaluates the true residual
    zero = np.zeros((3, wall.nvert))
    orc.set_wall_density(zero)
    b = -assemble(orc.compute_wall_residual_vel(), wall)
    for prec in (FP64, FP32D, FP32M):
        gctx.set_wall_density(zero)
        st, code = gctx.no_slip_wall(1e-8, 900, 300, prec=prec)
        assert code == 0 and st.converged == 1
        assert abs(st.bnorm - np.linalg.norm(b)) <= 1e-10 * np.linalg.norm(b)
        f = gctx.get_wall_density(wall.nvert)
        orc.set_wall_density(f)
        r = assemble(orc.compute_wall_residual_vel(), wall)
        assert np.linalg.norm(r) <= 1.02e-8 * np.linalg.norm(b), (prec, np.linalg.norm(r) / np.linalg.norm(b))
        print(f"C3 NoSlipWall prec {prec}: {st.iterations} its, GPU residual {st.rnorm / st.bnorm:.2e}, "
              f"oracle residual of the GPU density {np.linalg.norm(r) / np.linalg.norm(b):.2e}")
    orc.close()
    gctx.close()
