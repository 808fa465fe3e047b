"""Membrane mechanics (RBC_ComputeGeometry, Shell_ResForce with the Skalak
law and bending, ModRbc.F90:404-963): the oracle against analytic geometry
and the equilibrium identities, and the GPU against the oracle."""
import math

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import Context

MODULI = (1.0, 50.0, 5.4e-3)  # ES (shear), ED (area dilation), EB (bending)


def _ctx(lib, ncell=2):
    prm, cells, _ = G.config("C1", ncell=ncell)
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    return ctx, cells


def _reference():
    th, phi, _ = G.gauss_grid(25, 50)
    x0, _, _ = G.biconcave_surface(th, phi, np.eye(3), np.zeros(3))
    return G._to_points(x0[None]), x0


def _deformed(ncell, seed=4, amp=0.08):
    """Rotated, translated biconcave cells with a smooth random deformation (degree <= 4)."""
    rng = np.random.default_rng(seed)
    th, phi, _ = G.gauss_grid(25, 50)
    X = []
    for c in range(ncell):
        x, _, _ = G.biconcave_surface(th, phi, G.random_rotation(rng), rng.uniform(-2, 2, 3))
        d = np.stack([G.sh_eval(G.random_sh_coeffs(rng, lmax=4), th, phi) for _ in range(3)], axis=-1)
        X.append(x + amp * d)
    return G._to_points(np.array(X))


def test_oracle_geometry_matches_analytic(oracle):
    ctx, cells = _ctx(oracle)
    a3, dj, area, vol = ctx.cell_geometry(cells.x, cells.ncell)
    # the biconcave surface is a degree-5 expansion: the Gauss-grid derivatives are exact
    assert np.abs(a3 - cells.a3).max() < 1e-10
    assert np.abs(dj - cells.detJ).max() < 1e-10
    assert np.allclose(area, cells.area, rtol=1e-12, atol=0)
    sph = G.make_sphere_cells([np.array([1.0, -2.0, 0.5])], radius=1.3)
    a3s, djs, ars, vos = ctx.cell_geometry(sph.x, 1)
    assert np.abs(a3s - sph.a3).max() < 1e-10 and np.abs(djs - 1.3 ** 2).max() < 1e-10
    assert abs(ars[0] - 4 * math.pi * 1.3 ** 2) < 1e-11 and abs(vos[0] - 4 / 3 * math.pi * 1.3 ** 3) < 1e-11
    ctx.close()


def test_oracle_force_vanishes_at_reference_and_balances(oracle):
    ctx, cells = _ctx(oracle)
    xref, _ = _reference()
    ctx.set_ref_cells(xref, *MODULI)
    # the reference shape, also moved rigidly, carries no force (frame invariance)
    assert np.abs(ctx.shell_res_force(xref, [0])).max() < 1e-11
    rng = np.random.default_rng(2)
    th, phi, w = G.gauss_grid(25, 50)
    x1, _, _ = G.biconcave_surface(th, phi, G.random_rotation(rng), np.array([0.3, -0.2, 0.5]))
    assert np.abs(ctx.shell_res_force(G._to_points(x1[None]), [0])).max() < 1e-9
    # deformed cells: membrane forces are in equilibrium (zero net force and torque) up to
    # the truncation of the degree < nlat expansion (about 1e-5 of the force scale here)
    X = _deformed(3)
    f = ctx.shell_res_force(X, [0, 0, 0])
    _, dj, _, _ = ctx.cell_geometry(X, 3)
    ds = dj * np.tile(w, 50 * 3)
    nv = 25 * 50
    for c in range(3):
        sl = slice(c * nv, (c + 1) * nv)
        scale = np.sum(np.linalg.norm(f[:, sl], axis=0) * ds[sl])
        F = (f[:, sl] * ds[sl]).sum(1)
        xc = X[:, sl] - X[:, sl].mean(1, keepdims=True)
        T = (np.cross(xc.T, f[:, sl].T).T * ds[sl]).sum(1)
        assert scale > 100.0
        assert np.linalg.norm(F) < 1e-4 * scale and np.linalg.norm(T) < 1e-4 * scale
    ctx.close()


@pytest.mark.gpu
def test_gpu_geometry_and_force_match_oracle(gpu, oracle):
    xref, _ = _reference()
    X = _deformed(5, seed=7)
    ct = [0, 0, 0, 0, 0]
    out = {}
    for name, lib in (("o", oracle), ("g", gpu)):
        ctx, _ = _ctx(lib)
        ctx.set_ref_cells(xref, *MODULI)
        out[name] = ctx.cell_geometry(X, 5) + (ctx.shell_res_force(X, ct),)
        ctx.close()
    o, g = out["o"], out["g"]
    for a, b in zip(g[:4], o[:4]):
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())
    assert np.linalg.norm(g[4] - o[4]) <= 1e-11 * np.linalg.norm(o[4])


def test_host_sph_transforms():
    from rbc3d_gb300.dynamics import SphTransform, to_grid
    rng = np.random.default_rng(3)
    prm, cells, _ = G.config("C1", ncell=2)
    T = SphTransform(cells.th, cells.phi, cells.w, 12)
    # a degree < 12 field is reproduced by the filter
    f = 0.7 + G.sh_eval(G.random_sh_coeffs(rng, lmax=11), cells.th, cells.phi)
    assert np.abs(T.project(f) - f).max() < 1e-12
    # positions of the biconcave cells (degree 5): the filtered equiangular spline
    # equals the table built from the exact surface
    X = to_grid(cells.x, cells.ncell, cells.nlat, cells.nlon)
    assert np.abs(T.spline(X) - cells.spl_x).max() < 1e-11


def _dyn_case(lib, ncell=1):
    prm, _, _ = G.config("C1", ncell=ncell)
    X = _deformed(ncell, seed=11, amp=0.06)
    X[:, :] += 6.0  # inside the box
    prm0, cells, _ = G.config("C1", ncell=ncell)
    cells.x = X
    ctx = Context(lib, prm)
    return ctx, cells


@pytest.mark.gpu
def test_gpu_rk2_step_matches_oracle(gpu, oracle):
    from rbc3d_gb300.dynamics import CellDynamics
    xref, _ = _reference()
    xs, fr = {}, {}
    for name, lib in (("o", oracle), ("g", gpu)):
        ctx, cells = _dyn_case(lib, 2)
        ctx.set_cells(cells)
        dyn = CellDynamics(ctx, cells, xref, MODULI, rtol=1e-11, force_coef=0.8)
        forces = []
        for _ in range(2):
            dyn.rk2(5e-3)
            forces.append(dyn.last["force_rms"])
        xs[name], fr[name] = dyn.x, forces
        ctx.close()
    assert np.abs(xs["g"] - xs["o"]).max() < 1e-10
    assert np.allclose(fr["g"], fr["o"], rtol=1e-9)
    assert fr["g"][1] < fr["g"][0]  # the deformed cells relax towards the reference shape


def _pinched(ncell=2, seed=5):
    """Cells whose two dimples are pushed towards each other (the biconcave
    faces approach within the repulsion range) plus a generic deformation."""
    rng = np.random.default_rng(seed)
    th, phi, _ = G.gauss_grid(25, 50)
    X = []
    for c in range(ncell):
        x, _, _ = G.biconcave_surface(th, phi, np.eye(3), np.zeros(3))
        x = x.copy()
        x[..., 2] *= 0.35  # flatten: the dimples' faces 0.07 apart
        d = np.stack([G.sh_eval(G.random_sh_coeffs(rng, lmax=3), th, phi) for _ in range(3)], axis=-1)
        X.append(x + 0.01 * d + 4.0 * c + 3.0)
    return G._to_points(np.array(X))


def test_oracle_intra_cell_repulsion(oracle):
    ctx, _ = _ctx(oracle)
    X = _pinched()
    a3, dj, area, _ = ctx.cell_geometry(X, 2)
    f = np.zeros_like(X)
    n = ctx.intra_cell_repulsion(X, a3, area, 10.0, f)
    assert n > 0
    pushed = np.linalg.norm(f, axis=0) > 0
    assert pushed.sum() == n
    # the push is along the outward normal with magnitude ForceCoef exp(1 - d/eps) in (10, 10e]
    mag = np.linalg.norm(f[:, pushed], axis=0)
    assert mag.min() > 10.0 and mag.max() <= 10.0 * math.e + 1e-9
    assert np.allclose(f[:, pushed] / mag, a3[:, pushed], atol=1e-12)
    # a sphere has no opposite faces within epsDist: no point is pushed
    sph = G.make_sphere_cells([np.array([3.0, 3.0, 3.0])], radius=1.0)
    a3s, _, ars, _ = ctx.cell_geometry(sph.x, 1)
    fs = np.zeros_like(sph.x)
    assert ctx.intra_cell_repulsion(sph.x, a3s, ars, 10.0, fs) == 0 and not fs.any()
    ctx.close()


@pytest.mark.gpu
def test_gpu_intra_cell_repulsion_matches_oracle(gpu, oracle):
    X = _pinched(3, seed=9)
    out = {}
    for name, lib in (("o", oracle), ("g", gpu)):
        ctx, _ = _ctx(lib)
        a3, dj, area, _ = ctx.cell_geometry(X, 3)
        f = np.full_like(X, 0.25)
        n = ctx.intra_cell_repulsion(X, a3, area, 10.0, f)
        out[name] = (n, f)
        ctx.close()
    assert out["g"][0] == out["o"][0] > 0
    assert np.abs(out["g"][1] - out["o"][1]).max() <= 1e-12 * np.abs(out["o"][1]).max()


# ---------------------------------------------------------------------------
# The reference's sample sickle cell (tests/golden/sickle_cell.npz, made by
# tests/golden/make_sickle.py from sample_files/sample_cells/SickleCell.dat):
# a strongly deformed shape on a 36 x 72 grid
def _sickle_ctx(lib):
    import os
    from conftest import ROOT
    z = np.load(os.path.join(ROOT, "tests", "golden", "sickle_cell.npz"))
    nlat, nlon = int(z["nlat"]), int(z["nlon"])
    prm, _, _ = G.config("C1", ncell=1)
    prm = dict(prm, nlat=nlat, nlon=nlon)
    ctx = Context(lib, prm)
    th, phi, w = G.gauss_grid(nlat, nlon)
    ctx.set_cell_grid(th, phi, w)
    X = G._to_points(np.asarray(z["x"])[None] + 6.0)  # inside the box
    return ctx, X, w, nlat, nlon


def test_oracle_sickle_cell_mechanics(oracle):
    ctx, X, w, nlat, nlon = _sickle_ctx(oracle)
    a3, dj, area, vol = ctx.cell_geometry(X, 1)
    # reduced volume of the sickle shape: between a biconcave disc (0.64) and a sphere (1)
    rv = vol[0] / (4 / 3 * math.pi * (area[0] / (4 * math.pi)) ** 1.5)
    assert area[0] > 0 and 0.5 < rv < 1.0
    # the shape as its own reference carries no force; shrunk by 2% it does, in equilibrium
    ctx.set_ref_cells(X, *MODULI)
    assert np.abs(ctx.shell_res_force(X, [0])).max() < 1e-8
    c = X.mean(axis=1, keepdims=True)
    Xs = c + 0.98 * (X - c)
    f = ctx.shell_res_force(Xs, [0])
    _, djs, _, _ = ctx.cell_geometry(Xs, 1)
    ds = djs * np.tile(w, nlon)
    scale = np.sum(np.linalg.norm(f, axis=0) * ds)
    assert scale > 1.0 and np.linalg.norm((f * ds).sum(1)) < 1e-3 * scale
    ctx.close()


@pytest.mark.gpu
def test_gpu_sickle_cell_matches_oracle(gpu, oracle):
    out = {}
    for name, lib in (("o", oracle), ("g", gpu)):
        ctx, X, w, nlat, nlon = _sickle_ctx(lib)
        c = X.mean(axis=1, keepdims=True)
        ctx.set_ref_cells(c + 1.03 * (X - c), *MODULI)
        a3, dj, area, vol = ctx.cell_geometry(X, 1)
        f = ctx.shell_res_force(X, [0])
        fr = np.zeros_like(X)
        n = ctx.intra_cell_repulsion(X, a3, area, 0.8, fr)
        out[name] = (a3, dj, area, vol, f, fr, n)
        ctx.close()
    o, g = out["o"], out["g"]
    # a degree-35 shape: the summation orders (FMA on the GPU, none in the oracle) differ by ~1e-12
    for a, b in zip(g[:4], o[:4]):
        assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max())
    assert np.linalg.norm(g[4] - o[4]) <= 1e-9 * np.linalg.norm(o[4])
    assert g[6] == o[6] and np.abs(g[5] - o[5]).max() <= 1e-10 * max(1.0, np.abs(o[5]).max())


def _packed(lib, wall=False):
    """Cells packed closer than their size (10 cells, centres at least 2.0
    apart in a 12^3 box), or 6 cells inside a radius-4 tube whose wall they
    come within a few tenths of: many points within the repulsion distance of
    another cell or of the wall.  Two cell types (viscRat 5 and 50)."""
    if wall:
        rng = np.random.default_rng(8)
        L = [9.0, 9.0, 12.0]
        prm = dict(Lb=L, alpha=G.alpha_for_cutoff(2.9, 1e-6), rc=2.9, eps=1e-6, Nb=[48, 48, 64], P=6, nlat=25,
                   nlon=50, ncelltypes=2, viscRat=[5.0, 50.0], vBkg=[0, 0, 0])
        w = G.make_tube(4.0, 12.0, 24, 48, (4.5, 4.5))
        cells = G.make_cells(rng, 6, L, 2.2, inside=lambda c: (c[0] - 4.5) ** 2 + (c[1] - 4.5) ** 2 < 2.5 ** 2)
    else:
        rng = np.random.default_rng(6)
        L = [12.0] * 3
        prm = dict(Lb=L, alpha=G.alpha_for_cutoff(3.0, 1e-6), rc=3.0, eps=1e-6, Nb=[32] * 3, P=6, nlat=25, nlon=50,
                   ncelltypes=2, viscRat=[5.0, 50.0], vBkg=[0, 0, 0])
        w = None
        cells = G.make_cells(rng, 10, L, 2.0)
    cells.celltype = (np.arange(cells.ncell) % 2).astype(np.int32)
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    if w is not None:
        ctx.set_walls(w)
    return ctx, cells


def test_oracle_inter_cell_repulsion_moves_close_points(oracle):
    ctx, cells = _packed(oracle)
    eps = 0.3
    x, dmin, n = ctx.inter_cell_repulsion(eps, 10.0, rigidsep=False)
    assert n > 0 and dmin < eps
    moved = np.linalg.norm(x - cells.x, axis=0)
    nv = cells.nlat * cells.nlon
    soft = np.repeat(cells.celltype == 0, nv)
    # type 1 (viscRat 50 >= 10, no rigidsep) stays; type 0 moves by at most eps / 2
    assert np.all(moved[~soft] == 0) and 0 < moved[soft].max() <= 0.5 * eps + 1e-12
    # with rigidsep the stiff cells move rigidly
    x2, _, n2 = ctx.inter_cell_repulsion(eps, 10.0, rigidsep=True)
    d = (x2 - cells.x).reshape(3, cells.ncell, nv)
    for c in np.flatnonzero(cells.celltype == 1):
        assert np.allclose(d[:, c, :], d[:, c, :1], atol=1e-14)
    assert n2 == n
    # the tube case: points near the wall move too
    ctx, cells = _packed(oracle, wall=True)
    x, dmin, n = ctx.inter_cell_repulsion(0.5, 10.0)
    assert n > 0


@pytest.mark.gpu
@pytest.mark.parametrize("wall,eps", [(False, 0.3), (True, 0.5)])
def test_gpu_inter_cell_repulsion_matches_oracle(gpu, oracle, wall, eps):
    out = {}
    for name, lib in (("o", oracle), ("g", gpu)):
        ctx, cells = _packed(lib, wall)
        out[name] = [ctx.inter_cell_repulsion(eps, 10.0, rigidsep=r) for r in (False, True)]
        ctx.close()
    for r in range(2):
        xo, do, no = out["o"][r]
        xg, dg, ng = out["g"][r]
        assert ng == no > 0
        assert abs(dg - do) <= 1e-12 * max(do, 1e-300)
        assert np.abs(xg - xo).max() <= 1e-12
