"""Cell velocity solve (Solve_RBC_Vel, ModVelSolver.F90:44-132): the
spherical-harmonic transforms and spline rebuild it needs, the oracle's
solve, and the GPU solve against the oracle."""
import ctypes
import math

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import FP32C, FP32D, FP32M, FP64, Context

_dp = ctypes.POINTER(ctypes.c_double)
NLAT0 = 12  # spherical-harmonic degree < 12 on the 25 x 50 grid


def _small(ncell=2, visc=5.0):
    prm, cells, _ = G.config("C1", ncell=ncell)
    prm["viscRat"] = [visc]
    return prm, cells


def test_pbar_matches_normalised_legendre(oracle):
    from scipy.special import lpmv
    f = oracle.lib.rbc3d_oracle_kat_pbar
    f.argtypes = [ctypes.c_int, ctypes.c_double, _dp]
    f.restype = None
    L = 14
    for th in np.linspace(0.03, 3.1, 11):
        P = np.zeros(L * L)
        f(L, th, P.ctypes.data_as(_dp))
        for m in range(L):
            for n in range(m, L):
                # Spherepack: sqrt((2n+1)/2 (n-m)!/(n+m)!) P_n^m without the Condon-Shortley phase
                ref = math.sqrt((2 * n + 1) / 2 * math.factorial(n - m) / math.factorial(n + m)) * (-1) ** m * lpmv(
                    m, n, math.cos(th))
                assert abs(P[m * L + n] - ref) < 1e-12


def test_sph_trans_roundtrip(oracle):
    prm, cells = _small()
    ctx = Context(oracle, prm)
    ctx.set_cells(cells)
    f = oracle.lib.rbc3d_oracle_kat_sph_trans
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_int]
    f.restype = ctypes.c_int
    N = cells.x.shape[1]
    c = np.random.default_rng(3).standard_normal(3 * NLAT0 * NLAT0 * cells.ncell)
    v = np.zeros(3 * N)
    f(ctx.h, NLAT0, v.ctypes.data_as(_dp), c.ctypes.data_as(_dp), 0)
    c2 = np.zeros_like(c)
    f(ctx.h, NLAT0, v.ctypes.data_as(_dp), c2.ctypes.data_as(_dp), 1)
    assert np.abs(c2 - c).max() < 1e-12  # Gauss quadrature is exact for degree < nlat0
    # a degree-0 field: a(0, 0) = 2 sqrt(2) c0 reproduces the constant c0 = 1
    cc = np.zeros_like(c)
    for cell in range(cells.ncell):
        cc[cell * 3 * NLAT0 * NLAT0:cell * 3 * NLAT0 * NLAT0 + 3] = 2 * math.sqrt(2.0)
    f(ctx.h, NLAT0, v.ctypes.data_as(_dp), cc.ctypes.data_as(_dp), 0)
    assert np.allclose(v, 1.0, atol=1e-13)
    ctx.close()


def test_spline_build_matches_fft_diff(oracle):
    f = oracle.lib.rbc3d_oracle_kat_spline_build
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]
    f.restype = None
    nlat, nlon = 25, 50
    fe = np.random.default_rng(1).standard_normal((nlat + 1, nlon, 3))
    tab = np.zeros(4 * 3 * 2 * nlat * nlon)
    fin = np.ascontiguousarray(fe.transpose(2, 1, 0)).reshape(-1)
    f(nlat, nlon, 3, fin.ctypes.data_as(_dp), tab.ctypes.data_as(_dp))
    ref = G.spline_on_sphere(fe)
    assert np.abs(tab - ref.reshape(-1)).max() < 1e-10 * np.abs(ref).max()


def test_oracle_cell_solve_converges_and_warm_starts(oracle):
    prm, cells = _small()
    ctx = Context(oracle, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
    sol, v, st, code = ctx.solve_rbc_vel(NLAT0, rtol=1e-11, max_it=200, restart=30)
    assert code == 0 and st.converged and st.rnorm < 1e-11 * st.bnorm
    assert 0 < st.iterations < 200
    sol2, v2, st2, code2 = ctx.solve_rbc_vel(NLAT0, rtol=1e-11, max_it=200, restart=30, sol=sol)
    assert st2.iterations == 0 and np.array_equal(v2, v)
    ctx.close()


def test_oracle_cell_solve_viscrat_one_is_projected_rhs(oracle):
    # viscRat = 1: sol = rhs, so v is the degree < nlat0 projection of the
    # single-layer velocity + 2 vBkg / Acoef (Acoef = 2)
    prm, cells = _small(visc=1.0)
    ctx = Context(oracle, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
    sol, v, st, code = ctx.solve_rbc_vel(NLAT0)
    assert code == 0 and st.iterations == 0
    u = ctx.matvec(0, 1 / (4 * math.pi), 0.0)
    f = oracle.lib.rbc3d_oracle_kat_sph_trans
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_int]
    f.restype = ctypes.c_int
    uu = np.ascontiguousarray(u.reshape(-1))
    c = np.zeros(3 * NLAT0 * NLAT0 * cells.ncell)
    f(ctx.h, NLAT0, uu.ctypes.data_as(_dp), c.ctypes.data_as(_dp), 1)
    assert np.allclose(c, sol, rtol=0, atol=1e-13 * np.abs(sol).max())
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("visc", [5.0, 1.0])
def test_gpu_cell_solve_matches_oracle(gpu, oracle, visc):
    prm, cells = _small(ncell=3, visc=visc)
    out = []
    for lib in (oracle, gpu):
        ctx = Context(lib, prm)
        ctx.set_cells(cells)
        ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
        out.append(ctx.solve_rbc_vel(NLAT0, rtol=1e-11, max_it=200, restart=30))
        if lib is gpu:
            # warm start from the converged solution: nothing left to do
            sol2, v2, st2, code2 = ctx.solve_rbc_vel(NLAT0, rtol=1e-11, max_it=200, restart=30, sol=out[-1][0])
            assert st2.iterations <= 1
        ctx.close()
    (so, vo, sto, co), (sg, vg, stg, cg) = out
    assert co == 0 and cg == 0
    if visc != 1.0:
        assert stg.rnorm < 1e-11 * stg.bnorm
    else:
        assert stg.iterations == 0  # sol = rhs, no GMRES
    assert abs(stg.iterations - sto.iterations) <= 1
    assert np.linalg.norm(vg - vo) <= 1e-9 * np.linalg.norm(vo)
    assert np.linalg.norm(sg - so) <= 1e-9 * np.linalg.norm(so)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [FP32C, FP32M, FP32D])
def test_gpu_cell_solve_mixed_precision(gpu, prec):
    # FP32 double-layer operator inside FP64 refinement, to the reference's 1e-11
    prm, cells = _small(ncell=3, visc=5.0)
    out = {}
    for p in (FP64, prec):
        ctx = Context(gpu, prm)
        ctx.set_cells(cells)
        ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
        out[p] = ctx.solve_rbc_vel(NLAT0, rtol=1e-11, max_it=200, restart=30, prec=p)
        ctx.close()
    (s, v, st, c), (s64, v64, st64, c64) = out[prec], out[FP64]
    assert c == 0 and c64 == 0 and st.converged == 1 and st.refinements >= 1
    assert st.rnorm < 1e-11 * st.bnorm
    assert np.linalg.norm(v - v64) <= 1e-9 * np.linalg.norm(v64)
    assert np.linalg.norm(s - s64) <= 1e-9 * np.linalg.norm(s64)
