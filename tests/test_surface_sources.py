"""The cells' geometry and spline tables derived on the device from the raw
surface fields (rbc3d_set_cells_x / rbc3d_set_cell_density_x:
RBC_ComputeGeometry + Rbc_BuildSurfaceSource, ModRbc.F90:404-509,716-807)
against the same derivation done on the host: RBC_ComputeGeometry on the GPU
(checked against the oracle in test_membrane.py) and the filtered
spherical-harmonic resampling plus Spline_Build_On_Sphere restated in numpy
(rbc3d_gb300.dynamics.SphTransform, checked against Spherepack's definitions
in test_cell_solve.py).  Both paths feed the same matvec."""
import math

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import Context, FP32D, FP64, TERM_ALL, TLIST_RBC
from rbc3d_gb300.dynamics import SphTransform, to_grid

pytestmark = pytest.mark.gpu
C = 1 / (4 * math.pi)


def host_sources(ctx, cells, nlat0):
    nc, nlat, nlon = cells.ncell, cells.nlat, cells.nlon
    a3, detJ, area, _ = ctx.cell_geometry(cells.x, nc)
    T = SphTransform(cells.th, cells.phi, cells.w, nlat0)
    Xg, Ag, Dg = to_grid(cells.x, nc, nlat, nlon), to_grid(a3, nc, nlat, nlon), to_grid(detJ[None], nc, nlat, nlon)
    Fg, Gg = to_grid(cells.f, nc, nlat, nlon), to_grid(cells.g, nc, nlat, nlon)
    return G.Cells(nlat=nlat, nlon=nlon, th=cells.th, phi=cells.phi, w=cells.w, ncell=nc, celltype=cells.celltype,
                   x=cells.x, a3=a3, detJ=detJ, area=area, meshSize=np.sqrt(area / nlat ** 2),
                   spl_x=T.spline(Xg), spl_a3=T.spline(Ag), spl_detJ=T.spline(Dg),
                   f=cells.f, g=cells.g, spl_F=T.spline(Fg * Dg), spl_G=T.spline(Gg * Dg))


@pytest.mark.parametrize("nlat0", [12, 8])
def test_device_surface_sources_match_host_derivation(gpu, nlat0):
    prm, cells, _ = G.config("C2", ncell=24)
    prm["Lb"] = [20.0] * 3
    ref_ctx = Context(gpu, prm)
    ref_ctx.set_cell_grid(cells.th, cells.phi, cells.w)
    hc = host_sources(ref_ctx, cells, nlat0)
    ref_ctx.set_cells(hc)
    ref_ctx.set_cell_density(f=hc.f, g=hc.g, spl_F=hc.spl_F, spl_G=hc.spl_G)
    dev = Context(gpu, prm)
    dev.set_cells_x(cells, nlat0)
    dev.set_cell_density_x(nlat0, f=cells.f, g=cells.g)
    # the two transforms sum in different orders: 1.7e-12 measured in FP64
    for prec, tol in ((FP64, 1e-11), (FP32D, 1e-6)):
        a = ref_ctx.matvec(TLIST_RBC, C, C, TERM_ALL, prec)
        ca = ref_ctx.counts()
        b = dev.matvec(TLIST_RBC, C, C, TERM_ALL, prec)
        cb = dev.counts()
        assert np.linalg.norm(a - b) <= tol * np.linalg.norm(a), prec
        for k in ("nbr_items", "nearsing_items", "self_items"):
            assert ca[k] == cb[k], k
    # the densities alone can change without new positions
    dev.set_cell_density_x(nlat0, f=2 * cells.f)
    ref_ctx.set_cell_density(f=2 * hc.f, spl_F=2 * hc.spl_F)
    a = ref_ctx.matvec(TLIST_RBC, C, 0.0, TERM_ALL, FP64)
    b = dev.matvec(TLIST_RBC, C, 0.0, TERM_ALL, FP64)
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a)
    ref_ctx.close()
    dev.close()


def test_device_surface_sources_of_the_synthetic_cells(gpu):
    """The synthetic workloads carry analytic tables; the device derivation
    filters every field to degree < nlat0 as the reference does (ShFilter),
    which moves the matvec by the truncation of that filter only: the
    difference shrinks as the kept degree grows (the oracle's 4-cell case:
    4.2e-3 at nlat0 12, 1.6e-4 at 20, 1.0e-4 at 24)."""
    prm, cells, _ = G.config("C2", ncell=24)
    prm["Lb"] = [20.0] * 3
    a_ctx = Context(gpu, prm)
    a_ctx.set_cells(cells)
    a_ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    a = a_ctx.matvec(TLIST_RBC, C, C, TERM_ALL, FP64)
    err = {}
    for nlat0 in (12, 24):
        d_ctx = Context(gpu, prm)
        d_ctx.set_cells_x(cells, nlat0)
        d_ctx.set_cell_density_x(nlat0, f=cells.f, g=cells.g)
        b = d_ctx.matvec(TLIST_RBC, C, C, TERM_ALL, FP64)
        err[nlat0] = np.linalg.norm(a - b) / np.linalg.norm(a)
        d_ctx.close()
    print(f"analytic vs device-derived tables: {err}")
    assert err[12] < 1e-2
    assert err[24] < 3e-4 and err[24] < 0.1 * err[12]
    a_ctx.close()


def test_back_to_back_updates_and_buffer_reuse(gpu):
    """set_cells_x / set_cell_density_x return while the derivation runs on
    the device: updates issued back to back, and host buffers overwritten as
    soon as the calls return, give the matvec of the last state as a fresh
    context computes it."""
    prm, cells, _ = G.config("C2", ncell=24)
    prm["Lb"] = [20.0] * 3
    rng = np.random.default_rng(7)
    moved = np.ascontiguousarray(cells.x + 0.05 * rng.standard_normal(cells.x.shape))
    f2 = np.ascontiguousarray(1.5 * cells.f)
    fresh = Context(gpu, prm)
    fresh.set_cell_grid(cells.th, cells.phi, cells.w)

    class Raw:
        pass

    def raw(x):
        r = Raw()
        for k in ("nlat", "nlon", "th", "phi", "w", "ncell", "celltype"):
            setattr(r, k, getattr(cells, k))
        r.x = x
        return r

    fresh.set_cells_x(raw(moved), 12)
    fresh.set_cell_density_x(12, f=f2, g=cells.g)
    ref = {p: fresh.matvec(TLIST_RBC, C, C, TERM_ALL, p) for p in (FP64, FP32D)}
    fresh.close()
    ctx = Context(gpu, prm)
    ctx.set_cell_grid(cells.th, cells.phi, cells.w)
    # pinned host buffers: the copies are asynchronous, the calls wait for them
    xbuf, fbuf, gbuf = gpu.pinned(cells.x.shape), gpu.pinned(cells.f.shape), gpu.pinned(cells.g.shape)
    xbuf[...] = cells.x
    fbuf[...] = cells.f
    gbuf[...] = cells.g
    ctx.set_cells_x(raw(xbuf), 12)
    ctx.set_cell_density_x(12, f=fbuf, g=gbuf)
    ctx.matvec(TLIST_RBC, C, C, TERM_ALL, FP32D)  # a matvec of the first state, then the second state
    xbuf[...] = moved
    ctx.set_cells_x(raw(xbuf), 12)
    xbuf[...] = 0.0          # the caller's buffers are free once the calls return
    fbuf[...] = f2
    ctx.set_cell_density_x(12, f=fbuf, g=gbuf)
    fbuf[...] = 0.0
    gbuf[...] = 0.0
    # FP64 to rounding; FP32D to its run-to-run spread (float atomics in the
    # PME spread, ~3e-8): a stale or half-written input moves it by far more
    for p, tol in ((FP64, 1e-12), (FP32D, 1e-6)):
        v = ctx.matvec(TLIST_RBC, C, C, TERM_ALL, p)
        assert np.linalg.norm(v - ref[p]) <= tol * np.linalg.norm(ref[p]), p
    # two density updates back to back without a matvec between them
    ctx.set_cell_density_x(12, f=cells.f, g=cells.g)
    ctx.set_cell_density_x(12, f=f2, g=cells.g)
    v = ctx.matvec(TLIST_RBC, C, C, TERM_ALL, FP64)
    assert np.linalg.norm(v - ref[FP64]) <= 1e-12 * np.linalg.norm(ref[FP64])
    ctx.close()
