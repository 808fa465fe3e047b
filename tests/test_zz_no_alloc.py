"""rbc3d_add_linear_int_noalloc: the allocation-free entry point for callers
that cannot allocate device memory (their device arrays are owned by another
runtime or pool).  The test owns its device buffers (it is the caller here),
calls the entry point twice in a row through the C ABI and compares each
result with the linear term of the regular matvec entry point."""
import ctypes
import dataclasses
import math
import os

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import Context, FP64, TERM_LINEAR, TLIST_RBC

pytestmark = pytest.mark.gpu


def cudart():
    for name in ("libcudart.so", "/usr/local/cuda/lib64/libcudart.so", "libcudart.so.13"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("CUDA runtime library not found")


class Dev:
    """Minimal device-buffer helper on the CUDA runtime (test side only)."""

    def __init__(self):
        self.rt = cudart()
        self.rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        self.rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        self.rt.cudaFree.argtypes = [ctypes.c_void_p]
        self.rt.cudaStreamCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        self.rt.cudaStreamSynchronize.argtypes = [ctypes.c_void_p]
        self.rt.cudaStreamDestroy.argtypes = [ctypes.c_void_p]
        self.bufs = []

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), max(a.nbytes, 8)) == 0
        assert self.rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0
        self.bufs.append(p)
        return p

    def get(self, p, like):
        out = np.empty_like(like)
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0
        return out

    def zero(self, p, like):
        z = np.zeros_like(like)
        assert self.rt.cudaMemcpy(p, z.ctypes.data, z.nbytes, 1) == 0

    def set(self, p, a):
        a = np.ascontiguousarray(a)
        assert self.rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0

    def stream(self):
        s = ctypes.c_void_p()
        assert self.rt.cudaStreamCreate(ctypes.byref(s)) == 0
        return s

    def free(self):
        for p in self.bufs:
            self.rt.cudaFree(p)


def entry(gpu):
    fn = gpu.lib.rbc3d_add_linear_int_noalloc
    fn.restype = ctypes.c_int
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp, ctypes.c_int, dp, dp,
                   ctypes.c_double, ctypes.c_int, vp, vp, vp]
    return fn


def linear_term(cells, B_of_type, L, c2, acoef):
    """AddLinearInt restated in numpy: v += c2 * xvint / Acoef with
    xvint = -8 pi / V * sum over cells of Bcoef * sum x (g.a3) detJ w."""
    nv = cells.nlat * cells.nlon
    ilat = np.arange(cells.x.shape[1]) % cells.nlat
    integrand = cells.x * np.sum(cells.g * cells.a3, axis=0) * cells.detJ * cells.w[ilat]
    per_cell = integrand.reshape(3, cells.ncell, nv).sum(axis=2)
    B = np.array([B_of_type.get(int(t), 0.0) for t in cells.celltype])
    xvint = -8 * math.pi / L ** 3 * (per_cell * B).sum(axis=1)
    return c2 * xvint[:, None] / acoef[None, :]


def test_noalloc_linear_term_matches_regular_path(gpu):
    rng = np.random.default_rng(23)
    L = 14.0
    cells = G.make_cells(rng, 5, [L] * 3, 2.8, with_g=True)
    prm = dict(Lb=[L] * 3, alpha=G.alpha_for_cutoff(3.0, 1e-6), rc=3.0, eps=1e-6, Nb=[32] * 3, P=6, nlat=25,
               nlon=50, ncelltypes=1, viscRat=[5.0], vBkg=[0, 0, 0])
    c2 = 1 / (4 * math.pi)
    ctx = Context(gpu, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    ref = ctx.matvec(TLIST_RBC, 0.0, c2, TERM_LINEAR, FP64)
    ctx.close()
    assert np.linalg.norm(ref) > 0

    fn = entry(gpu)
    dp = ctypes.POINTER(ctypes.c_double)
    N = cells.x.shape[1]
    dev = Dev()
    try:
        x, g, a3 = dev.put(cells.x), dev.put(cells.g), dev.put(cells.a3)
        detJ, w = dev.put(cells.detJ), dev.put(cells.w)
        ct = dev.put(cells.celltype.astype(np.int32))
        acoef = dev.put(np.full(N, 6.0))  # initCOEFs: Acoef = 1 + viscRat
        v = dev.put(np.zeros((3, N)))
        vr = np.array([5.0])
        Lb = np.array([L] * 3)
        for _ in range(2):  # two calls in a row share the scratch array
            dev.zero(v, ref)
            st = fn(cells.ncell, 25, 50, x, g, a3, detJ, w, ct, 1, vr.ctypes.data_as(dp), Lb.ctypes.data_as(dp),
                    c2, N, acoef, v, None)
            assert st == 0
            out = dev.get(v, ref)
            assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-12
        # sizes beyond the scratch capacity are rejected before any device work
        st = fn(8193, 25, 50, x, g, a3, detJ, w, ct, 1, vr.ctypes.data_as(dp), Lb.ctypes.data_as(dp), c2, N,
                acoef, v, None)
        assert st == 1
    finally:
        dev.free()


def test_noalloc_mixed_cell_types_on_a_stream(gpu):
    """Two cell types (one rigid: viscRat <= 0 gives Bcoef = -1, Acoef = 1),
    a caller-created stream, accumulation into a nonzero v, an out-of-range
    cell type (contributes nothing) and the early returns (v unchanged)."""
    rng = np.random.default_rng(29)
    L = 15.0
    cells = G.make_cells(rng, 6, [L] * 3, 2.8, with_g=True)
    cells.celltype = np.array([0, 1, 0, 1, 1, 0], dtype=np.int32)
    visc = [5.0, 0.0]
    prm = dict(Lb=[L] * 3, alpha=G.alpha_for_cutoff(3.0, 1e-6), rc=3.0, eps=1e-6, Nb=[32] * 3, P=6, nlat=25,
               nlon=50, ncelltypes=2, viscRat=visc, vBkg=[0, 0, 0])
    c2 = 1 / (4 * math.pi)
    ctx = Context(gpu, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    ref = ctx.matvec(TLIST_RBC, 0.0, c2, TERM_LINEAR, FP64)
    ctx.close()
    N = cells.x.shape[1]
    nv = cells.nlat * cells.nlon
    acoef = np.repeat(np.where(cells.celltype == 0, 6.0, 1.0), nv)
    B = {0: 1.0 - 5.0, 1: -1.0}
    expect = linear_term(cells, B, L, c2, acoef)
    assert np.linalg.norm(expect - ref) / np.linalg.norm(ref) < 1e-12  # the restatement is the regular path

    fn = entry(gpu)
    dp = ctypes.POINTER(ctypes.c_double)
    dev = Dev()
    stream = dev.stream()
    try:
        x, g, a3 = dev.put(cells.x), dev.put(cells.g), dev.put(cells.a3)
        detJ, w = dev.put(cells.detJ), dev.put(cells.w)
        ct = dev.put(cells.celltype)
        acoef_d = dev.put(acoef)
        v0 = rng.standard_normal((3, N))
        v = dev.put(v0)
        vr = np.array(visc)
        Lb = np.array([L] * 3)

        def call(ncell, c2_):
            return fn(ncell, 25, 50, x, g, a3, detJ, w, ct, 2, vr.ctypes.data_as(dp), Lb.ctypes.data_as(dp), c2_,
                      N, acoef_d, v, stream)

        for _ in range(2):
            dev.set(v, v0)
            assert call(cells.ncell, c2) == 0
            assert dev.rt.cudaStreamSynchronize(stream) == 0
            out = dev.get(v, v0) - v0
            assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-12

        # a cell type outside [0, ncelltypes) contributes nothing
        bad = cells.celltype.copy()
        bad[2] = 7
        dev.set(ct, bad)
        dev.set(v, v0)
        assert call(cells.ncell, c2) == 0
        assert dev.rt.cudaStreamSynchronize(stream) == 0
        cells_bad = dataclasses.replace(cells, celltype=bad)
        expect_bad = linear_term(cells_bad, B, L, c2, acoef)
        out = dev.get(v, v0) - v0
        assert np.linalg.norm(out - expect_bad) / np.linalg.norm(expect_bad) < 1e-12
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) > 1e-3

        # early returns leave v untouched
        dev.set(v, v0)
        assert call(0, c2) == 0
        assert call(cells.ncell, 0.0) == 0
        assert dev.rt.cudaStreamSynchronize(stream) == 0
        assert np.array_equal(dev.get(v, v0), v0)
    finally:
        dev.rt.cudaStreamDestroy(stream)
        dev.free()
