"""rbc3d_add_linear_int_noalloc: the allocation-free entry point for callers
that cannot allocate device memory (their device arrays are owned by another
runtime or pool).  The test owns its device buffers (it is the caller here),
calls the entry point twice in a row through the C ABI and compares each
result with the linear term of the regular matvec entry point."""
import ctypes
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

    def free(self):
        for p in self.bufs:
            self.rt.cudaFree(p)


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

    fn = gpu.lib.rbc3d_add_linear_int_noalloc
    fn.restype = ctypes.c_int
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp, ctypes.c_int, dp, dp,
                   ctypes.c_double, ctypes.c_int, vp, vp, vp]
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
