"""Learned initial guess for the wall no-slip GMRES (no counterpart in the
reference).

The wall solve of NoSlipWall (ModNoSlip.F90:45-150) finds the density
increment x with A x = b, b the residual wall velocity with the previous
density (ModNoSlip.F90:110-113).  Every solved step of a run gives a pair
(b_i, x_i) with A x_i = b_i to the solve tolerance; the learned guess is
trained on those pairs as the run goes:

* spectral operator (rbc3d_wall_spectral_*, device): the tube wall is a
  uniform stack of rings along the periodic axis, so A is block diagonal in
  the axial Fourier modes; per mode the model keeps an orthonormal basis of
  the transformed right-hand sides seen and the matching solutions, and
  predicts x_s for a new b mode by mode (a pair seen at one position of the
  tube teaches every position).  It learns the exact pairs (A x_i, x_i) and
  also returns the part r_s of b outside the learned span.
* network: a per-vertex MLP (BF16 tensor-core GEMMs, FP32 accumulation,
  rbc3d_mlp_*) maps local-frame features of r_s (r_s and two graph-Laplacian
  powers of it, plus x_s) to the remainder e = x - x_s, trained online on
  the pairs of the solved steps.

GMRES then starts from p x_s + q e_hat with the least-squares p, q (guess
mode 3 of rbc3d_no_slip_wall, one extra matvec) and runs to the same
absolute tolerance rtol * ||b|| as the plain solve.  A solve that does not
reach it within the iteration budget is redone from the previous density
(the plain guess, a zero increment), which stays the fallback and the
yardstick.  The history projection of the previous design (least squares
over the last K right-hand sides, no symmetry) is kept as the comparison
arm "history".
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from .abi import FP64, RBC3DError, _ptr

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)


def _bind(lib):
    L = lib.lib
    sig = {
        "rbc3d_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
        "rbc3d_mlp_destroy": (C.c_int, [C.c_void_p]),
        "rbc3d_mlp_num_params": (C.c_longlong, [C.c_void_p]),
        "rbc3d_mlp_params": (C.c_int, [C.c_void_p, _fp, C.c_int]),
        "rbc3d_mlp_forward": (C.c_int, [C.c_void_p, C.c_int, _fp, _fp]),
        "rbc3d_mlp_gradients": (C.c_int, [C.c_void_p, C.c_int, _fp, _fp, _fp, _fp]),
        "rbc3d_mlp_train_step": (C.c_int, [C.c_void_p, C.c_int, _fp, _fp, C.c_float, _fp]),
        "rbc3d_wall_rhs": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "rbc3d_wall_spectral_init": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int]),
        "rbc3d_wall_spectral_add": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_int)]),
        "rbc3d_wall_spectral_predict": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
        "rbc3d_wall_spectral_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                               C.POINTER(C.c_longlong)]),
    }
    out = {}
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
        out[name] = f
    return out


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """GPU MLP (BF16 tensor-core GEMMs, FP32 master weights, Adam)."""

    def __init__(self, lib, nin, width, depth, nout, seed=0):
        self.fn = _bind(lib)
        self.dims = (nin, width, depth, nout)
        self.h = C.c_void_p()
        st = self.fn["rbc3d_mlp_create"](nin, width, depth, nout, seed, C.byref(self.h))
        if st:
            raise RBC3DError(st, "rbc3d_mlp_create")
        self.nparam = self.fn["rbc3d_mlp_num_params"](self.h)

    def close(self):
        if self.h:
            self.fn["rbc3d_mlp_destroy"](self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, values=None):
        if values is None:
            out = np.empty(self.nparam, np.float32)
            self._ok(self.fn["rbc3d_mlp_params"](self.h, out.ctypes.data_as(_fp), 1))
            return out
        v = _f32(values)
        self._ok(self.fn["rbc3d_mlp_params"](self.h, v.ctypes.data_as(_fp), 0))

    def forward(self, x):
        x = _f32(x)
        y = np.empty((x.shape[0], self.dims[3]), np.float32)
        self._ok(self.fn["rbc3d_mlp_forward"](self.h, x.shape[0], x.ctypes.data_as(_fp), y.ctypes.data_as(_fp)))
        return y

    def gradients(self, x, t):
        x, t = _f32(x), _f32(t)
        g = np.empty(self.nparam, np.float32)
        loss = C.c_float()
        self._ok(self.fn["rbc3d_mlp_gradients"](self.h, x.shape[0], x.ctypes.data_as(_fp), t.ctypes.data_as(_fp),
                                                g.ctypes.data_as(_fp), C.byref(loss)))
        return loss.value, g

    def train_step(self, x, t, lr):
        x, t = _f32(x), _f32(t)
        loss = C.c_float()
        self._ok(self.fn["rbc3d_mlp_train_step"](self.h, x.shape[0], x.ctypes.data_as(_fp), t.ctypes.data_as(_fp),
                                                 C.c_float(lr), C.byref(loss)))
        return loss.value

    @staticmethod
    def _ok(st):
        if st:
            raise RBC3DError(st, "mlp")


def vertex_frames(wall):
    """Unit normal, axial and azimuthal tangents per unique wall vertex."""
    x = wall.x.T
    e2v = wall.e2v.T - 1
    n = np.zeros_like(x)
    a, b, c = x[e2v[:, 0]], x[e2v[:, 1]], x[e2v[:, 2]]
    fn = np.cross(b - a, c - a)  # area-weighted element normals
    for k in range(3):
        np.add.at(n, e2v[:, k], fn)
    nu = np.zeros((wall.ndof // 3, 3))
    np.add.at(nu, wall.glb - 1, n)  # merge periodic duplicates
    nu /= np.linalg.norm(nu, axis=1, keepdims=True)
    ez = np.array([0.0, 0.0, 1.0])
    t1 = ez - (nu @ ez)[:, None] * nu
    bad = np.linalg.norm(t1, axis=1) < 1e-6
    t1[bad] = np.array([1.0, 0.0, 0.0]) - nu[bad, 0:1] * nu[bad]
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(nu, t1)
    return np.stack([nu, t1, t2], axis=1)  # (nv, 3 axes, 3 components)


def vertex_smoother(wall):
    """Random-walk graph Laplacian (mean of the edge neighbours minus the
    vertex) on the unique wall vertices, periodic duplicates merged."""
    import scipy.sparse as sp
    nv = wall.ndof // 3
    e2v = wall.glb[wall.e2v.T - 1] - 1  # element corners as unique vertices
    i = np.concatenate([e2v[:, 0], e2v[:, 1], e2v[:, 2], e2v[:, 1], e2v[:, 2], e2v[:, 0]])
    j = np.concatenate([e2v[:, 1], e2v[:, 2], e2v[:, 0], e2v[:, 0], e2v[:, 1], e2v[:, 2]])
    A = sp.csr_matrix((np.ones(i.size), (i, j)), shape=(nv, nv))
    A.data[:] = 1.0  # edges shared by two elements count once
    deg = np.asarray(A.sum(axis=1)).ravel()
    return sp.diags(1.0 / deg) @ A - sp.identity(nv, format="csr")


def ring_count(wall):
    """Number of rings when the unique wall vertices form a stack of rings
    along z (unique id = ring * nper + i, as make_tube and periodic Exodus
    tubes number them), else None.  The library checks the mesh itself."""
    nu = wall.ndof // 3
    x = np.zeros((nu, 3))
    x[wall.glb - 1] = wall.x.T
    z = x[:, 2]
    nper = int(np.sum(np.abs(z - z[0]) < 1e-9 * (1 + abs(z[0]))))
    if nper < 1 or nu % nper:
        return None
    return nu // nper


class WallGuess:
    """Online-trained initial guess for rbc3d_no_slip_wall: the learned
    spectral operator (device) and the MLP correction of its remainder; the
    history projection is kept as a comparison arm."""

    def __init__(self, lib, ctx, wall, width=512, depth=4, seed=0, history=48, buffer_steps=32, nlap=2, tau=1e-7):
        self.nlap = nlap
        self.mlp = MLP(lib, 3 * (nlap + 2), width, depth, 3, seed)
        self.fn = self.mlp.fn
        self.ctx = ctx
        self.frames = vertex_frames(wall)
        self.lap = vertex_smoother(wall)
        self.nv = wall.ndof // 3
        self.glb = wall.glb - 1
        self.K = history
        self.hist_b, self.hist_x = [], []
        self.buf = []
        self.buffer_steps = buffer_steps
        self.k = None  # rms(e) / rms(r_s), set from data
        self.lap_scale = None
        self.pairs = 0
        nring = ring_count(wall)
        if nring is None:
            raise RBC3DError(1, "the learned spectral operator needs a tube wall meshed as a stack of rings")
        self._ok(self.fn["rbc3d_wall_spectral_init"](ctx.h, nring, tau, 0), "rbc3d_wall_spectral_init")

    def _ok(self, st, what):
        if st:
            raise RBC3DError(st, f"{what}: {self.ctx.L.fn['last_error'](self.ctx.h).decode()}")

    def _to_local(self, v3):  # (nv,3) -> (nv,3) in the local frame
        return np.einsum("vac,vc->va", self.frames, v3)

    def _to_global(self, l3):
        return np.einsum("vac,va->vc", self.frames, l3)

    @staticmethod
    def _rms(a):
        return np.sqrt(np.mean(a * a)) + 1e-300

    def project(self, b):
        """History arm: least squares over the last K right-hand sides,
        (x_h, r_h) (zeros if no history)."""
        if not self.hist_b:
            return np.zeros_like(b), b.copy()
        Bm = np.stack(self.hist_b, 1)
        Xm = np.stack(self.hist_x, 1)
        c, *_ = np.linalg.lstsq(Bm, b, rcond=None)
        return Xm @ c, b - Bm @ c

    def spectral(self, b):
        """Spectral operator: (x_s, r_s), the prediction for b and the part of
        b outside the learned span."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        xs, rs = np.empty_like(b), np.empty_like(b)
        self._ok(self.fn["rbc3d_wall_spectral_predict"](self.ctx.h, _ptr(b), _ptr(xs), _ptr(rs)),
                 "rbc3d_wall_spectral_predict")
        return xs, rs

    def basis_sizes(self):
        nm = C.c_int()
        self._ok(self.fn["rbc3d_wall_spectral_size"](self.ctx.h, C.byref(nm), None, None), "rbc3d_wall_spectral_size")
        nb = np.zeros(nm.value, dtype=np.int32)
        pairs = C.c_longlong()
        self._ok(self.fn["rbc3d_wall_spectral_size"](self.ctx.h, C.byref(nm), nb.ctypes.data_as(C.POINTER(C.c_int)),
                                                     C.byref(pairs)), "rbc3d_wall_spectral_size")
        return nb, pairs.value

    def features(self, r, xs):
        g = r.reshape(self.nv, 3)
        rl = self._to_local(g)
        sr = self._rms(rl)
        cols = [rl / sr]
        lap = []
        for _ in range(self.nlap):
            g = self.lap @ g
            lap.append(self._to_local(g) / sr)
        if self.lap_scale is None:  # fixed per-order scales: the stencil map stays linear in r
            self.lap_scale = [self._rms(l3) for l3 in lap]
        cols += [l3 / c for l3, c in zip(lap, self.lap_scale)]
        xl = self._to_local(xs.reshape(self.nv, 3))
        cols.append(xl / self._rms(xl))
        return np.concatenate(cols, axis=1), sr

    def record(self, b, x):
        """A solved step (A x = b to the solve tolerance): a training pair for
        the network (from the spectral prediction made before the pair is
        learned), then the pair for the spectral operator and the history."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        if self.pairs >= 2:
            xs, rs = self.spectral(b)
            X, sr = self.features(rs, xs)
            el = self._to_local((x - xs).reshape(self.nv, 3)) / sr
            k = self._rms(el)
            self.k = k if self.k is None else 0.8 * self.k + 0.2 * k
            self.buf.append((X.astype(np.float32), el))
            if len(self.buf) > self.buffer_steps:
                self.buf.pop(0)
        self.learn(x)
        self.pairs += 1
        self.hist_b.append(b.copy())
        self.hist_x.append(x.copy())
        if len(self.hist_b) > self.K:
            self.hist_b.pop(0)
            self.hist_x.pop(0)

    def learn(self, x):
        """The spectral operator learns the exact pair (A x, x), A x formed on
        the device with the FP64 wall operator."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._ok(self.fn["rbc3d_wall_spectral_add"](self.ctx.h, _ptr(x), None), "rbc3d_wall_spectral_add")

    def train(self, iters=10, batch=4096, lr=1e-3, rng=None):
        if not self.buf:
            return None
        rng = rng or np.random.default_rng(0)
        X = np.concatenate([a for a, _ in self.buf])
        T = np.concatenate([t for _, t in self.buf]) / self.k
        loss = None
        for _ in range(iters):
            idx = rng.integers(0, X.shape[0], min(batch, X.shape[0]))
            loss = self.mlp.train_step(X[idx], T[idx], lr)
        return loss

    def predict(self, b):
        """(x_s, e_hat): the spectral prediction and the network's correction."""
        xs, rs = self.spectral(b)
        if self.k is None:
            return xs, np.zeros_like(b)
        X, sr = self.features(rs, xs)
        y = self.mlp.forward(X)
        return xs, np.ascontiguousarray(self._to_global(y.astype(np.float64) * (self.k * sr)).reshape(-1))

    def rhs(self, ctx, prec):
        # the solves' right-hand side is FP64 in every mode (the mixed-precision
        # solves form b and their residuals with the FP64 operator)
        b = np.empty(3 * self.nv)
        st = self.fn["rbc3d_wall_rhs"](ctx.h, FP64, b.ctypes.data_as(_dp))
        if st:
            raise RBC3DError(st, "rbc3d_wall_rhs")
        return b

    def solve(self, ctx, wall, rtol, max_it, restart, prec, mode="learned"):
        """One NoSlipWall step from the guess `mode`: "learned" (spectral
        operator + network, least-squares combination), "spectral" (the
        spectral operator alone, predicted on the device: guess mode 4),
        "preconditioned" (the spectral operator as x0 and as the right
        preconditioner of GMRES: guess mode 5) or "history" (the history
        projection, scaled).  Returns (stats, accepted, total_ms, b); with
        accepted False the plain solve (zero increment) was run."""
        t0 = time.perf_counter()
        f0 = ctx.get_wall_density(wall.nvert)
        b = None
        if self.pairs:
            if mode in ("spectral", "preconditioned"):
                st, code = ctx.no_slip_wall(rtol, max_it, restart, prec, check=False,
                                            guess_mode=4 if mode == "spectral" else 5)
            else:
                b = self.rhs(ctx, prec)
                if mode == "learned":
                    xs, eh = self.predict(b)
                    st, code = ctx.no_slip_wall(rtol, max_it, restart, prec, guess=np.concatenate([xs, eh]),
                                                check=False, guess_mode=3)
                else:
                    xh, _ = self.project(b)
                    st, code = ctx.no_slip_wall(rtol, max_it, restart, prec, guess=xh, check=False, guess_mode=2)
            if code == 0 and st.converged and st.rnorm <= rtol * st.bnorm:
                return st, True, (time.perf_counter() - t0) * 1e3, b
            ctx.set_wall_density(f0)  # fallback: the plain guess
        st, code = ctx.no_slip_wall(rtol, max_it, restart, prec, check=False)
        return st, False, (time.perf_counter() - t0) * 1e3, b
