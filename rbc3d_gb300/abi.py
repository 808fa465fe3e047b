"""ctypes binding of the C ABI in include/rbc3d_gpu.h.

``Library(path, prefix)`` binds one shared library exporting the ABI under a
symbol prefix.  The product library is ``librbc3d_gb300.so`` (prefix
``rbc3d_``).  The test suite binds the FP64 CPU oracle through the same class
with the prefix ``rbc3d_oracle_``; product code never does.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

MAX_CELLTYPES = 8
FP64, FP32C, FP32M, FP32D = 0, 1, 2, 3
TLIST_RBC, TLIST_WALL, TLIST_RAW = 0, 1, 2
TERM_REAL, TERM_CORR, TERM_LINEAR, TERM_PME, TERM_WALLS = 1, 2, 4, 8, 16
TERM_ALL = 31
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_TIMEOUT", 4: "ERR_NOCONV",
          5: "ERR_OVERFLOW", 6: "ERR_STATE", 7: "ERR_NOMEM"}


class Params(C.Structure):
    _fields_ = [("Lb", C.c_double * 3), ("alpha", C.c_double), ("rc", C.c_double),
                ("eps", C.c_double), ("Nb", C.c_int * 3), ("P", C.c_int),
                ("nlat", C.c_int), ("nlon", C.c_int), ("ncelltypes", C.c_int),
                ("viscRat", C.c_double * MAX_CELLTYPES), ("vBkg", C.c_double * 3)]


class Counts(C.Structure):
    _fields_ = [("pairs_within_rc", C.c_longlong), ("nbr_items", C.c_longlong),
                ("nearsing_items", C.c_longlong), ("self_items", C.c_longlong),
                ("wall_pairs", C.c_longlong), ("wall_duffy", C.c_longlong),
                ("nbr_overflow", C.c_int), ("kernel_launches", C.c_longlong),
                ("screen_misses", C.c_longlong), ("near_replays", C.c_longlong),
                ("near_projections", C.c_longlong)]


class SolveOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("max_it", C.c_int), ("restart", C.c_int),
                ("prec", C.c_int), ("guess", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("rnorm0", C.c_double),
                ("rnorm", C.c_double), ("bnorm", C.c_double), ("ms", C.c_double),
                ("matvecs", C.c_int), ("refinements", C.c_int)]


class RBC3DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def make_params(d: dict) -> Params:
    p = Params()
    p.Lb[:] = [float(v) for v in d["Lb"]]
    p.alpha = float(d["alpha"]); p.rc = float(d["rc"]); p.eps = float(d.get("eps", 1e-6))
    p.Nb[:] = [int(v) for v in d["Nb"]]
    p.P = int(d["P"]); p.nlat = int(d["nlat"]); p.nlon = int(d["nlon"])
    vr = list(d.get("viscRat", [1.0]))
    p.ncelltypes = int(d.get("ncelltypes", len(vr)))
    p.viscRat[:len(vr)] = [float(v) for v in vr]
    p.vBkg[:] = [float(v) for v in d.get("vBkg", [0.0, 0.0, 0.0])]
    return p


# Exported C-ABI entry points (name, restype, argtypes).  Shared between the
# product library and the oracle.
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
SIGNATURES = [
    ("abi_version", C.c_int, []),
    ("ewald_prms", C.c_int, [C.c_double, C.c_double, _dp, C.c_int, _dp, _ip]),
    ("create", C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    ("destroy", C.c_int, [_vp]),
    ("last_error", C.c_char_p, [_vp]),
    ("set_cell_grid", C.c_int, [_vp, _dp, _dp, _dp]),
    ("set_cells", C.c_int, [_vp, C.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("set_cell_density", C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    ("set_walls", C.c_int, [_vp, C.c_int, C.c_int, _dp, _ip, _ip]),
    ("set_wall_density", C.c_int, [_vp, _dp]),
    ("get_wall_density", C.c_int, [_vp, _dp]),
    ("set_raw_targets", C.c_int, [_vp, C.c_int, _dp]),
    ("num_targets", C.c_int, [_vp, C.c_int]),
    ("add_int_on_rbcs", C.c_int, [_vp, C.c_int, C.c_double, C.c_double, C.c_int, _dp]),
    ("add_int_on_walls", C.c_int, [_vp, C.c_int, C.c_double, C.c_int, _dp]),
    ("prepare_sing_int_on_wall", C.c_int, [_vp]),
    ("pme_distrib_source", C.c_int, [_vp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int]),
    ("pme_transform", C.c_int, [_vp]),
    ("pme_add_interp_vel", C.c_int, [_vp, C.c_int, _dp]),
    ("matvec", C.c_int, [_vp, C.c_int, C.c_double, C.c_double, C.c_uint, C.c_int, _dp]),
    ("compute_wall_residual_vel", C.c_int, [_vp, C.c_int, _dp]),
    ("no_slip_wall", C.c_int, [_vp, C.POINTER(SolveOpts), _dp, C.POINTER(SolveStats)]),
    ("wall_matmult", C.c_int, [_vp, C.c_int, _dp, _dp]),
    ("calc_velocity_field", C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    ("get_counts", C.c_int, [_vp, C.POINTER(Counts)]),
    ("cell_dof", C.c_int, [_vp, C.c_int]),
    ("solve_rbc_vel", C.c_int, [_vp, C.POINTER(SolveOpts), C.c_int, _dp, _dp, C.POINTER(SolveStats)]),
    ("set_ref_cells", C.c_int, [_vp, C.c_int, _dp, _dp, _dp, _dp]),
    ("cell_geometry", C.c_int, [_vp, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    ("shell_res_force", C.c_int, [_vp, C.c_int, _ip, _dp, _dp]),
    ("intra_cell_repulsion", C.c_int, [_vp, C.c_int, _dp, _dp, _dp, C.c_double, _dp, _ip]),
    ("inter_cell_repulsion", C.c_int, [_vp, C.c_double, C.c_double, C.c_int, _dp, _dp, _ip]),
]
# Device-timing entry points of the GPU library only.
GPU_SIGNATURES = [
    ("set_profiling", C.c_int, [_vp, C.c_int]),
    ("stage_times", C.c_int, [_vp, _dp, _ip]),
    ("timer_start", C.c_int, [_vp]),
    ("timer_stop", C.c_int, [_vp, _dp]),
    ("host_alloc", C.c_int, [C.c_ulonglong, C.POINTER(C.c_void_p)]),
    ("host_free", C.c_int, [_vp]),
    ("fma_peak", C.c_int, [C.c_int, _dp]),
    ("h2d_bandwidth", C.c_int, [C.c_ulonglong, _dp]),
    ("set_cells_x", C.c_int, [_vp, C.c_int, _ip, C.c_int, _dp]),
    ("set_cell_density_x", C.c_int, [_vp, C.c_int, _dp, _dp]),
]
STAGES = ["pair", "self", "near", "linear", "walls", "pme_spread", "pme_fft_infl", "pme_gather"]


def _ptr(a, dtype=np.float64):
    if a is None:
        return None
    assert a.dtype == dtype and a.flags.c_contiguous, (a.dtype, a.flags)
    ct = C.c_double if dtype == np.float64 else C.c_int
    return a.ctypes.data_as(C.POINTER(ct))


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


class Library:
    def __init__(self, path: str, prefix: str):
        self.path = path
        self.prefix = prefix
        self.lib = C.CDLL(path)
        self.fn = {}
        for name, res, args in SIGNATURES:
            f = getattr(self.lib, prefix + name)
            f.restype = res
            f.argtypes = args
            self.fn[name] = f
        for name, res, args in GPU_SIGNATURES:
            f = getattr(self.lib, prefix + name, None)
            if f is not None:
                f.restype = res
                f.argtypes = args
                self.fn[name] = f

    def h2d_bandwidth(self, nbytes):
        """Measured pinned host-to-device copy bandwidth, GB/s."""
        t = C.c_double()
        st = self.fn["h2d_bandwidth"](int(nbytes), C.byref(t))
        if st:
            raise RBC3DError(st, "h2d_bandwidth")
        return t.value

    def fma_peak(self, prec):
        t = C.c_double()
        st = self.fn["fma_peak"](prec, C.byref(t))
        if st:
            raise RBC3DError(st, "fma_peak")
        return t.value

    def pinned(self, shape, dtype=np.float64):
        """numpy array in page-locked host memory (freed with the library)."""
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        st = self.fn["host_alloc"](n, C.byref(p))
        if st:
            raise RBC3DError(st, "host_alloc")
        self._pinned = getattr(self, "_pinned", [])
        self._pinned.append(p)
        buf = (C.c_char * n).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    def ewald_prms(self, alpha, eps, Lb, P):
        rc = C.c_double()
        Nb = (C.c_int * 3)()
        Lbv = (C.c_double * 3)(*Lb)
        self.fn["ewald_prms"](alpha, eps, Lbv, P, C.byref(rc), Nb)
        return rc.value, list(Nb)


class Context:
    """One rbc3d context (one GPU stream, or one oracle instance)."""

    def __init__(self, lib: Library, params: dict):
        self.L = lib
        self.params = params
        self.h = C.c_void_p()
        self._keep = []
        self._check(lib.fn["create"](C.byref(make_params(params)), C.byref(self.h)), nullctx=True)

    def _check(self, st, nullctx=False):
        if st != 0:
            msg = "" if nullctx else self.L.fn["last_error"](self.h).decode()
            raise RBC3DError(st, msg)

    def close(self):
        if self.h:
            self.L.fn["destroy"](self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- surfaces
    def set_cell_grid(self, th, phi, w):
        """The cell grid alone (RBC_Create's colatitudes, longitudes, weights)."""
        th, phi, w = f64(th), f64(phi), f64(w)
        self._check(self.L.fn["set_cell_grid"](self.h, _ptr(th), _ptr(phi), _ptr(w)))
        self._grid = (th.copy(), phi.copy(), w.copy())

    def set_cells(self, cells):
        th, phi, w = f64(cells.th), f64(cells.phi), f64(cells.w)
        # RbcPolarPatch_Create and the grid tables: once per grid, not per position update
        grid = getattr(self, "_grid", None)
        if grid is None or not all(a.shape == b.shape and np.array_equal(a, b) for a, b in zip(grid, (th, phi, w))):
            self._check(self.L.fn["set_cell_grid"](self.h, _ptr(th), _ptr(phi), _ptr(w)))
            self._grid = (th.copy(), phi.copy(), w.copy())
        ct = i32(cells.celltype)
        arrs = [f64(cells.x), f64(cells.a3), f64(cells.detJ), f64(cells.area), f64(cells.meshSize),
                f64(cells.spl_x), f64(cells.spl_a3), f64(cells.spl_detJ)]
        self._check(self.L.fn["set_cells"](self.h, int(cells.ncell), _ptr(ct, np.int32),
                                           *[_ptr(a) for a in arrs]))

    def set_cells_x(self, cells, nlat0, x=None):
        """Cells from positions alone (GPU library): geometry and spline tables
        derived on the device as RBC_ComputeGeometry + Rbc_BuildSurfaceSource
        (degree < nlat0).  `cells` supplies the grid and cell types; x (3, N)
        defaults to cells.x."""
        th, phi, w = f64(cells.th), f64(cells.phi), f64(cells.w)
        grid = getattr(self, "_grid", None)
        if grid is None or not all(a.shape == b.shape and np.array_equal(a, b) for a, b in zip(grid, (th, phi, w))):
            self._check(self.L.fn["set_cell_grid"](self.h, _ptr(th), _ptr(phi), _ptr(w)))
            self._grid = (th.copy(), phi.copy(), w.copy())
        ct = i32(cells.celltype)
        x = f64(cells.x if x is None else x)
        self._check(self.L.fn["set_cells_x"](self.h, int(cells.ncell), _ptr(ct, np.int32), int(nlat0), _ptr(x)))

    def set_cell_density_x(self, nlat0, f=None, g=None):
        """Raw densities alone (GPU library): the f detJ / g detJ tables derived
        on the device as Rbc_BuildSurfaceSource (degree < nlat0)."""
        f, g = f64(f), f64(g)
        self._check(self.L.fn["set_cell_density_x"](self.h, int(nlat0), _ptr(f), _ptr(g)))

    def set_cell_density(self, f=None, g=None, spl_F=None, spl_G=None):
        f, g, sF, sG = f64(f), f64(g), f64(spl_F), f64(spl_G)
        self._check(self.L.fn["set_cell_density"](self.h, _ptr(f), _ptr(g), _ptr(sF), _ptr(sG)))

    def set_walls(self, wall):
        x, e2v, glb = f64(wall.x), i32(wall.e2v), i32(wall.glb)
        self._check(self.L.fn["set_walls"](self.h, int(wall.nvert), int(wall.nele), _ptr(x),
                                           _ptr(e2v, np.int32), _ptr(glb, np.int32)))

    def set_wall_density(self, f):
        f = f64(f)
        self._check(self.L.fn["set_wall_density"](self.h, _ptr(f)))

    def get_wall_density(self, nvert):
        out = np.zeros((3, nvert))
        self._check(self.L.fn["get_wall_density"](self.h, _ptr(out)))
        return out

    def set_raw_targets(self, x):
        x = f64(x)
        self._check(self.L.fn["set_raw_targets"](self.h, int(x.shape[1]), _ptr(x)))

    def num_targets(self, tlist):
        return self.L.fn["num_targets"](self.h, tlist)

    def _vout(self, tlist, v):
        n = self.num_targets(tlist)
        if n < 0:
            raise RBC3DError(1, f"bad target list {tlist}")
        if v is None:
            v = np.zeros((3, n))
        assert v.dtype == np.float64 and v.flags.c_contiguous
        return v

    # ---- L2
    def add_int_on_rbcs(self, tlist, c1, c2, prec=FP64, v=None):
        v = self._vout(tlist, v)
        self._check(self.L.fn["add_int_on_rbcs"](self.h, tlist, c1, c2, prec, _ptr(v)))
        return v

    def add_int_on_walls(self, tlist, c1, prec=FP64, v=None):
        v = self._vout(tlist, v)
        self._check(self.L.fn["add_int_on_walls"](self.h, tlist, c1, prec, _ptr(v)))
        return v

    def prepare_sing_int_on_wall(self):
        self._check(self.L.fn["prepare_sing_int_on_wall"](self.h))

    def pme(self, tlist, c1, c2, cells=True, walls=False, prec=FP64, v=None):
        v = self._vout(tlist, v)
        self._check(self.L.fn["pme_distrib_source"](self.h, c1, c2, int(cells), int(walls), prec))
        self._check(self.L.fn["pme_transform"](self.h))
        self._check(self.L.fn["pme_add_interp_vel"](self.h, tlist, _ptr(v)))
        return v

    def matvec(self, tlist, c1, c2, terms=TERM_ALL, prec=FP64, v=None, device_only=False):
        if device_only:
            self._check(self.L.fn["matvec"](self.h, tlist, c1, c2, terms, prec, None))
            return None
        v = self._vout(tlist, v)
        self._check(self.L.fn["matvec"](self.h, tlist, c1, c2, terms, prec, _ptr(v)))
        return v

    # ---- device timing (GPU library)
    def set_profiling(self, on):
        self._check(self.L.fn["set_profiling"](self.h, int(on)))

    def stage_times(self):
        ms = (C.c_double * 8)()
        cnt = (C.c_int * 8)()
        self._check(self.L.fn["stage_times"](self.h, ms, cnt))
        return {s: (ms[i], cnt[i]) for i, s in enumerate(STAGES)}

    def timer_start(self):
        self._check(self.L.fn["timer_start"](self.h))

    def timer_stop(self):
        ms = C.c_double()
        self._check(self.L.fn["timer_stop"](self.h, C.byref(ms)))
        return ms.value

    # ---- L3
    def calc_velocity_field(self, tlist, prec=FP64):
        v = self._vout(tlist, None)
        self._check(self.L.fn["calc_velocity_field"](self.h, tlist, prec, _ptr(v)))
        return v

    def compute_wall_residual_vel(self, prec=FP64):
        v = self._vout(TLIST_WALL, None)
        self._check(self.L.fn["compute_wall_residual_vel"](self.h, prec, _ptr(v)))
        return v

    def wall_matmult(self, u, prec=FP64):
        u = f64(u)
        y = np.zeros_like(u)
        self._check(self.L.fn["wall_matmult"](self.h, prec, _ptr(u), _ptr(y)))
        return y

    def no_slip_wall(self, rtol, max_it, restart=30, prec=FP64, guess=None, check=True, guess_mode=1):
        o = SolveOpts(rtol=rtol, max_it=max_it, restart=restart, prec=prec,
                      guess=0 if (guess is None and guess_mode not in (4, 5)) else guess_mode)
        st = SolveStats()
        g = f64(guess)
        code = self.L.fn["no_slip_wall"](self.h, C.byref(o), _ptr(g), C.byref(st))
        if check and code not in (0, 4):
            self._check(code)
        return st, code

    def solve_rbc_vel(self, nlat0, rtol=1e-11, max_it=200, restart=30, sol=None, check=True, prec=FP64):
        """Solve_RBC_Vel: returns (sol, v (N,3) as (3,N) SoA, stats, code).  sol, when
        given, is the warm start (the reference keeps its solution vector
        between calls, KSPSetInitialGuessNonzero).  prec FP32C / FP32M: the
        mixed-precision solve (FP32 operator inside, FP64 residual)."""
        n = self.L.fn["cell_dof"](self.h, nlat0)
        x = np.zeros(n) if sol is None else f64(sol).copy()
        o = SolveOpts(rtol=rtol, max_it=max_it, restart=restart, prec=prec, guess=0 if sol is None else 1)
        st = SolveStats()
        N = self.L.fn["num_targets"](self.h, 0)
        v = np.zeros(3 * N)
        code = self.L.fn["solve_rbc_vel"](self.h, C.byref(o), nlat0, _ptr(x), _ptr(v), C.byref(st))
        if check and code not in (0, 4):
            self._check(code)
        return x, v.reshape(3, N), st, code

    def set_ref_cells(self, xref, ES, ED, EB):
        """Reference cells (one per cell type, positions 3 x ntypes*nlat*nlon) and
        their moduli for Shell_ResForce."""
        xref = f64(xref)
        ES, ED, EB = (f64(np.atleast_1d(v)) for v in (ES, ED, EB))
        nt = ES.size
        self._check(self.L.fn["set_ref_cells"](self.h, nt, _ptr(xref), _ptr(ES), _ptr(ED), _ptr(EB)))

    def cell_geometry(self, x, ncell):
        """RBC_ComputeGeometry: (a3 (3,N), detJ (N,), area (ncell,), vol (ncell,))."""
        x = f64(x)
        N = x.shape[1]
        a3, dj, ar, vo = np.zeros((3, N)), np.zeros(N), np.zeros(ncell), np.zeros(ncell)
        self._check(self.L.fn["cell_geometry"](self.h, ncell, _ptr(x), _ptr(a3), _ptr(dj), _ptr(ar), _ptr(vo)))
        return a3, dj, ar, vo

    def shell_res_force(self, x, celltype):
        """Shell_ResForce of every cell at positions x: f (3, N), Cartesian."""
        x = f64(x)
        ct = i32(celltype)
        f = np.zeros_like(x)
        self._check(self.L.fn["shell_res_force"](self.h, int(ct.size), _ptr(ct, np.int32), _ptr(x), _ptr(f)))
        return f

    def intra_cell_repulsion(self, x, a3, area, force_coef, f):
        """AddIntraCellRepulsionForce: adds to f (3, N) in place; returns the
        number of points pushed."""
        x, a3, area = f64(x), f64(a3), f64(area)
        assert f.dtype == np.float64 and f.flags.c_contiguous
        n = C.c_int(0)
        self._check(self.L.fn["intra_cell_repulsion"](self.h, int(area.size), _ptr(x), _ptr(a3), _ptr(area),
                                                      float(force_coef), _ptr(f), C.byref(n)))
        return n.value

    def inter_cell_repulsion(self, eps_dist, visc_thresh, rigidsep=False):
        """InterCellRepulsion on the context's cells and wall: (moved positions
        (3, N), minimum surface separation, points moved)."""
        n = self.num_targets(0)
        x = np.zeros((3, max(n, 0)))
        dmin = C.c_double()
        nm = C.c_int()
        self._check(self.L.fn["inter_cell_repulsion"](self.h, float(eps_dist), float(visc_thresh), int(rigidsep),
                                                      _ptr(x), C.byref(dmin), C.byref(nm)))
        return x, dmin.value, nm.value

    def counts(self):
        c = Counts()
        self._check(self.L.fn["get_counts"](self.h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in Counts._fields_}
