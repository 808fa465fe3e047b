"""Host-side FP64 producers of the matvec inputs.

These replace, for analytically described cells, the geometry and spline
builders of RBC3D that run before every matvec:

* ``RBC_Create`` grid (Gauss colatitudes x uniform longitudes, weights with the
  2*pi/nlon factor), ModRbc.F90:44-104;
* ``RBC_MakeBiConcave`` (Evans-Fung / Pozrikidis shape), ModRbc.F90:368-398;
* ``RBC_ComputeGeometry`` outputs used by the matvec: unit normal a3,
  detJ = |x_theta x x_phi| / sin(theta), area, meshSize, ModRbc.F90:404-509
  (here from the analytic surface derivatives instead of an SH gradient);
* ``Spline_Build_on_Sphere`` (doubled-sphere bicubic Hermite tables with FFT
  derivatives, Nyquist mode zeroed), ModSpline.F90:121-143 and
  ModFFT.F90:25-93, fed from samples on the equiangular grid of
  ``ShSynthEqu`` (nlat+1 colatitudes including both poles), ModRbc.F90:716-807;
* ``Wall_ComputeGeometry``-ready Tri3 tube meshes with the periodic duplicate
  vertex map of ``Wall_Build_V2V`` / ``GlobData_Init``, ModWall.F90:66-113,
  ModData.F90:47-58.

Everything is seeded (``numpy.random.default_rng``) so the oracle and the GPU
consume bit-identical inputs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ALPH_BICONCAVE = 1.3858189  # ModRbc.F90:375


# ---------------------------------------------------------------------------
# Ewald parameters
def ewald_s(eps: float) -> float:
    """Fixed-point iteration of SetEwaldPrms (ModConf.F90:364-369)."""
    s = 1.0
    for _ in range(10):
        s = 0.75 * math.sqrt(math.pi) * eps / (s ** 3 + 1.5 * s + 0.75 / s)
        s = math.sqrt(-math.log(s))
    return s


def alpha_for_cutoff(rc: float, eps: float) -> float:
    """alpha such that SetEwaldPrms derives the cut-off rc from eps."""
    s = ewald_s(eps)
    return math.pi * (rc / s) ** 2


# ---------------------------------------------------------------------------
# Cell grid
def gauss_grid(nlat: int, nlon: int):
    """Gauss-Legendre colatitudes (increasing), longitudes and weights
    w = gauss_weight * 2*pi/nlon (RBC_Create, ModRbc.F90:92-94)."""
    x, wg = np.polynomial.legendre.leggauss(nlat)
    th = np.arccos(x)[::-1].copy()
    wg = wg[::-1].copy()
    phi = np.arange(nlon) * (2 * np.pi / nlon)
    w = (2 * np.pi / nlon) * wg
    return th, phi, w


def _biconcave_profile(th, rc=1.0):
    """r(th), z(th) and derivatives of RBC_MakeBiConcave (ModRbc.F90:368-398)."""
    a = ALPH_BICONCAVE
    s, c = np.sin(th), np.cos(th)
    P = 0.207 + 2.003 * s ** 2 - 1.123 * s ** 4
    dP = 4.006 * s - 4.492 * s ** 3
    r = rc * a * s
    z = rc * 0.5 * a * P * c
    dr = rc * a * c
    dz = rc * 0.5 * a * (dP * c * c - P * s)
    return r, z, dr, dz


def biconcave_surface(th, phi, R, xc, rc=1.0):
    """Position, unit normal and detJ of a rotated, translated biconcave cell
    at colatitudes th (any grid) and longitudes phi.  Arrays (nth, nphi, 3)."""
    r, z, dr, dz = _biconcave_profile(th, rc)
    cp, sp = np.cos(phi), np.sin(phi)
    X = np.stack([r[:, None] * cp[None, :], r[:, None] * sp[None, :],
                  np.broadcast_to(z[:, None], (th.size, phi.size))], axis=-1)
    nrm = np.sqrt(dr ** 2 + dz ** 2)
    N = np.stack([-dz[:, None] * cp[None, :] / nrm[:, None],
                  -dz[:, None] * sp[None, :] / nrm[:, None],
                  np.broadcast_to((dr / nrm)[:, None], (th.size, phi.size))], axis=-1)
    detJ = np.broadcast_to((rc * ALPH_BICONCAVE * nrm)[:, None], (th.size, phi.size)).copy()
    X = X @ R.T + xc
    N = N @ R.T
    return X, N, detJ


def sphere_surface(th, phi, radius, xc):
    """Sphere of given radius (RBC_MakeSphere, ModRbc.F90:147-171): position,
    unit normal and detJ = |x_th x x_phi| / sin(th) = radius^2."""
    st, ct = np.sin(th), np.cos(th)
    cp, sp = np.cos(phi), np.sin(phi)
    N = np.stack([st[:, None] * cp[None, :], st[:, None] * sp[None, :],
                  np.broadcast_to(ct[:, None], (th.size, phi.size))], axis=-1)
    X = radius * N + xc
    detJ = np.full((th.size, phi.size), radius * radius)
    return X, N.copy(), detJ


def make_sphere_cells(centres, radius=1.0, nlat=25, nlon=50):
    """Spherical cells (zero densities) in the C-ABI layout."""
    th, phi, w = gauss_grid(nlat, nlon)
    the = equi_theta(nlat)
    X, A3, DJ, SX, SA, SD, areas, msz = [], [], [], [], [], [], [], []
    for c in centres:
        x, n, dj = sphere_surface(th, phi, radius, c)
        xe, ne, dje = sphere_surface(the, phi, radius, c)
        X.append(x); A3.append(n); DJ.append(dj[..., None])
        SX.append(spline_on_sphere(xe)); SA.append(spline_on_sphere(ne)); SD.append(spline_on_sphere(dje[..., None]))
        area = float(np.sum(dj * w[:, None]))
        areas.append(area)
        msz.append(math.sqrt(area / nlat ** 2))
    nc = len(centres)
    cells = Cells(nlat=nlat, nlon=nlon, th=th, phi=phi, w=w, ncell=nc, celltype=np.zeros(nc, dtype=np.int32),
                  x=_to_points(np.array(X)), a3=_to_points(np.array(A3)), detJ=_to_points(np.array(DJ))[0].copy(),
                  area=np.array(areas), meshSize=np.array(msz), spl_x=np.ascontiguousarray(np.array(SX)),
                  spl_a3=np.ascontiguousarray(np.array(SA)), spl_detJ=np.ascontiguousarray(np.array(SD)),
                  centres=np.asarray(centres))
    cells.f = np.zeros_like(cells.x)
    cells.g = np.zeros_like(cells.x)
    cells.spl_F = np.zeros((nc, 4, 3, nlon, 2 * nlat))
    cells.spl_G = np.zeros_like(cells.spl_F)
    return cells


def sphere_uniform_spline(cells, fvec, radius=1.0):
    """FdetJ spline of a constant density fvec on spherical cells."""
    the = equi_theta(cells.nlat)
    v = np.broadcast_to(np.asarray(fvec) * radius * radius, (the.size, cells.nlon, 3)).copy()
    tab = spline_on_sphere(v)
    return np.ascontiguousarray(np.broadcast_to(tab, (cells.ncell,) + tab.shape).copy())


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


# ---------------------------------------------------------------------------
# Real spherical-harmonic fields
def _assoc_legendre(lmax, x):
    """Orthonormalised associated Legendre functions Nbar_lm(x) for m<=l<=lmax,
    such that Y_lm = Nbar_lm(cos th) * {1, sqrt2 cos(m phi), sqrt2 sin(m phi)} is
    orthonormal on the unit sphere.  Own recursion (stable for small lmax)."""
    x = np.asarray(x, dtype=np.float64)
    s = np.sqrt(np.maximum(0.0, 1 - x * x))
    P = {}
    P[(0, 0)] = np.full_like(x, math.sqrt(1 / (4 * math.pi)))
    for m in range(1, lmax + 1):
        P[(m, m)] = -math.sqrt((2 * m + 1) / (2 * m)) * s * P[(m - 1, m - 1)]
    for m in range(0, lmax):
        P[(m + 1, m)] = math.sqrt(2 * m + 3) * x * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4 * l * l - 1) / (l * l - m * m))
            b = math.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
            P[(l, m)] = a * (x * P[(l - 1, m)] - b * P[(l - 2, m)])
    return P


def random_sh_coeffs(rng, lmax=6, lmin=1):
    """Coefficients a_lm ~ N(0, l^-2) of a real SH field, l in [lmin, lmax]."""
    out = {}
    for l in range(lmin, lmax + 1):
        sd = 1.0 / l
        for m in range(-l, l + 1):
            out[(l, m)] = rng.normal(0.0, sd)
    return out


_SH_BASIS = {}


def _sh_basis(keys, th, phi):
    """Y_lm on the (th, phi) grid for the ordered (l, m) keys, cached per grid."""
    ck = (tuple(keys), th.size, phi.size, float(th[0]), float(th[-1]), float(phi[-1]))
    B = _SH_BASIS.get(ck)
    if B is None:
        lmax = max(l for l, _ in keys)
        P = _assoc_legendre(lmax, np.cos(th))
        B = np.empty((len(keys), th.size, phi.size))
        for i, (l, m) in enumerate(keys):
            am = abs(m)
            if m == 0:
                ang = np.ones_like(phi)
            elif m > 0:
                ang = math.sqrt(2) * np.cos(m * phi)
            else:
                ang = math.sqrt(2) * np.sin(am * phi)
            B[i] = P[(l, am)][:, None] * ang[None, :]
        _SH_BASIS[ck] = B
    return B


def sh_eval(coeffs, th, phi):
    keys = list(coeffs)
    B = _sh_basis(keys, th, phi)
    a = np.array([coeffs[k] for k in keys])
    return np.tensordot(a, B, axes=(0, 0))


# ---------------------------------------------------------------------------
# Splines
def fft_diff(u, axis):
    """FFT_Diff of ModFFT.F90:25-93 along one axis (domain mapped to 2*pi):
    modes k < n/2 times i k, mode n/2 (integer division, odd n too) zeroed."""
    n = u.shape[axis]
    U = np.fft.rfft(u, axis=axis)
    k = np.arange(n // 2 + 1, dtype=np.float64)
    k[-1] = 0.0
    shape = [1] * u.ndim
    shape[axis] = k.size
    U = U * (1j * k).reshape(shape)
    return np.fft.irfft(U, n=n, axis=axis)


def spline_on_sphere(v):
    """Spline_Build_on_Sphere (ModSpline.F90:121-143).

    v: values on the equiangular grid, shape (nlat+1, nlon, nvar), rows at
    th_i = i*pi/nlat (both poles included).  Returns the table
    (4, nvar, nlon, 2*nlat) = u, u1, u2, u12 each Fortran-ordered (m, n, nvar).
    """
    nlat = v.shape[0] - 1
    nlon = v.shape[1]
    m = 2 * nlat
    u = np.empty((m, nlon, v.shape[2]))
    u[:nlat] = v[:nlat]
    for i in range(nlat):
        u[nlat + i] = np.roll(v[nlat - i], -(nlon // 2), axis=0)
    u1 = fft_diff(u, 0)
    u2 = fft_diff(u, 1)
    u12 = fft_diff(u1, 1)
    tab = np.stack([u, u1, u2, u12])          # (4, m, n, nvar)
    return np.ascontiguousarray(tab.transpose(0, 3, 2, 1))  # (4, nvar, n, m)


def spline_on_sphere_batch(V):
    """spline_on_sphere over a stack of cells: V (ncell, nlat+1, nlon, nvar)
    -> (ncell, 4, nvar, nlon, 2*nlat)."""
    ncell, nl1, nlon, nvar = V.shape
    nlat = nl1 - 1
    m = 2 * nlat
    u = np.empty((ncell, m, nlon, nvar))
    u[:, :nlat] = V[:, :nlat]
    u[:, nlat:] = np.roll(V[:, nlat:0:-1], -(nlon // 2), axis=2)
    u1 = fft_diff(u, 1)
    u2 = fft_diff(u, 2)
    u12 = fft_diff(u1, 2)
    tab = np.stack([u, u1, u2, u12], axis=1)  # (ncell, 4, m, n, nvar)
    return np.ascontiguousarray(tab.transpose(0, 1, 4, 3, 2))


def equi_theta(nlat):
    return np.arange(nlat + 1) * (np.pi / nlat)


# ---------------------------------------------------------------------------
@dataclass
class Cells:
    """Cell surfaces in the C-ABI layout (see include/rbc3d_gpu.h)."""
    nlat: int
    nlon: int
    th: np.ndarray
    phi: np.ndarray
    w: np.ndarray
    ncell: int
    celltype: np.ndarray      # (ncell,) int32
    x: np.ndarray             # (3, N)
    a3: np.ndarray            # (3, N)
    detJ: np.ndarray          # (N,)
    area: np.ndarray          # (ncell,)
    meshSize: np.ndarray      # (ncell,)
    spl_x: np.ndarray         # (ncell, 4, 3, nlon, 2nlat)
    spl_a3: np.ndarray
    spl_detJ: np.ndarray      # (ncell, 4, 1, nlon, 2nlat)
    f: np.ndarray = None      # (3, N)
    g: np.ndarray = None
    spl_F: np.ndarray = None
    spl_G: np.ndarray = None
    centres: np.ndarray = None
    rotations: list = field(default_factory=list)


def _to_points(a):
    """(ncell, nlat, nlon, k) -> (k, N) with p = cell*nv + ilon*nlat + ilat."""
    nc, nlat, nlon, k = a.shape
    return np.ascontiguousarray(a.transpose(3, 0, 2, 1).reshape(k, nc * nlat * nlon))


def place_cells(rng, ncell, L, min_dist, inside=None, max_tries=2_000_000):
    """Uniform centres in the box with rejection at a minimum periodic centre
    distance; ``inside(c)`` optionally restricts the region (tube)."""
    L = np.asarray(L, dtype=np.float64)
    C = []
    tries = 0
    nb = np.maximum(1, np.floor(L / max(min_dist, 1e-12)).astype(int))
    bs = L / nb
    offs = [np.array((i, j, k)) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)]
    bins = {}
    while len(C) < ncell:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("cell placement did not converge")
        c = rng.uniform(0, 1, 3) * L
        if inside is not None and not inside(c):
            continue
        ok = True
        # the accepted centres in the neighbouring bins (bin edge >= min_dist)
        # are the only ones that can be closer than min_dist
        b = np.floor(c / bs).astype(int) % nb
        for off in offs:
            for d in bins.get(tuple((b + off) % nb), ()):
                dd = c - d
                dd -= np.round(dd / L) * L
                if np.dot(dd, dd) < min_dist ** 2:
                    ok = False
                    break
            if not ok:
                break
        if ok:
            C.append(c)
            bins.setdefault(tuple(b), []).append(c)
    return np.array(C)


def make_cells(rng, ncell, L, min_dist, nlat=25, nlon=50, celltype=0, rc=1.0,
               inside=None, with_g=False, centres=None, rotations=None):
    th, phi, w = gauss_grid(nlat, nlon)
    the = equi_theta(nlat)
    if centres is None:
        centres = place_cells(rng, ncell, L, min_dist, inside)
    X, A3, DJ, SX, SA, SD, F, G, SF, SG = [], [], [], [], [], [], [], [], [], []
    rots = []
    areas, msz = [], []
    for ic in range(ncell):
        R = random_rotation(rng) if rotations is None else np.asarray(rotations[ic])
        rots.append(R)
        x, n, dj = biconcave_surface(th, phi, R, centres[ic], rc)
        xe, ne, dje = biconcave_surface(the, phi, R, centres[ic], rc)
        X.append(x); A3.append(n); DJ.append(dj[..., None])
        SX.append(xe); SA.append(ne); SD.append(dje[..., None])
        area = float(np.sum(dj * w[:, None]))
        areas.append(area)
        msz.append(math.sqrt(area / nlat ** 2))
        coeff = [random_sh_coeffs(rng) for _ in range(3)]
        f = np.stack([sh_eval(cf, th, phi) for cf in coeff], axis=-1)
        fe = np.stack([sh_eval(cf, the, phi) for cf in coeff], axis=-1)
        F.append(f); SF.append(fe * dje[..., None])
        if with_g:
            coeffg = [random_sh_coeffs(rng) for _ in range(3)]
            g = np.stack([sh_eval(cf, th, phi) for cf in coeffg], axis=-1)
            ge = np.stack([sh_eval(cf, the, phi) for cf in coeffg], axis=-1)
            G.append(g); SG.append(ge * dje[..., None])
    cells = Cells(
        nlat=nlat, nlon=nlon, th=th, phi=phi, w=w, ncell=ncell,
        celltype=np.full(ncell, celltype, dtype=np.int32),
        x=_to_points(np.array(X)), a3=_to_points(np.array(A3)),
        detJ=_to_points(np.array(DJ))[0].copy(),
        area=np.array(areas), meshSize=np.array(msz),
        spl_x=spline_on_sphere_batch(np.array(SX)), spl_a3=spline_on_sphere_batch(np.array(SA)),
        spl_detJ=spline_on_sphere_batch(np.array(SD)),
        f=_to_points(np.array(F)), spl_F=spline_on_sphere_batch(np.array(SF)),
        centres=centres, rotations=rots)
    if with_g:
        cells.g = _to_points(np.array(G))
        cells.spl_G = spline_on_sphere_batch(np.array(SG))
    else:
        cells.g = np.zeros_like(cells.f)
        cells.spl_G = np.zeros_like(cells.spl_F)
    return cells


# ---------------------------------------------------------------------------
@dataclass
class Wall:
    nvert: int
    nele: int
    x: np.ndarray          # (3, nvert)
    e2v: np.ndarray        # (3, nele) int32, 1-based
    glb: np.ndarray        # (nvert,) int32, 1-based unique vertex id
    ndof: int


def make_tube(radius, Lz, ntheta, nz, centre_xy):
    """Straight periodic tube along z meshed with ntheta x nz quads split into
    two Tri3 each.  The ring at z = Lz duplicates the ring at z = 0
    (indxVertGlb points back to it, as Wall_Build_V2V / GlobData_Init)."""
    th = np.arange(ntheta) * (2 * np.pi / ntheta)
    zs = np.arange(nz + 1) * (Lz / nz)
    nvert = ntheta * (nz + 1)
    x = np.empty((3, nvert))
    glb = np.empty(nvert, dtype=np.int32)
    for k in range(nz + 1):
        for i in range(ntheta):
            v = k * ntheta + i
            x[0, v] = centre_xy[0] + radius * np.cos(th[i])
            x[1, v] = centre_xy[1] + radius * np.sin(th[i])
            x[2, v] = zs[k]
            kk = 0 if k == nz else k
            glb[v] = kk * ntheta + i + 1
    tris = []
    for k in range(nz):
        for i in range(ntheta):
            a = k * ntheta + i
            b = k * ntheta + (i + 1) % ntheta
            c = (k + 1) * ntheta + i
            d = (k + 1) * ntheta + (i + 1) % ntheta
            tris.append((a, b, d))
            tris.append((a, d, c))
    e2v = np.ascontiguousarray(np.array(tris, dtype=np.int32).T + 1)
    return Wall(nvert=nvert, nele=e2v.shape[1], x=x, e2v=e2v, glb=glb, ndof=3 * ntheta * nz)


# ---------------------------------------------------------------------------
# Named workloads (sizes of the benchmark configurations)
def config(name: str, seed: int = 20261203, ncell: int | None = None, L: float | None = None):
    """Build a named workload.  Returns (params dict, Cells, Wall|None).
    ``ncell`` / ``L`` override the cell count and the periodic box side."""
    L_override = L
    rng = np.random.default_rng(seed)
    eps = 1e-6
    rc = 3.0
    alpha = alpha_for_cutoff(rc, eps)
    if name == "C1":        # 8 cells, L=12, SL only, 64^3
        L = [12.0] * 3; n = ncell or 8; Nb = [64] * 3; md = 3.0; vr = 1.0; g = False
    elif name == "C2":      # 256 cells, L=40, SL+DL, 128^3, viscRat 5
        L = [40.0] * 3; n = ncell or 256; Nb = [128] * 3; md = 2.6; vr = 5.0; g = True
    elif name == "C5":      # 2048 cells, L=80, SL+DL, 256^3
        L = [80.0] * 3; n = ncell or 2048; Nb = [256] * 3; md = 2.6; vr = 5.0; g = True
    elif name == "C3":      # 64 cells in a tube of radius 8, length 48
        L = [16.5, 16.5, 48.0]; n = ncell or 64; Nb = [96, 96, 256]; md = 3.0; vr = 1.0; g = False
    else:
        raise ValueError(name)
    if L_override is not None:
        L = [float(L_override)] * 3
    prm = dict(Lb=L, alpha=alpha, rc=rc, eps=eps, Nb=Nb, P=6, nlat=25, nlon=50,
               ncelltypes=1, viscRat=[vr], vBkg=[0.0, 0.0, 8.0] if name == "C3" else [0.0, 0.0, 0.0])
    wall = None
    inside = None
    if name == "C3":
        cxy = (L[0] / 2, L[1] / 2)
        inside = lambda c: (c[0] - cxy[0]) ** 2 + (c[1] - cxy[1]) ** 2 < 6.5 ** 2
        wall = make_tube(8.0, L[2], 48, 192, cxy)
    cells = make_cells(rng, n, L, md, inside=inside, with_g=g)
    return prm, cells, wall


# ---------------------------------------------------------------------------
# Rigid motion of cells (a kinematic stand-in for the membrane dynamics of
# TimeInt_RK2, used to produce sequences of correlated wall solves)
def _rot(axis, angle):
    axis = np.asarray(axis, dtype=np.float64)
    n = np.linalg.norm(axis)
    if n < 1e-300 or angle == 0.0:
        return np.eye(3)
    k = axis / n
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * (K @ K)


def move_cells(cells, dx, dR):
    """New Cells with cell c rotated by dR[c] about its centre and shifted by
    dx[c]: positions, normals and tractions transform exactly, and so do
    their spline tables (the bicubic tables are linear in the values)."""
    nv = cells.nlat * cells.nlon
    out = Cells(**{k: getattr(cells, k) for k in cells.__dataclass_fields__})
    x = cells.x.copy(); a3 = cells.a3.copy(); f = cells.f.copy(); g = cells.g.copy()
    sx = cells.spl_x.copy(); sa = cells.spl_a3.copy(); sF = cells.spl_F.copy(); sG = cells.spl_G.copy()
    cen = np.asarray(cells.centres, dtype=np.float64).copy()
    for c in range(cells.ncell):
        R, d, c0 = dR[c], dx[c], cen[c]
        sl = slice(c * nv, (c + 1) * nv)
        x[:, sl] = R @ (cells.x[:, sl] - c0[:, None]) + (c0 + d)[:, None]
        a3[:, sl] = R @ cells.a3[:, sl]
        f[:, sl] = R @ cells.f[:, sl]
        g[:, sl] = R @ cells.g[:, sl]
        # tables (4 kinds, 3 vars, n, m): rotate the var axis; translate the u kind of x
        for tab, src in ((sx, cells.spl_x), (sa, cells.spl_a3), (sF, cells.spl_F), (sG, cells.spl_G)):
            tab[c] = np.einsum("ij,kjnm->kinm", R, src[c])
        sx[c, 0] = np.einsum("ij,jnm->inm", R, cells.spl_x[c, 0] - c0[:, None, None]) + (c0 + d)[:, None, None]
        cen[c] = c0 + d
    out.x, out.a3, out.f, out.g = x, a3, f, g
    out.spl_x, out.spl_a3, out.spl_F, out.spl_G = sx, sa, sF, sG
    out.centres = cen
    return out


def poiseuille_step(cells, axis_xy, radius, umax, dt):
    """Advect cell centres along z with u = umax (1 - r^2/R^2) and rotate them
    with the local shear rate (about e_z x e_r)."""
    cen = np.asarray(cells.centres)
    dx, dR = [], []
    for c in cen:
        rx, ry = c[0] - axis_xy[0], c[1] - axis_xy[1]
        r2 = rx * rx + ry * ry
        u = umax * max(0.0, 1 - r2 / radius ** 2)
        shear = 2 * umax * math.sqrt(r2) / radius ** 2
        dx.append(np.array([0.0, 0.0, u * dt]))
        dR.append(_rot([-ry, rx, 0.0], -0.5 * shear * dt))
    return move_cells(cells, dx, dR)
