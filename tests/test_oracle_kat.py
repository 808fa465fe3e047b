"""Known-answer tests that pin the FP64 oracle.

RBC3D ships no tests, fixtures or golden vectors, and its Fortran/PETSc/FFTW
build cannot run here, so the oracle is pinned by mathematics: tables against
their exact functions (ModEwaldFunc.F90:25-80, ModBasicMath.F90:332-346),
quadrature exactness (ModQuadRule.F90), the FFT against numpy, PME against a
direct Ewald k-sum, Ewald-split invariance, and the periodic sphere-drag law
(Hasimoto 1959)."""
import ctypes as C
import math

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300.abi import Context, TLIST_RAW, TLIST_RBC, FP64

dp = C.POINTER(C.c_double)


def _f(lib, name, res, args):
    f = getattr(lib.lib, "rbc3d_oracle_" + name)
    f.restype = res
    f.argtypes = args
    return f


def p(a):
    return a.ctypes.data_as(dp)


def test_ewald_tables_vs_exact(oracle):
    alpha, rc = G.alpha_for_cutoff(3.0, 1e-6), 3.0
    r = np.linspace(1e-2, rc * 0.999, 4001)
    A, B, Ae, Be = (np.zeros_like(r) for _ in range(4))
    sl = _f(oracle, "kat_ewald_sl", None, [C.c_double, C.c_double, C.c_int, dp, dp, dp, C.c_int])
    sl(alpha, rc, r.size, p(r), p(A), p(B), 0)
    sl(alpha, rc, r.size, p(r), p(Ae), p(Be), 1)
    # lerp on 8193 nodes: relative error far below the FP32 target
    assert np.max(np.abs(A - Ae) * r ** 3) < 1e-7
    assert np.max(np.abs(B - Be) * r) < 1e-7
    D, De = np.zeros_like(r), np.zeros_like(r)
    dl = _f(oracle, "kat_ewald_dl", None, [C.c_double, C.c_double, C.c_int, dp, dp, C.c_int])
    dl(alpha, rc, r.size, p(r), p(D), 0)
    dl(alpha, rc, r.size, p(r), p(De), 1)
    assert np.max(np.abs(D - De) * r ** 5) < 1e-6
    # exact values at the nodes; zero beyond the cut-off and below r_eps
    rn = np.array([3.0 * 100 / 8192, 3.0 * 5000 / 8192, 3.0, 3.5, 1e-5])
    An, Bn, Ane, Bne = (np.zeros_like(rn) for _ in range(4))
    sl(alpha, rc, rn.size, p(rn), p(An), p(Bn), 0)
    sl(alpha, rc, rn.size, p(rn), p(Ane), p(Bne), 1)
    assert np.allclose(An[:2], Ane[:2], rtol=1e-13) and np.allclose(Bn[:2], Bne[:2], rtol=1e-13)
    assert An[2] == 0 and Bn[2] == 0 and An[3] == 0 and An[4] == 0
    # the free-space limit: alpha -> 0 gives the Oseen tensor coefficients
    Ao, Bo = np.zeros(1), np.zeros(1)
    sl(0.0, rc, 1, p(np.array([0.7])), p(Ao), p(Bo), 1)
    assert math.isclose(Ao[0], 1 / 0.7 ** 3) and math.isclose(Bo[0], 1 / 0.7)


def test_mask_table(oracle):
    x = np.linspace(0, 1.2, 2001)
    m, me = np.zeros_like(x), np.zeros_like(x)
    f = _f(oracle, "kat_mask", None, [C.c_int, dp, dp, C.c_int])
    f(x.size, p(x), p(m), 0)
    f(x.size, p(x), p(me), 1)
    assert np.max(np.abs(m - me)) < 1e-6
    assert m[0] == 1.0 and np.all(m[x >= 1.0] == 0.0)


def test_bspline_partition_of_unity(oracle):
    f = _f(oracle, "kat_bspline", None, [C.c_double, C.c_int, C.POINTER(C.c_int), dp])
    for P in (4, 6, 8):
        for xc in np.linspace(-3.3, 17.9, 97):
            w = np.zeros(P)
            imin = C.c_int()
            f(xc, P, C.byref(imin), p(w))
            assert abs(w.sum() - 1) < 1e-14
            assert np.all(w >= -1e-15)
            assert imin.value == math.floor(xc) - (P - 1)
            # first moment of the cardinal B-spline M_P centred at xc - P/2
            nodes = imin.value + np.arange(P)
            assert abs((w * nodes).sum() - (xc - P / 2)) < 1e-12


def test_gauleg_exactness(oracle):
    f = _f(oracle, "kat_gauleg", None, [C.c_double, C.c_double, C.c_int, dp, dp])
    for n in (4, 10, 16, 25):
        x, w = np.zeros(n), np.zeros(n)
        f(-1.0, 1.0, n, p(x), p(w))
        xn, wn = np.polynomial.legendre.leggauss(n)
        assert np.allclose(x, xn, atol=1e-14) and np.allclose(w, wn, atol=1e-14)
        f(0.0, 0.7, n, p(x), p(w))
        for k in range(2 * n):
            assert abs((w * x ** k).sum() - 0.7 ** (k + 1) / (k + 1)) < 1e-13


def test_gauleg_sinh(oracle):
    f = _f(oracle, "kat_gauleg_sinh", None, [C.c_double] * 4 + [C.c_int, dp, dp])
    x, w = np.zeros(16), np.zeros(16)
    f(0.0, 0.6, 0.0, 0.01, 16, p(x), p(w))
    # maps into the interval and integrates smooth functions exactly enough
    assert np.all((x > 0) & (x < 0.6))
    assert abs(w.sum() - 0.6) < 1e-10
    # clusters nodes towards the near-singular end
    xg, wg = np.zeros(16), np.zeros(16)
    _f(oracle, "kat_gauleg", None, [C.c_double, C.c_double, C.c_int, dp, dp])(0.0, 0.6, 16, p(xg), p(wg))
    assert x[0] < xg[0]


def test_gqtri7_degree5(oracle):
    r, s, w = np.zeros(7), np.zeros(7), np.zeros(7)
    _f(oracle, "kat_gqtri7", None, [dp, dp, dp])(p(r), p(s), p(w))
    assert abs(w.sum() - 0.5) < 1e-15
    # int_T r^a s^b = a! b! / (a+b+2)!
    for a in range(6):
        for b in range(6 - a):
            ex = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
            assert abs((w * r ** a * s ** b).sum() - ex) < 1e-15


def test_fft_vs_numpy(oracle):
    f = _f(oracle, "kat_fft", None, [dp, dp, C.c_int, C.c_int])
    rng = np.random.default_rng(0)
    for n in (8, 12, 30, 64, 96, 7, 49):
        z = rng.normal(size=n) + 1j * rng.normal(size=n)
        re, im = z.real.copy(), z.imag.copy()
        f(p(re), p(im), n, -1)
        assert np.allclose(re + 1j * im, np.fft.fft(z), atol=1e-12 * n)
        re, im = z.real.copy(), z.imag.copy()
        f(p(re), p(im), n, +1)
        assert np.allclose(re + 1j * im, np.fft.ifft(z) * n, atol=1e-12 * n)


def test_min_dist_to_tri_bruteforce(oracle):
    f = _f(oracle, "kat_min_dist_to_tri", C.c_double, [dp, dp, dp, dp])
    rng = np.random.default_rng(3)
    a = np.linspace(0, 1, 301)
    S, T = np.meshgrid(a, a)
    m = S + T <= 1
    S, T = S[m], T[m]
    for _ in range(40):
        tri = rng.normal(size=(3, 3))
        xt = rng.normal(size=3) * 1.5
        s0, t0 = C.c_double(), C.c_double()
        x = np.ascontiguousarray(tri)  # x(l, c) column-major -> tri.T flattened
        xf = np.ascontiguousarray(tri.T.reshape(-1))
        d = f(p(xt), p(xf), C.byref(s0), C.byref(t0))
        P = (1 - S - T)[:, None] * tri[0] + S[:, None] * tri[1] + T[:, None] * tri[2]
        dmin = np.sqrt(((P - xt) ** 2).sum(1)).min()
        assert d <= dmin + 1e-12 and d > dmin - 5e-3
        q = (1 - s0.value - t0.value) * tri[0] + s0.value * tri[1] + t0.value * tri[2]
        assert abs(np.linalg.norm(q - xt) - d) < 1e-10


def test_spline_interp_reproduces_nodes(oracle):
    """Spline_Interp returns the tabulated values at the equiangular nodes and
    approximates the surface between them (bicubic Hermite, O(h^4))."""
    rng = np.random.default_rng(1)
    nlat, nlon = 25, 50
    R = G.random_rotation(rng)
    th = G.equi_theta(nlat)
    phi = np.arange(nlon) * 2 * np.pi / nlon
    xe, _, _ = G.biconcave_surface(th, phi, R, np.zeros(3))
    tab = G.spline_on_sphere(xe)
    f = _f(oracle, "kat_spline_interp", None, [C.c_int, C.c_int, C.c_int, dp, C.c_int, dp, dp, dp])
    T, PH = np.meshgrid(th[:-1], phi, indexing="ij")
    tt, pp = np.ascontiguousarray(T.ravel()), np.ascontiguousarray(PH.ravel())
    out = np.zeros((tt.size, 3))
    f(2 * nlat, nlon, 3, p(tab), tt.size, p(tt), p(pp), p(out))
    assert np.allclose(out, xe[:-1].reshape(-1, 3), atol=1e-12)
    # off-node: compare with the exact surface
    tq = np.ascontiguousarray(rng.uniform(0.05, np.pi - 0.05, 200))
    pq = np.ascontiguousarray(rng.uniform(0, 2 * np.pi, 200))
    out = np.zeros((200, 3))
    f(2 * nlat, nlon, 3, p(tab), 200, p(tq), p(pq), p(out))
    ex = np.array([G.biconcave_surface(np.array([a]), np.array([b]), R, np.zeros(3))[0][0, 0] for a, b in zip(tq, pq)])
    assert np.max(np.abs(out - ex)) < 2e-3


def _direct_ksum(alpha, L, xs, F, T, xt, q2t_max=40.0):
    """Direct Ewald k-space sum of the Stokeslet (F) and stresslet (T, 3x3 per
    source) densities at targets xt, with the influence of PME_Transform
    (ModPME.F90:165-206) and q = k/L."""
    vol = L ** 3
    K = int(math.ceil(math.sqrt(q2t_max / (math.pi * alpha)) * L)) + 1
    k = np.arange(-K, K + 1)
    q = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3) / L
    q2 = (q ** 2).sum(1)
    keep = (q2 > 0) & (math.pi * alpha * q2 < q2t_max)
    q, q2 = q[keep], q2[keep]
    q2t = math.pi * alpha * q2
    e = np.exp(-q2t)
    phi0 = e / q2t
    phi1 = (e + phi0) / q2t
    qt = math.sqrt(math.pi * alpha) * q
    ph = np.exp(-2j * np.pi * (q @ xs))
    Fh = ph @ F.T
    V = 2 * alpha / vol * phi1[:, None] * (q2t[:, None] * Fh - qt * (qt * Fh).sum(1)[:, None])
    if T is not None:
        Th = np.einsum("qs,sab->qab", ph, T)
        tr = np.einsum("qaa->q", Th)
        qT = np.einsum("qa,qab->qb", q, Th)
        Tq = np.einsum("qab,qb->qa", Th, q)
        qTq = np.einsum("qa,qa->q", q, Tq)
        tmp = 1j * 4 * math.pi * alpha / vol * phi0[:, None] * (q * tr[:, None] + qT + Tq)
        tmp -= 1j * 8 * math.pi ** 2 * alpha ** 2 / vol * (phi1 * qTq)[:, None] * q
        V = V - tmp
    return np.real(np.exp(2j * np.pi * (xt.T @ q.T)) @ V).T


def _one_cell(viscrat=1.0, with_g=False, seed=2, L=12.0, Nb=64, rc=3.0, eps=1e-6):
    rng = np.random.default_rng(seed)
    cells = G.make_cells(rng, 1, [L] * 3, 3.0, with_g=with_g, centres=np.array([[6.1, 5.7, 6.3]]))
    prm = dict(Lb=[L] * 3, alpha=G.alpha_for_cutoff(rc, eps), rc=rc, eps=eps, Nb=[Nb] * 3, P=6, nlat=25,
               nlon=50, ncelltypes=1, viscRat=[viscrat], vBkg=[0, 0, 0])
    return prm, cells


@pytest.mark.parametrize("dl", [False, True])
def test_pme_vs_direct_ksum(oracle, dl):
    prm, cells = _one_cell(viscrat=5.0, with_g=dl)
    ctx = Context(oracle, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g if dl else None, spl_F=cells.spl_F, spl_G=cells.spl_G if dl else None)
    rng = np.random.default_rng(11)
    xt = rng.uniform(0, 12, (3, 6))
    ctx.set_raw_targets(xt)
    c1, c2 = (0.0, 1.0) if dl else (1.0, 0.0)
    v = ctx.pme(TLIST_RAW, c1, c2)
    N = cells.x.shape[1]
    ds = cells.detJ * np.tile(cells.w, N // cells.nlat)
    F = cells.f * ds * c1
    T = None
    if dl:
        B = 1 - 5.0
        T = np.einsum("sa,sb->sab", (cells.g * ds).T, cells.a3.T * B) * c2
    u = _direct_ksum(prm["alpha"], 12.0, cells.x, F, T, xt) / 2.0
    assert np.linalg.norm(v - u) / np.linalg.norm(u) < 1e-6


def test_ewald_split_invariance(oracle):
    """Real space + k space is independent of alpha (FP64, targets away from
    the cell so no correction applies): pins the real-space tables and the
    k-space influence (SL and DL, incl. the stresslet sign) against each other."""
    prm, cells = _one_cell(viscrat=5.0, with_g=True)
    rng = np.random.default_rng(4)
    xt = np.array([[1.0, 2.0, 10.5], [10.9, 1.1, 2.2], [1.5, 10.0, 9.0], [6.1, 5.7, 9.9]]).T
    N = cells.x.shape[1]
    ds = cells.detJ * np.tile(cells.w, N // cells.nlat)
    B = 1 - 5.0
    out = []
    for rc, eps in ((3.9, 1e-11), (3.0, 1e-11)):
        prm2 = dict(prm, alpha=G.alpha_for_cutoff(rc, eps), rc=rc)
        ctx = Context(oracle, prm2)
        ctx.set_cells(cells)
        ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
        ctx.set_raw_targets(xt)
        vr = ctx.add_int_on_rbcs(TLIST_RAW, 1.0, 1.0)
        T = np.einsum("sa,sb->sab", (cells.g * ds).T, cells.a3.T * B)
        vk = _direct_ksum(prm2["alpha"], 12.0, cells.x, cells.f * ds, T, xt, q2t_max=-math.log(1e-13)) / 2.0
        out.append(vr + vk)
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[0]) < 1e-8


def test_hasimoto_sphere_drag(oracle):
    """Uniform traction on a sphere (radius 1) in a periodic cube: the surface
    velocity is F/(6 pi a) (1 - 2.837297 a/L + 4.19 (a/L)^3) (Hasimoto 1959);
    exercises real space + self-patch correction + PME with c1 = 1/(4 pi)."""
    L = 12.0
    cells = G.make_sphere_cells(np.array([[6.0, 6.0, 6.0]]), radius=1.0)
    Ftot = 1.0
    cells.f = np.zeros_like(cells.x)
    cells.f[2] = Ftot / (4 * math.pi)
    cells.spl_F = G.sphere_uniform_spline(cells, np.array([0.0, 0.0, Ftot / (4 * math.pi)]))
    prm = dict(Lb=[L] * 3, alpha=G.alpha_for_cutoff(3.0, 1e-8), rc=3.0, eps=1e-8, Nb=[64] * 3, P=6, nlat=25,
               nlon=50, ncelltypes=1, viscRat=[1.0], vBkg=[0, 0, 0])
    ctx = Context(oracle, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, spl_F=cells.spl_F)
    v = ctx.calc_velocity_field(TLIST_RBC)
    a_L = 1.0 / L
    expect = Ftot / (6 * math.pi) * (1 - 2.837297 * a_L + 4.19 * a_L ** 3)
    assert abs(np.mean(v[2]) - expect) / expect < 2e-3
    assert np.std(v[2]) / expect < 2e-3
    assert np.max(np.abs(v[:2])) / expect < 2e-3
