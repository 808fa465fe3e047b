"""Cell dynamics on the GPU library: Compute_Rbc_Vel (ModTimeInt.F90:716-808)
and the RK2 step of TimeInt_RK2 (ModTimeInt.F90:183-271).

One Compute_Rbc_Vel at positions x:
  RBC_ComputeGeometry + Rbc_BuildSurfaceSource(x)  -> rbc3d_set_cells_x on the GPU
      (a3, detJ, area and the x / a3 / detJ spline tables of the filtered
      expansion, SourceList_UpdateCoord, TargetList_Update); with the oracle
      the same derivation runs on the host;
  Shell_ResForce, f = -f                           -> rbc3d_shell_res_force on the GPU;
  AddIntraCellRepulsionForce                       -> rbc3d_intra_cell_repulsion on the GPU;
  Rbc_SphProject(f) + Rbc_BuildSurfaceSource(f)    -> ShFilter to degree < nlat0 on the
      Gauss grid (host), the f detJ spline and SourceList_UpdateDensity on the
      GPU (rbc3d_set_cell_density_x);
  Solve_RBC_Vel                                    -> rbc3d_solve_rbc_vel (g := v on the cells).
The spherical-harmonic filter and the equiangular synthesis
that feed the spline tables are small host transforms in the conventions of
Spherepack's shags / shsgs / shses:
  g = 1/2 sum_n a(0,n) pbar(0,n) + sum_{m>=1} sum_n pbar(m,n) (a(m,n) cos m phi - b(m,n) sin m phi).
"""
from __future__ import annotations

import math

import numpy as np

from . import geometry as G
from .abi import FP64


def pbar(L, th):
    """Spherepack pbar(m, n, theta) for 0 <= m <= n < L: array (len(th), L, L)."""
    th = np.atleast_1d(np.asarray(th, dtype=np.float64))
    x, s = np.cos(th), np.sin(th)
    P = np.zeros((th.size, L, L))
    pmm = np.full(th.size, math.sqrt(0.5))
    for m in range(L):
        if m > 0:
            pmm = pmm * math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s
        P[:, m, m] = pmm
        if m + 1 < L:
            P[:, m, m + 1] = math.sqrt(2.0 * m + 3.0) * x * pmm
        for n in range(m + 2, L):
            a = math.sqrt((4.0 * n * n - 1.0) / (n * n - m * m))
            b = math.sqrt(((n - 1.0) ** 2 - m * m) / (4.0 * (n - 1.0) ** 2 - 1.0))
            P[:, m, n] = a * (x * P[:, m, n - 1] - b * P[:, m, n - 2])
    return P


class SphTransform:
    """ShAnalGau + ShFilter (degree < nlat0) and ShSynthGau / ShSynthEqu on
    the cell grid; fields are arrays (..., nlat, nlon)."""

    def __init__(self, th, phi, w, nlat0):
        self.nlat, self.nlon, self.L = th.size, phi.size, nlat0
        L = nlat0
        self.PG = pbar(L, th)                                    # (nlat, m, n)
        self.PE = pbar(L, G.equi_theta(self.nlat))               # (nlat+1, m, n)
        m = np.arange(L)
        self.cs = np.cos(np.outer(m, phi))                       # (m, j)
        self.sn = np.sin(np.outer(m, phi))
        self.wf = np.asarray(w) / math.pi                        # Gauss weight x 2 / nlon
        tri = np.triu(np.ones((L, L)))                           # n >= m
        self.PGw = self.PG * self.wf[:, None, None] * tri

    def anal(self, F):
        C = np.einsum("...ij,mj->...im", F, self.cs)
        S = np.einsum("...ij,mj->...im", F, self.sn)
        a = np.einsum("imn,...im->...mn", self.PGw, C)
        b = -np.einsum("imn,...im->...mn", self.PGw, S)
        return a, b

    def synth(self, a, b, equi=False):
        P = self.PE if equi else self.PG
        Gm = np.einsum("imn,...mn->...im", P, a)
        Hm = np.einsum("imn,...mn->...im", P, b)
        Gm[..., 0] *= 0.5
        return np.einsum("...im,mj->...ij", Gm, self.cs) - np.einsum("...im,mj->...ij", Hm, self.sn)

    def project(self, F):
        """Rbc_SphProject: analysis, ShFilter, synthesis on the Gauss grid."""
        return self.synth(*self.anal(F))

    def spline(self, F):
        """Rbc_BuildSurfaceSource's table of F (ncell, nvar, nlat, nlon): filtered
        expansion on the equiangular rows, Spline_Build_On_Sphere."""
        E = self.synth(*self.anal(F), equi=True)                 # (ncell, nvar, nlat+1, nlon)
        return G.spline_on_sphere_batch(np.ascontiguousarray(E.transpose(0, 2, 3, 1)))


def to_grid(v, ncell, nlat, nlon):
    """SoA point layout (k, N) -> (ncell, k, nlat, nlon)."""
    k = v.shape[0]
    return np.ascontiguousarray(v.reshape(k, ncell, nlon, nlat).transpose(1, 0, 3, 2))


def to_points(F):
    """(ncell, k, nlat, nlon) -> SoA point layout (k, N)."""
    nc, k, nlat, nlon = F.shape
    return np.ascontiguousarray(F.transpose(1, 0, 3, 2).reshape(k, nc * nlon * nlat))


class CellDynamics:
    """Compute_Rbc_Vel and the RK2 step for the cells of a context whose cell
    grid, walls and wall density are set.  ``cells`` supplies the grid and the
    cell types; its positions are the initial state."""

    def __init__(self, ctx, cells, xref, moduli, nlat0=12, rtol=1e-11, prec=FP64, max_it=200, force_coef=0.0):
        self.ctx, self.nlat0, self.rtol, self.prec, self.max_it = ctx, nlat0, rtol, prec, max_it
        self.force_coef = force_coef  # ForceCoef of AddIntraCellRepulsionForce (0: no repulsion)
        self.cells = cells
        self.nlat, self.nlon, self.ncell = cells.nlat, cells.nlon, cells.ncell
        self.T = SphTransform(cells.th, cells.phi, cells.w, nlat0)
        ctx.set_ref_cells(xref, *moduli)
        self.x = np.array(cells.x, dtype=np.float64)
        self.sol = None
        self.last = {}

    def compute_rbc_vel(self, x):
        ctx, c, T = self.ctx, self.cells, self.T
        nc, nlat, nlon = self.ncell, self.nlat, self.nlon
        device = "set_cells_x" in ctx.L.fn  # the GPU library derives the sources itself
        if device:
            # RBC_ComputeGeometry + Rbc_BuildSurfaceSource(xFlag) + the list
            # updates on the device (rbc3d_set_cells_x)
            ctx.set_cells_x(c, self.nlat0, x=x)
        else:
            # the same derivation on the host (the oracle's path)
            a3, detJ, area, _ = ctx.cell_geometry(x, nc)
            Xg, Ag, Dg = to_grid(x, nc, nlat, nlon), to_grid(a3, nc, nlat, nlon), to_grid(detJ[None], nc, nlat, nlon)
            ctx.set_cells(G.Cells(nlat=nlat, nlon=nlon, th=c.th, phi=c.phi, w=c.w, ncell=nc, celltype=c.celltype,
                                  x=x, a3=a3, detJ=detJ, area=area, meshSize=np.sqrt(area / nlat ** 2),
                                  spl_x=T.spline(Xg), spl_a3=T.spline(Ag), spl_detJ=T.spline(Dg)))
        f = -ctx.shell_res_force(x, c.celltype)
        if self.force_coef:
            if device:
                a3, _, area, _ = ctx.cell_geometry(x, nc)  # host arrays of the repulsion call
            pushed = ctx.intra_cell_repulsion(x, a3, area, self.force_coef, f)
        else:
            pushed, area = 0, None
        # Rbc_SphProject(f), then Rbc_BuildSurfaceSource(fFlag) + SourceList_UpdateDensity
        Fg = T.project(to_grid(f, nc, nlat, nlon))
        f = to_points(Fg)
        if device:
            ctx.set_cell_density_x(self.nlat0, f=f)
        else:
            ctx.set_cell_density(f=f, spl_F=T.spline(Fg * Dg))
        sol, v, st, _ = ctx.solve_rbc_vel(self.nlat0, rtol=self.rtol, max_it=self.max_it, restart=30, sol=self.sol,
                                          prec=self.prec)
        self.sol = sol
        self.last = dict(force_rms=float(np.sqrt(np.mean(f * f))), solve_its=st.iterations, area=area,
                         repulsion_points=pushed)
        return v

    def rk2(self, dt, alpha=0.5, after_stage=None):
        """One TimeInt_RK2 step (c2 = alpha, b2 = 1 / (2 alpha), b1 = 1 - b2);
        after_stage(stage) runs after each Compute_Rbc_Vel, where the reference
        calls NoSlipWall."""
        b2 = 1.0 / (2.0 * alpha)
        b1 = 1.0 - b2
        k1 = self.compute_rbc_vel(self.x)
        if after_stage:
            after_stage(0)
        k2 = self.compute_rbc_vel(self.x + alpha * dt * k1)
        if after_stage:
            after_stage(1)
        self.x = self.x + dt * (b1 * k1 + b2 * k2)
        return k1, k2
