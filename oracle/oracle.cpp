// oracle.cpp -- FP64 CPU restatement of RBC3D's Ewald-split boundary-integral
// matvec and the wall no-slip GMRES, behind the same C ABI as the GPU library
// (include/rbc3d_gpu.h) with the prefix rbc3d_oracle_.
//
// TEST INFRASTRUCTURE ONLY: this is the parity checker of the GPU library and
// the timed CPU baseline of the benchmark.  No product code links or calls it.
//
// Reference routines restated (paths relative to the RBC3D source tree):
//   AddIntOnRbcs / AddLinearInt          common/ModIntOnRbcs.F90:25-201
//   RBC_SingInt / RBC_NearSingInt*       common/ModRbcSingInt.F90:29-310
//   NbrRbcList_*                          common/ModRbcSingInt.F90:316-362
//   HashTable_*                           common/ModHashTable.F90:23-126
//   SourceList_UpdateCoord/UpdateDensity  common/ModSourceList.F90:92-189
//   TargetList_Update / CreateFromRaw     common/ModTargetList.F90:95-166
//   RbcPolarPatch_Create                  common/ModPolarPatch.F90:27-75
//   PME_*                                 common/ModPME.F90:58-489
//   Get_That / Get_R (sign, normalisation) common/ModPFFTW.F90:110-185
//   AddIntOnWalls / PrepareSingIntOnWall  common/ModIntOnWalls.F90:37-308
//   NoSlipWall / MyMatMult / Compute_Wall_Residual_Vel / AssembleArray
//                                         common/ModNoSlip.F90:45-384
//   initCOEFs / SetEwaldPrms              common/ModConf.F90:327-408
//   CalcVelocityField                     common/ModPostProcess.F90:29-63
//   PETSc KSPGMRES (restart 30, classical Gram-Schmidt, PCNONE, x0 = 0,
//   ||r|| <= rtol*||r0||) is restated in gmres() below.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../include/rbc3d_gpu.h"
#include "oracle_math.hpp"

using namespace orc;
using cplx = std::complex<double>;

#define API(name) rbc3d_oracle_##name

struct NbrEntry { int surf, ilat, ilon; double dist; };

struct HashList {
  int Nc[3] = {0, 0, 0};
  double iLbNc[3] = {0, 0, 0};
  std::vector<int> hoc;   // (Nc1+2)*(Nc2+2)*(Nc3+2), 0-based point id or -1
  std::vector<int> next;  // per point
  int id(int i1, int i2, int i3) const { return i1 + (Nc[0] + 2) * (i2 + (Nc[1] + 2) * i3); }
};

struct rbc3d_oracle_ctx {
  rbc3d_params prm{};
  double iLb[3]{};
  double Acoef[RBC3D_MAX_CELLTYPES]{}, Bcoef[RBC3D_MAX_CELLTYPES]{};
  EwaldTables E;
  std::string err;
  // cell grid
  int nlat = 0, nlon = 0;
  std::vector<double> th, phi, w;
  // polar patch (RbcPolarPatch_Create)
  int nrad = 0, nazm = 0;
  double radius = 0;
  std::vector<double> pw, thG, phiG;  // thG[(irad + nrad*iazm) + nrad*nazm*(ilat + nlat*ilon)]
  // cells
  int ncell = 0, npt = 0;
  std::vector<int> celltype;
  std::vector<double> x, a3, detJ, f, g, area, meshSize;
  std::vector<double> spl_x, spl_a3, spl_detJ, spl_F, spl_G;
  bool has_f = false, has_g = false;
  // cell source list
  std::vector<double> sf, sg;  // f*dS, g*dS (N x 3)
  HashList hcell;
  // walls (single wall, id = ncell + 1)
  int nvert = 0, nele = 0, ndof = 0;
  std::vector<double> wx, wf, warea, weps;
  std::vector<int> e2v, glb;
  HashList hwall;
  std::vector<double> wsrc;  // centroids (nele x 3)
  // self-wall operator (CSR, 3nvert x 3nvert, component-major rows/cols)
  bool wall_prepared = false;
  std::vector<int> rowptr, colidx;
  std::vector<double> vals;
  // raw targets
  int nraw = 0;
  std::vector<double> rawx;
  // PME
  int N1 = 0, N2 = 0, N3 = 0, NH = 0;
  std::vector<double> ff, tt, vv;  // real grids, x fastest
  std::vector<cplx> ffC, ttC, vvC;
  std::vector<double> bbx, bby, bbz;
  bool flag_sl = false, flag_dl = false;
  rbc3d_counts counts{};
  // membrane mechanics: reference cells (rbcRefs) per cell type
  int nref = 0;
  std::vector<double> ref_ar, ref_b;  // a_rcp and b of each reference cell, [type][4][nv]
  std::vector<double> ES, ED, EB;
};
typedef rbc3d_oracle_ctx Ctx;

static rbc3d_status fail(Ctx* c, int code, const std::string& m) { if (c) c->err = m; return code; }

// ---------------------------------------------------------------------------
// Hash table, ModHashTable.F90:23-126 (single node: z handled like x, y)
static void hash_setup(Ctx* c, HashList& h) {
  for (int d = 0; d < 3; ++d) {
    h.Nc[d] = std::max((int)std::floor(c->prm.Lb[d] / c->prm.rc), 3);
    h.iLbNc[d] = c->iLb[d] * h.Nc[d];
  }
}
static inline void hash_index(const HashList& h, const double* x, int& i1, int& i2, int& i3) {
  i1 = fmod_pos(ifloor(x[0] * h.iLbNc[0]), h.Nc[0]) + 1;
  i2 = fmod_pos(ifloor(x[1] * h.iLbNc[1]), h.Nc[1]) + 1;
  i3 = fmod_pos(ifloor(x[2] * h.iLbNc[2]), h.Nc[2]) + 1;
}
// x(N,3) column-major, head insertion in point order as HashTable_Build
static void hash_build(HashList& h, int n, const double* x) {
  h.hoc.assign((size_t)(h.Nc[0] + 2) * (h.Nc[1] + 2) * (h.Nc[2] + 2), -1);
  h.next.assign(n, -1);
  for (int p = 0; p < n; ++p) {
    double xp[3] = {x[p], x[p + n], x[p + 2 * (size_t)n]};
    int i1, i2, i3;
    hash_index(h, xp, i1, i2, i3);
    int id = h.id(i1, i2, i3);
    h.next[p] = h.hoc[id];
    h.hoc[id] = p;
  }
  int N1 = h.Nc[0], N2 = h.Nc[1], N3 = h.Nc[2];
  for (int k = 0; k <= N3 + 1; ++k)
    for (int j = 0; j <= N2 + 1; ++j) {
      h.hoc[h.id(0, j, k)] = h.hoc[h.id(N1, j, k)];
      h.hoc[h.id(N1 + 1, j, k)] = h.hoc[h.id(1, j, k)];
    }
  for (int k = 0; k <= N3 + 1; ++k)
    for (int i = 0; i <= N1 + 1; ++i) {
      h.hoc[h.id(i, 0, k)] = h.hoc[h.id(i, N2, k)];
      h.hoc[h.id(i, N2 + 1, k)] = h.hoc[h.id(i, 1, k)];
    }
  for (int j = 0; j <= N2 + 1; ++j)
    for (int i = 0; i <= N1 + 1; ++i) {
      h.hoc[h.id(i, j, 0)] = h.hoc[h.id(i, j, N3)];
      h.hoc[h.id(i, j, N3 + 1)] = h.hoc[h.id(i, j, 1)];
    }
}

// ---------------------------------------------------------------------------
// Target lists
struct TView {
  int n = 0;
  std::vector<double> x;      // N x 3
  std::vector<double> Acoef;  // N
  std::vector<int> surf, i1, i2;
};
static bool make_tlist(Ctx* c, int which, TView& t) {
  if (which == RBC3D_TLIST_RBC) {
    t.n = c->npt; t.x = c->x; t.Acoef.resize(t.n); t.surf.resize(t.n); t.i1.resize(t.n); t.i2.resize(t.n);
    int nv = c->nlat * c->nlon;
    for (int p = 0; p < t.n; ++p) {
      int cell = p / nv, r = p % nv;
      t.Acoef[p] = c->Acoef[c->celltype[cell]];
      t.surf[p] = cell + 1; t.i1[p] = r % c->nlat; t.i2[p] = r / c->nlat;
    }
    return true;
  }
  if (which == RBC3D_TLIST_WALL) {
    t.n = c->nvert; t.x = c->wx; t.Acoef.assign(t.n, 2.); t.surf.assign(t.n, c->ncell + 1);
    t.i1.resize(t.n); t.i2.assign(t.n, -1);
    for (int p = 0; p < t.n; ++p) t.i1[p] = p;
    return true;
  }
  if (which == RBC3D_TLIST_RAW) {
    t.n = c->nraw; t.x = c->rawx; t.Acoef.assign(t.n, 2.); t.surf.assign(t.n, -1);
    t.i1.assign(t.n, -1); t.i2.assign(t.n, -1);
    return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Cell helpers
static inline void cell_spline(const Ctx* c, const std::vector<double>& tab, int nvar, int cell, Spline& s) {
  int m = 2 * c->nlat, n = c->nlon;
  s.set(m, n, nvar, tab.data() + (size_t)cell * 4 * m * n * nvar);
}
static inline void cellx(const Ctx* c, const std::vector<double>& a, int cell, int ilat, int ilon, double* out) {
  size_t p = (size_t)cell * c->nlat * c->nlon + (size_t)ilon * c->nlat + ilat;
  for (int k = 0; k < 3; ++k) out[k] = a[p + (size_t)k * c->npt];
}

// RBC_SingInt, ModRbcSingInt.F90:29-90
static void rbc_sing_int(const Ctx* c, double c1, double c2, int cell, int ilat0, int ilon0, double* dv) {
  Spline sx, sF, sG, sa3;
  cell_spline(c, c->spl_x, 3, cell, sx);
  if (c1 != 0) cell_spline(c, c->spl_F, 3, cell, sF);
  if (c2 != 0) { cell_spline(c, c->spl_G, 3, cell, sG); cell_spline(c, c->spl_a3, 3, cell, sa3); }
  dv[0] = dv[1] = dv[2] = 0;
  double xi[3];
  spline_interp(sx, c->th[ilat0], c->phi[ilon0], xi);
  size_t base = (size_t)c->nrad * c->nazm * (ilat0 + (size_t)c->nlat * ilon0);
  for (int irad = 0; irad < c->nrad; ++irad)
    for (int iazm = 0; iazm < c->nazm; ++iazm) {
      double th_j = c->thG[base + irad + c->nrad * iazm], phi_j = c->phiG[base + irad + c->nrad * iazm];
      double xj[3], xx[3];
      spline_interp(sx, th_j, phi_j, xj);
      for (int k = 0; k < 3; ++k) xx[k] = xj[k] - xi[k];
      double rr = std::sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
      if (rr >= c->prm.rc) continue;
      if (c1 != 0) {
        double fj[3], EA, EB;
        spline_interp(sF, th_j, phi_j, fj);
        for (int k = 0; k < 3; ++k) fj[k] = c->pw[irad] * fj[k];
        c->E.sl(rr, EA, EB);
        double d = xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2];
        for (int k = 0; k < 3; ++k) dv[k] = dv[k] + c1 * (EA * xx[k] * d + EB * fj[k]);
      }
      if (c2 != 0) {
        double gj[3], aj[3];
        spline_interp(sG, th_j, phi_j, gj);
        for (int k = 0; k < 3; ++k) gj[k] = c->pw[irad] * gj[k];
        spline_interp(sa3, th_j, phi_j, aj);
        double EA = c->E.dl(rr);
        double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
        double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
        for (int k = 0; k < 3; ++k) dv[k] = dv[k] + c2 * (EA * xx[k] * dg * da);
      }
    }
}

// RBC_NearSingInt_Subtract, ModRbcSingInt.F90:175-226
static void near_subtract(const Ctx* c, double c1, double c2, int cell, const double* xi, double th0,
                          double phi0, double radPat, double* dv) {
  dv[0] = dv[1] = dv[2] = 0;
  std::vector<int> il, jl;
  polar_patch_find_points(th0, phi0, radPat, c->th.data(), c->nlat, c->phi.data(), c->nlon, il, jl);
  for (size_t p = 0; p < il.size(); ++p) {
    int ilat = il[p], ilon = jl[p];
    double xj[3], xx[3];
    cellx(c, c->x, cell, ilat, ilon, xj);
    for (int k = 0; k < 3; ++k) xx[k] = xj[k] - xi[k];
    double rr = std::sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
    if (rr > c->prm.rc) continue;
    double dth = dist_on_sphere(th0, phi0, c->th[ilat], c->phi[ilon]);
    double mask = MaskFunc(dth / radPat);
    size_t q = (size_t)cell * c->nlat * c->nlon + (size_t)ilon * c->nlat + ilat;
    if (c1 != 0) {
      double fj[3], EA, EB;
      cellx(c, c->f, cell, ilat, ilon, fj);
      for (int k = 0; k < 3; ++k) fj[k] = fj[k] * c->detJ[q] * c->w[ilat];
      c->E.sl(rr, EA, EB);
      double d = xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2];
      for (int k = 0; k < 3; ++k) dv[k] = dv[k] - c1 * mask * (EA * xx[k] * d + EB * fj[k]);
    }
    if (c2 != 0) {
      double gj[3], aj[3];
      cellx(c, c->g, cell, ilat, ilon, gj);
      for (int k = 0; k < 3; ++k) gj[k] = gj[k] * c->detJ[q] * c->w[ilat];
      cellx(c, c->a3, cell, ilat, ilon, aj);
      double EA = c->E.dl(rr);
      double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
      double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
      for (int k = 0; k < 3; ++k) dv[k] = dv[k] - c2 * mask * (EA * xx[k] * dg * da);
    }
  }
}

// RBC_NearSingInt_ReAdd, ModRbcSingInt.F90:232-310
static void near_readd(const Ctx* c, double c1, double c2, int cell, const double* xi, const double* x0,
                       double th0, double phi0, double radPat, double* dv) {
  double d = std::sqrt((xi[0] - x0[0]) * (xi[0] - x0[0]) + (xi[1] - x0[1]) * (xi[1] - x0[1]) +
                       (xi[2] - x0[2]) * (xi[2] - x0[2]));
  double sizePat = radPat * std::sqrt(c->area[cell] / (4 * PI));
  dv[0] = dv[1] = dv[2] = 0;
  const int nrad = 16, nazm = 2 * nrad;
  double thP[nrad], wtP[nrad], phiP[nazm], thPG[nrad * nazm], phiPG[nrad * nazm];
  if (d > 2.2250738585072014e-308) {
    d = d * (radPat / sizePat);
    gauleg_sinh(0., radPat, 0., d, nrad, thP, wtP);
  } else {
    gauleg(0., radPat, nrad, thP, wtP);
  }
  for (int i = 0; i < nrad; ++i) {
    wtP[i] = wtP[i] * std::sin(thP[i]) * (TWO_PI / nazm);
    wtP[i] = wtP[i] * MaskFunc(thP[i] / radPat);
  }
  for (int j = 0; j < nazm; ++j) phiP[j] = j * TWO_PI / nazm;
  polar_patch_build(th0, phi0, thP, nrad, phiP, nazm, thPG, phiPG);
  Spline sx, sF, sG, sa3;
  cell_spline(c, c->spl_x, 3, cell, sx);
  if (c1 != 0) cell_spline(c, c->spl_F, 3, cell, sF);
  if (c2 != 0) { cell_spline(c, c->spl_G, 3, cell, sG); cell_spline(c, c->spl_a3, 3, cell, sa3); }
  for (int irad = 0; irad < nrad; ++irad)
    for (int iazm = 0; iazm < nazm; ++iazm) {
      double th_j = thPG[irad + nrad * iazm], phi_j = phiPG[irad + nrad * iazm];
      double xj[3], xx[3];
      spline_interp(sx, th_j, phi_j, xj);
      for (int k = 0; k < 3; ++k) xx[k] = xj[k] - xi[k];
      double rr = std::sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
      if (rr > c->prm.rc) continue;
      if (c1 != 0) {
        double fj[3], EA, EB;
        spline_interp(sF, th_j, phi_j, fj);
        for (int k = 0; k < 3; ++k) fj[k] = wtP[irad] * fj[k];
        c->E.sl(rr, EA, EB);
        double dd = xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2];
        for (int k = 0; k < 3; ++k) dv[k] = dv[k] + c1 * (EA * xx[k] * dd + EB * fj[k]);
      }
      if (c2 != 0) {
        double aj[3], gj[3];
        spline_interp(sa3, th_j, phi_j, aj);
        spline_interp(sG, th_j, phi_j, gj);
        for (int k = 0; k < 3; ++k) gj[k] = wtP[irad] * gj[k];
        double EA = c->E.dl(rr);
        double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
        double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
        for (int k = 0; k < 3; ++k) dv[k] = dv[k] + c2 * (EA * xx[k] * dg * da);
      }
    }
}

// RBC_NearSingInt, ModRbcSingInt.F90:103-166.  Returns 1 if a correction was made.
static int rbc_near_sing_int(const Ctx* c, double c1, double c2, int cell, const double* xi, const double* x0,
                             double th0, double phi0, double* dv) {
  Spline sa3;
  cell_spline(c, c->spl_a3, 3, cell, sa3);
  double a30[3];
  spline_interp(sa3, th0, phi0, a30);
  double dist = a30[0] * (xi[0] - x0[0]) + a30[1] * (xi[1] - x0[1]) + a30[2] * (xi[2] - x0[2]);
  if (dist > 2 * c->meshSize[cell]) { dv[0] = dv[1] = dv[2] = 0; return 0; }
  double sizePat = c->radius * std::sqrt(c->area[cell] / (4 * PI));
  double dist1 = std::copysign(std::fabs(0.01 * sizePat), dist);
  double tmp[3];
  near_subtract(c, c1, c2, cell, xi, th0, phi0, c->radius, tmp);
  for (int k = 0; k < 3; ++k) dv[k] = tmp[k];
  if (std::fabs(dist) >= std::fabs(dist1)) {
    near_readd(c, c1, c2, cell, xi, x0, th0, phi0, c->radius, tmp);
    for (int k = 0; k < 3; ++k) dv[k] += tmp[k];
  } else {
    double xi1[3], dv1[3], dv0[3];
    for (int k = 0; k < 3; ++k) xi1[k] = x0[k] + dist1 * a30[k];
    near_readd(c, c1, c2, cell, xi1, x0, th0, phi0, c->radius, dv1);
    near_readd(c, c1, c2, cell, x0, x0, th0, phi0, c->radius, dv0);
    if (c2 != 0) {
      Spline sd, sG;
      cell_spline(c, c->spl_detJ, 1, cell, sd);
      cell_spline(c, c->spl_G, 3, cell, sG);
      double dJ0, g0[3];
      spline_interp(sd, th0, phi0, &dJ0);
      spline_interp(sG, th0, phi0, g0);
      for (int k = 0; k < 3; ++k) g0[k] = g0[k] / dJ0;
      for (int k = 0; k < 3; ++k) dv0[k] = (dist > 0) ? dv0[k] + c2 * 4 * PI * g0[k] : dv0[k] - c2 * 4 * PI * g0[k];
    }
    for (int k = 0; k < 3; ++k) dv[k] += dv0[k] + dist / dist1 * (dv1[k] - dv0[k]);
  }
  return 1;
}

// NbrRbcList_Insert, ModRbcSingInt.F90:341-362
static void nbr_insert(std::vector<NbrEntry>& L, int surf, int ilat, int ilon, double dist) {
  for (auto& e : L)
    if (e.surf == surf) {
      if (dist < e.dist) { e.ilat = ilat; e.ilon = ilon; e.dist = dist; }
      return;
    }
  L.push_back({surf, ilat, ilon, dist});
}

// AddLinearInt, ModIntOnRbcs.F90:162-201
static void add_linear_int(Ctx* c, double c1, double c2, const TView& t, double* v) {
  (void)c1;
  if (c2 == 0 || !c->has_g) return;
  double xv[3] = {0, 0, 0};
  for (int cell = 0; cell < c->ncell; ++cell)
    for (int ilon = 0; ilon < c->nlon; ++ilon)
      for (int ilat = 0; ilat < c->nlat; ++ilat) {
        size_t p = (size_t)cell * c->nlat * c->nlon + (size_t)ilon * c->nlat + ilat;
        double ds = c->w[ilat] * c->detJ[p];
        double gg[3], aa[3], xx[3];
        cellx(c, c->g, cell, ilat, ilon, gg);
        cellx(c, c->a3, cell, ilat, ilon, aa);
        cellx(c, c->x, cell, ilat, ilon, xx);
        double vn = gg[0] * aa[0] + gg[1] * aa[1] + gg[2] * aa[2];
        for (int k = 0; k < 3; ++k) xv[k] = xv[k] + c->Bcoef[c->celltype[cell]] * xx[k] * vn * ds;
      }
  double pil = c->iLb[0] * c->iLb[1] * c->iLb[2];
  for (int k = 0; k < 3; ++k) xv[k] = -8 * PI * pil * xv[k];
  for (int i = 0; i < t.n; ++i)
    for (int k = 0; k < 3; ++k) v[i + (size_t)k * t.n] += c2 * xv[k] / t.Acoef[i];
}

// AddIntOnRbcs, ModIntOnRbcs.F90:25-156
static rbc3d_status add_int_on_rbcs(Ctx* c, const TView& t, double c1, double c2, double* v) {
  if (c->ncell == 0) return RBC3D_OK;
  // a density that was never set is zero
  if (!c->has_f) c1 = 0;
  if (!c->has_g) c2 = 0;
  const int nv = c->nlat * c->nlon;
  const int N = c->npt;
  const double rc = c->prm.rc;
  long long npairs = 0, nnbr = 0, nnear = 0, nself = 0;
  int overflow = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : npairs, nnbr, nnear, nself, overflow)
  for (int i = 0; i < t.n; ++i) {
    double xi[3] = {t.x[i], t.x[i + t.n], t.x[i + 2 * (size_t)t.n]};
    int surf_i = t.surf[i];
    int cell_i = surf_i - 1;
    bool own = cell_i >= 0 && cell_i < c->ncell;
    double th_i = 0, phi_i = 0;
    if (own) { th_i = c->th[t.i1[i]]; phi_i = c->phi[t.i2[i]]; }
    std::vector<NbrEntry> L;
    double vi[3] = {0, 0, 0};
    int i1, i2, i3;
    hash_index(c->hcell, xi, i1, i2, i3);
    const HashList& h = c->hcell;
    for (int j1 = std::max(i1 - 1, 0); j1 <= std::min(i1 + 1, h.Nc[0] + 1); ++j1)
      for (int j2 = std::max(i2 - 1, 0); j2 <= std::min(i2 + 1, h.Nc[1] + 1); ++j2)
        for (int j3 = std::max(i3 - 1, 0); j3 <= std::min(i3 + 1, h.Nc[2] + 1); ++j3)
          for (int j = h.hoc[h.id(j1, j2, j3)]; j >= 0; j = h.next[j]) {
            double xx[3];
            for (int k = 0; k < 3; ++k) {
              xx[k] = c->x[j + (size_t)k * N] - xi[k];
              xx[k] = xx[k] - nint(xx[k] * c->iLb[k]) * c->prm.Lb[k];
            }
            double rr = std::sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
            if (rr > rc) continue;
            ++npairs;
            int cell_j = j / nv, r = j % nv, ilat_j = r % c->nlat, ilon_j = r / c->nlat;
            int surf_j = cell_j + 1;
            double mask;
            if (surf_i == surf_j) {
              double dth = dist_on_sphere(th_i, phi_i, c->th[ilat_j], c->phi[ilon_j]);
              mask = MaskFunc(dth / c->radius);
            } else {
              mask = 0.;
              nbr_insert(L, surf_j, ilat_j, ilon_j, rr);
            }
            if (c1 != 0) {
              double EA, EB, fj[3] = {c->sf[j], c->sf[j + N], c->sf[j + 2 * (size_t)N]};
              c->E.sl(rr, EA, EB);
              double d = xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2];
              double s = (1. - mask) * c1 / t.Acoef[i];
              for (int k = 0; k < 3; ++k) vi[k] = vi[k] + s * (EA * xx[k] * d + EB * fj[k]);
            }
            if (c2 != 0) {
              double EA = c->E.dl(rr);
              double gj[3] = {c->sg[j], c->sg[j + N], c->sg[j + 2 * (size_t)N]};
              double aj[3] = {c->a3[j], c->a3[j + N], c->a3[j + 2 * (size_t)N]};
              double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
              double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
              double s = (1. - mask) * c2 * c->Bcoef[c->celltype[cell_j]] / t.Acoef[i];
              for (int k = 0; k < 3; ++k) vi[k] = vi[k] + s * (EA * xx[k] * dg * da);
            }
          }
    if (own) {
      double c2m = c2 * c->Bcoef[c->celltype[cell_i]], dv[3];
      rbc_sing_int(c, c1, c2m, cell_i, t.i1[i], t.i2[i], dv);
      for (int k = 0; k < 3; ++k) vi[k] += dv[k] / t.Acoef[i];
      ++nself;
    }
    if ((int)L.size() > RBC3D_NBR_MAX) ++overflow;
    for (const auto& e : L) {
      ++nnbr;
      int cj = e.surf - 1;
      double th0 = c->th[e.ilat], phi0 = c->phi[e.ilon];
      double x0[3], xt[3];
      cellx(c, c->x, cj, e.ilat, e.ilon, x0);
      for (int k = 0; k < 3; ++k) {
        double xx = xi[k] - x0[k];
        xx = xx - nint(xx * c->iLb[k]) * c->prm.Lb[k];
        xt[k] = x0[k] + xx;
      }
      Spline sx;
      cell_spline(c, c->spl_x, 3, cj, sx);
      spline_find_projection(sx, xt, th0, phi0, x0);
      double c2m = c2 * c->Bcoef[c->celltype[cj]], dv[3];
      nnear += rbc_near_sing_int(c, c1, c2m, cj, xt, x0, th0, phi0, dv);
      for (int k = 0; k < 3; ++k) vi[k] += dv[k] / t.Acoef[i];
    }
    for (int k = 0; k < 3; ++k) v[i + (size_t)k * t.n] += vi[k];
  }
  c->counts.pairs_within_rc = npairs;
  c->counts.nbr_items = nnbr;
  c->counts.nearsing_items = nnear;
  c->counts.self_items = nself;
  c->counts.nbr_overflow = overflow;
  add_linear_int(c, c1, c2, t, v);
  if (overflow) return fail(c, RBC3D_ERR_OVERFLOW, "neighbour-cell list above NMax=32");
  return RBC3D_OK;
}

// ---------------------------------------------------------------------------
// Walls
static void wall_geometry(Ctx* c) {
  c->warea.resize(c->nele); c->weps.resize(c->nele); c->wsrc.resize(3 * (size_t)c->nele);
  for (int e = 0; e < c->nele; ++e) {
    double xe[3][3];
    for (int l = 0; l < 3; ++l) {
      int iv = c->e2v[e + (size_t)l * c->nele] - 1;
      for (int k = 0; k < 3; ++k) xe[l][k] = c->wx[iv + (size_t)k * c->nvert];
    }
    double a[3], b[3];
    for (int k = 0; k < 3; ++k) { a[k] = xe[1][k] - xe[0][k]; b[k] = xe[2][k] - xe[0][k]; }
    double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    double an = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    c->warea[e] = 0.5 * an;
    c->weps[e] = std::sqrt(c->warea[e]);
    for (int k = 0; k < 3; ++k) c->wsrc[e + (size_t)k * c->nele] = THRD * (xe[0][k] + xe[1][k] + xe[2][k]);
  }
  hash_setup(c, c->hwall);
  hash_build(c->hwall, c->nele, c->wsrc.data());
}

static inline void tri_coords(const Ctx* c, int e, double* xe /*3x3 col-major*/, double* fe) {
  for (int l = 0; l < 3; ++l) {
    int iv = c->e2v[e + (size_t)l * c->nele] - 1;
    for (int k = 0; k < 3; ++k) {
      xe[l + 3 * k] = c->wx[iv + (size_t)k * c->nvert];
      if (fe) fe[l + 3 * k] = c->wf[iv + (size_t)k * c->nvert];
    }
  }
}

// PrepareSingIntOnWall, ModIntOnWalls.F90:181-308
static void prepare_sing_int_on_wall(Ctx* c) {
  const int nv = c->nvert, nrow = 3 * nv;
  std::vector<std::map<int, double>> rows(nrow);
  const HashList& h = c->hwall;
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < nv; ++i) {
    double xi[3] = {c->wx[i], c->wx[i + nv], c->wx[i + 2 * (size_t)nv]};
    int i1, i2, i3;
    hash_index(h, xi, i1, i2, i3);
    for (int j1 = std::max(i1 - 1, 0); j1 <= std::min(i1 + 1, h.Nc[0] + 1); ++j1)
      for (int j2 = std::max(i2 - 1, 0); j2 <= std::min(i2 + 1, h.Nc[1] + 1); ++j2)
        for (int j3 = std::max(i3 - 1, 0); j3 <= std::min(i3 + 1, h.Nc[2] + 1); ++j3)
          for (int e = h.hoc[h.id(j1, j2, j3)]; e >= 0; e = h.next[e]) {
            double xe[9], fe[9] = {0};
            tri_coords(c, e, xe, nullptr);
            for (int k = 0; k < 3; ++k) {
              double sh = nint((xi[k] - xe[0 + 3 * k]) * c->iLb[k]) * c->prm.Lb[k];
              for (int l = 0; l < 3; ++l) xe[l + 3 * k] += sh;
            }
            double s0, t0;
            double rr = min_dist_to_tri(xi, xe, s0, t0);
            if (rr > c->prm.rc) continue;
            double rhs[3], lhs[27];
            if (rr > c->weps[e]) tri_int_regular(c->E, xe, fe, xi, rhs, lhs);
            else tri_int_duffy(c->E, xe, fe, xi, s0, t0, rhs, lhs);
            for (int l = 0; l < 3; ++l) {
              int iv = c->e2v[e + (size_t)l * c->nele] - 1;
              for (int r = 0; r < 3; ++r)
                for (int cc = 0; cc < 3; ++cc) rows[i + r * nv][iv + cc * nv] += lhs[l + 3 * (r + 3 * cc)];
            }
          }
  }
  c->rowptr.assign(nrow + 1, 0);
  c->colidx.clear(); c->vals.clear();
  for (int r = 0; r < nrow; ++r) {
    for (auto& kv : rows[r]) { c->colidx.push_back(kv.first); c->vals.push_back(kv.second); }
    c->rowptr[r + 1] = (int)c->colidx.size();
  }
  c->wall_prepared = true;
}

// AddIntOnWalls, ModIntOnWalls.F90:37-128
static rbc3d_status add_int_on_walls(Ctx* c, int which, const TView& t, double c1, double* v) {
  if (c->nvert == 0) return RBC3D_OK;
  if (which == RBC3D_TLIST_WALL) {
    if (!c->wall_prepared) return fail(c, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
    const int nv = c->nvert;
    for (int r = 0; r < 3 * nv; ++r) {
      double s = 0;
      for (int q = c->rowptr[r]; q < c->rowptr[r + 1]; ++q) s += c->vals[q] * c->wf[c->colidx[q]];
      int i = r % nv;
      v[r] += c1 * s / t.Acoef[i];
    }
    return RBC3D_OK;  // a single wall: all wall-wall interactions are self interactions
  }
  const HashList& h = c->hwall;
  long long np = 0, nd = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : np, nd)
  for (int i = 0; i < t.n; ++i) {
    double xi[3] = {t.x[i], t.x[i + t.n], t.x[i + 2 * (size_t)t.n]};
    double vi[3] = {0, 0, 0};
    int i1, i2, i3;
    hash_index(h, xi, i1, i2, i3);
    for (int j1 = std::max(i1 - 1, 0); j1 <= std::min(i1 + 1, h.Nc[0] + 1); ++j1)
      for (int j2 = std::max(i2 - 1, 0); j2 <= std::min(i2 + 1, h.Nc[1] + 1); ++j2)
        for (int j3 = std::max(i3 - 1, 0); j3 <= std::min(i3 + 1, h.Nc[2] + 1); ++j3)
          for (int e = h.hoc[h.id(j1, j2, j3)]; e >= 0; e = h.next[e]) {
            if (t.surf[i] == c->ncell + 1) continue;
            double xe[9], fe[9];
            tri_coords(c, e, xe, fe);
            for (int k = 0; k < 3; ++k) {
              double sh = nint((xi[k] - xe[0 + 3 * k]) * c->iLb[k]) * c->prm.Lb[k];
              for (int l = 0; l < 3; ++l) xe[l + 3 * k] += sh;
            }
            double s0, t0;
            double rr = min_dist_to_tri(xi, xe, s0, t0);
            if (rr > c->prm.rc) continue;
            ++np;
            double dv[3];
            if (rr < c->weps[e]) { tri_int_duffy(c->E, xe, fe, xi, s0, t0, dv, nullptr); ++nd; }
            else tri_int_regular(c->E, xe, fe, xi, dv, nullptr);
            for (int k = 0; k < 3; ++k) vi[k] += c1 * dv[k] / t.Acoef[i];
          }
    for (int k = 0; k < 3; ++k) v[i + (size_t)k * t.n] += vi[k];
  }
  c->counts.wall_pairs = np;
  c->counts.wall_duffy = nd;
  return RBC3D_OK;
}

// ---------------------------------------------------------------------------
// PME, ModPME.F90
static void pme_init(Ctx* c) {
  c->N1 = c->prm.Nb[0]; c->N2 = c->prm.Nb[1]; c->N3 = c->prm.Nb[2];
  c->NH = c->N1 / 2 + 1;
  const int P = c->prm.P;
  // B-factor, ModPME.F90:306-336
  std::vector<double> MP(P);
  int imin;
  bspline((double)P + 2.220446049250313e-16, P, imin, MP.data());
  auto bfac = [&](int N, int kmax, std::vector<double>& out) {
    out.resize(kmax + 1);
    for (int k = 0; k <= kmax; ++k) {
      cplx b = 0.;
      for (int m = 0; m <= P - 2; ++m) {
        double ang = TWO_PI * k * m / (double)N;
        b += MP[m] * cplx(std::cos(ang), std::sin(ang));
      }
      double ang = TWO_PI * k * (P - 1.) / (double)N;
      b = cplx(std::cos(ang), std::sin(ang)) / b;
      out[k] = std::norm(b);
    }
  };
  bfac(c->N1, c->N1 / 2, c->bbx);
  bfac(c->N2, c->N2 - 1, c->bby);
  bfac(c->N3, c->N3 - 1, c->bbz);
}

static inline size_t gidx(const Ctx* c, int i, int j, int k) { return (size_t)i + (size_t)c->N1 * (j + (size_t)c->N2 * k); }
static inline size_t cidx(const Ctx* c, int i, int j, int k) { return (size_t)i + (size_t)c->NH * (j + (size_t)c->N2 * k); }

// Distrib_Source, ModPME.F90:405-443
static void distrib_source(Ctx* c, const double* x, double c1, double c2, const double* f, const double* t) {
  const int P = c->prm.P;
  double wx[32], wy[32], wz[32];
  int imin, jmin, kmin;
  double ih[3];
  for (int d = 0; d < 3; ++d) ih[d] = c->prm.Nb[d] / c->prm.Lb[d];
  bspline(x[0] * ih[0], P, imin, wx);
  bspline(x[1] * ih[1], P, jmin, wy);
  bspline(x[2] * ih[2], P, kmin, wz);
  const size_t G = (size_t)c->N1 * c->N2 * c->N3;
  for (int k0 = 0; k0 < P; ++k0) {
    int k = fmod_pos(kmin + k0, c->N3);
    for (int j0 = 0; j0 < P; ++j0)
      for (int i0 = 0; i0 < P; ++i0) {
        int j = fmod_pos(jmin + j0, c->N2), i = fmod_pos(imin + i0, c->N1);
        double wxyz = wx[i0] * wy[j0] * wz[k0];
        size_t q = gidx(c, i, j, k);
        if (c->flag_sl)
          for (int a = 0; a < 3; ++a) c->ff[q + a * G] += (c1 * wxyz) * f[a];
        if (c->flag_dl)
          for (int a = 0; a < 9; ++a) c->tt[q + a * G] += (c2 * wxyz) * t[a];
      }
  }
}

// PME_Distrib_Source, ModPME.F90:58-133
static rbc3d_status pme_distrib_source(Ctx* c, double c1, double c2, int cells, int walls) {
  c->flag_sl = std::fabs(c1) > 1.e-10;
  c->flag_dl = std::fabs(c2) > 1.e-10;
  const size_t G = (size_t)c->N1 * c->N2 * c->N3;
  c->ff.assign(3 * G, 0.);
  c->tt.assign(9 * G, 0.);
  if (cells && c->ncell > 0 && ((c->flag_sl && c->has_f) || (c->flag_dl && c->has_g))) {
    const int N = c->npt, nv = c->nlat * c->nlon;
    for (int p = 0; p < N; ++p) {
      double xp[3] = {c->x[p], c->x[p + N], c->x[p + 2 * (size_t)N]};
      double fp[3] = {0, 0, 0}, tp[9] = {0};
      if (c->flag_sl && c->has_f) for (int k = 0; k < 3; ++k) fp[k] = c->sf[p + (size_t)k * N];
      if (c->flag_dl && c->has_g) {
        double B = c->Bcoef[c->celltype[p / nv]];
        double gp[3], ap[3];
        for (int k = 0; k < 3; ++k) { gp[k] = c->sg[p + (size_t)k * N]; ap[k] = c->a3[p + (size_t)k * N] * B; }
        for (int ii = 0; ii < 3; ++ii)
          for (int jj = 0; jj < 3; ++jj) tp[ii + 3 * jj] = gp[ii] * ap[jj];
      }
      distrib_source(c, xp, c1, c2, fp, tp);
    }
  }
  if (walls && c->nvert > 0) {
    for (int e = 0; e < c->nele; ++e) {
      double xe[9], fe[9];
      tri_coords(c, e, xe, fe);
      double xp[3], fp[3] = {0, 0, 0}, tp[9] = {0};
      for (int k = 0; k < 3; ++k) xp[k] = THRD * (xe[0 + 3 * k] + xe[1 + 3 * k] + xe[2 + 3 * k]);
      if (c->flag_sl)
        for (int k = 0; k < 3; ++k) fp[k] = THRD * (fe[0 + 3 * k] + fe[1 + 3 * k] + fe[2 + 3 * k]) * c->warea[e];
      distrib_source(c, xp, c1, c2, fp, tp);
    }
  }
  return RBC3D_OK;
}

// Get_That, ModPFFTW.F90:148: 2-D r2c over (x,y) (sign -1), then c2c along z (sign +1)
static void get_that(Ctx* c, const double* r, cplx* out) {
  const int N1 = c->N1, N2 = c->N2, N3 = c->N3, NH = c->NH;
#pragma omp parallel
  {
    std::vector<cplx> line(std::max({N1, N2, N3}));
#pragma omp for
    for (int k = 0; k < N3; ++k)
      for (int j = 0; j < N2; ++j) {
        for (int i = 0; i < N1; ++i) line[i] = r[gidx(c, i, j, k)];
        fft_c2c(line.data(), N1, 1, -1);
        for (int i = 0; i < NH; ++i) out[cidx(c, i, j, k)] = line[i];
      }
#pragma omp for
    for (int k = 0; k < N3; ++k)
      for (int i = 0; i < NH; ++i) fft_c2c(out + cidx(c, i, 0, k), N2, NH, -1);
#pragma omp for
    for (int j = 0; j < N2; ++j)
      for (int i = 0; i < NH; ++i) fft_c2c(out + cidx(c, i, j, 0), N3, NH * N2, +1);
  }
}
// Get_R, ModPFFTW.F90:170: c2c along z (sign -1), 2-D c2r over (x,y) (c2c along
// y sign +1, then the 1-D c2r along x that ignores Im at kx = 0 and N1/2).
// Unnormalised.
static void get_r(Ctx* c, cplx* in, double* r) {
  const int N1 = c->N1, N2 = c->N2, N3 = c->N3, NH = c->NH;
#pragma omp parallel
  {
    std::vector<cplx> line(std::max({N1, N2, N3}));
#pragma omp for
    for (int j = 0; j < N2; ++j)
      for (int i = 0; i < NH; ++i) fft_c2c(in + cidx(c, i, j, 0), N3, NH * N2, -1);
#pragma omp for
    for (int k = 0; k < N3; ++k)
      for (int i = 0; i < NH; ++i) fft_c2c(in + cidx(c, i, 0, k), N2, NH, +1);
#pragma omp for
    for (int k = 0; k < N3; ++k)
      for (int j = 0; j < N2; ++j) {
        for (int i = 0; i < N1; ++i) line[i] = 0.;
        for (int i = 0; i < NH; ++i) {
          cplx vv = in[cidx(c, i, j, k)];
          if (i == 0 || 2 * i == N1) line[i] = cplx(vv.real(), 0.);
          else { line[i] = vv; line[N1 - i] = std::conj(vv); }
        }
        fft_c2c(line.data(), N1, 1, +1);
        for (int i = 0; i < N1; ++i) r[gidx(c, i, j, k)] = line[i].real();
      }
  }
}

// PME_Transform, ModPME.F90:137-222
static void pme_transform(Ctx* c) {
  const int N1 = c->N1, N2 = c->N2, N3 = c->N3, NH = c->NH;
  const size_t G = (size_t)N1 * N2 * N3, GC = (size_t)NH * N2 * N3;
  c->ffC.assign(3 * GC, 0.);
  c->ttC.assign(9 * GC, 0.);
  if (c->flag_sl)
    for (int a = 0; a < 3; ++a) get_that(c, c->ff.data() + a * G, c->ffC.data() + a * GC);
  if (c->flag_dl)
    for (int a = 0; a < 9; ++a) get_that(c, c->tt.data() + a * G, c->ttC.data() + a * GC);
  c->vvC.assign(3 * GC, 0.);
  const double alpha = c->prm.alpha, vol = c->prm.Lb[0] * c->prm.Lb[1] * c->prm.Lb[2];
  const cplx iota(0., 1.);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < N3; ++k)
    for (int j = 0; j < N2; ++j)
      for (int i = 0; i < NH; ++i) {
        size_t q = cidx(c, i, j, k);
        if (i == 0 && j == 0 && k == 0) continue;
        double qv[3];
        qv[0] = i * c->iLb[0];
        qv[1] = (j < N2 / 2) ? j * c->iLb[1] : (j - N2) * c->iLb[1];
        double q3 = (k < N3 / 2) ? k * c->iLb[2] : (k - N3) * c->iLb[2];
        qv[2] = -q3;  // ModPME.F90:303
        double qt[3];
        for (int d = 0; d < 3; ++d) qt[d] = std::sqrt(PI * alpha) * qv[d];
        double q2 = qv[0] * qv[0] + qv[1] * qv[1] + qv[2] * qv[2];
        double q2t = PI * alpha * q2, e = std::exp(-q2t);
        double phi0 = e / q2t, phi1 = (e + phi0) / q2t;
        cplx vres[3] = {0., 0., 0.};
        if (c->flag_sl) {
          cplx F[3] = {c->ffC[q], c->ffC[q + GC], c->ffC[q + 2 * GC]};
          cplx qf = qt[0] * F[0] + qt[1] * F[1] + qt[2] * F[2];
          for (int d = 0; d < 3; ++d) vres[d] += 2 * alpha / vol * phi1 * (q2t * F[d] - qt[d] * qf);
        }
        if (c->flag_dl) {
          cplx T[3][3];
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) T[a][b] = c->ttC[q + (a + 3 * b) * GC];
          cplx tr = T[0][0] + T[1][1] + T[2][2];
          cplx tmp[3];
          for (int d = 0; d < 3; ++d) {
            cplx qT = qv[0] * T[0][d] + qv[1] * T[1][d] + qv[2] * T[2][d];
            cplx Tq = T[d][0] * qv[0] + T[d][1] * qv[1] + T[d][2] * qv[2];
            tmp[d] = iota * 4. * PI * alpha / vol * phi0 * (qv[d] * tr + qT + Tq);
          }
          cplx qTq = 0.;
          for (int a = 0; a < 3; ++a) qTq += qv[a] * (T[a][0] * qv[0] + T[a][1] * qv[1] + T[a][2] * qv[2]);
          for (int d = 0; d < 3; ++d) tmp[d] -= iota * 8. * PI * PI * alpha * alpha / vol * phi1 * qTq * qv[d];
          for (int d = 0; d < 3; ++d) vres[d] -= tmp[d];
        }
        double bb = c->bbx[i] * c->bby[j] * c->bbz[k];
        for (int d = 0; d < 3; ++d) c->vvC[q + d * GC] = bb * vres[d];
      }
  c->vv.assign(3 * G, 0.);
  for (int a = 0; a < 3; ++a) get_r(c, c->vvC.data() + a * GC, c->vv.data() + a * G);
}

// Interp_Vel, ModPME.F90:450-489 and PME_Add_Interp_Vel :228-248
static void pme_add_interp_vel(Ctx* c, const TView& t, double* v) {
  const int P = c->prm.P;
  const size_t G = (size_t)c->N1 * c->N2 * c->N3;
  double ih[3];
  for (int d = 0; d < 3; ++d) ih[d] = c->prm.Nb[d] / c->prm.Lb[d];
#pragma omp parallel for schedule(static)
  for (int p = 0; p < t.n; ++p) {
    double wx[32], wy[32], wz[32];
    int imin, jmin, kmin;
    bspline(t.x[p + 2 * (size_t)t.n] * ih[2], P, kmin, wz);
    bspline(t.x[p + (size_t)t.n] * ih[1], P, jmin, wy);
    bspline(t.x[p] * ih[0], P, imin, wx);
    double dv[3] = {0, 0, 0};
    for (int k0 = 0; k0 < P; ++k0) {
      int k = fmod_pos(kmin + k0, c->N3);
      for (int j0 = 0; j0 < P; ++j0)
        for (int i0 = 0; i0 < P; ++i0) {
          int j = fmod_pos(jmin + j0, c->N2), i = fmod_pos(imin + i0, c->N1);
          double wxyz = wx[i0] * wy[j0] * wz[k0];
          size_t q = gidx(c, i, j, k);
          for (int d = 0; d < 3; ++d) dv[d] = dv[d] + wxyz * c->vv[q + d * G];
        }
    }
    for (int d = 0; d < 3; ++d) v[p + (size_t)d * t.n] += dv[d] / t.Acoef[p];
  }
}

// ---------------------------------------------------------------------------
// Wall solve
static void assemble_to_1d(const Ctx* c, const double* u /*nvert x 3*/, double* u1d) {
  for (int iv = 0; iv < c->nvert; ++iv) {
    int g = c->glb[iv] - 1;
    for (int k = 0; k < 3; ++k) u1d[3 * g + k] = u[iv + (size_t)k * c->nvert];
  }
}
static void assemble_from_1d(const Ctx* c, const double* u1d, double* u) {
  for (int iv = 0; iv < c->nvert; ++iv) {
    int g = c->glb[iv] - 1;
    for (int k = 0; k < 3; ++k) u[iv + (size_t)k * c->nvert] = u1d[3 * g + k];
  }
}

// MyMatMult, ModNoSlip.F90:255-308
static rbc3d_status wall_matmult(Ctx* c, const double* u, double* y) {
  std::vector<double> f(3 * (size_t)c->nvert), v(3 * (size_t)c->nvert, 0.);
  assemble_from_1d(c, u, f.data());
  c->wf = f;
  TView t;
  make_tlist(c, RBC3D_TLIST_WALL, t);
  double c1 = 1. / (4. * PI);
  rbc3d_status s = add_int_on_walls(c, RBC3D_TLIST_WALL, t, c1, v.data());
  if (s) return s;
  if ((s = pme_distrib_source(c, c1, 0., 0, 1))) return s;
  pme_transform(c);
  pme_add_interp_vel(c, t, v.data());
  assemble_to_1d(c, v.data(), y);
  return RBC3D_OK;
}

// Compute_Wall_Residual_Vel, ModNoSlip.F90:153-193
static rbc3d_status wall_residual(Ctx* c, double* v) {
  TView t;
  make_tlist(c, RBC3D_TLIST_WALL, t);
  std::fill(v, v + 3 * (size_t)t.n, 0.);
  double c1 = 1. / (4. * PI), c2 = 1. / (4. * PI);
  rbc3d_status s;
  if ((s = add_int_on_rbcs(c, t, c1, c2, v))) return s;
  if ((s = add_int_on_walls(c, RBC3D_TLIST_WALL, t, c1, v))) return s;
  if ((s = pme_distrib_source(c, c1, c2, 1, 1))) return s;
  pme_transform(c);
  pme_add_interp_vel(c, t, v);
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < t.n; ++i) v[i + (size_t)k * t.n] += c->prm.vBkg[k];
  return RBC3D_OK;
}

static double nrm2(const std::vector<double>& a) { double s = 0; for (double x : a) s += x * x; return std::sqrt(s); }

// Restarted GMRES with PETSc KSPGMRES defaults (classical Gram-Schmidt without
// refinement, PCNONE, convergence ||r_k|| < max(rtol*||b||, abstol)); a cycle
// ends on the Givens estimate and the true residual after it decides.
template <class MV>
static int gmres(int n, MV&& A, const std::vector<double>& b, std::vector<double>& x, double rtol, int max_it,
                 int restart, rbc3d_solve_stats* st, rbc3d_status* err) {
  std::vector<double> r(n), w(n);
  auto resid = [&]() -> bool {
    if ((*err = A(x.data(), w.data()))) return false;
    st->matvecs++;
    for (int i = 0; i < n; ++i) r[i] = b[i] - w[i];
    return true;
  };
  if (!resid()) return -1;
  // KSPConvergedDefault: ||r|| < max(rtol * ||b||, abstol) with ||b|| of the right-hand side
  double rnorm0 = nrm2(r), ttol = std::max(rtol * nrm2(b), 1.e-50);
  st->rnorm0 = rnorm0;
  int its = 0;
  double beta = rnorm0;
  if (beta <= ttol) { st->iterations = 0; st->converged = 1; return 0; }
  std::vector<std::vector<double>> V(restart + 1, std::vector<double>(n));
  std::vector<double> H((size_t)(restart + 1) * restart, 0.), cs(restart), sn(restart), gv(restart + 1);
  bool conv = false;
  while (!conv && its < max_it) {
    for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    std::fill(gv.begin(), gv.end(), 0.);
    gv[0] = beta;
    int k;
    for (k = 0; k < restart && its < max_it; ++k) {
      if ((*err = A(V[k].data(), w.data()))) return -1;
      st->matvecs++;
      for (int j = 0; j <= k; ++j) {
        double h = 0;
        for (int i = 0; i < n; ++i) h += w[i] * V[j][i];
        H[j + (restart + 1) * k] = h;
      }
      for (int j = 0; j <= k; ++j) {
        double h = H[j + (restart + 1) * k];
        for (int i = 0; i < n; ++i) w[i] -= h * V[j][i];
      }
      double hn = 0;
      for (int i = 0; i < n; ++i) hn += w[i] * w[i];
      hn = std::sqrt(hn);
      H[k + 1 + (restart + 1) * k] = hn;
      if (hn > 0) for (int i = 0; i < n; ++i) V[k + 1][i] = w[i] / hn;
      for (int j = 0; j < k; ++j) {
        double a = H[j + (restart + 1) * k], bb = H[j + 1 + (restart + 1) * k];
        H[j + (restart + 1) * k] = cs[j] * a + sn[j] * bb;
        H[j + 1 + (restart + 1) * k] = -sn[j] * a + cs[j] * bb;
      }
      double a = H[k + (restart + 1) * k], bb = H[k + 1 + (restart + 1) * k];
      double den = std::sqrt(a * a + bb * bb);
      cs[k] = den > 0 ? a / den : 1.; sn[k] = den > 0 ? bb / den : 0.;
      H[k + (restart + 1) * k] = den; H[k + 1 + (restart + 1) * k] = 0.;
      gv[k + 1] = -sn[k] * gv[k];
      gv[k] = cs[k] * gv[k];
      ++its;
      if (std::fabs(gv[k + 1]) <= ttol || hn == 0) { ++k; conv = true; break; }
    }
    // back substitution and update
    std::vector<double> yv(k);
    for (int i = k - 1; i >= 0; --i) {
      double s = gv[i];
      for (int j = i + 1; j < k; ++j) s -= H[i + (restart + 1) * j] * yv[j];
      yv[i] = s / H[i + (restart + 1) * i];
    }
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < n; ++i) x[i] += yv[j] * V[j][i];
    if (!resid()) return -1;
    beta = nrm2(r);
    conv = beta <= ttol;  // the true residual decides, not the Givens estimate
  }
  st->iterations = its;
  st->converged = conv ? 1 : 0;
  st->rnorm = beta;
  st->bnorm = nrm2(b);
  return 0;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// Cell velocity solve (Solve_RBC_Vel, ModVelSolver.F90:44-132): spherical
// harmonic transforms on the Gauss grid (Glob_Sph_Trans :641-719 through
// Spherepack shags / shsgs, restated from their documented definitions with
// pbar_table) and the g spline rebuild of Rbc_BuildSurfaceSource
// (ModRbc.F90:716-807: analysis, ShFilter to degree < nlat0, synthesis on the
// equiangular grid with both poles, Spline_Build_On_Sphere).
struct ShTab {
  int L = 0, nlat = 0, nlon = 0;
  std::vector<double> PG, PE;  // [row][m][n], Gauss rows and equiangular rows (nlat+1)
  std::vector<double> cs, sn;  // cos(m phi_j), sin(m phi_j): [m * nlon + j]
};
static void sh_setup(const Ctx* c, int L, ShTab& T) {
  T.L = L; T.nlat = c->nlat; T.nlon = c->nlon;
  T.PG.assign((size_t)c->nlat * L * L, 0.);
  T.PE.assign((size_t)(c->nlat + 1) * L * L, 0.);
  for (int i = 0; i < c->nlat; ++i) pbar_table(L, c->th[i], &T.PG[(size_t)i * L * L]);
  for (int i = 0; i <= c->nlat; ++i) pbar_table(L, i * PI / c->nlat, &T.PE[(size_t)i * L * L]);
  T.cs.resize((size_t)L * c->nlon); T.sn.resize((size_t)L * c->nlon);
  for (int m = 0; m < L; ++m)
    for (int j = 0; j < c->nlon; ++j) { T.cs[m * c->nlon + j] = std::cos(m * c->phi[j]); T.sn[m * c->nlon + j] = std::sin(m * c->phi[j]); }
}
// shags restricted to m, n < L: v[ilat + nlat*ilon] -> a, b [m*L + n]
static void sh_anal(const Ctx* c, const ShTab& T, const double* v, double* a, double* b) {
  const int L = T.L, nlat = T.nlat, nlon = T.nlon;
  std::fill(a, a + L * L, 0.); std::fill(b, b + L * L, 0.);
  for (int i = 0; i < nlat; ++i)
    for (int m = 0; m < L; ++m) {
      double C = 0, S = 0;
      for (int j = 0; j < nlon; ++j) { C += v[i + nlat * j] * T.cs[m * nlon + j]; S += v[i + nlat * j] * T.sn[m * nlon + j]; }
      // Gauss weight x 2/nlon; the grid's w is the Gauss weight x 2 pi/nlon (RBC_Create, ModRbc.F90:94)
      const double wf = c->w[i] / PI;
      for (int n = m; n < L; ++n) {
        const double P = T.PG[((size_t)i * L + m) * L + n];
        a[m * L + n] += wf * P * C;
        b[m * L + n] -= wf * P * S;
      }
    }
}
// shsgs / shses restricted to m, n < L on the rows of P: out[i + nrow*j]
static void sh_synth(const ShTab& T, const std::vector<double>& P, int nrow, const double* a, const double* b, double* out) {
  const int L = T.L, nlon = T.nlon;
  for (int i = 0; i < nrow; ++i) {
    std::vector<double> G(L, 0.), H(L, 0.);
    for (int m = 0; m < L; ++m)
      for (int n = m; n < L; ++n) {
        const double p = P[((size_t)i * L + m) * L + n];
        G[m] += p * a[m * L + n];
        H[m] += p * b[m * L + n];
      }
    for (int j = 0; j < nlon; ++j) {
      double s = 0.5 * G[0];
      for (int m = 1; m < L; ++m) s += G[m] * T.cs[m * nlon + j] - H[m] * T.sn[m * nlon + j];
      out[i + nrow * j] = s;
    }
  }
}
// Glob_Sph_Trans layout of one cell's coefficients: a(m, n) for m < L, n >= m,
// then b(m, n) for 1 <= m < L, n >= m; 3 components each.
static void sh_pack(int L, const double* a /*3 x L*L*/, const double* b, double* cvec) {
  size_t pc = 0;
  for (int m = 0; m < L; ++m)
    for (int n = m; n < L; ++n)
      for (int k = 0; k < 3; ++k) cvec[pc++] = a[(size_t)k * L * L + m * L + n];
  for (int m = 1; m < L; ++m)
    for (int n = m; n < L; ++n)
      for (int k = 0; k < 3; ++k) cvec[pc++] = b[(size_t)k * L * L + m * L + n];
}
static void sh_unpack(int L, const double* cvec, double* a, double* b) {
  std::fill(a, a + 3 * L * L, 0.); std::fill(b, b + 3 * L * L, 0.);
  size_t pc = 0;
  for (int m = 0; m < L; ++m)
    for (int n = m; n < L; ++n)
      for (int k = 0; k < 3; ++k) a[(size_t)k * L * L + m * L + n] = cvec[pc++];
  for (int m = 1; m < L; ++m)
    for (int n = m; n < L; ++n)
      for (int k = 0; k < 3; ++k) b[(size_t)k * L * L + m * L + n] = cvec[pc++];
}
// Glob_Sph_Trans over all cells: v (N x 3, point layout) <-> c (3 L^2 per cell)
static void glob_sph_trans(const Ctx* c, const ShTab& T, double* v, double* cv, bool to_four) {
  const int L = T.L, nv = c->nlat * c->nlon;
  const size_t N = c->npt;
  std::vector<double> a(3 * L * L), b(3 * L * L);
  for (int cell = 0; cell < c->ncell; ++cell) {
    double* cc = cv + (size_t)cell * 3 * L * L;
    if (to_four) {
      for (int k = 0; k < 3; ++k) sh_anal(c, T, v + (size_t)cell * nv + k * N, &a[(size_t)k * L * L], &b[(size_t)k * L * L]);
      sh_pack(L, a.data(), b.data(), cc);
    } else {
      sh_unpack(L, cc, a.data(), b.data());
      for (int k = 0; k < 3; ++k)
        sh_synth(T, T.PG, c->nlat, &a[(size_t)k * L * L], &b[(size_t)k * L * L], v + (size_t)cell * nv + k * N);
    }
  }
}
// rbc%g <- g, Rbc_BuildSurfaceSource(gFlag), SourceList_UpdateDensity(updateG)
static void set_g_from_grid(Ctx* c, const ShTab& T, const double* g) {
  const int L = T.L, nlat = c->nlat, nlon = c->nlon, nv = nlat * nlon;
  const size_t N = c->npt, S = (size_t)4 * 2 * nlat * nlon;  // per cell and variable
  c->g.assign(g, g + 3 * N);
  c->sg.resize(3 * N);
  c->spl_G.resize(3 * S * c->ncell);
  std::vector<double> gd(nv), a(L * L), b(L * L), fe((size_t)(nlat + 1) * nlon * 3), tab(3 * S);
  for (int cell = 0; cell < c->ncell; ++cell) {
    for (int k = 0; k < 3; ++k) {
      for (int r = 0; r < nv; ++r) gd[r] = g[(size_t)cell * nv + r + k * N] * c->detJ[(size_t)cell * nv + r];
      sh_anal(c, T, gd.data(), a.data(), b.data());  // ShAnalGau + ShFilter (degree < nlat0)
      sh_synth(T, T.PE, nlat + 1, a.data(), b.data(), &fe[(size_t)(nlat + 1) * nlon * k]);
    }
    spline_build_on_sphere(nlat, nlon, 3, fe.data(), tab.data());
    std::copy(tab.begin(), tab.end(), c->spl_G.begin() + (size_t)cell * 3 * S);
  }
  for (size_t p = 0; p < N; ++p) {
    const int ilat = (int)((p % nv) % nlat);
    const double ds = c->detJ[p] * c->w[ilat];
    for (int k = 0; k < 3; ++k) c->sg[p + k * N] = c->g[p + k * N] * ds;
  }
  c->has_g = true;
}

// ---------------------------------------------------------------------------
// Membrane mechanics: RBC_ComputeGeometry (ModRbc.F90:404-509),
// RBC_CovarGrad_Vec / RBC_CovarGrad_Tensor (:527-658), Shell_ResForce,
// Shell_ElasStrs, Shell_Bend (:815-963).  Surface derivatives through
// ShAnalGau + ShGradGau (ModSphpk.F90:74-105, 377-417: Spherepack gradgs
// with the sin(theta) factor restored, so v = d/dtheta and w = d/dphi of the
// degree < nlat expansion).  Per-cell fields are [k][nv], r = ilat + nlat*ilon;
// 2x2 tensors [ij][nv] with ij = 2*(i-1) + (j-1).

// d pbar(m, n, theta) / d theta from (1 - x^2) dP_n^m/dx = (n + m) P_{n-1}^m - n x P_n^m
// in the orthonormal normalisation (sin(theta) > 0 on the Gauss rows)
static void dpbar_table(int L, double theta, const double* P, double* dP) {
  const double x = std::cos(theta), s = std::sin(theta);
  for (int i = 0; i < L * L; ++i) dP[i] = 0.;
  for (int m = 0; m < L; ++m)
    for (int n = m; n < L; ++n) {
      const double q = n > m ? std::sqrt((2.0 * n + 1.0) * (n + m) * (n - m) / (2.0 * n - 1.0)) * P[m * L + n - 1] : 0.0;
      dP[m * L + n] = (n * x * P[m * L + n] - q) / s;
    }
}
struct MbTab {
  ShTab T;                 // degree < nlat (no ShFilter in the geometry and force)
  std::vector<double> DG;  // dpbar at the Gauss rows, [i][m][n]
};
static void mb_setup(const Ctx* c, MbTab& M) {
  const int L = c->nlat;
  sh_setup(c, L, M.T);
  M.DG.assign((size_t)c->nlat * L * L, 0.);
  for (int i = 0; i < c->nlat; ++i) dpbar_table(L, c->th[i], &M.T.PG[(size_t)i * L * L], &M.DG[(size_t)i * L * L]);
}
// ShAnalGau + ShGradGau of one field: vt = d/dtheta, vp = d/dphi at the Gauss points
static void sh_grad(const Ctx* c, const MbTab& M, const double* v, double* vt, double* vp) {
  const int L = M.T.L, nlat = c->nlat, nlon = c->nlon;
  std::vector<double> a(L * L), b(L * L), G(L), H(L), Gt(L), Ht(L);
  sh_anal(c, M.T, v, a.data(), b.data());
  for (int i = 0; i < nlat; ++i) {
    for (int m = 0; m < L; ++m) {
      G[m] = H[m] = Gt[m] = Ht[m] = 0.;
      for (int n = m; n < L; ++n) {
        const size_t q = ((size_t)i * L + m) * L + n;
        G[m] += M.T.PG[q] * a[m * L + n]; H[m] += M.T.PG[q] * b[m * L + n];
        Gt[m] += M.DG[q] * a[m * L + n]; Ht[m] += M.DG[q] * b[m * L + n];
      }
    }
    for (int j = 0; j < nlon; ++j) {
      double st = 0.5 * Gt[0], sp = 0.;
      for (int m = 1; m < L; ++m) {
        const double cm = M.T.cs[m * nlon + j], sm = M.T.sn[m * nlon + j];
        st += Gt[m] * cm - Ht[m] * sm;
        sp += -m * (G[m] * sm + H[m] * cm);
      }
      vt[i + nlat * j] = st;
      vp[i + nlat * j] = sp;
    }
  }
}
struct CellGeom {
  std::vector<double> a1, a2, a3, a1r, a2r;  // [k][nv]
  std::vector<double> a, ar, b;              // [ij][nv]
  std::vector<double> detJ;                  // [nv]
  double area = 0, vol = 0, xc[3] = {0, 0, 0}, meshSize = 0;
};
static inline double dot3(const double* u, const double* v, int nv, int r) {
  return u[r] * v[r] + u[r + nv] * v[r + nv] + u[r + 2 * nv] * v[r + 2 * nv];
}
// RBC_ComputeGeometry of one cell, x [k][nv]
static void compute_geometry(const Ctx* c, const MbTab& M, const double* x, CellGeom& G) {
  const int nlat = c->nlat, nlon = c->nlon, nv = nlat * nlon;
  G.a1.assign(3 * nv, 0.); G.a2.assign(3 * nv, 0.); G.a3.assign(3 * nv, 0.);
  G.a1r.assign(3 * nv, 0.); G.a2r.assign(3 * nv, 0.);
  G.a.assign(4 * nv, 0.); G.ar.assign(4 * nv, 0.); G.b.assign(4 * nv, 0.); G.detJ.assign(nv, 0.);
  for (int k = 0; k < 3; ++k) sh_grad(c, M, x + (size_t)k * nv, &G.a1[(size_t)k * nv], &G.a2[(size_t)k * nv]);
  for (int r = 0; r < nv; ++r) {
    const int ilat = r % nlat;
    const double* a1 = G.a1.data();
    const double* a2 = G.a2.data();
    const double a11 = dot3(a1, a1, nv, r), a12 = dot3(a1, a2, nv, r), a22 = dot3(a2, a2, nv, r);
    const double detA = a11 * a22 - a12 * a12, idet = 1. / detA;
    const double r11 = idet * a22, r12 = -idet * a12, r21 = -idet * a12, r22 = idet * a11;
    G.a[r] = a11; G.a[nv + r] = a12; G.a[2 * nv + r] = a12; G.a[3 * nv + r] = a22;
    G.ar[r] = r11; G.ar[nv + r] = r12; G.ar[2 * nv + r] = r21; G.ar[3 * nv + r] = r22;
    double n[3];
    for (int k = 0; k < 3; ++k) {
      G.a1r[k * nv + r] = r11 * a1[k * nv + r] + r12 * a2[k * nv + r];
      G.a2r[k * nv + r] = r21 * a1[k * nv + r] + r22 * a2[k * nv + r];
    }
    n[0] = a1[nv + r] * a2[2 * nv + r] - a1[2 * nv + r] * a2[nv + r];
    n[1] = a1[2 * nv + r] * a2[r] - a1[r] * a2[2 * nv + r];
    n[2] = a1[r] * a2[nv + r] - a1[nv + r] * a2[r];
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) G.a3[k * nv + r] = n[k] / nn;
    G.detJ[r] = std::sqrt(detA) / std::sin(c->th[ilat]);
  }
  // curvature tensor b = -(a_i . d a3 / d theta_j)
  std::vector<double> a31(3 * nv), a32(3 * nv);
  for (int k = 0; k < 3; ++k) sh_grad(c, M, &G.a3[(size_t)k * nv], &a31[(size_t)k * nv], &a32[(size_t)k * nv]);
  for (int r = 0; r < nv; ++r) {
    G.b[r] = -dot3(G.a1.data(), a31.data(), nv, r);
    G.b[nv + r] = -dot3(G.a1.data(), a32.data(), nv, r);
    G.b[2 * nv + r] = -dot3(G.a2.data(), a31.data(), nv, r);
    G.b[3 * nv + r] = -dot3(G.a2.data(), a32.data(), nv, r);
  }
  // centroid and area (ilat outer, ilon inner), then volume
  G.area = 0; G.xc[0] = G.xc[1] = G.xc[2] = 0;
  for (int i = 0; i < nlat; ++i)
    for (int j = 0; j < nlon; ++j) {
      const int r = i + nlat * j;
      const double ds = G.detJ[r] * c->w[i];
      G.area += ds;
      for (int k = 0; k < 3; ++k) G.xc[k] += ds * x[(size_t)k * nv + r];
    }
  for (int k = 0; k < 3; ++k) G.xc[k] /= G.area;
  G.vol = 0;
  for (int j = 0; j < nlon; ++j)
    for (int i = 0; i < nlat; ++i) {
      const int r = i + nlat * j;
      const double ds = G.detJ[r] * c->w[i];
      double d = 0;
      for (int k = 0; k < 3; ++k) d += G.a3[(size_t)k * nv + r] * (x[(size_t)k * nv + r] - G.xc[k]);
      G.vol += ds * d;
    }
  G.vol *= THRD;
  G.meshSize = std::sqrt(G.area / ((double)nlat * nlat));
}
// RBC_CovarGrad_Tensor: t [ij][nv] (contravariant) -> dt [ij][kd][nv], kd = derivative direction
static void covar_grad_tensor(const Ctx* c, const MbTab& M, const CellGeom& G, const double* t, double* dt) {
  const int nv = c->nlat * c->nlon;
  std::vector<double> tc(9 * (size_t)nv), t1(9 * (size_t)nv), t2(9 * (size_t)nv);
  for (int r = 0; r < nv; ++r)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double a1i = G.a1[i * nv + r], a2i = G.a2[i * nv + r], a1j = G.a1[j * nv + r], a2j = G.a2[j * nv + r];
        tc[(size_t)(3 * i + j) * nv + r] = t[r] * a1i * a1j + t[nv + r] * a1i * a2j + t[2 * nv + r] * a2i * a1j +
                                          t[3 * nv + r] * a2i * a2j;
      }
  for (int q = 0; q < 9; ++q) sh_grad(c, M, &tc[(size_t)q * nv], &t1[(size_t)q * nv], &t2[(size_t)q * nv]);
  for (int r = 0; r < nv; ++r) {
    double u[2][3];
    for (int k = 0; k < 3; ++k) { u[0][k] = G.a1r[k * nv + r]; u[1][k] = G.a2r[k * nv + r]; }
    for (int kd = 0; kd < 2; ++kd) {
      const std::vector<double>& td = kd == 0 ? t1 : t2;
      for (int al = 0; al < 2; ++al)
        for (int be = 0; be < 2; ++be) {
          double s = 0;
          for (int i = 0; i < 3; ++i) {
            double mv = 0;
            for (int j = 0; j < 3; ++j) mv += td[(size_t)(3 * i + j) * nv + r] * u[be][j];
            s += u[al][i] * mv;
          }
          dt[(size_t)((2 * al + be) * 2 + kd) * nv + r] = s;
        }
    }
  }
}
// RBC_CovarGrad_Vec: v [i][nv] (contravariant) -> dv [ij][nv], dv(i, j) = dv^i_j
static void covar_grad_vec(const Ctx* c, const MbTab& M, const CellGeom& G, const double* v, double* dv) {
  const int nv = c->nlat * c->nlon;
  std::vector<double> vc(3 * (size_t)nv), v1(3 * (size_t)nv), v2(3 * (size_t)nv);
  for (int r = 0; r < nv; ++r)
    for (int k = 0; k < 3; ++k) vc[(size_t)k * nv + r] = v[r] * G.a1[k * nv + r] + v[nv + r] * G.a2[k * nv + r];
  for (int k = 0; k < 3; ++k) sh_grad(c, M, &vc[(size_t)k * nv], &v1[(size_t)k * nv], &v2[(size_t)k * nv]);
  for (int r = 0; r < nv; ++r) {
    dv[r] = dot3(G.a1r.data(), v1.data(), nv, r);
    dv[nv + r] = dot3(G.a1r.data(), v2.data(), nv, r);
    dv[2 * nv + r] = dot3(G.a2r.data(), v1.data(), nv, r);
    dv[3 * nv + r] = dot3(G.a2r.data(), v2.data(), nv, r);
  }
}
static inline void mm2(const double* A, const double* B, double* C) {  // 2x2 row-major products
  C[0] = A[0] * B[0] + A[1] * B[2]; C[1] = A[0] * B[1] + A[1] * B[3];
  C[2] = A[2] * B[0] + A[3] * B[2]; C[3] = A[2] * B[1] + A[3] * B[3];
}
// Shell_ResForce of one cell (geometry G) against its reference (ar_ref, b_ref
// [ij][nv]): f [k][nv], Cartesian
static void shell_res_force(const Ctx* c, const MbTab& M, const CellGeom& G, const double* ar_ref, const double* b_ref,
                            double ES, double ED, double EB, double* f) {
  const int nlat = c->nlat, nlon = c->nlon, nv = nlat * nlon;
  std::vector<double> tau(4 * (size_t)nv), bnd(4 * (size_t)nv), dtau(8 * (size_t)nv), dbnd(8 * (size_t)nv);
  std::vector<double> taun(2 * (size_t)nv), dtaun(4 * (size_t)nv), fl(3 * (size_t)nv);
  for (int r = 0; r < nv; ++r) {
    double a[4], ar[4], arr[4], b[4], brf[4], V2[4];
    for (int q = 0; q < 4; ++q) {
      a[q] = G.a[q * nv + r]; ar[q] = G.ar[q * nv + r]; arr[q] = ar_ref[q * nv + r];
      b[q] = G.b[q * nv + r]; brf[q] = b_ref[q * nv + r];
    }
    // Shell_ElasStrs (:906-942)
    mm2(a, arr, V2);
    const double lbd1 = V2[0] + V2[3] - 2.0;
    const double lbd2 = V2[0] * V2[3] - V2[1] * V2[2] - 1.0;
    const double JS = std::sqrt(V2[0] * V2[3] - V2[1] * V2[2]);
    for (int q = 0; q < 4; ++q) tau[q * nv + r] = 0.5 * ES / JS * (lbd1 + 1.0) * arr[q] + 0.5 * JS * (ED * lbd2 - ES) * ar[q];
    // Shell_Bend (:949-963)
    double bm[4], bmr[4], d[4], o[4];
    mm2(ar, b, bm);
    mm2(arr, brf, bmr);
    for (int q = 0; q < 4; ++q) d[q] = bm[q] - bmr[q];
    mm2(d, ar, o);
    for (int q = 0; q < 4; ++q) bnd[q * nv + r] = -EB * o[q];
  }
  covar_grad_tensor(c, M, G, bnd.data(), dbnd.data());
  auto D = [&](const std::vector<double>& t, int i, int j, int kd, int r) { return t[(size_t)((2 * i + j) * 2 + kd) * nv + r]; };
  for (int r = 0; r < nv; ++r) {
    taun[r] = D(dbnd, 0, 0, 0, r) + D(dbnd, 1, 0, 1, r);
    taun[nv + r] = D(dbnd, 0, 1, 0, r) + D(dbnd, 1, 1, 1, r);
  }
  covar_grad_tensor(c, M, G, tau.data(), dtau.data());
  for (int r = 0; r < nv; ++r) {
    double f1 = -D(dtau, 0, 0, 0, r) - D(dtau, 1, 0, 1, r);
    double f2 = -D(dtau, 0, 1, 0, r) - D(dtau, 1, 1, 1, r);
    const double b11 = G.b[r], b12 = G.b[nv + r], b21 = G.b[2 * nv + r], b22 = G.b[3 * nv + r];
    const double bt1 = b11 * taun[r] + b12 * taun[nv + r], bt2 = b21 * taun[r] + b22 * taun[nv + r];
    f1 += G.ar[r] * bt1 + G.ar[nv + r] * bt2;
    f2 += G.ar[2 * nv + r] * bt1 + G.ar[3 * nv + r] * bt2;
    fl[r] = f1;
    fl[nv + r] = f2;
  }
  covar_grad_vec(c, M, G, taun.data(), dtaun.data());
  for (int r = 0; r < nv; ++r) {
    double tb = 0;
    for (int q = 0; q < 4; ++q) tb += tau[q * nv + r] * G.b[q * nv + r];
    fl[2 * nv + r] = -dtaun[r] - dtaun[3 * nv + r] - tb;
  }
  // subtract the average normal force (ilon outer, ilat inner)
  double fnTot = 0;
  for (int j = 0; j < nlon; ++j)
    for (int i = 0; i < nlat; ++i) fnTot += fl[2 * nv + i + nlat * j] * G.detJ[i + nlat * j] * c->w[i];
  for (int r = 0; r < nv; ++r) fl[2 * nv + r] -= fnTot / G.area;
  for (int r = 0; r < nv; ++r)
    for (int k = 0; k < 3; ++k)
      f[(size_t)k * nv + r] = fl[r] * G.a1[k * nv + r] + fl[nv + r] * G.a2[k * nv + r] + fl[2 * nv + r] * G.a3[k * nv + r];
}
// gather cell `cell` of an SoA point array (3 x n) into [k][nv]
static void gather_cell(const double* x, size_t n, int cell, int nv, double* out) {
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < nv; ++r) out[(size_t)k * nv + r] = x[(size_t)cell * nv + r + k * n];
}

extern "C" {

int API(abi_version)(void) { return RBC3D_ABI_VERSION; }

rbc3d_status API(ewald_prms)(double alpha, double eps, const double Lb[3], int P, double* rc, int Nb[3]) {
  double s = 1.;
  for (int it = 0; it < 10; ++it) {
    s = 0.75 * std::sqrt(PI) * eps / (s * s * s + 1.5 * s + 0.75 / s);
    s = std::sqrt(-std::log(s));
  }
  double r = std::sqrt(alpha / PI) * s;
  r = std::min(std::min(Lb[0] / 3.001, Lb[1] / 3.001), std::min(Lb[2] / 3.001, r));
  *rc = r;
  for (int d = 0; d < 3; ++d) Nb[d] = 2 * (int)std::ceil(std::sqrt(-std::log(eps) / (PI * alpha)) * Lb[d]);
  Nb[2] = std::max(Nb[2], P);
  return RBC3D_OK;
}

rbc3d_status API(create)(const rbc3d_params* prm, Ctx** out) {
  if (!prm || !out) return RBC3D_ERR_ARG;
  Ctx* c = new Ctx();
  c->prm = *prm;
  for (int d = 0; d < 3; ++d) c->iLb[d] = 1. / prm->Lb[d];
  if (prm->ncelltypes < 1 || prm->ncelltypes > RBC3D_MAX_CELLTYPES) { delete c; return RBC3D_ERR_ARG; }
  for (int l = 0; l < prm->ncelltypes; ++l) {  // initCOEFs, ModConf.F90:327
    if (prm->viscRat[l] > 0) { c->Acoef[l] = 1. + prm->viscRat[l]; c->Bcoef[l] = 1. - prm->viscRat[l]; }
    else { c->Acoef[l] = 1.; c->Bcoef[l] = -1.; }
  }
  c->E.build(prm->alpha, prm->rc);
  c->nlat = prm->nlat; c->nlon = prm->nlon;
  pme_init(c);
  hash_setup(c, c->hcell);
  *out = c;
  return RBC3D_OK;
}

rbc3d_status API(destroy)(Ctx* c) { delete c; return RBC3D_OK; }
const char* API(last_error)(const Ctx* c) { return c ? c->err.c_str() : "null context"; }

// RBC_Create grid + RbcPolarPatch_Create, ModPolarPatch.F90:27-75
rbc3d_status API(set_cell_grid)(Ctx* c, const double* th, const double* phi, const double* w) {
  int nlat = c->nlat, nlon = c->nlon;
  c->th.assign(th, th + nlat); c->phi.assign(phi, phi + nlon); c->w.assign(w, w + nlat);
  c->radius = PI / std::sqrt((double)nlat);
  double h = PI / nlat;
  c->nrad = 2 * (int)nint(c->radius / h);
  c->nazm = 2 * c->nrad;
  std::vector<double> thL(c->nrad), phiL(c->nazm);
  c->pw.resize(c->nrad);
  gauleg(0., c->radius, c->nrad, thL.data(), c->pw.data());
  for (int i = 0; i < c->nrad; ++i) {
    c->pw[i] = c->pw[i] * std::sin(thL[i]) * (TWO_PI / c->nazm);
    c->pw[i] = c->pw[i] * MaskFunc(thL[i] / c->radius);
  }
  for (int j = 0; j < c->nazm; ++j) phiL[j] = j * TWO_PI / c->nazm;
  size_t np = (size_t)c->nrad * c->nazm;
  c->thG.resize(np * nlat * nlon); c->phiG.resize(np * nlat * nlon);
  for (int ilon = 0; ilon < nlon; ++ilon)
    for (int ilat = 0; ilat < nlat; ++ilat) {
      size_t b = np * (ilat + (size_t)nlat * ilon);
      polar_patch_build(c->th[ilat], c->phi[ilon], thL.data(), c->nrad, phiL.data(), c->nazm,
                        c->thG.data() + b, c->phiG.data() + b);
    }
  return RBC3D_OK;
}

rbc3d_status API(set_cells)(Ctx* c, int ncell, const int* celltype, const double* x, const double* a3,
                            const double* detJ, const double* area, const double* meshSize,
                            const double* spl_x, const double* spl_a3, const double* spl_detJ) {
  if (c->th.empty()) return fail(c, RBC3D_ERR_STATE, "cell grid not set");
  c->ncell = ncell;
  int nv = c->nlat * c->nlon;
  c->npt = ncell * nv;
  size_t N = c->npt, S = (size_t)ncell * 4 * 2 * c->nlat * c->nlon;
  c->celltype.assign(celltype, celltype + ncell);
  for (int t : c->celltype) if (t < 0 || t >= c->prm.ncelltypes) return fail(c, RBC3D_ERR_ARG, "bad celltype");
  c->x.assign(x, x + 3 * N); c->a3.assign(a3, a3 + 3 * N); c->detJ.assign(detJ, detJ + N);
  c->area.assign(area, area + ncell); c->meshSize.assign(meshSize, meshSize + ncell);
  c->spl_x.assign(spl_x, spl_x + 3 * S); c->spl_a3.assign(spl_a3, spl_a3 + 3 * S);
  c->spl_detJ.assign(spl_detJ, spl_detJ + S);
  hash_build(c->hcell, c->npt, c->x.data());
  c->has_f = c->has_g = false;
  return RBC3D_OK;
}

rbc3d_status API(set_cell_density)(Ctx* c, const double* f, const double* g, const double* spl_F, const double* spl_G) {
  if ((f && !spl_F) || (g && !spl_G)) return fail(c, RBC3D_ERR_ARG, "density without spline table");
  size_t N = c->npt, S = (size_t)c->ncell * 4 * 2 * c->nlat * c->nlon;
  int nv = c->nlat * c->nlon;
  auto mk = [&](const double* src, std::vector<double>& raw, std::vector<double>& scaled) {
    raw.assign(src, src + 3 * N);
    scaled.resize(3 * N);
    for (size_t p = 0; p < N; ++p) {
      int ilat = (int)((p % nv) % c->nlat);
      double ds = c->detJ[p] * c->w[ilat];
      for (int k = 0; k < 3; ++k) scaled[p + k * N] = raw[p + k * N] * ds;
    }
  };
  if (f) { mk(f, c->f, c->sf); c->spl_F.assign(spl_F, spl_F + 3 * S); c->has_f = true; }
  if (g) { mk(g, c->g, c->sg); c->spl_G.assign(spl_G, spl_G + 3 * S); c->has_g = true; }
  return RBC3D_OK;
}

rbc3d_status API(set_walls)(Ctx* c, int nvert, int nele, const double* x, const int* e2v, const int* glb) {
  c->nvert = nvert; c->nele = nele;
  c->wx.assign(x, x + 3 * (size_t)nvert);
  c->e2v.assign(e2v, e2v + 3 * (size_t)nele);
  c->glb.assign(glb, glb + nvert);
  c->ndof = 0;
  for (int g : c->glb) c->ndof = std::max(c->ndof, 3 * g);
  c->wf.assign(3 * (size_t)nvert, 0.);
  wall_geometry(c);
  c->wall_prepared = false;
  return RBC3D_OK;
}
rbc3d_status API(set_wall_density)(Ctx* c, const double* f) { c->wf.assign(f, f + 3 * (size_t)c->nvert); return RBC3D_OK; }
rbc3d_status API(get_wall_density)(Ctx* c, double* f) { std::copy(c->wf.begin(), c->wf.end(), f); return RBC3D_OK; }
rbc3d_status API(set_raw_targets)(Ctx* c, int n, const double* x) { c->nraw = n; c->rawx.assign(x, x + 3 * (size_t)n); return RBC3D_OK; }
int API(num_targets)(const Ctx* c, int which) {
  return which == RBC3D_TLIST_RBC ? c->npt : which == RBC3D_TLIST_WALL ? c->nvert : which == RBC3D_TLIST_RAW ? c->nraw : -1;
}

rbc3d_status API(add_int_on_rbcs)(Ctx* c, int which, double c1, double c2, int prec, double* v) {
  (void)prec;
  TView t;
  if (!make_tlist(c, which, t)) return fail(c, RBC3D_ERR_ARG, "bad tlist");
  return add_int_on_rbcs(c, t, c1, c2, v);
}
rbc3d_status API(add_int_on_walls)(Ctx* c, int which, double c1, int prec, double* v) {
  (void)prec;
  TView t;
  if (!make_tlist(c, which, t)) return fail(c, RBC3D_ERR_ARG, "bad tlist");
  return add_int_on_walls(c, which, t, c1, v);
}
rbc3d_status API(prepare_sing_int_on_wall)(Ctx* c) { if (c->nvert) prepare_sing_int_on_wall(c); return RBC3D_OK; }
rbc3d_status API(pme_distrib_source)(Ctx* c, double c1, double c2, int cells, int walls, int prec) {
  (void)prec;
  return pme_distrib_source(c, c1, c2, cells, walls);
}
rbc3d_status API(pme_transform)(Ctx* c) { pme_transform(c); return RBC3D_OK; }
rbc3d_status API(pme_add_interp_vel)(Ctx* c, int which, double* v) {
  TView t;
  if (!make_tlist(c, which, t)) return fail(c, RBC3D_ERR_ARG, "bad tlist");
  pme_add_interp_vel(c, t, v);
  return RBC3D_OK;
}

rbc3d_status API(matvec)(Ctx* c, int which, double c1, double c2, unsigned terms, int prec, double* v) {
  (void)prec;
  TView t;
  if (!make_tlist(c, which, t)) return fail(c, RBC3D_ERR_ARG, "bad tlist");
  rbc3d_status s;
  if (terms & (RBC3D_TERM_REAL | RBC3D_TERM_CORR | RBC3D_TERM_LINEAR)) {
    if ((terms & 7u) != 7u) return fail(c, RBC3D_ERR_ARG, "oracle evaluates REAL|CORR|LINEAR together");
    if ((s = add_int_on_rbcs(c, t, c1, c2, v))) return s;
  }
  if (terms & RBC3D_TERM_WALLS)
    if ((s = add_int_on_walls(c, which, t, c1, v))) return s;
  if (terms & RBC3D_TERM_PME) {
    if ((s = pme_distrib_source(c, c1, c2, 1, (terms & RBC3D_TERM_WALLS) ? 1 : 0))) return s;
    pme_transform(c);
    pme_add_interp_vel(c, t, v);
  }
  return RBC3D_OK;
}

rbc3d_status API(calc_velocity_field)(Ctx* c, int which, int prec, double* v) {
  (void)prec;
  TView t;
  if (!make_tlist(c, which, t)) return fail(c, RBC3D_ERR_ARG, "bad tlist");
  std::fill(v, v + 3 * (size_t)t.n, 0.);
  double c1 = 1.0 / (4. * PI), c2 = 1.0 / (4. * PI);
  rbc3d_status s;
  if ((s = add_int_on_rbcs(c, t, c1, c2, v))) return s;
  if ((s = add_int_on_walls(c, which, t, c1, v))) return s;
  if ((s = pme_distrib_source(c, c1, c2, 1, 1))) return s;
  pme_transform(c);
  pme_add_interp_vel(c, t, v);
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < t.n; ++i) v[i + (size_t)k * t.n] += c->prm.vBkg[k];
  return RBC3D_OK;
}

rbc3d_status API(compute_wall_residual_vel)(Ctx* c, int prec, double* v) { (void)prec; return wall_residual(c, v); }

rbc3d_status API(wall_matmult)(Ctx* c, int prec, const double* u, double* y) {
  (void)prec;
  std::vector<double> fsave = c->wf;
  rbc3d_status s = wall_matmult(c, u, y);
  c->wf = fsave;
  return s;
}

// NoSlipWall, ModNoSlip.F90:45-150
rbc3d_status API(no_slip_wall)(Ctx* c, const rbc3d_solve_opts* o, const double* guess, rbc3d_solve_stats* st) {
  if (c->nvert == 0) return RBC3D_OK;
  if (!c->wall_prepared) return fail(c, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
  auto t0 = std::chrono::steady_clock::now();
  rbc3d_solve_stats s{};
  const int nv = c->nvert, n = c->ndof;
  std::vector<double> f0 = c->wf, v(3 * (size_t)nv), rhs(n), x(n, 0.);
  rbc3d_status err = wall_residual(c, v.data());
  if (err) return err;
  for (double& a : v) a = -a;
  assemble_to_1d(c, v.data(), rhs.data());
  if (o->guess && guess) x.assign(guess, guess + n);
  auto A = [&](const double* u, double* y) -> rbc3d_status { return wall_matmult(c, u, y); };
  int r = gmres(n, A, rhs, x, o->rtol, o->max_it, o->restart > 0 ? o->restart : 30, &s, &err);
  if (r < 0) return err;
  std::vector<double> finc(3 * (size_t)nv);
  assemble_from_1d(c, x.data(), finc.data());
  for (size_t i = 0; i < finc.size(); ++i) c->wf[i] = f0[i] + finc[i];
  s.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = s;
  return s.converged ? RBC3D_OK : fail(c, RBC3D_ERR_NOCONV, "GMRES reached max_it");
}

rbc3d_status API(get_counts)(const Ctx* c, rbc3d_counts* out) { *out = c->counts; return RBC3D_OK; }

int API(cell_dof)(const Ctx* c, int nlat0) { return 3 * nlat0 * nlat0 * c->ncell; }

rbc3d_status API(set_ref_cells)(Ctx* c, int ntypes, const double* xref, const double* ES, const double* ED,
                                const double* EB) {
  if (!c || ntypes < 1 || ntypes > RBC3D_MAX_CELLTYPES || !xref || !ES || !ED || !EB) return fail(c, RBC3D_ERR_ARG, "set_ref_cells");
  if (c->th.empty()) return fail(c, RBC3D_ERR_STATE, "cell grid not set");
  const int nv = c->nlat * c->nlon;
  MbTab M;
  mb_setup(c, M);
  c->nref = ntypes;
  c->ref_ar.assign((size_t)ntypes * 4 * nv, 0.);
  c->ref_b.assign((size_t)ntypes * 4 * nv, 0.);
  c->ES.assign(ES, ES + ntypes); c->ED.assign(ED, ED + ntypes); c->EB.assign(EB, EB + ntypes);
  std::vector<double> xc(3 * (size_t)nv);
  for (int t = 0; t < ntypes; ++t) {
    gather_cell(xref, (size_t)ntypes * nv, t, nv, xc.data());
    CellGeom G;
    compute_geometry(c, M, xc.data(), G);
    std::copy(G.ar.begin(), G.ar.end(), c->ref_ar.begin() + (size_t)t * 4 * nv);
    std::copy(G.b.begin(), G.b.end(), c->ref_b.begin() + (size_t)t * 4 * nv);
  }
  return RBC3D_OK;
}

rbc3d_status API(cell_geometry)(Ctx* c, int ncell, const double* x, double* a3, double* detJ, double* area, double* vol) {
  if (!c || ncell < 0 || (ncell > 0 && !x)) return fail(c, RBC3D_ERR_ARG, "cell_geometry");
  if (c->th.empty()) return fail(c, RBC3D_ERR_STATE, "cell grid not set");
  const int nv = c->nlat * c->nlon;
  const size_t n = (size_t)ncell * nv;
  MbTab M;
  mb_setup(c, M);
  std::vector<double> xc(3 * (size_t)nv);
  for (int cell = 0; cell < ncell; ++cell) {
    gather_cell(x, n, cell, nv, xc.data());
    CellGeom G;
    compute_geometry(c, M, xc.data(), G);
    for (int r = 0; r < nv; ++r) {
      const size_t p = (size_t)cell * nv + r;
      if (a3) for (int k = 0; k < 3; ++k) a3[p + k * n] = G.a3[(size_t)k * nv + r];
      if (detJ) detJ[p] = G.detJ[r];
    }
    if (area) area[cell] = G.area;
    if (vol) vol[cell] = G.vol;
  }
  return RBC3D_OK;
}

// AddIntraCellRepulsionForce (ModRepulsion.F90:126-266): every point of a
// cell against the points of the same cell (those in the 27 hash cells
// around it include every point within epsDist, the only ones that count)
rbc3d_status API(intra_cell_repulsion)(Ctx* c, int ncell, const double* x, const double* a3, const double* area,
                                       double force_coef, double* f, int* count) {
  if (!c || ncell < 0 || (ncell > 0 && (!x || !a3 || !area || !f))) return fail(c, RBC3D_ERR_ARG, "intra_cell_repulsion");
  if (c->th.empty() || c->radius <= 0) return fail(c, RBC3D_ERR_STATE, "cell grid not set");
  const int nlat = c->nlat, nlon = c->nlon, nv = nlat * nlon;
  const size_t n = (size_t)ncell * nv;
  int cnt = 0;
  for (int cell = 0; cell < ncell; ++cell) {
    const double epsDist = 2 * std::sqrt(area[cell]) / nlat, epsRef = c->radius;
    for (int ri = 0; ri < nv; ++ri) {
      const size_t pi = (size_t)cell * nv + ri;
      const int ilat = ri % nlat, ilon = ri / nlat;
      double dist = HUGE_VAL;
      for (int rj = 0; rj < nv; ++rj) {
        const size_t pj = (size_t)cell * nv + rj;
        const int jlat = rj % nlat, jlon = rj / nlat;
        if (dist_on_sphere(c->th[ilat], c->phi[ilon], c->th[jlat], c->phi[jlon]) < epsRef) continue;
        double xx[3], rr = 0;
        for (int k = 0; k < 3; ++k) { xx[k] = x[pi + k * n] - x[pj + k * n]; rr += xx[k] * xx[k]; }
        rr = std::sqrt(rr);
        if (rr > epsDist) continue;
        const double xxn = -(xx[0] * a3[pj] + xx[1] * a3[pj + n] + xx[2] * a3[pj + 2 * n]);
        if (xxn / rr < 0.707) continue;
        dist = std::min(dist, rr);
      }
      if (dist < epsDist) {
        const double FF = force_coef * std::exp(1 - dist / epsDist);
        for (int k = 0; k < 3; ++k) f[pi + k * n] += FF * a3[pi + k * n];
        ++cnt;
      }
    }
  }
  if (count) *count = cnt;
  return RBC3D_OK;
}

// InterCellRepulsion (ModRepulsion.F90:270-402) with Closest_Neighbor_Cell
// (:480-551) and Closest_Neighbor_Wall (:556-613), one rank (every target
// active): each cell point finds the nearest point of another cell over the
// 27 hash cells around it (projected onto that cell's spline surface when
// within 2 epsDist) and the nearest point of the wall's triangles; closer
// than epsDist it moves by 0.5 xx (epsDist - rr) / rr.  Cells of types with
// |viscRat| < viscRatThresh move pointwise, others (rigidsep) by the mean
// move of their moved points.  xout: the moved positions (3 x N).
rbc3d_status API(inter_cell_repulsion)(Ctx* c, double epsDist, double viscRatThresh, int rigidsep, double* xout,
                                       double* distMin, int* nmoved) {
  if (!c || !xout) return fail(c, RBC3D_ERR_ARG, "inter_cell_repulsion");
  const int nv = c->nlat * c->nlon, N = c->npt;
  std::vector<double> dx(3 * (size_t)N, 0.);
  double dmin = HUGE_VAL;
  int cnt = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(min : dmin) reduction(+ : cnt)
  for (int i = 0; i < N; ++i) {
    const double xi[3] = {c->x[i], c->x[i + (size_t)N], c->x[i + 2 * (size_t)N]};
    const int surf_i = i / nv;
    // Closest_Neighbor_Cell
    double dist1 = HUGE_VAL, x1[3] = {0, 0, 0};
    int j0 = -1;
    {
      const HashList& h = c->hcell;
      int i1, i2, i3;
      hash_index(h, xi, i1, i2, i3);
      for (int j1 = std::max(i1 - 1, 0); j1 <= std::min(i1 + 1, h.Nc[0] + 1); ++j1)
        for (int j2 = std::max(i2 - 1, 0); j2 <= std::min(i2 + 1, h.Nc[1] + 1); ++j2)
          for (int j3 = std::max(i3 - 1, 0); j3 <= std::min(i3 + 1, h.Nc[2] + 1); ++j3)
            for (int j = h.hoc[h.id(j1, j2, j3)]; j >= 0; j = h.next[j]) {
              if (j / nv == surf_i) continue;
              double xx[3], rr = 0;
              for (int k = 0; k < 3; ++k) {
                xx[k] = xi[k] - c->x[j + (size_t)k * N];
                xx[k] = xx[k] - nint(xx[k] * c->iLb[k]) * c->prm.Lb[k];
                rr += xx[k] * xx[k];
              }
              rr = std::sqrt(rr);
              if (rr < dist1) { dist1 = rr; j0 = j; }
            }
    }
    if (j0 >= 0 && dist1 <= 2 * epsDist) {
      const int cell0 = j0 / nv, r = j0 % nv, ilat0 = r % c->nlat, ilon0 = r / c->nlat;
      double x0[3], xtar[3];
      cellx(c, c->x, cell0, ilat0, ilon0, x0);
      for (int k = 0; k < 3; ++k) {
        double xx = xi[k] - x0[k];
        xx = xx - nint(xx * c->iLb[k]) * c->prm.Lb[k];
        xtar[k] = x0[k] + xx;
      }
      double th0 = c->th[ilat0], phi0 = c->phi[ilon0];
      Spline sx;
      cell_spline(c, c->spl_x, 3, cell0, sx);
      spline_find_projection(sx, xtar, th0, phi0, x1);
      double d2 = 0;
      for (int k = 0; k < 3; ++k) d2 += (xtar[k] - x1[k]) * (xtar[k] - x1[k]);
      dist1 = std::sqrt(d2);
    }
    // Closest_Neighbor_Wall
    double dist2 = HUGE_VAL, x2[3] = {0, 0, 0};
    if (c->nvert > 0) {
      const HashList& h = c->hwall;
      int i1, i2, i3;
      hash_index(h, xi, i1, i2, i3);
      for (int j1 = std::max(i1 - 1, 0); j1 <= std::min(i1 + 1, h.Nc[0] + 1); ++j1)
        for (int j2 = std::max(i2 - 1, 0); j2 <= std::min(i2 + 1, h.Nc[1] + 1); ++j2)
          for (int j3 = std::max(i3 - 1, 0); j3 <= std::min(i3 + 1, h.Nc[2] + 1); ++j3)
            for (int e = h.hoc[h.id(j1, j2, j3)]; e >= 0; e = h.next[e]) {
              double xe[9], fe[9], xtar[3];
              tri_coords(c, e, xe, fe);
              for (int k = 0; k < 3; ++k) {
                double xx = xi[k] - xe[0 + 3 * k];
                xx = xx - nint(xx * c->iLb[k]) * c->prm.Lb[k];
                xtar[k] = xe[0 + 3 * k] + xx;
              }
              double s0, t0;
              const double rr = min_dist_to_tri(xtar, xe, s0, t0);
              if (rr < dist2) {
                dist2 = rr;
                for (int k = 0; k < 3; ++k) x2[k] = (1 - s0 - t0) * xe[0 + 3 * k] + s0 * xe[1 + 3 * k] + t0 * xe[2 + 3 * k];
              }
            }
    }
    const bool cellwin = dist1 < dist2;
    const double dist = cellwin ? dist1 : dist2;
    const double* xj = cellwin ? x1 : x2;
    dmin = std::min(dmin, dist);
    if (dist < epsDist) {
      double xx[3], rr = 0;
      for (int k = 0; k < 3; ++k) {
        xx[k] = xi[k] - xj[k];
        xx[k] = xx[k] - nint(xx[k] * c->iLb[k]) * c->prm.Lb[k];
        rr += xx[k] * xx[k];
      }
      rr = std::sqrt(rr);
      for (int k = 0; k < 3; ++k) dx[i + (size_t)k * N] = 0.5 * xx[k] * (epsDist - rr) / rr;
      ++cnt;
    }
  }
  for (size_t q = 0; q < 3 * (size_t)N; ++q) xout[q] = c->x[q];
  for (int cell = 0; cell < c->ncell; ++cell) {
    const size_t p0 = (size_t)cell * nv;
    if (std::fabs(c->prm.viscRat[c->celltype[cell]]) < viscRatThresh) {
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < nv; ++r) xout[p0 + r + (size_t)k * N] += dx[p0 + r + (size_t)k * N];
    } else if (rigidsep) {
      double m[3] = {0, 0, 0};
      int nd = 0;
      for (int r = 0; r < nv; ++r) {
        const double a = dx[p0 + r], b = dx[p0 + r + (size_t)N], d = dx[p0 + r + 2 * (size_t)N];
        if (a * a + b * b + d * d > 0.) { m[0] += a; m[1] += b; m[2] += d; ++nd; }
      }
      if (nd > 0)
        for (int k = 0; k < 3; ++k)
          for (int r = 0; r < nv; ++r) xout[p0 + r + (size_t)k * N] += m[k] / nd;
    }
  }
  if (distMin) *distMin = dmin;
  if (nmoved) *nmoved = cnt;
  return RBC3D_OK;
}

rbc3d_status API(shell_res_force)(Ctx* c, int ncell, const int* celltype, const double* x, double* f) {
  if (!c || ncell < 0 || (ncell > 0 && (!celltype || !x || !f))) return fail(c, RBC3D_ERR_ARG, "shell_res_force");
  if (c->nref == 0) return fail(c, RBC3D_ERR_STATE, "reference cells not set");
  const int nv = c->nlat * c->nlon;
  const size_t n = (size_t)ncell * nv;
  for (int cell = 0; cell < ncell; ++cell)
    if (celltype[cell] < 0 || celltype[cell] >= c->nref) return fail(c, RBC3D_ERR_ARG, "bad celltype");
  MbTab M;
  mb_setup(c, M);
  std::vector<double> xc(3 * (size_t)nv), fc(3 * (size_t)nv);
  for (int cell = 0; cell < ncell; ++cell) {
    gather_cell(x, n, cell, nv, xc.data());
    CellGeom G;
    compute_geometry(c, M, xc.data(), G);
    const int t = celltype[cell];
    shell_res_force(c, M, G, &c->ref_ar[(size_t)t * 4 * nv], &c->ref_b[(size_t)t * 4 * nv], c->ES[t], c->ED[t], c->EB[t],
                    fc.data());
    for (int k = 0; k < 3; ++k)
      for (int r = 0; r < nv; ++r) f[(size_t)cell * nv + r + k * n] = fc[(size_t)k * nv + r];
  }
  return RBC3D_OK;
}

// Solve_RBC_Vel, ModVelSolver.F90:44-132 (Deflate off)
rbc3d_status API(solve_rbc_vel)(Ctx* c, const rbc3d_solve_opts* o, int nlat0, double* sol, double* v,
                                rbc3d_solve_stats* st) {
  if (!o || !v || nlat0 < 1 || nlat0 > c->nlat || 2 * (nlat0 - 1) >= c->nlon) return fail(c, RBC3D_ERR_ARG, "bad nlat0");
  if (c->npt == 0) return RBC3D_OK;
  auto t0 = std::chrono::steady_clock::now();
  rbc3d_solve_stats s{};
  ShTab T;
  sh_setup(c, nlat0, T);
  TView t;
  make_tlist(c, RBC3D_TLIST_RBC, t);
  const size_t N = c->npt;
  const int dof = 3 * nlat0 * nlat0 * c->ncell;
  const double ip4 = 1.0 / (4. * PI);
  rbc3d_status err;
  // Compute_Rhs (:455-515)
  std::vector<double> vv(3 * N, 0.), rhs(dof), x(dof, 0.);
  if ((err = add_int_on_rbcs(c, t, ip4, 0., vv.data()))) return err;
  if ((err = add_int_on_walls(c, RBC3D_TLIST_RBC, t, ip4, vv.data()))) return err;
  if ((err = pme_distrib_source(c, ip4, 0., 1, 1))) return err;
  pme_transform(c);
  pme_add_interp_vel(c, t, vv.data());
  for (int k = 0; k < 3; ++k)
    for (size_t i = 0; i < N; ++i) vv[i + k * N] += 2. * c->prm.vBkg[k] / t.Acoef[i];
  glob_sph_trans(c, T, vv.data(), rhs.data(), true);
  bool all_one = true;
  for (int l = 0; l < c->prm.ncelltypes; ++l) all_one = all_one && c->prm.viscRat[l] == 1.0;
  if (all_one) {
    x = rhs;
    s.converged = 1;
  } else {
    if (o->guess && sol) x.assign(sol, sol + dof);
    // MyMatMult (:523-601)
    std::vector<double> g(3 * N);
    auto A = [&](const double* u, double* y) -> rbc3d_status {
      glob_sph_trans(c, T, g.data(), const_cast<double*>(u), false);
      set_g_from_grid(c, T, g.data());
      std::fill(vv.begin(), vv.end(), 0.);
      rbc3d_status e;
      if ((e = add_int_on_rbcs(c, t, 0., -ip4, vv.data()))) return e;
      if ((e = pme_distrib_source(c, 0., -ip4, 1, 0))) return e;
      pme_transform(c);
      pme_add_interp_vel(c, t, vv.data());
      for (size_t i = 0; i < 3 * N; ++i) vv[i] += g[i];
      glob_sph_trans(c, T, vv.data(), y, true);
      return RBC3D_OK;
    };
    int r = gmres(dof, A, rhs, x, o->rtol, o->max_it, o->restart > 0 ? o->restart : 30, &s, &err);
    if (r < 0) return err;
  }
  if (sol) std::copy(x.begin(), x.end(), sol);
  glob_sph_trans(c, T, v, x.data(), false);
  s.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = s;
  return s.converged ? RBC3D_OK : fail(c, RBC3D_ERR_NOCONV, "GMRES reached max_it");
}

// Test hooks for the known-answer tests of the building blocks.
void API(kat_ewald_sl)(double alpha, double rc, int n, const double* r, double* A, double* B, int exact) {
  EwaldTables E;
  if (!exact) E.build(alpha, rc);
  for (int i = 0; i < n; ++i) {
    if (exact) ewald_sl_exact(r[i], alpha, A[i], B[i]);
    else E.sl(r[i], A[i], B[i]);
  }
}
void API(kat_ewald_dl)(double alpha, double rc, int n, const double* r, double* A, int exact) {
  EwaldTables E;
  if (!exact) E.build(alpha, rc);
  for (int i = 0; i < n; ++i) A[i] = exact ? ewald_dl_exact(r[i], alpha) : E.dl(r[i]);
}
void API(kat_mask)(int n, const double* x, double* f, int exact) {
  for (int i = 0; i < n; ++i) f[i] = exact ? mask_exact(x[i]) : MaskFunc(x[i]);
}
void API(kat_bspline)(double xc, int P, int* imin, double* w) { bspline(xc, P, *imin, w); }
void API(kat_gauleg)(double x1, double x2, int n, double* x, double* w) { gauleg(x1, x2, n, x, w); }
void API(kat_gauleg_sinh)(double xmin, double xmax, double a, double b, int n, double* x, double* w) {
  gauleg_sinh(xmin, xmax, a, b, n, x, w);
}
void API(kat_gqtri7)(double* r, double* s, double* w) {
  TriRule q = gq_tri7();
  for (int i = 0; i < 7; ++i) { r[i] = q.r[i]; s[i] = q.s[i]; w[i] = q.w[i]; }
}
void API(kat_fft)(double* re, double* im, int n, int sign) {
  std::vector<cplx> a(n);
  for (int i = 0; i < n; ++i) a[i] = cplx(re[i], im[i]);
  fft_c2c(a.data(), n, 1, sign);
  for (int i = 0; i < n; ++i) { re[i] = a[i].real(); im[i] = a[i].imag(); }
}
double API(kat_min_dist_to_tri)(const double* xtar, const double* x, double* s0, double* t0) {
  return min_dist_to_tri(xtar, x, *s0, *t0);
}
void API(kat_tri_int)(double alpha, double rc, const double* x, const double* f, const double* xtar, int duffy,
                      double s0, double t0, double* rhs, double* lhs) {
  EwaldTables E;
  E.build(alpha, rc);
  if (duffy) tri_int_duffy(E, x, f, xtar, s0, t0, rhs, lhs);
  else tri_int_regular(E, x, f, xtar, rhs, lhs);
}
// Spline interpolation of one cell's table at (th, phi): test hook.
void API(kat_spline_interp)(int m, int n, int nvar, const double* tab, int npt, const double* th,
                            const double* phi, double* out) {
  Spline s;
  s.set(m, n, nvar, tab);
  for (int p = 0; p < npt; ++p) spline_interp(s, th[p], phi[p], out + (size_t)p * nvar);
}
void API(kat_find_projection)(int m, int n, const double* tab, const double* xtar, double* th0, double* phi0,
                              double* x0) {
  Spline s;
  s.set(m, n, 3, tab);
  spline_find_projection(s, xtar, *th0, *phi0, x0);
}
// PME grid after PME_Transform (3 x G, x fastest) for white-box tests.
void API(pme_velocity_grid)(const Ctx* c, double* out) { std::copy(c->vv.begin(), c->vv.end(), out); }
void API(kat_pbar)(int L, double theta, double* P) { pbar_table(L, theta, P); }
void API(kat_spline_build)(int nlat, int nlon, int nvar, const double* f, double* tab) {
  spline_build_on_sphere(nlat, nlon, nvar, f, tab);
}
// Glob_Sph_Trans of the context's cells (to_four = 1: v -> c, else c -> v)
rbc3d_status API(kat_sph_trans)(Ctx* c, int nlat0, double* v, double* cv, int to_four) {
  ShTab T;
  sh_setup(c, nlat0, T);
  glob_sph_trans(c, T, v, cv, to_four != 0);
  return RBC3D_OK;
}
int API(set_threads)(int n) { if (n > 0) omp_set_num_threads(n); return omp_get_max_threads(); }

}  // extern "C"
