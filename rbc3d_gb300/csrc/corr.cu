// corr.cu -- FP64 singular and near-singular polar-patch corrections on the
// GPU: RBC_SingInt (ModRbcSingInt.F90:29-90) and RBC_NearSingInt with its
// Subtract / ReAdd halves (ModRbcSingInt.F90:103-310), including
// Spline_FindProjection (ModSpline.F90:203-269) and QuadFit_2D (normal
// equations + Cholesky, ModBasicMath.F90:234-284).
//
// Mapping: one warp per target for the self patch (nrad*nazm quadrature points
// spread over the lanes), one warp per (target, neighbour cell) work item for
// the near-singular correction.  In the projection the 17 fit points sit on
// lanes 0..16 and the 27 normal-equation sums are butterfly warp reductions,
// which leave bit-identical values on every lane so the subsequent 6x6 solve
// and every branch stay warp-uniform.  In ReAdd lane = azimuth (nazm = 32).
#include <cmath>
#include <cstring>

#include "ctx.hpp"

namespace {

struct CorrArgs {
  int nt;
  const double* tx;
  const double* tA;
  const int4* tmeta;
  double* v;
  int ncell, nlat, nlon, m;
  SplGrid G;  // Spline_Create constants of the (2 nlat, nlon) spline grid
  double rc2;
  unsigned long long* queue;  // k_near's item counter
  const SelfW64* W64;         // k_self: tabulated patch weights (uniform longitudes), or null
  const int* list;            // k_near: items to process (indices), or null for all
  long long list_start;       // k_near over a list: its first entry (the staged pass takes those before)
  int stage_cap;              // the staged pass: entries it takes from the list's head
  const float* rep;           // k_near_replay: x and a3 node values in FP32, 24 floats a node
  const unsigned long long* nlist;
  const double* th;
  const double* phi;
  const double* w;
  const double* x;
  const double* a3;
  const double* detJ;
  const double* f;
  const double* g;
  const double* area;
  const double* meshSize;
  const int* celltype;
  const double* Bc;
  const double* spl;  // ncell * SPL_NSET * m*nlon * SPL_NODE
  int npt;
  // patch
  int nrad, nazm;
  double radius;
  const double* pw;
  const double* thG;
  const double* phiA;
  const double* rd_s;
  const double* rd_w;
  const double* rd_x0;
  const double* rd_w0;
  double c1, c2;
  double L[3], iL[3];
  Tables T;
  const int4* items;
  const unsigned long long* nitems;
  int cap;
  unsigned long long* cnt;
  int screen;  // screen items before the FP64 projection (FP32C path)
  double rthr;  // FP32C path: cross-surface pairs closer than rthr are added here in FP64
  int verify;  // evaluate screened items in FP64 anyway and count disagreements
};

__device__ __forceinline__ const double* set_ptr(const CorrArgs& a, int cell, int set) {
  return a.spl + ((size_t)cell * SPL_NSET + set) * (size_t)a.m * a.nlon * SPL_NODE;
}

// RBC_SingInt: one warp per cell target
__global__ void __launch_bounds__(256) k_self(CorrArgs a) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= a.nt) return;
  int4 mt = a.tmeta[warp];
  int cell = mt.x - 1;
  if (cell < 0 || cell >= a.ncell || mt.y < 0) return;
  const int ilat0 = mt.y, ilon0 = mt.z;
  const double c1 = a.c1, c2m = a.c2 * a.Bc[a.celltype[cell]];
  const double* sx = set_ptr(a, cell, SPL_X);
  const double* sF = set_ptr(a, cell, SPL_F);
  const double* sG = set_ptr(a, cell, SPL_G);
  const double* sA = set_ptr(a, cell, SPL_A3);
  SplW W;
  double xi[3];
  spline_weights(a.th[ilat0], a.phi[ilon0], a.m, a.nlon, W);
  spline_eval(sx, W, 3, xi);
  const int NQ = a.nrad * a.nazm;
  const double phi0 = a.phi[ilon0];
  double dv[3] = {0, 0, 0};
  const Tables& T = a.T;
  for (int q = lane; q < NQ; q += 32) {
    const int irad = q % a.nrad;
    double w16[16];
    if (a.W64) {
      // weight products tabulated per (latitude, patch point); longitudes shift the stencil
      const SelfW64& e = a.W64[(size_t)ilat0 * NQ + q];
      const int j1 = imod(e.j1b + ilon0, a.nlon), j2 = (j1 + 1 == a.nlon) ? 0 : j1 + 1;
      const int i2 = (e.i1 + 1 == a.m) ? 0 : e.i1 + 1;
      W.n11 = e.i1 + a.m * j1; W.n12 = e.i1 + a.m * j2; W.n21 = i2 + a.m * j1; W.n22 = i2 + a.m * j2;
#pragma unroll
      for (int k = 0; k < 16; ++k) w16[k] = e.w[k];
    } else {
      const double th_j = a.thG[(size_t)ilat0 * NQ + q];
      const double p = a.phiA[(size_t)ilat0 * NQ + q] + phi0;  // PolarPatch_Build: atan2(...) + phi0
      const double phi_j = p - floor(p * RBC3D_I_2PI) * RBC3D_TWO_PI;
      spline_weights_g(th_j, phi_j, a.G, W);
      spline_w16(W, w16);
    }
    double xj[3], xx[3];
    spline_eval16(sx, W, w16, 3, xj);
    for (int k = 0; k < 3; ++k) xx[k] = xj[k] - xi[k];
    const double r2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    if (r2 >= a.rc2) continue;  // rr >= rc (ModRbcSingInt.F90:65)
    const double ir = rsqrt(r2), rr = r2 > 0. ? r2 * ir : 0.;
    // EwaldCoeff_SL / EwaldCoeff_DL share the table position (ModEwaldFunc.F90:86-180);
    // below r_eps or beyond the table both are zero
    if (!(rr >= T.r_eps)) continue;
    const double sp = rr * T.ntab_over_rc;
    const int it = (int)floor(sp);
    if (it < 0 || it >= EWALD_NTAB) continue;
    const double f1 = sp - it, f0 = (it + 1) - sp;
    const double ir2 = ir * ir;
    const double wq = a.pw[irad];
    if (c1 != 0.) {
      const double cs1 = __ldg(T.sl_c1 + it) * f0 + __ldg(T.sl_c1 + it + 1) * f1;
      const double cs2 = __ldg(T.sl_c2 + it) * f0 + __ldg(T.sl_c2 + it + 1) * f1;
      const double EA = (cs1 * ir + cs2) * ir2, EB = cs1 * ir - cs2;
      double fj[3];
      spline_eval16(sF, W, w16, 3, fj);
      // c1 wq (EA xx (xx . f) + EB f)
      const double sw = c1 * wq, t = EA * (xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2]);
      for (int k = 0; k < 3; ++k) dv[k] = fma(sw, fma(t, xx[k], EB * fj[k]), dv[k]);
    }
    if (c2m != 0.) {
      const double cd = __ldg(T.dl_c1 + it) * f0 + __ldg(T.dl_c1 + it + 1) * f1;
      const double EA = cd * (ir2 * ir2 * ir);
      double gj[3], aj[3];
      spline_eval16(sG, W, w16, 3, gj);
      spline_eval16(sA, W, w16, 3, aj);
      // c2 Bcoef wq EA xx (xx . g)(xx . a3)
      const double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
      const double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
      const double t = c2m * wq * EA * dg * da;
      for (int k = 0; k < 3; ++k) dv[k] = fma(t, xx[k], dv[k]);
    }
  }
  for (int k = 0; k < 3; ++k) dv[k] = warp_sum(dv[k]);
  if (lane == 0) {
    double iA = 1.0 / a.tA[warp];
    for (int k = 0; k < 3; ++k) a.v[warp + (size_t)k * a.nt] += dv[k] * iA;
  }
}

// One point of PolarPatch_Build (ModPolarPatch.F90:99-148)
__device__ __forceinline__ void patch_point(double st0, double ct0, double phi0, double sth, double cth, double cph,
                                            double sph, double& thG, double& phiG) {
  double x0 = sth * cph, x1 = sth * sph, x2 = cth;
  double y0 = ct0 * x0 + st0 * x2;
  double y1 = x1;
  double y2 = -st0 * x0 + ct0 * x2;
  y2 = fmax(-1.0, fmin(1.0, y2));
  thG = acos(y2);
  double p = atan2(y1, y0) + phi0;
  phiG = p - floor(p * RBC3D_I_2PI) * RBC3D_TWO_PI;
}

// PolarPatch_Map (ModPolarPatch.F90:218-244)
__device__ __forceinline__ void patch_map(double th0, double phi0, double dth, double dphi, double& th, double& phi) {
  double st0 = sin(th0), ct0 = cos(th0), sp0 = sin(phi0), cp0 = cos(phi0);
  double s1[3] = {ct0 * cp0, ct0 * sp0, -st0};
  double s2[3] = {-sp0, cp0, 0.};
  double x0[3] = {st0 * cp0, st0 * sp0, ct0};
  double x[3] = {sin(dth) * cos(dphi), sin(dth) * sin(dphi), cos(dth)};
  double y[3];
  for (int c = 0; c < 3; ++c) y[c] = x[0] * s1[c] + x[1] * s2[c] + x[2] * x0[c];
  double nrm = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
  for (int c = 0; c < 3; ++c) y[c] /= nrm;
  y[2] = fmax(-1., fmin(1., y[2]));
  th = acos(y[2]);
  phi = atan2(y[1], y[0]);
  if (phi < 0) phi += RBC3D_TWO_PI;
}

// dposv on the 6x6 normal equations (upper Cholesky); leaves b unchanged when
// the matrix is not positive definite, as LAPACK does for info > 0.
__device__ void chol6(const double* A /*21 packed upper, row-major a<=b*/, double* b) {
  double U[6][6];
  double M[6][6];
  int p = 0;
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j) { M[i][j] = A[p]; M[j][i] = A[p]; ++p; }
  for (int j = 0; j < 6; ++j) {
    double s = M[j][j];
    for (int k = 0; k < j; ++k) s -= U[k][j] * U[k][j];
    if (!(s > 0)) return;
    U[j][j] = sqrt(s);
    for (int i = j + 1; i < 6; ++i) {
      double t = M[j][i];
      for (int k = 0; k < j; ++k) t -= U[k][j] * U[k][i];
      U[j][i] = t / U[j][j];
    }
  }
  double y[6];
  for (int i = 0; i < 6; ++i) {
    double t = b[i];
    for (int k = 0; k < i; ++k) t -= U[k][i] * y[k];
    y[i] = t / U[i][i];
  }
  for (int i = 5; i >= 0; --i) {
    double t = y[i];
    for (int k = i + 1; k < 6; ++k) t -= U[i][k] * b[k];
    b[i] = t / U[i][i];
  }
}

// Spline_FindProjection, warp-cooperative.  All lanes return the same result.
__device__ void find_projection(const double* sx, int m, int n, const double* xt, double& th0, double& phi0,
                                double* x0) {
  const int lane = threadIdx.x & 31;
  SplW W;
  spline_weights(th0, phi0, m, n, W);
  spline_eval(sx, W, 3, x0);
  double h = fmax(RBC3D_TWO_PI / m, RBC3D_TWO_PI / n);
  for (int iter = 0; iter < 3; ++iter) {
    double px = 0, py = 0, d2 = 0;
    bool on = lane <= 16;
    if (lane < 16) {
      int ith = lane % 2, iphi = lane / 2;
      double thL = (ith + 1) * h / 2;
      double phL = iphi * RBC3D_TWO_PI / 8;
      double thP, phP;
      patch_point(sin(th0), cos(th0), phi0, sin(thL), cos(thL), cos(phL), sin(phL), thP, phP);
      px = thL * cos(phL);
      py = thL * sin(phL);
      double xx[3];
      spline_weights(thP, phP, m, n, W);
      spline_eval(sx, W, 3, xx);
      for (int k = 0; k < 3; ++k) xx[k] -= xt[k];
      d2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    } else if (lane == 16) {
      double xx[3];
      spline_weights(th0, phi0, m, n, W);
      spline_eval(sx, W, 3, xx);
      for (int k = 0; k < 3; ++k) xx[k] -= xt[k];
      d2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    }
    double d2c = __shfl_sync(0xffffffffu, d2, 16);
    double u[6] = {on ? 1. : 0., px, py, px * px, px * py, py * py};
    double A[21], b[6];
    int p = 0;
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j) A[p++] = warp_sum(u[i] * u[j]);
    for (int i = 0; i < 6; ++i) b[i] = warp_sum(u[i] * d2);
    chol6(A, b);
    // Min_Quad_2D
    double l11 = 2. * b[3], l12 = b[4], l22 = 2. * b[5];
    double det = l11 * l22 - l12 * l12;
    double xm0 = 0., xm1 = 0.;
    if (det > 0) {
      double idet = 1. / det;
      xm0 = idet * (l22 * (-b[1]) - l12 * (-b[2]));
      xm1 = idet * (-l12 * (-b[1]) + l11 * (-b[2]));
    }
    double thMinL = sqrt(xm0 * xm0 + xm1 * xm1), phiMinL = atan2(xm1, xm0);
    double thMin, phiMin, xMin[3];
    patch_map(th0, phi0, thMinL, phiMinL, thMin, phiMin);
    spline_weights(thMin, phiMin, m, n, W);
    spline_eval(sx, W, 3, xMin);
    double e0 = xMin[0] - xt[0], e1 = xMin[1] - xt[1], e2 = xMin[2] - xt[2];
    double d2Min = e0 * e0 + e1 * e1 + e2 * e2;
    if (d2Min > d2c) break;
    th0 = thMin; phi0 = phiMin;
    for (int k = 0; k < 3; ++k) x0[k] = xMin[k];
    h = 0.5 * h;
  }
}

// RBC_NearSingInt_Subtract: lane = latitude row of PolarPatch_FindPoints
__device__ void near_subtract(const CorrArgs& a, int cell, double c1, double c2, const double* xi, double th0,
                              double phi0, double radPat, double rthr, double* dv) {
  const int lane = threadIdx.x & 31;
  dv[0] = dv[1] = dv[2] = 0.;
  const double eps = 1.e-10;
  const double h_phi = RBC3D_TWO_PI / a.nlon, ih_phi = 1.0 / h_phi;
  const double cosr0 = cos(radPat);
  const size_t cb = (size_t)cell * a.nlat * a.nlon;
  for (int i = lane; i < a.nlat; i += 32) {
    double thi = a.th[i];
    if (thi <= th0 - radPat || thi >= th0 + radPat) continue;
    double dth = thi - th0;
    double dphi = 1. - (cos(dth) - cosr0) / ((sin(thi) + eps) * (sin(th0) + eps));
    dphi = fmax(-1., fmin(1., dphi));
    dphi = acos(dphi);
    int jmin, jmax;
    if (dphi > RBC3D_PI - eps) { jmin = 1; jmax = a.nlon; }
    else {
      jmin = (int)ceil((phi0 - dphi - a.phi[0]) * ih_phi) + 1;
      jmax = (int)floor((phi0 + dphi - a.phi[0]) * ih_phi) + 1;
    }
    for (int j = jmin; j <= jmax; ++j) {
      int ilon = imod(j - 1, a.nlon);
      size_t q = cb + (size_t)ilon * a.nlat + i;
      double xx[3];
      for (int k = 0; k < 3; ++k) xx[k] = a.x[q + (size_t)k * a.npt] - xi[k];
      double rr = sqrt(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]);
      if (rr > a.T.rc) continue;
      double dd = dist_on_sphere(th0, phi0, thi, a.phi[ilon]);
      double mask = mask64(a.T, dd / radPat);
      // FP32C: the pair sum skipped this point (rr < rthr); weight 1 - mask here
      // (each mesh point once: the index range of a row may wrap past nlon)
      if (rr < rthr && j - jmin < a.nlon) mask -= 1.0;
      double ds1 = a.detJ[q], ds2 = a.w[i];
      if (c1 != 0.) {
        double fj[3], EA, EB;
        for (int k = 0; k < 3; ++k) fj[k] = a.f[q + (size_t)k * a.npt] * ds1 * ds2;
        ewald_sl64(a.T, rr, EA, EB);
        double d = xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2];
        for (int k = 0; k < 3; ++k) dv[k] -= c1 * mask * (EA * xx[k] * d + EB * fj[k]);
      }
      if (c2 != 0.) {
        double gj[3], aj[3];
        for (int k = 0; k < 3; ++k) {
          gj[k] = a.g[q + (size_t)k * a.npt] * ds1 * ds2;
          aj[k] = a.a3[q + (size_t)k * a.npt];
        }
        double EA = ewald_dl64(a.T, rr);
        double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
        double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
        for (int k = 0; k < 3; ++k) dv[k] -= c2 * mask * (EA * xx[k] * dg * da);
      }
    }
  }
  for (int k = 0; k < 3; ++k) dv[k] = warp_sum(dv[k]);
}

// RBC_NearSingInt_ReAdd: nrad = 16, nazm = 32, lane = azimuth
__device__ void near_readd(const CorrArgs& a, int cell, double c1, double c2, const double* xi, const double* x0,
                           double th0, double phi0, double radPat, double* dv) {
  const int lane = threadIdx.x & 31;
  const int nrad = 16, nazm = 32;
  double d = sqrt((xi[0] - x0[0]) * (xi[0] - x0[0]) + (xi[1] - x0[1]) * (xi[1] - x0[1]) +
                  (xi[2] - x0[2]) * (xi[2] - x0[2]));
  double sizePat = radPat * sqrt(a.area[cell] / (4 * RBC3D_PI));
  // GauLeg_Sinh(0, radPat, 0, d*(radPat/sizePat), 16) (ModQuadRule.F90:223-263)
  bool sinh_rule = d > 2.2250738585072014e-308;
  double xm = 0.5 * radPat, xl = 0.5 * radPat, a0 = 0, b0 = 0, mu = 0, eta = 0;
  if (sinh_rule) {
    d = d * (radPat / sizePat);
    a0 = (0. - xm) / xl;
    b0 = d * xl;
    double f1 = (1 + a0) / b0, f2 = (1 - a0) / b0;
    double u1 = log(f1 + sqrt(1 + f1 * f1)), u2 = log(f2 + sqrt(1 + f2 * f2));
    mu = 0.5 * (u1 + u2);
    eta = 0.5 * (u1 - u2);
  }
  const double* sx = set_ptr(a, cell, SPL_X);
  const double* sF = set_ptr(a, cell, SPL_F);
  const double* sG = set_ptr(a, cell, SPL_G);
  const double* sA = set_ptr(a, cell, SPL_A3);
  const double st0 = sin(th0), ct0 = cos(th0);
  const double phL = lane * RBC3D_TWO_PI / nazm;
  const double cph = cos(phL), sph = sin(phL);
  // the radial rule and its weights depend on irad only: lane irad (< 16)
  // evaluates them once and the loop takes them by shuffle
  double rth = 0, rwt = 0, rs = 0, rc = 1;
  if (lane < nrad) {
    if (sinh_rule) {
      double s = a.rd_s[lane];
      rth = a0 + b0 * sinh(mu * s - eta);
      rwt = a.rd_w[lane] * b0 * mu * cosh(mu * s - eta);
      rwt = xl * rwt;
      rth = xm + xl * rth;
    } else {
      rth = a.rd_x0[lane];
      rwt = a.rd_w0[lane];
    }
    rs = sin(rth);
    rc = cos(rth);
    rwt = rwt * rs * (RBC3D_TWO_PI / nazm);
    rwt = rwt * mask64(a.T, rth / radPat);
  }
  double acc[3] = {0, 0, 0};
  for (int irad = 0; irad < nrad; ++irad) {
    const double wt = __shfl_sync(0xffffffffu, rwt, irad);
    const double sthP = __shfl_sync(0xffffffffu, rs, irad), cthP = __shfl_sync(0xffffffffu, rc, irad);
    double thG, phG;
    patch_point(st0, ct0, phi0, sthP, cthP, cph, sph, thG, phG);
    SplW W;
    spline_weights_g(thG, phG, a.G, W);
    double xj[3], xx[3];
    spline_eval(sx, W, 3, xj);
    for (int k = 0; k < 3; ++k) xx[k] = xj[k] - xi[k];
    const double r2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    if (r2 > a.rc2) continue;  // rr > rc
    const double ir = rsqrt(r2), rr = r2 > 0. ? r2 * ir : 0.;
    if (c1 != 0.) {
      double fj[3], EA, EB;
      spline_eval(sF, W, 3, fj);
      for (int k = 0; k < 3; ++k) fj[k] = wt * fj[k];
      ewald_sl64r(a.T, rr, ir, EA, EB);
      double dd = xx[0] * fj[0] + xx[1] * fj[1] + xx[2] * fj[2];
      for (int k = 0; k < 3; ++k) acc[k] += c1 * (EA * xx[k] * dd + EB * fj[k]);
    }
    if (c2 != 0.) {
      double aj[3], gj[3];
      spline_eval(sA, W, 3, aj);
      spline_eval(sG, W, 3, gj);
      for (int k = 0; k < 3; ++k) gj[k] = wt * gj[k];
      double EA = ewald_dl64r(a.T, rr, ir);
      double dg = xx[0] * gj[0] + xx[1] * gj[1] + xx[2] * gj[2];
      double da = xx[0] * aj[0] + xx[1] * aj[1] + xx[2] * aj[2];
      for (int k = 0; k < 3; ++k) acc[k] += c2 * (EA * xx[k] * dg * da);
    }
  }
  for (int k = 0; k < 3; ++k) dv[k] = warp_sum(acc[k]);
}

// ---- FP32 replay of Spline_FindProjection, used only to screen items whose
// projection distance is clearly above 2*meshSize (no correction) -----------
__device__ __forceinline__ void spline_weights32(float x, float y, int m, int n, int& n11, int& n12, int& n21,
                                                 int& n22, float* cx, float* cy) {
  const float hx = (float)(RBC3D_TWO_PI / m), hy = (float)(RBC3D_TWO_PI / n);
  const float ihx = 1.f / hx, ihy = 1.f / hy;
  int i1 = (int)floorf(x * ihx), j1 = (int)floorf(y * ihy);
  float s = x * ihx - i1, t = y * ihy - j1;
  i1 = imod(i1, m); j1 = imod(j1, n);
  int i2 = imod(i1 + 1, m), j2 = imod(j1 + 1, n);
  cx[0] = 1 + s * s * (-3.f + 2.f * s); cx[1] = s * s * (3.f - 2.f * s);
  cx[2] = hx * s * (1.f + s * (-2.f + s)); cx[3] = hx * s * s * (-1.f + s);
  cy[0] = 1 + t * t * (-3.f + 2.f * t); cy[1] = t * t * (3.f - 2.f * t);
  cy[2] = hy * t * (1.f + t * (-2.f + t)); cy[3] = hy * t * t * (-1.f + t);
  n11 = i1 + m * j1; n12 = i1 + m * j2; n21 = i2 + m * j1; n22 = i2 + m * j2;
}
__device__ __forceinline__ void spline_eval32(const double* __restrict__ spl, float th, float ph, int m, int n,
                                              float* f) {
  int n11, n12, n21, n22;
  float cx[4], cy[4];
  spline_weights32(th, ph, m, n, n11, n12, n21, n22, cx, cy);
  const double* a = spl + (size_t)n11 * SPL_NODE;
  const double* b = spl + (size_t)n12 * SPL_NODE;
  const double* c = spl + (size_t)n21 * SPL_NODE;
  const double* d = spl + (size_t)n22 * SPL_NODE;
  for (int l = 0; l < 3; ++l) {
    float r0 = (float)a[l] * cy[0] + (float)b[l] * cy[1] + (float)a[6 + l] * cy[2] + (float)b[6 + l] * cy[3];
    float r1 = (float)c[l] * cy[0] + (float)d[l] * cy[1] + (float)c[6 + l] * cy[2] + (float)d[6 + l] * cy[3];
    float r2 = (float)a[3 + l] * cy[0] + (float)b[3 + l] * cy[1] + (float)a[9 + l] * cy[2] + (float)b[9 + l] * cy[3];
    float r3 = (float)c[3 + l] * cy[0] + (float)d[3 + l] * cy[1] + (float)c[9 + l] * cy[2] + (float)d[9 + l] * cy[3];
    f[l] = cx[0] * r0 + cx[1] * r1 + cx[2] * r2 + cx[3] * r3;
  }
}
// the same from the replay's FP32 node records (24 floats a node: the x
// slots' 12 values, then a3's; off 0 for x, 12 for a3), with no conversions
__device__ __forceinline__ void spline_eval32f(const float* __restrict__ rec, int off, float th, float ph, int m,
                                               int n, float* f) {
  int n11, n12, n21, n22;
  float cx[4], cy[4];
  spline_weights32(th, ph, m, n, n11, n12, n21, n22, cx, cy);
  const float* a = rec + (size_t)n11 * 24 + off;
  const float* b = rec + (size_t)n12 * 24 + off;
  const float* c = rec + (size_t)n21 * 24 + off;
  const float* d = rec + (size_t)n22 * 24 + off;
  for (int l = 0; l < 3; ++l) {
    float r0 = a[l] * cy[0] + b[l] * cy[1] + a[6 + l] * cy[2] + b[6 + l] * cy[3];
    float r1 = c[l] * cy[0] + d[l] * cy[1] + c[6 + l] * cy[2] + d[6 + l] * cy[3];
    float r2 = a[3 + l] * cy[0] + b[3 + l] * cy[1] + a[9 + l] * cy[2] + b[9 + l] * cy[3];
    float r3 = c[3 + l] * cy[0] + d[3 + l] * cy[1] + c[9 + l] * cy[2] + d[9 + l] * cy[3];
    f[l] = cx[0] * r0 + cx[1] * r1 + cx[2] * r2 + cx[3] * r3;
  }
}
__device__ __forceinline__ float warp_sumf_(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Returns the projection's signed distance a3(x0).(xt - x0) in FP32, from
// the cell's FP32 node records (x at offset 0, a3 at 12).
__device__ float projection_dist32(const float* rc, int m, int n, const double* xtd, double th0d, double phi0d) {
  const int lane = threadIdx.x & 31;
  const float TWO_PI_F = (float)RBC3D_TWO_PI;
  float xt[3] = {(float)xtd[0], (float)xtd[1], (float)xtd[2]};
  float th0 = (float)th0d, phi0 = (float)phi0d;
  float x0[3];
  spline_eval32f(rc, 0, th0, phi0, m, n, x0);
  float h = fmaxf(TWO_PI_F / m, TWO_PI_F / n);
  for (int iter = 0; iter < 3; ++iter) {
    float px = 0, py = 0, d2 = 0;
    float st0 = sinf(th0), ct0 = cosf(th0);
    if (lane < 16) {
      int ith = lane % 2, iphi = lane / 2;
      float thL = (ith + 1) * h / 2;
      float phL = iphi * TWO_PI_F / 8;
      float sth = sinf(thL), cth = cosf(thL), cph = cosf(phL), sph = sinf(phL);
      float q0 = sth * cph, q1 = sth * sph, q2 = cth;
      float y0 = ct0 * q0 + st0 * q2, y1 = q1, y2 = fmaxf(-1.f, fminf(1.f, -st0 * q0 + ct0 * q2));
      float thP = acosf(y2), pp = atan2f(y1, y0) + phi0;
      float phP = pp - floorf(pp / TWO_PI_F) * TWO_PI_F;
      px = thL * cph;
      py = thL * sph;
      float xx[3];
      spline_eval32f(rc, 0, thP, phP, m, n, xx);
      d2 = (xx[0] - xt[0]) * (xx[0] - xt[0]) + (xx[1] - xt[1]) * (xx[1] - xt[1]) + (xx[2] - xt[2]) * (xx[2] - xt[2]);
    } else if (lane == 16) {
      float xx[3];
      spline_eval32f(rc, 0, th0, phi0, m, n, xx);
      d2 = (xx[0] - xt[0]) * (xx[0] - xt[0]) + (xx[1] - xt[1]) * (xx[1] - xt[1]) + (xx[2] - xt[2]) * (xx[2] - xt[2]);
    }
    float d2c = __shfl_sync(0xffffffffu, d2, 16);
    float u[6] = {lane <= 16 ? 1.f : 0.f, px, py, px * px, px * py, py * py};
    float M[6][6], b[6];
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j) { M[i][j] = warp_sumf_(u[i] * u[j]); M[j][i] = M[i][j]; }
    for (int i = 0; i < 6; ++i) b[i] = warp_sumf_(u[i] * d2);
    // Cholesky
    float U[6][6];
    bool ok = true;
    for (int j = 0; j < 6 && ok; ++j) {
      float s = M[j][j];
      for (int k = 0; k < j; ++k) s -= U[k][j] * U[k][j];
      if (!(s > 0)) { ok = false; break; }
      U[j][j] = sqrtf(s);
      for (int i = j + 1; i < 6; ++i) {
        float t = M[j][i];
        for (int k = 0; k < j; ++k) t -= U[k][j] * U[k][i];
        U[j][i] = t / U[j][j];
      }
    }
    if (ok) {
      float y[6];
      for (int i = 0; i < 6; ++i) {
        float t = b[i];
        for (int k = 0; k < i; ++k) t -= U[k][i] * y[k];
        y[i] = t / U[i][i];
      }
      for (int i = 5; i >= 0; --i) {
        float t = y[i];
        for (int k = i + 1; k < 6; ++k) t -= U[i][k] * b[k];
        b[i] = t / U[i][i];
      }
    }
    float l11 = 2.f * b[3], l12 = b[4], l22 = 2.f * b[5];
    float det = l11 * l22 - l12 * l12;
    float xm0 = 0.f, xm1 = 0.f;
    if (det > 0) {
      float idet = 1.f / det;
      xm0 = idet * (l22 * (-b[1]) - l12 * (-b[2]));
      xm1 = idet * (-l12 * (-b[1]) + l11 * (-b[2]));
    }
    float dth = sqrtf(xm0 * xm0 + xm1 * xm1), dph = atan2f(xm1, xm0);
    float sp0 = sinf(phi0), cp0 = cosf(phi0);
    float s1[3] = {ct0 * cp0, ct0 * sp0, -st0}, s2[3] = {-sp0, cp0, 0.f}, e0[3] = {st0 * cp0, st0 * sp0, ct0};
    float qx[3] = {sinf(dth) * cosf(dph), sinf(dth) * sinf(dph), cosf(dth)};
    float yv[3];
    for (int c = 0; c < 3; ++c) yv[c] = qx[0] * s1[c] + qx[1] * s2[c] + qx[2] * e0[c];
    float nr = sqrtf(yv[0] * yv[0] + yv[1] * yv[1] + yv[2] * yv[2]);
    yv[2] = fmaxf(-1.f, fminf(1.f, yv[2] / nr));
    float thMin = acosf(yv[2]), phiMin = atan2f(yv[1] / nr, yv[0] / nr);
    if (phiMin < 0) phiMin += TWO_PI_F;
    float xMin[3];
    spline_eval32f(rc, 0, thMin, phiMin, m, n, xMin);
    float d2Min = (xMin[0] - xt[0]) * (xMin[0] - xt[0]) + (xMin[1] - xt[1]) * (xMin[1] - xt[1]) +
                  (xMin[2] - xt[2]) * (xMin[2] - xt[2]);
    if (d2Min > d2c) break;
    th0 = thMin; phi0 = phiMin;
    for (int k = 0; k < 3; ++k) x0[k] = xMin[k];
    h = 0.5f * h;
  }
  float a30[3];
  spline_eval32f(rc, 12, th0, phi0, m, n, a30);
  return a30[0] * (xt[0] - x0[0]) + a30[1] * (xt[1] - x0[1]) + a30[2] * (xt[2] - x0[2]);
}

// RBC_NearSingInt over the work list (persistent warps)
// Target position in the item's cell frame (minimum image about the closest
// mesh point x0), as RBC_NearSingInt receives it.
__device__ __forceinline__ void item_geometry(const CorrArgs& a, int4 item, double* x0, double* xt, size_t& q0) {
  const int t = item.x, cell = item.y - 1, ilat0 = item.z, ilon0 = item.w;
  q0 = (size_t)cell * a.nlat * a.nlon + (size_t)ilon0 * a.nlat + ilat0;
  for (int k = 0; k < 3; ++k) {
    x0[k] = a.x[q0 + (size_t)k * a.npt];
    double xx = a.tx[t + (size_t)k * a.nt] - x0[k];
    xx = xx - round(xx * a.iL[k]) * a.L[k];
    xt[k] = x0[k] + xx;
  }
}

// FP32 modes, stage 1 (one thread per candidate): screen (1) -- a target
// farther than 6*meshSize from its closest mesh point, on its outer side,
// projects farther than 2*meshSize -- and the survivors listed for stage 2.
__global__ void k_near_screen(CorrArgs a, int* __restrict__ out, unsigned long long* __restrict__ nout) {
  unsigned long long nitem = *a.nitems;
  if (nitem > (unsigned long long)a.cap) nitem = a.cap;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nitem) return;
  const int4 item = a.items[i];
  const int cell = item.y - 1;
  if (cell < 0 || cell >= a.ncell) return;
  double x0[3], xt[3];
  size_t q0;
  item_geometry(a, item, x0, xt, q0);
  const double msz = a.meshSize[cell];
  const double dx0 = xt[0] - x0[0], dx1 = xt[1] - x0[1], dx2 = xt[2] - x0[2];
  const double d = sqrt(dx0 * dx0 + dx1 * dx1 + dx2 * dx2);
  const double nd = a.a3[q0] * dx0 + a.a3[q0 + a.npt] * dx1 + a.a3[q0 + 2 * (size_t)a.npt] * dx2;
  if (d > 6.0 * msz && nd > 0.9 * d) return;
  out[atomicAdd(nout, 1ull)] = (int)i;
}

// stage 2 (one warp per listed candidate): the FP32 replay of the projection;
// candidates within 2.3*meshSize are listed for the FP64 stage.
__global__ void __launch_bounds__(128) k_near_replay(CorrArgs a, const int* __restrict__ in,
                                                     const unsigned long long* __restrict__ nin,
                                                     int* __restrict__ out, unsigned long long* __restrict__ nout) {
  const int lane = threadIdx.x & 31;
  const long long n = (long long)*nin;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += nw) {
    const int idx = in[w];
    const int4 item = a.items[idx];
    const int cell = item.y - 1;
    double x0[3], xt[3];
    size_t q0;
    item_geometry(a, item, x0, xt, q0);
    const double msz = a.meshSize[cell];
    const float d32 = projection_dist32(a.rep + (size_t)cell * a.m * a.nlon * 24, a.m, a.nlon, xt, a.th[item.z],
                                        a.phi[item.w]);
    if ((double)d32 > 2.3 * msz) continue;
    if (lane == 0) out[atomicAdd(nout, 1ull)] = idx;
  }
}

__global__ void __launch_bounds__(128) k_near(CorrArgs a) {
  const int lane = threadIdx.x & 31;
  unsigned long long nitem = a.list ? *a.nlist : *a.nitems;
  if (nitem > (unsigned long long)a.cap) nitem = a.cap;
  // warps take items from a shared counter (the grid is one resident wave):
  // corrected items cost ~100x screened ones, so a static split leaves a tail
  // items per counter update: 4 over the full candidate list; 1 over the short
  // list of the FP32 modes, so its few expensive items spread over all SMs
  const int GRAB = a.list ? 1 : 4;
  long long it = 0, it_end = 0;
  for (;;) {
    if (it == it_end) {
      unsigned long long g0 = 0;
      if (lane == 0) g0 = atomicAdd(a.queue, (unsigned long long)GRAB);
      it = (long long)__shfl_sync(0xffffffffu, g0, 0);
      it_end = it + GRAB;
    }
    if (it + a.list_start >= (long long)nitem) break;
    const long long cur = a.list_start + it++;
    int4 item = a.items[a.list ? a.list[cur] : cur];
    int t = item.x, cell = item.y - 1, ilat0 = item.z, ilon0 = item.w;
    if (cell < 0 || cell >= a.ncell) continue;
    double th0 = a.th[ilat0], phi0 = a.phi[ilon0];
    size_t q0 = (size_t)cell * a.nlat * a.nlon + (size_t)ilon0 * a.nlat + ilat0;
    double x0[3], xt[3];
    for (int k = 0; k < 3; ++k) {
      x0[k] = a.x[q0 + (size_t)k * a.npt];
      double xx = a.tx[t + (size_t)k * a.nt] - x0[k];
      xx = xx - round(xx * a.iL[k]) * a.L[k];
      xt[k] = x0[k] + xx;
    }
    const double* sx = set_ptr(a, cell, SPL_X);
    const double msz = a.meshSize[cell];
    bool skip = false;
    if (a.screen) {
      // (1) far target on the outer side of its closest mesh point: the
      //     projection distance is ~|xt - x0| >= 6*meshSize > 2*meshSize
      double dx0 = xt[0] - x0[0], dx1 = xt[1] - x0[1], dx2 = xt[2] - x0[2];
      double d = sqrt(dx0 * dx0 + dx1 * dx1 + dx2 * dx2);
      double nd = a.a3[q0] * dx0 + a.a3[q0 + a.npt] * dx1 + a.a3[q0 + 2 * (size_t)a.npt] * dx2;
      if (d > 6.0 * msz && nd > 0.9 * d) skip = true;
      // (2) FP32 replay of the projection, margin 0.3*meshSize
      else {
        if (lane == 0) atomicAdd(a.cnt + 8, 1ull);
        if ((double)projection_dist32(a.rep + (size_t)cell * a.m * a.nlon * 24, a.m, a.nlon, xt, th0, phi0) >
            2.3 * msz)
          skip = true;
      }
      if (skip && !a.verify) continue;
    }
    if (lane == 0) atomicAdd(a.cnt + 9, 1ull);
    find_projection(sx, a.m, a.nlon, xt, th0, phi0, x0);
    const double c1 = a.c1, c2 = a.c2 * a.Bc[a.celltype[cell]];
    SplW W;
    double a30[3];
    spline_weights(th0, phi0, a.m, a.nlon, W);
    spline_eval(set_ptr(a, cell, SPL_A3), W, 3, a30);
    double dist = a30[0] * (xt[0] - x0[0]) + a30[1] * (xt[1] - x0[1]) + a30[2] * (xt[2] - x0[2]);
    if (dist > 2 * msz) continue;
    if (lane == 0) {
      atomicAdd(a.cnt + 3, 1ull);
      if (skip) atomicAdd(a.cnt + 6, 1ull);  // a screened item that needs a correction
    }
    double sizePat = a.radius * sqrt(a.area[cell] / (4 * RBC3D_PI));
    double dist1 = copysign(fabs(0.01 * sizePat), dist);
    double dv[3], tmp[3];
    near_subtract(a, cell, c1, c2, xt, th0, phi0, a.radius, a.rthr, dv);
    if (fabs(dist) >= fabs(dist1)) {
      near_readd(a, cell, c1, c2, xt, x0, th0, phi0, a.radius, tmp);
      for (int k = 0; k < 3; ++k) dv[k] += tmp[k];
    } else {
      double xi1[3], dv1[3], dv0[3];
      for (int k = 0; k < 3; ++k) xi1[k] = x0[k] + dist1 * a30[k];
      near_readd(a, cell, c1, c2, xi1, x0, th0, phi0, a.radius, dv1);
      near_readd(a, cell, c1, c2, x0, x0, th0, phi0, a.radius, dv0);
      if (c2 != 0.) {
        double dJ0[3], g0[3];
        spline_eval(set_ptr(a, cell, SPL_DJ), W, 1, dJ0);
        spline_eval(set_ptr(a, cell, SPL_G), W, 3, g0);
        for (int k = 0; k < 3; ++k) g0[k] = g0[k] / dJ0[0];
        for (int k = 0; k < 3; ++k) dv0[k] = (dist > 0) ? dv0[k] + c2 * 4 * RBC3D_PI * g0[k] : dv0[k] - c2 * 4 * RBC3D_PI * g0[k];
      }
      for (int k = 0; k < 3; ++k) dv[k] += dv0[k] + dist / dist1 * (dv1[k] - dv0[k]);
    }
    if (lane == 0) {
      double iA = 1.0 / a.tA[t];
      for (int k = 0; k < 3; ++k) atomicAdd(a.v + t + (size_t)k * a.nt, dv[k] * iA);
    }
  }
}

// The FP32 modes' FP64 pass over their short list, staged so that its work
// spreads evenly over the SMs: with one warp per item the pass waited on its
// slowest items.  (1) k_near_proj, one warp per item: the projection and the
// correction test; (2) k_near_units, one warp per quadrature (the first
// re-adds of every item, then the second ones, then the subtracts), each
// keeping its warp sum; (3) k_near_fin, one thread per item: the combination
// of RBC_NearSingInt (ModRbcSingInt.F90:103-160) in the order k_near uses, so the
// sums are k_near's.  Entries past its capacity (NEAR_STAGE_CAP, or less when
// RBC3D_NEAR_STAGE_CAP asks for it) go through k_near.
struct NearPlan {
  double th0, phi0, x0[3], xt[3], a30[3], dist, dist1;
  int t, cell, two, ok;
};
static_assert(sizeof(NearPlan) <= 16 * sizeof(double), "plan slot");

__device__ __forceinline__ long long near_stage_count(const CorrArgs& a) {
  unsigned long long n = *a.nlist;
  if (n > (unsigned long long)a.cap) n = a.cap;
  if (n > (unsigned long long)a.stage_cap) n = a.stage_cap;
  return (long long)n;
}

__global__ void __launch_bounds__(128) k_near_proj(CorrArgs a, NearPlan* __restrict__ plan) {
  const int lane = threadIdx.x & 31;
  const long long n = near_stage_count(a);
  for (;;) {
    unsigned long long g0 = 0;
    if (lane == 0) g0 = atomicAdd(a.queue, 1ull);
    const long long cur = (long long)__shfl_sync(0xffffffffu, g0, 0);
    if (cur >= n) break;
    NearPlan P{};
    const int4 item = a.items[a.list[cur]];
    const int t = item.x, cell = item.y - 1, ilat0 = item.z, ilon0 = item.w;
    if (cell >= 0 && cell < a.ncell) {
      double th0 = a.th[ilat0], phi0 = a.phi[ilon0];
      const size_t q0 = (size_t)cell * a.nlat * a.nlon + (size_t)ilon0 * a.nlat + ilat0;
      double x0[3], xt[3];
      for (int k = 0; k < 3; ++k) {
        x0[k] = a.x[q0 + (size_t)k * a.npt];
        double xx = a.tx[t + (size_t)k * a.nt] - x0[k];
        xx = xx - round(xx * a.iL[k]) * a.L[k];
        xt[k] = x0[k] + xx;
      }
      if (lane == 0) atomicAdd(a.cnt + 9, 1ull);
      find_projection(set_ptr(a, cell, SPL_X), a.m, a.nlon, xt, th0, phi0, x0);
      SplW W;
      double a30[3];
      spline_weights(th0, phi0, a.m, a.nlon, W);
      spline_eval(set_ptr(a, cell, SPL_A3), W, 3, a30);
      const double dist = a30[0] * (xt[0] - x0[0]) + a30[1] * (xt[1] - x0[1]) + a30[2] * (xt[2] - x0[2]);
      if (!(dist > 2 * a.meshSize[cell])) {
        if (lane == 0) atomicAdd(a.cnt + 3, 1ull);
        const double sizePat = a.radius * sqrt(a.area[cell] / (4 * RBC3D_PI));
        P.dist = dist;
        P.dist1 = copysign(fabs(0.01 * sizePat), dist);
        P.two = fabs(dist) < fabs(P.dist1) ? 1 : 0;
        P.th0 = th0;
        P.phi0 = phi0;
        for (int k = 0; k < 3; ++k) {
          P.x0[k] = x0[k];
          P.xt[k] = xt[k];
          P.a30[k] = a30[k];
        }
        P.t = t;
        P.cell = cell;
        P.ok = 1;
      }
    }
    if (lane == 0) plan[cur] = P;
  }
}

__global__ void __launch_bounds__(128) k_near_units(CorrArgs a, const NearPlan* __restrict__ plan,
                                                    double* __restrict__ part, unsigned long long* __restrict__ queue) {
  const int lane = threadIdx.x & 31;
  const long long n = near_stage_count(a);
  for (;;) {
    unsigned long long g0 = 0;
    if (lane == 0) g0 = atomicAdd(queue, 1ull);
    const long long u = (long long)__shfl_sync(0xffffffffu, g0, 0);
    if (u >= 3 * n) break;
    const long long i = u % n;
    // kind 0: re-add at xt (at xi1 when the target is within dist1);
    // kind 1: re-add at x0 (only then); kind 2: subtract
    const int kind = (int)(u / n);
    const NearPlan P = plan[i];
    if (!P.ok || (kind == 1 && !P.two)) continue;
    const double c2 = a.c2 * a.Bc[a.celltype[P.cell]];
    double dv[3];
    if (kind == 0) {
      double xi1[3];
      for (int k = 0; k < 3; ++k) xi1[k] = P.x0[k] + P.dist1 * P.a30[k];
      near_readd(a, P.cell, a.c1, c2, P.two ? xi1 : P.xt, P.x0, P.th0, P.phi0, a.radius, dv);
    } else if (kind == 1) {
      near_readd(a, P.cell, a.c1, c2, P.x0, P.x0, P.th0, P.phi0, a.radius, dv);
    } else {
      near_subtract(a, P.cell, a.c1, c2, P.xt, P.th0, P.phi0, a.radius, a.rthr, dv);
    }
    if (lane == 0) {
      const int o = kind == 2 ? 0 : (kind == 0 ? 3 : 6);
      for (int k = 0; k < 3; ++k) part[9 * i + o + k] = dv[k];
    }
  }
}

__global__ void k_near_fin(CorrArgs a, const NearPlan* __restrict__ plan, const double* __restrict__ part) {
  const long long n = near_stage_count(a);
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const NearPlan& P = plan[i];
  if (!P.ok) return;
  const double* S = part + 9 * i;
  double dv[3] = {S[0], S[1], S[2]};
  if (!P.two) {
    for (int k = 0; k < 3; ++k) dv[k] += S[3 + k];
  } else {
    const double c2 = a.c2 * a.Bc[a.celltype[P.cell]];
    double dv1[3] = {S[3], S[4], S[5]}, dv0[3] = {S[6], S[7], S[8]};
    if (c2 != 0.) {
      SplW W;
      double dJ0[3], g0[3];
      spline_weights(P.th0, P.phi0, a.m, a.nlon, W);
      spline_eval(set_ptr(a, P.cell, SPL_DJ), W, 1, dJ0);
      spline_eval(set_ptr(a, P.cell, SPL_G), W, 3, g0);
      for (int k = 0; k < 3; ++k) g0[k] = g0[k] / dJ0[0];
      for (int k = 0; k < 3; ++k)
        dv0[k] = (P.dist > 0) ? dv0[k] + c2 * 4 * RBC3D_PI * g0[k] : dv0[k] - c2 * 4 * RBC3D_PI * g0[k];
    }
    for (int k = 0; k < 3; ++k) dv[k] += dv0[k] + P.dist / P.dist1 * (dv1[k] - dv0[k]);
  }
  const double iA = 1.0 / a.tA[P.t];
  for (int k = 0; k < 3; ++k) atomicAdd(a.v + P.t + (size_t)k * a.nt, dv[k] * iA);
}

// The FP32 replay's node records: x and a3 of every spline node in FP32,
// rounded once here instead of at every interpolation (the double-to-float
// conversions kept the replay on GB300's FP64 pipe: 1.42 -> 1.17 ms for the
// near-singular stage at 256 cells, the same decisions).
__global__ void k_rep_rec(long long nn, int per, const double* __restrict__ spl, float* __restrict__ rep) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nn) return;
  const long long cell = q / per, node = q - cell * per;
  const double* sx = spl + ((cell * SPL_NSET + SPL_X) * per + node) * SPL_NODE;
  const double* sa = spl + ((cell * SPL_NSET + SPL_A3) * per + node) * SPL_NODE;
  float* o = rep + q * 24;
  for (int k = 0; k < 12; ++k) {
    o[k] = (float)sx[k];
    o[12 + k] = (float)sa[k];
  }
}

// InterCellRepulsion (ModRepulsion.F90:270-402): one warp per cell point.
struct RepArgs {
  int n, nv, nlat, nlon, m;
  const double* x;      // cell points, point layout (3 x n)
  const double* sx;     // sorted source positions (3 x n)
  const int4* smeta;    // (surf 1-based, ilat, ilon, point index)
  const int* cs;
  const int* ce;
  const double* spl;
  const double* th;
  const double* phi;
  int Nc[3];
  double L[3], iL[3];
  double eps;
  // wall (one), or nele == 0
  int nvert, nele;
  const double* wx;     // vertices (3 x nvert)
  const int* e2v;       // (nele x 3), 0-based
  const int* wcs;
  const int* wce;
  const int* worder;
  double* dx;           // 3 x n, moves (zero where none)
  unsigned long long* dmin;   // minimum surface separation (double bits)
  unsigned long long* nmoved;
};

__device__ __forceinline__ double rep_minimg(double d, double L, double iL) { return d - round(d * iL) * L; }

// lexicographic warp minimum of (d, key): all lanes receive the winner
__device__ __forceinline__ void warp_argmin(double& d, int& key) {
  for (int o = 16; o > 0; o >>= 1) {
    const double d2 = __shfl_xor_sync(0xffffffffu, d, o);
    const int k2 = __shfl_xor_sync(0xffffffffu, key, o);
    if (d2 < d || (d2 == d && k2 < key)) { d = d2; key = k2; }
  }
}

__global__ void __launch_bounds__(128) k_inter_rep(RepArgs a) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= a.n) return;
  const double xi[3] = {a.x[i], a.x[i + (size_t)a.n], a.x[i + 2 * (size_t)a.n]};
  const int surf_i = i / a.nv + 1;
  int ci[3];
  for (int d = 0; d < 3; ++d) ci[d] = imod((int)floor(xi[d] * a.Nc[d] * a.iL[d]), a.Nc[d]);
  // Closest_Neighbor_Cell: the nearest mesh point of another cell over the
  // 27 hash cells around xi (lanes over the sources of each hash cell)
  double dist1 = 1e300;
  int q1 = 0x7fffffff;
  for (int nb = 0; nb < 27; ++nb) {
    const int hc = imod(ci[0] + nb % 3 - 1, a.Nc[0]) +
                   a.Nc[0] * (imod(ci[1] + (nb / 3) % 3 - 1, a.Nc[1]) + a.Nc[1] * imod(ci[2] + nb / 9 - 1, a.Nc[2]));
    for (int q = a.cs[hc] + lane; q < a.ce[hc]; q += 32) {
      if (a.smeta[q].x == surf_i) continue;
      double r2 = 0;
      for (int d = 0; d < 3; ++d) {
        const double xx = rep_minimg(xi[d] - a.sx[q + (size_t)d * a.n], a.L[d], a.iL[d]);
        r2 += xx * xx;
      }
      const double rr = sqrt(r2);
      if (rr < dist1 || (rr == dist1 && q < q1)) { dist1 = rr; q1 = q; }
    }
  }
  warp_argmin(dist1, q1);
  double x1[3] = {0, 0, 0};
  if (q1 != 0x7fffffff && dist1 <= 2 * a.eps) {
    // projection onto that cell's spline surface (Spline_FindProjection)
    const int4 m = a.smeta[q1];
    const int cell0 = m.x - 1, p0 = m.w;
    double xtar[3];
    for (int d = 0; d < 3; ++d) {
      const double x0 = a.x[p0 + (size_t)d * a.n];
      xtar[d] = x0 + rep_minimg(xi[d] - x0, a.L[d], a.iL[d]);
    }
    double th0 = a.th[m.y], phi0 = a.phi[m.z];
    const double* sx = a.spl + ((size_t)cell0 * SPL_NSET + SPL_X) * (size_t)a.m * a.nlon * SPL_NODE;
    find_projection(sx, a.m, a.nlon, xtar, th0, phi0, x1);
    double d2 = 0;
    for (int d = 0; d < 3; ++d) d2 += (xtar[d] - x1[d]) * (xtar[d] - x1[d]);
    dist1 = sqrt(d2);
  }
  // Closest_Neighbor_Wall: the nearest point of the wall's triangles whose
  // centroids lie in the 27 hash cells around xi
  double dist2 = 1e300;
  int e2 = 0x7fffffff;
  double x2[3] = {0, 0, 0};
  if (a.nele > 0) {
    double best[3] = {0, 0, 0};
    for (int nb = 0; nb < 27; ++nb) {
      const int hc = imod(ci[0] + nb % 3 - 1, a.Nc[0]) +
                     a.Nc[0] * (imod(ci[1] + (nb / 3) % 3 - 1, a.Nc[1]) + a.Nc[1] * imod(ci[2] + nb / 9 - 1, a.Nc[2]));
      for (int q = a.wcs[hc] + lane; q < a.wce[hc]; q += 32) {
        const int e = a.worder[q];
        double xv[3][3], xtar[3];
        for (int l = 0; l < 3; ++l) {
          const int iv = a.e2v[e + (size_t)l * a.nele];
          for (int d = 0; d < 3; ++d) xv[l][d] = a.wx[iv + (size_t)d * a.nvert];
        }
        for (int d = 0; d < 3; ++d) xtar[d] = xv[0][d] + rep_minimg(xi[d] - xv[0][d], a.L[d], a.iL[d]);
        double s0, t0;
        const double rr = min_dist_to_tri(xtar, xv, s0, t0);
        if (rr < dist2 || (rr == dist2 && e < e2)) {
          dist2 = rr;
          e2 = e;
          for (int d = 0; d < 3; ++d) best[d] = (1 - s0 - t0) * xv[0][d] + s0 * xv[1][d] + t0 * xv[2][d];
        }
      }
    }
    const int emine = e2;
    warp_argmin(dist2, e2);
    // the winning lane's closest point
    const unsigned ball = __ballot_sync(0xffffffffu, emine == e2 && e2 != 0x7fffffff);
    if (ball) {
      const int src = __ffs(ball) - 1;
      for (int d = 0; d < 3; ++d) x2[d] = __shfl_sync(0xffffffffu, best[d], src);
    }
  }
  if (lane != 0) return;
  const bool cellwin = dist1 < dist2;
  const double dist = cellwin ? dist1 : dist2;
  const double* xj = cellwin ? x1 : x2;
  if (dist < 1e300) atomicMin(a.dmin, (unsigned long long)__double_as_longlong(dist));
  if (dist < a.eps) {
    double xx[3], r2 = 0;
    for (int d = 0; d < 3; ++d) {
      xx[d] = rep_minimg(xi[d] - xj[d], a.L[d], a.iL[d]);
      r2 += xx[d] * xx[d];
    }
    const double rr = sqrt(r2);
    for (int d = 0; d < 3; ++d) a.dx[i + (size_t)d * a.n] = 0.5 * xx[d] * (a.eps - rr) / rr;
    atomicAdd(a.nmoved, 1ull);
  }
}

// The moves applied per cell: pointwise for |viscRat| < thresh, else (rigidsep)
// the mean move of the cell's moved points for every point; xo = x + move.
__global__ void __launch_bounds__(256) k_inter_rep_apply(int nv, int n, const double* __restrict__ x,
                                                         const double* __restrict__ dx, const int* __restrict__ celltype,
                                                         const double* __restrict__ visc, double thresh, int rigidsep,
                                                         double* __restrict__ xo) {
  const int cell = blockIdx.x;
  const size_t p0 = (size_t)cell * nv;
  const bool soft = fabs(visc[celltype[cell]]) < thresh;
  __shared__ double red[4][256];
  double m[4] = {0, 0, 0, 0};
  if (!soft && rigidsep) {
    for (int r = threadIdx.x; r < nv; r += blockDim.x) {
      const double a = dx[p0 + r], b = dx[p0 + r + (size_t)n], c = dx[p0 + r + 2 * (size_t)n];
      if (a * a + b * b + c * c > 0.) { m[0] += a; m[1] += b; m[2] += c; m[3] += 1.0; }
    }
    for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = m[k];
    __syncthreads();
    for (int hh = blockDim.x / 2; hh > 0; hh >>= 1) {
      if ((int)threadIdx.x < hh)
        for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + hh];
      __syncthreads();
    }
    for (int k = 0; k < 4; ++k) m[k] = red[k][0];
  }
  for (int r = threadIdx.x; r < nv; r += blockDim.x)
    for (int d = 0; d < 3; ++d) {
      const size_t q = p0 + r + (size_t)d * n;
      double v = x[q];
      if (soft) v += dx[q];
      else if (rigidsep && m[3] > 0) v += m[d] / m[3];
      xo[q] = v;
    }
}

void fill_args(rbc3d_ctx* ctx, int tlist, double c1, double c2, CorrArgs& a, const double* Bc) {
  TargetSet& t = ctx->tl[tlist];
  a.nt = t.n; a.tx = t.x.p; a.tA = t.Acoef.p; a.tmeta = t.meta.p; a.v = t.v.p;
  a.ncell = ctx->ncell; a.nlat = ctx->nlat; a.nlon = ctx->nlon; a.m = ctx->m;
  a.G = spl_grid(ctx->m, ctx->nlon);
  a.W64 = ctx->phi_uniform ? reinterpret_cast<const SelfW64*>(ctx->self_w64.p) : nullptr;
  a.rc2 = ctx->prm.rc * ctx->prm.rc;
  a.th = ctx->th.p; a.phi = ctx->phi.p; a.w = ctx->w.p;
  a.x = ctx->x.p; a.a3 = ctx->a3.p; a.detJ = ctx->detJ.p; a.f = ctx->f.p; a.g = ctx->g.p;
  a.area = ctx->area.p; a.meshSize = ctx->meshSize.p; a.celltype = ctx->celltype.p; a.Bc = Bc;
  a.spl = ctx->spl.p; a.npt = ctx->npt;
  a.nrad = ctx->nrad; a.nazm = ctx->nazm; a.radius = ctx->radius; a.pw = ctx->pw.p; a.thG = ctx->thG.p; a.phiA = ctx->phiA.p;
  a.rd_s = ctx->rd_s.p; a.rd_w = ctx->rd_w.p; a.rd_x0 = ctx->rd_x0.p; a.rd_w0 = ctx->rd_w0.p;
  a.c1 = c1; a.c2 = c2;
  for (int d = 0; d < 3; ++d) { a.L[d] = ctx->prm.Lb[d]; a.iL[d] = ctx->iLb[d]; }
  a.T = ctx->T;
  a.items = ctx->items.p; a.nitems = ctx->dcnt.p; a.cap = ctx->items_cap; a.cnt = ctx->dcnt.p;
}

}  // namespace

rbc3d_status run_self_corr(rbc3d_ctx* ctx, int tlist, double c1, double c2) {
  TargetSet& t = ctx->tl[tlist];
  if (tlist != RBC3D_TLIST_RBC || t.n == 0 || ctx->ncell == 0) return RBC3D_OK;
  const double* Bc = ctx->dBcoef.p;
  CorrArgs a;
  fill_args(ctx, tlist, c1, (c2 != 0 && ctx->has_g) ? c2 : 0.0, a, Bc);
  if (c1 != 0 && !ctx->has_f) a.c1 = 0;
  long long threads = (long long)t.n * 32;
  { k_self<<<(int)((threads + 255) / 256), 256, 0, ctx->st>>>(a); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

rbc3d_status run_near_corr(rbc3d_ctx* ctx, int tlist, double c1, double c2, int prec) {
  TargetSet& t = ctx->tl[tlist];
  if (t.n == 0 || ctx->ncell == 0) return RBC3D_OK;
  spl_wait(ctx);  // the near-singular quadrature interpolates the spline tables
  const double* Bc = ctx->dBcoef.p;
  CorrArgs a;
  fill_args(ctx, tlist, c1, (c2 != 0 && ctx->has_g) ? c2 : 0.0, a, Bc);
  if (c1 != 0 && !ctx->has_f) a.c1 = 0;
  a.screen = (prec != RBC3D_FP64) ? 1 : 0;
  // FP32 modes: pairs closer than rthr were left out of the FP32 pair sum and
  // are added back by the FP64 pass (-1: the FP64 plain form left nothing out)
  a.rthr = (prec != RBC3D_FP64) ? near_rthr_now(ctx) : -1.0;
  a.verify = ctx->verify_screen ? 1 : 0;
  a.list = nullptr;
  a.nlist = nullptr;
  int nsm = 0, per_sm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
  if (a.screen) {  // the FP32 replay reads x and a3 from FP32 node records
    const int per = ctx->m * ctx->nlon;
    const long long nn = (long long)ctx->ncell * per;
    if (!ctx->rep_valid || ctx->rep_rec.n < (size_t)nn * 24) {
      CUDA_TRY(ctx->rep_rec.alloc((size_t)nn * 24));
      { k_rep_rec<<<(int)((nn + 255) / 256), 256, 0, ctx->st>>>(nn, per, ctx->spl.p, ctx->rep_rec.p); ++ctx->launches; }
      CUDA_TRY(cudaGetLastError());
      ctx->rep_valid = true;
    }
    a.rep = ctx->rep_rec.p;
  }
  if (a.screen && !a.verify) {
    // FP32 modes: geometric screen per thread, FP32 replay per warp, then the
    // FP64 pass on what is left (counters: dcnt[8] replays, dcnt[10] listed)
    CUDA_TRY(ctx->near_l1.alloc(std::max(ctx->items_cap, 1)));
    CUDA_TRY(ctx->near_l2.alloc(std::max(ctx->items_cap, 1)));
    { k_near_screen<<<(ctx->items_cap + 255) / 256, 256, 0, ctx->st>>>(a, ctx->near_l1.p, ctx->dcnt.p + 8); ++ctx->launches; }
    { k_near_replay<<<nsm * 8, 128, 0, ctx->st>>>(a, ctx->near_l1.p, ctx->dcnt.p + 8, ctx->near_l2.p,
                                                   ctx->dcnt.p + 10); ++ctx->launches; }
    a.screen = 0;
    a.list = ctx->near_l2.p;
    a.nlist = ctx->dcnt.p + 10;
  }
  CUDA_TRY(ctx->near_queue.alloc(2));
  CUDA_TRY(cudaMemsetAsync(ctx->near_queue.p, 0, 2 * sizeof(unsigned long long), ctx->st));
  a.queue = ctx->near_queue.p;
  a.list_start = 0;
  a.stage_cap = std::max(0, std::min(ctx->near_stage_cap, NEAR_STAGE_CAP));
  if (a.list && a.stage_cap > 0) {  // the staged pass over the list's first stage_cap entries
    CUDA_TRY(ctx->near_plan.alloc((size_t)a.stage_cap * 16));
    CUDA_TRY(ctx->near_part.alloc((size_t)a.stage_cap * 9));
    NearPlan* plan = reinterpret_cast<NearPlan*>(ctx->near_plan.p);
    int ps = 0, us = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, k_near_proj, 128, 0));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&us, k_near_units, 128, 0));
    { k_near_proj<<<nsm * std::max(ps, 1), 128, 0, ctx->st>>>(a, plan); ++ctx->launches; }
    { k_near_units<<<nsm * std::max(us, 1), 128, 0, ctx->st>>>(a, plan, ctx->near_part.p, ctx->near_queue.p + 1);
      ++ctx->launches; }
    { k_near_fin<<<(a.stage_cap + 127) / 128, 128, 0, ctx->st>>>(a, plan, ctx->near_part.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
    // entries past the staged pass's capacity: k_near from there
    a.list_start = a.stage_cap;
    CUDA_TRY(cudaMemsetAsync(ctx->near_queue.p, 0, sizeof(unsigned long long), ctx->st));
  }
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_near, 128, 0));
  { k_near<<<nsm * std::max(per_sm, 1), 128, 0, ctx->st>>>(a); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// InterCellRepulsion (ModRepulsion.F90:270-402) with Closest_Neighbor_Cell and
// Closest_Neighbor_Wall (:480-613) on the context's cells and wall.
extern "C" rbc3d_status rbc3d_inter_cell_repulsion(rbc3d_ctx* ctx, double epsDist, double viscRatThresh,
                                                   int rigidsep, double* x, double* distMin, int* nmoved) {
  if (!ctx || !x || !(epsDist > 0)) return RBC3D_ERR_ARG;
  const int n = ctx->npt;
  if (distMin) *distMin = HUGE_VAL;
  if (nmoved) *nmoved = 0;
  if (n == 0) return RBC3D_OK;
  if (!ctx->src_sorted) return ctx_fail(ctx, RBC3D_ERR_STATE, "inter_cell_repulsion: cells not set");
  WallState& W = ctx->wall;
  if (W.nele > 0 && !W.cstart.p) return ctx_fail(ctx, RBC3D_ERR_STATE, "inter_cell_repulsion: wall lists not built");
  RepArgs a;
  a.n = n; a.nv = ctx->nlat * ctx->nlon; a.nlat = ctx->nlat; a.nlon = ctx->nlon; a.m = ctx->m;
  a.x = ctx->x.p; a.sx = ctx->s_x.p; a.smeta = ctx->s_meta.p; a.cs = ctx->s_cstart.p; a.ce = ctx->s_cend.p;
  a.spl = ctx->spl.p; a.th = ctx->th.p; a.phi = ctx->phi.p;
  for (int d = 0; d < 3; ++d) { a.Nc[d] = ctx->hg.Nc[d]; a.L[d] = ctx->prm.Lb[d]; a.iL[d] = ctx->iLb[d]; }
  a.eps = epsDist;
  a.nvert = W.nvert; a.nele = W.nele; a.wx = W.x.p; a.e2v = W.e2v.p;
  a.wcs = W.cstart.p; a.wce = W.cend.p; a.worder = W.order.p;
  spl_wait(ctx);  // Spline_FindProjection reads the x tables
  DBuf<double> dx, xo, visc;
  DBuf<unsigned long long> cnt;
  CUDA_TRY(dx.alloc(3 * (size_t)n)); CUDA_TRY(xo.alloc(3 * (size_t)n)); CUDA_TRY(cnt.alloc(2));
  CUDA_TRY(visc.upload(ctx->prm.viscRat, RBC3D_MAX_CELLTYPES, ctx->st));
  CUDA_TRY(cudaMemsetAsync(dx.p, 0, sizeof(double) * 3 * (size_t)n, ctx->st));
  unsigned long long init[2] = {0ull, 0ull};
  const double big = HUGE_VAL;
  std::memcpy(&init[0], &big, sizeof(big));  // positive doubles order as their bit patterns
  CUDA_TRY(cudaMemcpyAsync(cnt.p, init, sizeof(init), cudaMemcpyHostToDevice, ctx->st));
  a.dx = dx.p; a.dmin = cnt.p; a.nmoved = cnt.p + 1;
  { k_inter_rep<<<(int)(((long long)n * 32 + 127) / 128), 128, 0, ctx->st>>>(a); ++ctx->launches; }
  { k_inter_rep_apply<<<ctx->ncell, 256, 0, ctx->st>>>(a.nv, n, ctx->x.p, dx.p, ctx->celltype.p, visc.p, viscRatThresh,
                                                        rigidsep, xo.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  unsigned long long out[2] = {0, 0};
  CUDA_TRY(cudaMemcpyAsync(out, cnt.p, sizeof(out), cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaMemcpyAsync(x, xo.p, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  double dm;
  std::memcpy(&dm, &out[0], sizeof(dm));
  if (distMin) *distMin = dm;
  if (nmoved) *nmoved = (int)out[1];
  return RBC3D_OK;
}
