// oracle_math.cpp -- FP64 restatement of RBC3D numerical building blocks.
// TEST INFRASTRUCTURE ONLY (parity checker / CPU baseline); see oracle_math.hpp.
#include "oracle_math.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>

namespace orc {

const MaskTable& mask_table() {
  static const MaskTable t;
  return t;
}

// GauLeg, ModQuadRule.F90:135-214
void gauleg(double x1, double x2, int n, double* x, double* w) {
  const double EPS = 3.e-14;
  const int MAXIT = 10;
  int m = (n + 1) / 2;
  double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
  std::vector<double> p1(m), p2(m), p3(m), pp(m), z(m), z1(m);
  std::vector<char> unfinished(m, 1);
  for (int j = 0; j < m; ++j) z[j] = std::cos(PI * ((j + 1) - 0.25) / (n + 0.5));
  int its;
  for (its = 1; its <= MAXIT; ++its) {
    for (int k = 0; k < m; ++k)
      if (unfinished[k]) { p1[k] = 1.0; p2[k] = 0.0; }
    for (int j = 1; j <= n; ++j)
      for (int k = 0; k < m; ++k)
        if (unfinished[k]) {
          p3[k] = p2[k];
          p2[k] = p1[k];
          p1[k] = ((2.0 * j - 1.0) * z[k] * p2[k] - (j - 1.0) * p3[k]) / j;
        }
    bool any = false;
    for (int k = 0; k < m; ++k)
      if (unfinished[k]) {
        pp[k] = n * (z[k] * p1[k] - p2[k]) / (z[k] * z[k] - 1.0);
        z1[k] = z[k];
        z[k] = z1[k] - p1[k] / pp[k];
        unfinished[k] = std::fabs(z[k] - z1[k]) > EPS;
        any = any || unfinished[k];
      }
    if (!any) break;
  }
  for (int k = 0; k < m; ++k) {
    x[k] = xm - xl * z[k];
    x[n - 1 - k] = xm + xl * z[k];
    w[k] = 2.0 * xl / ((1.0 - z[k] * z[k]) * pp[k] * pp[k]);
    w[n - 1 - k] = w[k];
  }
}

static inline double my_asinh(double f) { return std::log(f + std::sqrt(1 + f * f)); }

// GauLeg_Sinh, ModQuadRule.F90:223-263
void gauleg_sinh(double xmin, double xmax, double a, double b, int n, double* x, double* w) {
  double xm = 0.5 * (xmin + xmax), xl = 0.5 * (xmax - xmin);
  double a0 = (a - xm) / xl;
  double b0 = b * xl;  // as written in the reference (:239)
  double u1 = my_asinh((1 + a0) / b0), u2 = my_asinh((1 - a0) / b0);
  double mu = 0.5 * (u1 + u2), eta = 0.5 * (u1 - u2);
  std::vector<double> s(n);
  gauleg(-1., 1., n, s.data(), w);
  for (int i = 0; i < n; ++i) {
    x[i] = a0 + b0 * std::sinh(mu * s[i] - eta);
    w[i] = w[i] * b0 * mu * std::cosh(mu * s[i] - eta);
  }
  for (int i = 0; i < n; ++i) { w[i] = xl * w[i]; x[i] = xm + xl * x[i]; }
}

// gqTri7, ModQuadRule.F90:69-94
TriRule gq_tri7() {
  TriRule q;
  q.n = 7;
  double r = (6. - std::sqrt(15.)) / 21., s = r, t = 1 - r - s;
  q.r[0] = r; q.r[1] = s; q.r[2] = t;
  q.s[0] = s; q.s[1] = t; q.s[2] = r;
  for (int i = 0; i < 3; ++i) q.w[i] = (155. - std::sqrt(15.)) / 2400.;
  r = (6. + std::sqrt(15.)) / 21.; s = r; t = 1 - r - s;
  q.r[3] = r; q.r[4] = s; q.r[5] = t;
  q.s[3] = s; q.s[4] = t; q.s[5] = r;
  for (int i = 3; i < 6; ++i) q.w[i] = (155. + std::sqrt(15.)) / 2400.;
  q.r[6] = 1. / 3.; q.s[6] = 1. / 3.; q.w[6] = 9. / 80.;
  return q;
}

// PolarPatch_Build, ModPolarPatch.F90:99-148
void polar_patch_build(double th0, double phi0, const double* thL, int nth, const double* phiL,
                       int nphi, double* thG, double* phiG) {
  double st0 = std::sin(th0), ct0 = std::cos(th0);
  for (int i = 0; i < nth; ++i) {
    double sth = std::sin(thL[i]), cth = std::cos(thL[i]);
    for (int j = 0; j < nphi; ++j) {
      double x0 = sth * std::cos(phiL[j]), x1 = sth * std::sin(phiL[j]), x2 = cth;
      double y0 = ct0 * x0 + 0. * x1 + st0 * x2;
      double y1 = 0. * x0 + 1. * x1 + 0. * x2;
      double y2 = -st0 * x0 + 0. * x1 + ct0 * x2;
      y2 = std::fmax(-1.0, std::fmin(1.0, y2));
      thG[i + nth * j] = std::acos(y2);
      double p = std::atan2(y1, y0) + phi0;
      phiG[i + nth * j] = p - std::floor(p * I_2PI) * TWO_PI;
    }
  }
}

// PolarPatch_Map, ModPolarPatch.F90:218-244
void polar_patch_map(double th0, double phi0, double dth, double dphi, double& th, double& phi) {
  double s1[3] = {std::cos(th0) * std::cos(phi0), std::cos(th0) * std::sin(phi0), -std::sin(th0)};
  double s2[3] = {-std::sin(phi0), std::cos(phi0), 0.};
  double x0[3] = {std::sin(th0) * std::cos(phi0), std::sin(th0) * std::sin(phi0), std::cos(th0)};
  double x[3] = {std::sin(dth) * std::cos(dphi), std::sin(dth) * std::sin(dphi), std::cos(dth)};
  double y[3];
  for (int c = 0; c < 3; ++c) y[c] = x[0] * s1[c] + x[1] * s2[c] + x[2] * x0[c];
  double nrm = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
  for (int c = 0; c < 3; ++c) y[c] /= nrm;
  y[2] = std::fmax(-1., std::fmin(1., y[2]));
  th = std::acos(y[2]);
  phi = std::atan2(y[1], y[0]);
  if (phi < 0) phi += TWO_PI;
}

// PolarPatch_FindPoints, ModPolarPatch.F90:161-209
void polar_patch_find_points(double th0, double phi0, double r0, const double* ths, int nth,
                             const double* phis, int nphi, std::vector<int>& ilat,
                             std::vector<int>& ilon) {
  const double eps = 1.e-10;
  double h_phi = TWO_PI / nphi, ih_phi = 1.0 / h_phi;
  double cosr0 = std::cos(r0);
  ilat.clear(); ilon.clear();
  for (int i = 0; i < nth; ++i) {
    if (ths[i] <= th0 - r0) continue;
    if (ths[i] >= th0 + r0) break;
    double dth = ths[i] - th0;
    double dphi = 1. - (std::cos(dth) - cosr0) / ((std::sin(ths[i]) + eps) * (std::sin(th0) + eps));
    dphi = std::fmax(-1., std::fmin(1., dphi));
    dphi = std::acos(dphi);
    int jmin, jmax;
    if (dphi > PI - eps) { jmin = 1; jmax = nphi; }
    else {
      jmin = (int)std::ceil((phi0 - dphi - phis[0]) * ih_phi) + 1;
      jmax = ifloor((phi0 + dphi - phis[0]) * ih_phi) + 1;
    }
    for (int j = jmin; j <= jmax; ++j) { ilat.push_back(i); ilon.push_back(fmod_pos(j - 1, nphi)); }
  }
}

// Spline_Interp, ModSpline.F90:150-191 (kx = ky = 0 for sphere splines)
void spline_interp(const Spline& s, double x, double y, double* f) {
  int i1 = ifloor(x * s.ihx), j1 = ifloor(y * s.ihy);
  double ss = x * s.ihx - i1, t = y * s.ihy - j1;
  i1 = fmod_pos(i1, s.m); j1 = fmod_pos(j1, s.n);
  int i2 = fmod_pos(i1 + 1, s.m), j2 = fmod_pos(j1 + 1, s.n);
  double cx[4] = {1 + ss * ss * (-3. + 2. * ss), ss * ss * (3. - 2. * ss), s.hx * ss * (1. + ss * (-2. + ss)),
                  s.hx * ss * ss * (-1. + ss)};
  double cy[4] = {1 + t * t * (-3. + 2. * t), t * t * (3. - 2. * t), s.hy * t * (1. + t * (-2. + t)),
                  s.hy * t * t * (-1. + t)};
  for (int l = 0; l < s.nvar; ++l) {
    double u[4][4] = {
        {s.at(0, i1, j1, l), s.at(0, i1, j2, l), s.at(2, i1, j1, l), s.at(2, i1, j2, l)},
        {s.at(0, i2, j1, l), s.at(0, i2, j2, l), s.at(2, i2, j1, l), s.at(2, i2, j2, l)},
        {s.at(1, i1, j1, l), s.at(1, i1, j2, l), s.at(3, i1, j1, l), s.at(3, i1, j2, l)},
        {s.at(1, i2, j1, l), s.at(1, i2, j2, l), s.at(3, i2, j1, l), s.at(3, i2, j2, l)}};
    double acc = 0;
    for (int a = 0; a < 4; ++a) {
      double r = 0;
      for (int b = 0; b < 4; ++b) r += u[a][b] * cy[b];
      acc += cx[a] * r;
    }
    f[l] = acc;
  }
}

// Cholesky solve of the 6x6 SPD system (LAPACK dposv 'U' semantics).
static void dposv6(double A[6][6], double* b) {
  double U[6][6] = {};
  for (int j = 0; j < 6; ++j) {
    double s = A[j][j];
    for (int k = 0; k < j; ++k) s -= U[k][j] * U[k][j];
    if (!(s > 0)) return;  // dposv leaves rhs unsolved when not SPD (info > 0)
    U[j][j] = std::sqrt(s);
    for (int i = j + 1; i < 6; ++i) {
      double t = A[j][i];
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

// QuadFit_2D, ModBasicMath.F90:234-284
void quadfit_2d(int npt, const double* xy, const double* f, double* c) {
  double lhs[6][6] = {}, rhs[6] = {};
  for (int i = 0; i < npt; ++i) {
    double xi = xy[i], yi = xy[i + npt];
    double u[6] = {1., xi, yi, xi * xi, xi * yi, yi * yi};
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b) lhs[a][b] += u[a] * u[b];
    for (int a = 0; a < 6; ++a) rhs[a] += u[a] * f[i];
  }
  for (int a = 1; a < 6; ++a)
    for (int b = 0; b < a; ++b) lhs[a][b] = lhs[b][a];
  dposv6(lhs, rhs);
  for (int a = 0; a < 6; ++a) c[a] = rhs[a];
}

// Min_Quad_2D, ModBasicMath.F90:296-327
void min_quad_2d(const double* c, double* xmin, double* fmin) {
  double a0 = c[0], a1 = c[1], a2 = c[2], a11 = c[3], a12 = c[4], a22 = c[5];
  double l11 = 2. * a11, l12 = a12, l21 = a12, l22 = 2. * a22;
  double det = l11 * l22 - l12 * l21;
  double r1 = -a1, r2 = -a2;
  if (det > 0) {
    double idet = 1. / det;
    xmin[0] = idet * (l22 * r1 - l12 * r2);
    xmin[1] = idet * (-l21 * r1 + l11 * r2);
  } else { xmin[0] = 0.; xmin[1] = 0.; }
  if (fmin)
    *fmin = a0 + a1 * xmin[0] + a2 * xmin[1] + a11 * xmin[0] * xmin[0] + a12 * xmin[0] * xmin[1] +
            a22 * xmin[1] * xmin[1];
}

// Spline_FindProjection, ModSpline.F90:203-269
void spline_find_projection(const Spline& s, const double* xtar, double& th0, double& phi0, double* x0) {
  const int iterMax = 3, nth = 2, nphi = 8;
  spline_interp(s, th0, phi0, x0);
  double h = std::max(s.hx, s.hy);
  double thL[nth], phiL[nphi], thP[nth * nphi], phiP[nth * nphi];
  double xy[(nth * nphi + 1) * 2], d2[nth * nphi + 1];
  const int npt = nth * nphi + 1;
  for (int iter = 1; iter <= iterMax; ++iter) {
    for (int i = 0; i < nth; ++i) thL[i] = (i + 1) * h / nth;
    for (int j = 0; j < nphi; ++j) phiL[j] = j * TWO_PI / nphi;
    polar_patch_build(th0, phi0, thL, nth, phiL, nphi, thP, phiP);
    double xx[3];
    xy[0] = 0.; xy[npt] = 0.;
    spline_interp(s, th0, phi0, xx);
    for (int c = 0; c < 3; ++c) xx[c] -= xtar[c];
    d2[0] = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    for (int j = 0; j < nphi; ++j)
      for (int i = 0; i < nth; ++i) {
        int k = 1 + i + nth * j;
        xy[k] = thL[i] * std::cos(phiL[j]);
        xy[k + npt] = thL[i] * std::sin(phiL[j]);
        spline_interp(s, thP[i + nth * j], phiP[i + nth * j], xx);
        for (int c = 0; c < 3; ++c) xx[c] -= xtar[c];
        d2[k] = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
      }
    double cf[6], xyMin[2], d2est;
    quadfit_2d(npt, xy, d2, cf);
    min_quad_2d(cf, xyMin, &d2est);
    double thMinL = std::sqrt(xyMin[0] * xyMin[0] + xyMin[1] * xyMin[1]);
    double phiMinL = std::atan2(xyMin[1], xyMin[0]);
    double thMin, phiMin, xMin[3];
    polar_patch_map(th0, phi0, thMinL, phiMinL, thMin, phiMin);
    spline_interp(s, thMin, phiMin, xMin);
    for (int c = 0; c < 3; ++c) xx[c] = xMin[c] - xtar[c];
    double d2Min = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    if (d2Min > d2[0]) break;
    th0 = thMin; phi0 = phiMin;
    for (int c = 0; c < 3; ++c) x0[c] = xMin[c];
    h = 0.5 * h;
  }
}

// ---------------------------------------------------------------------------
// FFT: recursive mixed radix (decimation in time), unnormalised, with a cached
// table of the n-th roots of unity exp(-2*pi*i*t/n).
static const std::vector<std::complex<double>>& roots(int n) {
  static std::mutex mu;
  static std::map<int, std::vector<std::complex<double>>> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(n);
  if (it != cache.end()) return it->second;
  std::vector<std::complex<double>> w(n);
  for (int t = 0; t < n; ++t) {
    double ang = -TWO_PI * (double)t / n;
    w[t] = std::complex<double>(std::cos(ang), std::sin(ang));
  }
  return cache.emplace(n, std::move(w)).first->second;
}

static void fft_rec(std::complex<double>* a, int n, int sign, std::complex<double>* tmp,
                    const std::complex<double>* W, int wstride) {
  if (n == 1) return;
  int p = 0;
  for (int f : {2, 3, 5}) if (n % f == 0) { p = f; break; }
  if (p == 0) {
    for (int f = 7; f * f <= n; f += 2) if (n % f == 0) { p = f; break; }
    if (p == 0) p = n;
  }
  int m = n / p;
  for (int r = 0; r < p; ++r)
    for (int k = 0; k < m; ++k) tmp[r * m + k] = a[k * p + r];
  for (int r = 0; r < p; ++r) fft_rec(tmp + r * m, m, sign, a, W, wstride * p);
  for (int q = 0; q < p; ++q)
    for (int k = 0; k < m; ++k) {
      int idx = k + q * m;
      std::complex<double> s = tmp[k];
      for (int r = 1; r < p; ++r) {
        std::complex<double> w = W[(size_t)(((long long)r * idx) % n) * wstride];
        if (sign > 0) w = std::conj(w);
        s += tmp[r * m + k] * w;
      }
      a[idx] = s;
    }
}

void fft_c2c(std::complex<double>* a, int n, int stride, int sign) {
  const auto& W = roots(n);
  std::vector<std::complex<double>> buf(n), tmp(n);
  for (int i = 0; i < n; ++i) buf[i] = a[(size_t)i * stride];
  fft_rec(buf.data(), n, sign, tmp.data(), W.data(), 1);
  for (int i = 0; i < n; ++i) a[(size_t)i * stride] = buf[i];
}

// ---------------------------------------------------------------------------
// Walls
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// MinDistToTri, ModIntOnWalls.F90:480-577
double min_dist_to_tri(const double* xTar, const double* x, double& s0, double& t0) {
  double x12[3], x13[3], x1T[3];
  for (int c = 0; c < 3; ++c) {
    x12[c] = x[1 + 3 * c] - x[0 + 3 * c];
    x13[c] = x[2 + 3 * c] - x[0 + 3 * c];
    x1T[c] = x[0 + 3 * c] - xTar[c];
  }
  double a = dot3(x12, x12), b = dot3(x12, x13), c = dot3(x13, x13);
  double det = a * c - b * b, invDet = 1. / det;
  double d = dot3(x12, x1T), e = dot3(x13, x1T), f = dot3(x1T, x1T);
  double s = b * e - c * d, t = b * d - a * e;
  int region;
  if (s + t <= det) {
    if (s < 0) region = (t < 0) ? 4 : 3;
    else if (t < 0) region = 5;
    else region = 0;
  } else {
    if (s < 0) region = 2;
    else if (t < 0) region = 6;
    else region = 1;
  }
  if (region == 2) region = (-(c + e) < 0) ? 3 : 1;
  else if (region == 4) region = (d < 0) ? 5 : 3;
  else if (region == 6) region = (b + e - a - d < 0) ? 1 : 5;
  switch (region) {
    case 0: s = invDet * s; t = invDet * t; break;
    case 1:
      s = (c + e - b - d) / (a - 2 * b + c);
      s = std::fmin(1., std::fmax(0., s));
      t = 1. - s;
      break;
    case 3:
      s = 0.; t = -e / c; t = std::fmin(1., std::fmax(0., t));
      break;
    case 5:
      t = 0.; s = -d / a; s = std::fmin(1., std::fmax(0., s));
      break;
  }
  s0 = s; t0 = t;
  return std::sqrt(a * s * s + 2 * b * s * t + c * t * t + 2 * d * s + 2 * e * t + f);
}

// Tri_Int_Regular, ModIntOnWalls.F90:319-363.  lhs (3,3,3) col-major: lhs[l + 3*(ii + 3*jj)].
void tri_int_regular(const EwaldTables& E, const double* x, const double* f, const double* xtar,
                     double* rhs, double* lhs) {
  static const TriRule GQ = gq_tri7();
  double xv[3][3], fv[3][3];
  for (int l = 0; l < 3; ++l)
    for (int c = 0; c < 3; ++c) { xv[l][c] = x[l + 3 * c]; fv[l][c] = f ? f[l + 3 * c] : 0.; }
  double a[3], b[3], cr[3];
  for (int c = 0; c < 3; ++c) { a[c] = xv[1][c] - xv[0][c]; b[c] = xv[2][c] - xv[0][c]; }
  cr[0] = a[1] * b[2] - a[2] * b[1]; cr[1] = a[2] * b[0] - a[0] * b[2]; cr[2] = a[0] * b[1] - a[1] * b[0];
  double detJ = 2 * (0.5 * std::sqrt(dot3(cr, cr)));
  rhs[0] = rhs[1] = rhs[2] = 0.;
  if (lhs) std::memset(lhs, 0, sizeof(double) * 27);
  for (int q = 0; q < GQ.n; ++q) {
    double s = GQ.r[q], t = GQ.s[q];
    double xg[3], fg[3], xx[3];
    for (int c = 0; c < 3; ++c) {
      xg[c] = (1. - s - t) * xv[0][c] + s * xv[1][c] + t * xv[2][c];
      fg[c] = (1. - s - t) * fv[0][c] + s * fv[1][c] + t * fv[2][c];
    }
    double ds = GQ.w[q] * detJ;
    for (int c = 0; c < 3; ++c) { fg[c] = ds * fg[c]; xx[c] = xtar[c] - xg[c]; }
    double rr = std::sqrt(dot3(xx, xx)), EA, EB;
    E.sl(rr, EA, EB);
    double xf = dot3(xx, fg);
    for (int c = 0; c < 3; ++c) rhs[c] += EA * xx[c] * xf + EB * fg[c];
    if (lhs) {
      double L[3][3];
      for (int ii = 0; ii < 3; ++ii)
        for (int jj = 0; jj < 3; ++jj) L[ii][jj] = EA * xx[ii] * xx[jj];
      for (int ii = 0; ii < 3; ++ii) L[ii][ii] += EB;
      double wv[3] = {1 - s - t, s, t};
      for (int l = 0; l < 3; ++l)
        for (int ii = 0; ii < 3; ++ii)
          for (int jj = 0; jj < 3; ++jj) lhs[l + 3 * (ii + 3 * jj)] += wv[l] * (ds * L[ii][jj]);
    }
  }
}

// Tri_Int_Duffy, ModIntOnWalls.F90:373-465
void tri_int_duffy(const EwaldTables& E, const double* x, const double* f, const double* xtar,
                   double s0, double t0, double* rhs, double* lhs) {
  static const int nGq = 4;
  static double rGq[4], wGq[4];
  static bool inited = [] { gauleg(0., 1., 4, rGq, wGq); return true; }();
  (void)inited;
  double xv[3][3], fv[3][3];
  for (int l = 0; l < 3; ++l)
    for (int c = 0; c < 3; ++c) { xv[l][c] = x[l + 3 * c]; fv[l][c] = f ? f[l + 3 * c] : 0.; }
  double x0[3], f0[3];
  for (int c = 0; c < 3; ++c) {
    x0[c] = (1 - s0 - t0) * xv[0][c] + s0 * xv[1][c] + t0 * xv[2][c];
    f0[c] = (1 - s0 - t0) * fv[0][c] + s0 * fv[1][c] + t0 * fv[2][c];
  }
  rhs[0] = rhs[1] = rhs[2] = 0.;
  if (lhs) std::memset(lhs, 0, sizeof(double) * 27);
  for (int n = 0; n < 3; ++n) {
    const double* x1 = xv[n];
    const double* x2 = xv[(n + 1) % 3];
    const double* f1 = fv[n];
    const double* f2 = fv[(n + 1) % 3];
    double a[3], b[3], nr[3];
    for (int c = 0; c < 3; ++c) { a[c] = x1[c] - x0[c]; b[c] = x2[c] - x0[c]; }
    nr[0] = a[1] * b[2] - a[2] * b[1]; nr[1] = a[2] * b[0] - a[0] * b[2]; nr[2] = a[0] * b[1] - a[1] * b[0];
    double detJ = std::sqrt(dot3(nr, nr));
    for (int i = 0; i < nGq; ++i)
      for (int j = 0; j < nGq; ++j) {
        double s = rGq[i], t = s * rGq[j];
        double xg[3], fg[3], xx[3];
        for (int c = 0; c < 3; ++c) {
          xg[c] = (1. - s) * x0[c] + (s - t) * x1[c] + t * x2[c];
          fg[c] = (1. - s) * f0[c] + (s - t) * f1[c] + t * f2[c];
        }
        double ds = wGq[i] * wGq[j] * detJ * s;
        for (int c = 0; c < 3; ++c) { fg[c] = ds * fg[c]; xx[c] = xtar[c] - xg[c]; }
        double rr = std::sqrt(dot3(xx, xx)), EA, EB;
        E.sl(rr, EA, EB);
        double xf = dot3(xx, fg);
        for (int c = 0; c < 3; ++c) rhs[c] += EA * xx[c] * xf + EB * fg[c];
        if (lhs) {
          double L[3][3];
          for (int ii = 0; ii < 3; ++ii)
            for (int jj = 0; jj < 3; ++jj) L[ii][jj] = EA * xx[ii] * xx[jj];
          for (int ii = 0; ii < 3; ++ii) L[ii][ii] += EB;
          double s1, t1, s2, t2;
          if (n == 0) { s1 = 0.; t1 = 0.; s2 = 1.; t2 = 0.; }
          else if (n == 1) { s1 = 1.; t1 = 0.; s2 = 0.; t2 = 1.; }
          else { s1 = 0.; t1 = 1.; s2 = 0.; t2 = 0.; }
          double sG = (1. - s) * s0 + (s - t) * s1 + t * s2;
          double tG = (1. - s) * t0 + (s - t) * t1 + t * t2;
          double wv[3] = {1. - sG - tG, sG, tG};
          for (int l = 0; l < 3; ++l)
            for (int ii = 0; ii < 3; ++ii)
              for (int jj = 0; jj < 3; ++jj) lhs[l + 3 * (ii + 3 * jj)] += wv[l] * (ds * L[ii][jj]);
        }
      }
  }
}


void pbar_table(int L, double theta, double* P) {
  const double x = std::cos(theta), sn = std::sin(theta);
  for (int i = 0; i < L * L; ++i) P[i] = 0.;
  double pmm = std::sqrt(0.5);  // pbar(0, 0)
  for (int m = 0; m < L; ++m) {
    if (m > 0) pmm *= std::sqrt((2.0 * m + 1.0) / (2.0 * m)) * sn;
    P[m * L + m] = pmm;
    if (m + 1 < L) P[m * L + m + 1] = std::sqrt(2.0 * m + 3.0) * x * pmm;
    for (int n = m + 2; n < L; ++n) {
      const double a = std::sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
      const double b = std::sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
      P[m * L + n] = a * (x * P[m * L + n - 1] - b * P[m * L + n - 2]);
    }
  }
}

void fft_diff(const double* u, int M, int stride, double* du) {
  std::vector<std::complex<double>> a(M);
  for (int i = 0; i < M; ++i) a[i] = u[(size_t)i * stride];
  fft_c2c(a.data(), M, 1, -1);
  // half spectrum k = 0 .. M/2: k < M/2 times i k / M, k = M/2 zeroed
  const int H = M / 2;
  std::vector<std::complex<double>> h(H + 1);
  for (int k = 0; k < H; ++k) h[k] = a[k] * std::complex<double>(0.0, (double)k / M);
  h[H] = 0.;
  // c2r: the Hermitian extension, imaginary parts of k = 0 (and M/2) ignored
  std::vector<std::complex<double>> b(M);
  b[0] = h[0].real();
  for (int k = 1; k <= H; ++k) {
    if (2 * k == M) { b[k] = h[k].real(); continue; }
    b[k] = h[k];
    b[M - k] = std::conj(h[k]);
  }
  fft_c2c(b.data(), M, 1, +1);
  for (int i = 0; i < M; ++i) du[(size_t)i * stride] = b[i].real();
}

void spline_build_on_sphere(int nlat, int nlon, int nvar, const double* f, double* tab) {
  const int m = 2 * nlat, n = nlon;
  const size_t per = (size_t)m * n * nvar;
  double* u = tab;
  double* u1 = tab + per;
  double* u2 = tab + 2 * per;
  double* u12 = tab + 3 * per;
  for (int l = 0; l < nvar; ++l)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < nlat; ++i) {
        u[i + (size_t)m * (j + (size_t)n * l)] = f[i + (size_t)(nlat + 1) * (j + (size_t)n * l)];
        u[nlat + i + (size_t)m * (j + (size_t)n * l)] =
            f[(nlat - i) + (size_t)(nlat + 1) * ((j + n / 2) % n + (size_t)n * l)];
      }
  for (int l = 0; l < nvar; ++l) {
    for (int j = 0; j < n; ++j) fft_diff(u + (size_t)m * (j + (size_t)n * l), m, 1, u1 + (size_t)m * (j + (size_t)n * l));
    for (int i = 0; i < m; ++i) {
      fft_diff(u + i + (size_t)m * n * l, n, m, u2 + i + (size_t)m * n * l);
      // u12 from u1 along the second axis (FFT_Diff(u1, u2=u12))
    }
  }
  for (int l = 0; l < nvar; ++l)
    for (int i = 0; i < m; ++i) fft_diff(u1 + i + (size_t)m * n * l, n, m, u12 + i + (size_t)m * n * l);
}
}  // namespace orc
