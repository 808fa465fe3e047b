// oracle_math.hpp -- FP64 restatement of the numerical building blocks of
// RBC3D's boundary-integral matvec.  TEST INFRASTRUCTURE: this code is the
// parity checker for the GPU implementation and the CPU baseline of the
// benchmark; nothing in the product path links or calls it.
//
// Each function follows the cited reference routine (paths relative to the
// RBC3D source tree) step by step, in FP64, including its quirks.
#pragma once
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

namespace orc {

constexpr double PI = 3.14159265358979323846;  // ModDataTypes.F90:17
constexpr double TWO_PI = 2 * PI;
constexpr double I_2PI = 1. / TWO_PI;
constexpr double THRD = 1.0 / 3;

inline int fmod_pos(int a, int b) { int r = a % b; return r < 0 ? r + b : r; }  // Fortran modulo
inline double nint(double x) { return std::round(x); }  // Fortran nint: half away from zero
inline int ifloor(double x) { return (int)std::floor(x); }

// ---------------------------------------------------------------------------
// Ewald coefficient tables, ModEwaldFunc.F90:86-180 (8193-entry lerp tables).
struct EwaldTables {
  static constexpr int N = 8192;  // Ntable, ModEwaldFunc.F90:9
  double alpha = 0, rc = 0, r_eps = 0;
  std::vector<double> sl_c1, sl_c2, dl_c1;
  void build(double alpha_, double rc_) {
    alpha = alpha_; rc = rc_;
    sl_c1.resize(N + 1); sl_c2.resize(N + 1); dl_c1.resize(N + 1);
    for (int i = 0; i <= N; ++i) {
      double r_t = std::sqrt(PI / alpha) * ((double)i * rc / N);
      sl_c1[i] = std::erfc(r_t);                                  // :101
      sl_c2[i] = 2 / std::sqrt(alpha) * std::exp(-(r_t * r_t));   // :102
      dl_c1[i] = -8 / std::sqrt(PI) *
                 (std::exp(-(r_t * r_t)) * (1.5 * r_t + r_t * r_t * r_t) +
                  0.75 * std::sqrt(PI) * std::erfc(r_t));          // :161
    }
    r_eps = 1.e-3 * std::sqrt(alpha / PI);
  }
  // EwaldCoeff_SL, ModEwaldFunc.F90:86
  inline void sl(double r, double& A, double& B) const {
    if (r < r_eps) { A = 0; B = 0; return; }
    double s = N * r / rc;
    int i = ifloor(s);
    if (i >= N) { A = 0; B = 0; return; }
    double c1 = sl_c1[i] * (i + 1 - s) + sl_c1[i + 1] * (s - i);
    double c2 = sl_c2[i] * (i + 1 - s) + sl_c2[i + 1] * (s - i);
    double ir = 1. / r, ir2 = ir * ir;
    A = c1 * ir * ir2 + c2 * ir2;
    B = c1 * ir - c2;
  }
  // EwaldCoeff_DL, ModEwaldFunc.F90:141
  inline double dl(double r) const {
    if (r < r_eps) return 0;
    double s = N * r / rc;
    int i = ifloor(s);
    if (i >= N) return 0;
    double c1 = dl_c1[i] * (i + 1 - s) + dl_c1[i + 1] * (s - i);
    double r2 = r * r;
    return c1 / (r2 * r2 * r);
  }
};

// EwaldCoeff_SL_Exact / EwaldCoeff_DL_Exact, ModEwaldFunc.F90:25-80
inline void ewald_sl_exact(double r, double alpha, double& A, double& B) {
  if (alpha <= 0) { A = 1 / (r * r * r); B = 1 / r; return; }
  double r_t = std::sqrt(PI / alpha) * r;
  if (r_t < 1.e-3) { A = 0; B = 0; return; }
  double c1 = std::erfc(r_t), c2 = 2. / std::sqrt(alpha) * std::exp(-(r_t * r_t));
  double ir = 1. / r, ir2 = ir * ir;
  A = c1 * ir * ir2 + c2 * ir2;
  B = c1 * ir - c2;
}
inline double ewald_dl_exact(double r, double alpha) {
  if (alpha <= 0) return -6 / std::pow(r, 5);
  double r_t = std::sqrt(PI / alpha) * r;
  if (r_t < 1.e-3) return 0;
  double A = std::exp(-(r_t * r_t)) * (1.5 * r_t + r_t * r_t * r_t) + 0.75 * std::sqrt(PI) * std::erfc(r_t);
  return -8 / std::sqrt(PI) * A / std::pow(r, 5);
}

// MaskFunc_Exact / MaskFunc, ModBasicMath.F90:332-379
inline double mask_exact(double x) {
  double t = std::fabs(x);
  if (t < 0.01) return 1.;
  if (t > 0.99) return 0.;
  return std::exp(2 * (std::exp(-1. / t)) / (t - 1));
}
struct MaskTable {
  static constexpr int N = 8192;
  std::vector<double> ftab;
  MaskTable() { ftab.resize(N + 1); for (int i = 0; i <= N; ++i) ftab[i] = mask_exact((double)i / N); }
  inline double operator()(double x) const {
    double s = std::fabs(x) * N;
    int i = ifloor(s);
    if (i >= N) return 0.;
    return ftab[i] * (i + 1 - s) + ftab[i + 1] * (s - i);
  }
};
const MaskTable& mask_table();
inline double MaskFunc(double x) { return mask_table()(x); }

// BsplineFunc, ModBasicMath.F90:392-417.  w[0..P-1] maps to mesh imin..imin+P-1.
inline void bspline(double xc, int P, int& imin, double* w) {
  double u[32];
  imin = ifloor(xc) - (P - 1);
  u[0] = imin - (xc - P);
  for (int j = 1; j < P; ++j) u[j] = u[j - 1] + 1;
  w[0] = 1.;
  for (int j = 1; j < P; ++j) w[j] = 0.;
  for (int pp = 2; pp <= P; ++pp) {
    for (int j = pp; j >= 2; --j)
      w[j - 1] = u[j - 1] / (pp - 1.) * w[j - 1] + (pp - u[j - 1]) / (pp - 1.) * w[j - 2];
    w[0] = u[0] / (pp - 1.) * w[0];
  }
}

// GauLeg, ModQuadRule.F90:135-214 (Numerical Recipes, simultaneous Newton).
void gauleg(double x1, double x2, int n, double* x, double* w);
// GauLeg_Sinh, ModQuadRule.F90:223-263 (b0 = b*xl as written at :239).
void gauleg_sinh(double xmin, double xmax, double a, double b, int n, double* x, double* w);

// gqTri7, ModQuadRule.F90:69-94
struct TriRule { int n; double r[7], s[7], w[7]; };
TriRule gq_tri7();

// DistOnSphere, ModPolarPatch.F90:249-257
inline double dist_on_sphere(double th0, double phi0, double th1, double phi1) {
  double d = std::cos(th0 - th1) - std::sin(th0) * std::sin(th1) * (1. - std::cos(phi0 - phi1));
  d = std::fmin(1., std::fmax(-1., d));
  return std::acos(d);
}

// PolarPatch_Build, ModPolarPatch.F90:99-148.  thG/phiG are (nth, nphi)
// column-major: thG[i + nth*j].
void polar_patch_build(double th0, double phi0, const double* thL, int nth, const double* phiL,
                       int nphi, double* thG, double* phiG);
// PolarPatch_Map, ModPolarPatch.F90:218-244
void polar_patch_map(double th0, double phi0, double dth, double dphi, double& th, double& phi);
// PolarPatch_FindPoints, ModPolarPatch.F90:161-209.  ijs holds 0-based (ilat, ilon).
void polar_patch_find_points(double th0, double phi0, double r0, const double* ths, int nth,
                             const double* phis, int nphi, std::vector<int>& ilat,
                             std::vector<int>& ilon);

// t_spline (ModDataStruct) view: u, u1, u2, u12 each (m, n, nvar) column-major.
struct Spline {
  int m = 0, n = 0, nvar = 0;
  double hx = 0, hy = 0, ihx = 0, ihy = 0;
  const double* u = nullptr;  // 4*m*n*nvar: u | u1 | u2 | u12
  void set(int m_, int n_, int nvar_, const double* data) {
    m = m_; n = n_; nvar = nvar_; u = data;
    hx = TWO_PI / m; hy = TWO_PI / n; ihx = 1. / hx; ihy = 1. / hy;  // Spline_Create
  }
  inline double at(int kind, int i, int j, int l) const { return u[(size_t)kind * m * n * nvar + i + (size_t)m * (j + (size_t)n * l)]; }
};
// Spline_Interp, ModSpline.F90:150-191
void spline_interp(const Spline& s, double x, double y, double* f);
// QuadFit_2D (normal equations + dposv 'U'), ModBasicMath.F90:234-284
void quadfit_2d(int npt, const double* xy /*(npt,2) col-major*/, const double* f, double* c);
// Min_Quad_2D, ModBasicMath.F90:296-327
void min_quad_2d(const double* c, double* xmin, double* fmin);
// Spline_FindProjection, ModSpline.F90:203-269 (th0, phi0 updated in place)
void spline_find_projection(const Spline& s, const double* xtar, double& th0, double& phi0, double* x0);

// Mixed-radix complex FFT (own implementation; radix 2/3/5 + direct DFT for
// other factors).  sign = -1 forward, +1 backward; unnormalised.
void fft_c2c(std::complex<double>* a, int n, int stride, int sign);

// Spherepack's normalised associated Legendre functions pbar(m, n, theta)
// (documentation of shags/shsgs: sqrt((2n+1)/2 (n-m)!/(n+m)!) sin^m(theta)
// d^m P_n / dx^m at x = cos(theta), no Condon-Shortley phase, so that
// int_{-1}^{1} pbar^2 dx = 1), for 0 <= m <= n < L, by the standard
// three-term recurrence in n.  P[m*L + n].
void pbar_table(int L, double theta, double* P);
// FFT_Diff, ModFFT.F90:25-93, along one axis of length M (stride in the
// array): the r2c transform, modes k < M/2 times i k / M, mode M/2 zeroed,
// the unnormalised c2r back (FFTW semantics).
void fft_diff(const double* u, int M, int stride, double* du);
// Spline_Build_On_Sphere, ModSpline.F90:121-143: f on the equiangular grid
// (nlat+1 rows with both poles, nlon columns, nvar; f[i + (nlat+1)*(j + nlon*l)])
// to the table u | u1 | u2 | u12, each (2 nlat, nlon, nvar) column-major.
void spline_build_on_sphere(int nlat, int nlon, int nvar, const double* f, double* tab);

// MinDistToTri (Eberly), ModIntOnWalls.F90:480-577.  x(3,3) col-major:
// x[l + 3*c] is vertex l component c.
double min_dist_to_tri(const double* xtar, const double* x, double& s0, double& t0);
// Tri_Int_Regular, ModIntOnWalls.F90:319-363 (lhs optional: (3,3,3) col-major)
void tri_int_regular(const EwaldTables& E, const double* x, const double* f, const double* xtar,
                     double* rhs, double* lhs);
// Tri_Int_Duffy, ModIntOnWalls.F90:373-465
void tri_int_duffy(const EwaldTables& E, const double* x, const double* f, const double* xtar,
                   double s0, double t0, double* rhs, double* lhs);

}  // namespace orc
