// common.cuh -- device helpers shared by the kernels of the GB300 Ewald matvec.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#define RBC3D_PI 3.14159265358979323846
#define RBC3D_TWO_PI (2.0 * RBC3D_PI)
#define RBC3D_I_2PI (1.0 / RBC3D_TWO_PI)
#define EWALD_NTAB 8192  // Ntable, ModEwaldFunc.F90:9
#define MASK_NTAB 8192   // MaskFunc table size, ModBasicMath.F90:356
#define NEAR_STAGE_CAP 65536  // list entries of the FP32 modes' staged near-singular pass

// Number of doubles per spline node per variable set: 4 kinds (u, u1, u2,
// u12) x 3 variables.  Sets: x, a3, FdetJ, GdetJ, detJ (detJ uses var 0).
#define SPL_NODE 12
enum { SPL_X = 0, SPL_A3 = 1, SPL_F = 2, SPL_G = 3, SPL_DJ = 4, SPL_NSET = 5 };

// Device view of the Ewald / mask tables.
struct Tables {
  // FP64 tables exactly as ModEwaldFunc / ModBasicMath build them (N+1 entries)
  const double* sl_c1;
  const double* sl_c2;
  const double* dl_c1;
  const double* mask;
  // FP32 lerp tables: {v_i, v_{i+1}-v_i} pairs
  const float4* sl32;  // {c1, dc1, c2, dc2}
  const float2* dl32;  // {dl, ddl}
  const float2* mask32;
  double rc, r_eps, ntab_over_rc;
  float rc_f, r_eps_f, ntab_over_rc_f;
};

// ---------------------------------------------------------------------------
// EwaldCoeff_SL / EwaldCoeff_DL (ModEwaldFunc.F90:86-180), FP64.
__device__ __forceinline__ void ewald_sl64(const Tables& T, double r, double& A, double& B) {
  if (r < T.r_eps) { A = 0.; B = 0.; return; }
  double s = EWALD_NTAB * r / T.rc;
  int i = (int)floor(s);
  if (i >= EWALD_NTAB) { A = 0.; B = 0.; return; }
  double c1 = __ldg(T.sl_c1 + i) * (i + 1 - s) + __ldg(T.sl_c1 + i + 1) * (s - i);
  double c2 = __ldg(T.sl_c2 + i) * (i + 1 - s) + __ldg(T.sl_c2 + i + 1) * (s - i);
  double ir = 1. / r, ir2 = ir * ir;
  A = c1 * ir * ir2 + c2 * ir2;
  B = c1 * ir - c2;
}
// The same with 1/r supplied (from rsqrt of r^2, 1 ulp) and the table index as
// r * (NTAB/rc): no FP64 division.
// Callers pass r = r2 * rsqrt(r2), which is NaN for r2 = 0 (a target that is
// its own source): !(r >= r_eps) catches it, and the index is range-checked.
__device__ __forceinline__ void ewald_sl64r(const Tables& T, double r, double ir, double& A, double& B) {
  if (!(r >= T.r_eps)) { A = 0.; B = 0.; return; }
  double s = r * T.ntab_over_rc;
  int i = (int)floor(s);
  if (i < 0 || i >= EWALD_NTAB) { A = 0.; B = 0.; return; }
  double c1 = __ldg(T.sl_c1 + i) * (i + 1 - s) + __ldg(T.sl_c1 + i + 1) * (s - i);
  double c2 = __ldg(T.sl_c2 + i) * (i + 1 - s) + __ldg(T.sl_c2 + i + 1) * (s - i);
  double ir2 = ir * ir;
  A = c1 * ir * ir2 + c2 * ir2;
  B = c1 * ir - c2;
}
__device__ __forceinline__ double ewald_dl64r(const Tables& T, double r, double ir) {
  if (!(r >= T.r_eps)) return 0.;
  double s = r * T.ntab_over_rc;
  int i = (int)floor(s);
  if (i < 0 || i >= EWALD_NTAB) return 0.;
  double c1 = __ldg(T.dl_c1 + i) * (i + 1 - s) + __ldg(T.dl_c1 + i + 1) * (s - i);
  double ir2 = ir * ir;
  return c1 * (ir2 * ir2 * ir);
}
__device__ __forceinline__ double ewald_dl64(const Tables& T, double r) {
  if (r < T.r_eps) return 0.;
  double s = EWALD_NTAB * r / T.rc;
  int i = (int)floor(s);
  if (i >= EWALD_NTAB) return 0.;
  double c1 = __ldg(T.dl_c1 + i) * (i + 1 - s) + __ldg(T.dl_c1 + i + 1) * (s - i);
  double r2 = r * r;
  return c1 / (r2 * r2 * r);
}
// MaskFunc (ModBasicMath.F90:351-379), FP64
__device__ __forceinline__ double mask64(const Tables& T, double x) {
  double s = fabs(x) * MASK_NTAB;
  int i = (int)floor(s);
  if (i >= MASK_NTAB) return 0.;
  return __ldg(T.mask + i) * (i + 1 - s) + __ldg(T.mask + i + 1) * (s - i);
}
// DistOnSphere (ModPolarPatch.F90:249-257)
__device__ __forceinline__ double dist_on_sphere(double th0, double phi0, double th1, double phi1) {
  double d = cos(th0 - th1) - sin(th0) * sin(th1) * (1. - cos(phi0 - phi1));
  d = fmin(1., fmax(-1., d));
  return acos(d);
}

// ---------------------------------------------------------------------------
// Bicubic Hermite interpolation on the doubled-sphere grid (Spline_Interp,
// ModSpline.F90:150-191).  Node layout: spl[node*SPL_NODE + kind*3 + var].
// Spline_Interp weights of one patch point for a target latitude: row i1,
// column offset j1b (before adding the target's longitude index), cx, cy.
struct SelfW64 {
  int i1, j1b;
  double w[16];  // the 16 Spline_Interp weight products in spline_w16's order
};
struct SplW {
  int n11, n12, n21, n22;  // node ids (i1,j1) (i1,j2) (i2,j1) (i2,j2)
  double cx[4], cy[4];
};
__device__ __forceinline__ int imod(int a, int b) { int r = a % b; return r < 0 ? r + b : r; }

// Spline_Create constants of the periodic (m, n) grid: h = 2 pi / m, ih = 1 / h.
struct SplGrid {
  int m, n;
  double hx, hy, ihx, ihy;
};
inline SplGrid spl_grid(int m, int n) {
  SplGrid g;
  g.m = m; g.n = n;
  g.hx = RBC3D_TWO_PI / m; g.hy = RBC3D_TWO_PI / n;
  g.ihx = 1. / g.hx; g.ihy = 1. / g.hy;
  return g;
}
// Spline_Interp weights (ModSpline.F90:150-191) with the grid constants
// precomputed (bitwise the same values as computing them here).
__device__ __forceinline__ void spline_weights_g(double x, double y, const SplGrid& G, SplW& W) {
  const int m = G.m, n = G.n;
  const double hx = G.hx, hy = G.hy, ihx = G.ihx, ihy = G.ihy;
  int i1 = (int)floor(x * ihx), j1 = (int)floor(y * ihy);
  double s = x * ihx - i1, t = y * ihy - j1;
  i1 = imod(i1, m); j1 = imod(j1, n);
  int i2 = imod(i1 + 1, m), j2 = imod(j1 + 1, n);
  W.cx[0] = 1 + s * s * (-3. + 2. * s); W.cx[1] = s * s * (3. - 2. * s);
  W.cx[2] = hx * s * (1. + s * (-2. + s)); W.cx[3] = hx * s * s * (-1. + s);
  W.cy[0] = 1 + t * t * (-3. + 2. * t); W.cy[1] = t * t * (3. - 2. * t);
  W.cy[2] = hy * t * (1. + t * (-2. + t)); W.cy[3] = hy * t * t * (-1. + t);
  W.n11 = i1 + m * j1; W.n12 = i1 + m * j2; W.n21 = i2 + m * j1; W.n22 = i2 + m * j2;
}
__device__ __forceinline__ void spline_weights(double x, double y, int m, int n, SplW& W) {
  const double hx = RBC3D_TWO_PI / m, hy = RBC3D_TWO_PI / n;
  const double ihx = 1. / hx, ihy = 1. / hy;
  int i1 = (int)floor(x * ihx), j1 = (int)floor(y * ihy);
  double s = x * ihx - i1, t = y * ihy - j1;
  i1 = imod(i1, m); j1 = imod(j1, n);
  int i2 = imod(i1 + 1, m), j2 = imod(j1 + 1, n);
  W.cx[0] = 1 + s * s * (-3. + 2. * s); W.cx[1] = s * s * (3. - 2. * s);
  W.cx[2] = hx * s * (1. + s * (-2. + s)); W.cx[3] = hx * s * s * (-1. + s);
  W.cy[0] = 1 + t * t * (-3. + 2. * t); W.cy[1] = t * t * (3. - 2. * t);
  W.cy[2] = hy * t * (1. + t * (-2. + t)); W.cy[3] = hy * t * t * (-1. + t);
  W.n11 = i1 + m * j1; W.n12 = i1 + m * j2; W.n21 = i2 + m * j1; W.n22 = i2 + m * j2;
}
// Interpolate nvar (<=3) variables of one spline set (pointer to node 0).
__device__ __forceinline__ void spline_eval(const double* __restrict__ spl, const SplW& W, int nvar, double* f) {
  const double* a = spl + (size_t)W.n11 * SPL_NODE;
  const double* b = spl + (size_t)W.n12 * SPL_NODE;
  const double* c = spl + (size_t)W.n21 * SPL_NODE;
  const double* d = spl + (size_t)W.n22 * SPL_NODE;
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    if (l >= nvar) break;
    // rows of u(4,4) in Spline_Interp: (u, u2 @ i1), (u, u2 @ i2), (u1, u12 @ i1), (u1, u12 @ i2)
    double r0 = __ldg(a + l) * W.cy[0] + __ldg(b + l) * W.cy[1] + __ldg(a + 6 + l) * W.cy[2] + __ldg(b + 6 + l) * W.cy[3];
    double r1 = __ldg(c + l) * W.cy[0] + __ldg(d + l) * W.cy[1] + __ldg(c + 6 + l) * W.cy[2] + __ldg(d + 6 + l) * W.cy[3];
    double r2 = __ldg(a + 3 + l) * W.cy[0] + __ldg(b + 3 + l) * W.cy[1] + __ldg(a + 9 + l) * W.cy[2] + __ldg(b + 9 + l) * W.cy[3];
    double r3 = __ldg(c + 3 + l) * W.cy[0] + __ldg(d + 3 + l) * W.cy[1] + __ldg(c + 9 + l) * W.cy[2] + __ldg(d + 9 + l) * W.cy[3];
    f[l] = W.cx[0] * r0 + W.cx[1] * r1 + W.cx[2] * r2 + W.cx[3] * r3;
  }
}

// The 16 products cx[.] cy[.] of Spline_Interp's weights, in record order:
// per node (n11, n12, n21, n22) the weights of (u, u1, u2, u12).
__device__ __forceinline__ void spline_w16(const SplW& W, double* w) {
  const double* cx = W.cx;
  const double* cy = W.cy;
  // node n11 = (i1, j1): u cx0 cy0, u1 cx2 cy0, u2 cx0 cy2, u12 cx2 cy2
  w[0] = cx[0] * cy[0]; w[1] = cx[2] * cy[0]; w[2] = cx[0] * cy[2]; w[3] = cx[2] * cy[2];
  // n12 = (i1, j2)
  w[4] = cx[0] * cy[1]; w[5] = cx[2] * cy[1]; w[6] = cx[0] * cy[3]; w[7] = cx[2] * cy[3];
  // n21 = (i2, j1)
  w[8] = cx[1] * cy[0]; w[9] = cx[3] * cy[0]; w[10] = cx[1] * cy[2]; w[11] = cx[3] * cy[2];
  // n22 = (i2, j2)
  w[12] = cx[1] * cy[1]; w[13] = cx[3] * cy[1]; w[14] = cx[1] * cy[3]; w[15] = cx[3] * cy[3];
}
// Spline_Interp with the products precomputed: 16 FMA per variable.
__device__ __forceinline__ void spline_eval16(const double* __restrict__ spl, const SplW& W, const double* w, int nvar,
                                              double* f) {
  const double* nd[4] = {spl + (size_t)W.n11 * SPL_NODE, spl + (size_t)W.n12 * SPL_NODE,
                         spl + (size_t)W.n21 * SPL_NODE, spl + (size_t)W.n22 * SPL_NODE};
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    if (l >= nvar) break;
    double s = 0.;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double* p = nd[k];
      s += w[4 * k] * __ldg(p + l) + w[4 * k + 1] * __ldg(p + 3 + l) + w[4 * k + 2] * __ldg(p + 6 + l) +
           w[4 * k + 3] * __ldg(p + 9 + l);
    }
    f[l] = s;
  }
}

// ---------------------------------------------------------------------------
// Warp reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Compensated (Kahan) accumulation in FP32.  Uses round-to-nearest intrinsics
// so the compiler can neither contract nor reassociate the error terms.
struct Kahan3 {
  float s[3], c[3];
  __device__ __forceinline__ void zero() { for (int k = 0; k < 3; ++k) { s[k] = 0.f; c[k] = 0.f; } }
  __device__ __forceinline__ void add(int k, float x) {
    float y = __fsub_rn(x, c[k]);
    float t = __fadd_rn(s[k], y);
    c[k] = __fsub_rn(__fsub_rn(t, s[k]), y);
    s[k] = t;
  }
};

// B-spline weights (BsplineFunc, ModBasicMath.F90:392-417).  w[0..P-1] maps
// to mesh indices imin..imin+P-1.
template <typename R>
__device__ __forceinline__ void bspline_w(R xc, int P, int& imin, R* w) {
  R u[8];
  imin = (int)floor(xc) - (P - 1);
  u[0] = (R)imin - (xc - (R)P);
#pragma unroll
  for (int j = 1; j < 8; ++j) u[j] = u[j - 1] + (R)1;
  w[0] = (R)1;
#pragma unroll
  for (int j = 1; j < 8; ++j) w[j] = (R)0;
  for (int pp = 2; pp <= P; ++pp) {
    R inv = (R)1 / (R)(pp - 1);
    for (int j = pp; j >= 2; --j) w[j - 1] = u[j - 1] * inv * w[j - 1] + ((R)pp - u[j - 1]) * inv * w[j - 2];
    w[0] = u[0] * inv * w[0];
  }
}


__host__ __device__ __forceinline__ double tri_dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
// MinDistToTri, ModIntOnWalls.F90:480-577.  xv[l][c]: vertex l component c.
__host__ __device__ inline double min_dist_to_tri(const double* xt, const double xv[3][3], double& s0, double& t0) {
  double x12[3], x13[3], x1T[3];
  for (int c = 0; c < 3; ++c) { x12[c] = xv[1][c] - xv[0][c]; x13[c] = xv[2][c] - xv[0][c]; x1T[c] = xv[0][c] - xt[c]; }
  double a = tri_dot3(x12, x12), b = tri_dot3(x12, x13), c = tri_dot3(x13, x13);
  double det = a * c - b * b, invDet = 1. / det;
  double d = tri_dot3(x12, x1T), e = tri_dot3(x13, x1T), f = tri_dot3(x1T, x1T);
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
    case 1: s = (c + e - b - d) / (a - 2 * b + c); s = fmin(1., fmax(0., s)); t = 1. - s; break;
    case 3: s = 0.; t = -e / c; t = fmin(1., fmax(0., t)); break;
    case 5: t = 0.; s = -d / a; s = fmin(1., fmax(0., s)); break;
  }
  s0 = s; t0 = t;
  return sqrt(a * s * s + 2 * b * s * t + c * t * t + 2 * d * s + 2 * e * t + f);
}


#define RBC3D_STR2(x) #x
#define RBC3D_STR(x) RBC3D_STR2(x)
#define CUDA_TRY(x)                                                                                  \
  do {                                                                                               \
    cudaError_t e__ = (x);                                                                           \
    if (e__ != cudaSuccess) return ctx_fail_cuda(ctx, e__, #x " (" __FILE__ ":" RBC3D_STR(__LINE__) ")"); \
  } while (0)
