// membrane.cu -- membrane mechanics of the red cells on the device, FP64:
// RBC_ComputeGeometry (ModRbc.F90:404-509), RBC_CovarGrad_Vec /
// RBC_CovarGrad_Tensor (:527-658), Shell_ResForce (:815-899), Shell_ElasStrs
// (:906-942, Skalak law) and Shell_Bend (:949-963); the intra-cell
// repulsion of AddIntraCellRepulsionForce (ModRepulsion.F90:126-266).
//
// Surface derivatives are ShAnalGau + ShGradGau (ModSphpk.F90:74-105,
// 377-417): Spherepack's Gauss-grid analysis to degree < nlat and gradgs with
// the sin(theta) factor restored, i.e. d/dtheta and d/dphi of the truncated
// expansion
//   g = 1/2 sum_n a(0,n) pbar(0,n) + sum_{m>=1} sum_n pbar(m,n) (a cos m phi - b sin m phi),
// with d pbar(m,n)/d theta from (1 - x^2) dP_n^m/dx = (n + m) P_{n-1}^m - n x P_n^m.
// One CTA per (cell, field) does the longitude sums, the Legendre sums and
// both derivative syntheses through shared memory; everything else is one
// thread per grid point.  Per-cell fields are stored field-major,
// F[(cell * K + k) * nv + r], r = ilat + nlat * ilon; 2x2 tensors as K = 4
// fields ij = 2 (i-1) + (j-1); derivatives of tensors as K = 8 fields
// ((2 (i-1) + (j-1)) * 2 + (k-1)).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.hpp"

namespace {

inline int mb_nblk(long long n, int b) { return (int)((n + b - 1) / b); }

struct MbArgs {
  int L, nlat, nlon, nv;
  const double* P;   // pbar at the Gauss rows [i][m][n]
  const double* DP;  // d pbar / d theta
  const double* wf;  // analysis weight of Gauss row i: wG_i * 2 / nlon
  const double* cs;  // cos(m phi_j) [m][j]
  const double* sn;
};

// ShAnalGau + ShGradGau of nf fields: F -> Vt = dF/dtheta, Vp = dF/dphi
__global__ void k_mb_grad(MbArgs a, const double* __restrict__ F, double* __restrict__ Vt, double* __restrict__ Vp) {
  extern __shared__ double sm[];
  const int L = a.L, nlat = a.nlat, nlon = a.nlon, nv = a.nv;
  double* g = sm;              // nv
  double* C = g + nv;          // [m][i]
  double* S = C + L * nlat;
  double* A = S + L * nlat;    // [m][n]
  double* B = A + L * L;
  double* G = B + L * L;       // [i][m]
  double* H = G + nlat * L;
  double* Gt = H + nlat * L;
  double* Ht = Gt + nlat * L;
  const size_t base = (size_t)blockIdx.x * nv;
  for (int r = threadIdx.x; r < nv; r += blockDim.x) g[r] = F[base + r];
  __syncthreads();
  for (int t = threadIdx.x; t < L * nlat; t += blockDim.x) {
    const int m = t / nlat, i = t % nlat;
    double c = 0, s = 0;
    for (int j = 0; j < nlon; ++j) {
      const double x = g[i + nlat * j];
      c += x * a.cs[m * nlon + j];
      s += x * a.sn[m * nlon + j];
    }
    C[t] = c;
    S[t] = s;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < L * L; t += blockDim.x) {
    const int m = t / L, n = t % L;
    double sa = 0, sb = 0;
    if (n >= m)
      for (int i = 0; i < nlat; ++i) {
        const double p = a.P[((size_t)i * L + m) * L + n] * a.wf[i];
        sa += p * C[m * nlat + i];
        sb -= p * S[m * nlat + i];
      }
    A[t] = sa;
    B[t] = sb;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nlat * L; t += blockDim.x) {
    const int i = t / L, m = t % L;
    double gs = 0, hs = 0, gt = 0, ht = 0;
    for (int n = m; n < L; ++n) {
      const size_t q = ((size_t)i * L + m) * L + n;
      const double p = a.P[q], dp = a.DP[q];
      gs += p * A[m * L + n]; hs += p * B[m * L + n];
      gt += dp * A[m * L + n]; ht += dp * B[m * L + n];
    }
    G[t] = gs; H[t] = hs; Gt[t] = gt; Ht[t] = ht;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nv; r += blockDim.x) {
    const int i = r % nlat, j = r / nlat;
    double st = 0.5 * Gt[i * L], sp = 0;
    for (int m = 1; m < L; ++m) {
      const double cm = a.cs[m * nlon + j], smv = a.sn[m * nlon + j];
      st += Gt[i * L + m] * cm - Ht[i * L + m] * smv;
      sp -= m * (G[i * L + m] * smv + H[i * L + m] * cm);
    }
    Vt[base + r] = st;
    Vp[base + r] = sp;
  }
}

// SoA point layout (3 x n) -> per-cell fields [cell][3][nv]
__global__ void k_mb_gather(int ncell, int nv, const double* __restrict__ x, double* __restrict__ X) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x, n = (long long)ncell * nv;
  if (t >= n) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  for (int k = 0; k < 3; ++k) X[((size_t)cell * 3 + k) * nv + r] = x[t + k * n];
}

__device__ __forceinline__ double fld(const double* F, int K, int cell, int k, int nv, int r) {
  return F[((size_t)cell * K + k) * nv + r];
}
__device__ __forceinline__ double& fldw(double* F, int K, int cell, int k, int nv, int r) {
  return F[((size_t)cell * K + k) * nv + r];
}

// metric, its inverse, reciprocal base vectors, unit normal, detJ (RBC_ComputeGeometry :425-454)
__global__ void k_mb_geom(int ncell, int nv, int nlat, const double* __restrict__ sinth, const double* __restrict__ A1,
                          const double* __restrict__ A2, double* __restrict__ Ga, double* __restrict__ Gar,
                          double* __restrict__ A1r, double* __restrict__ A2r, double* __restrict__ A3,
                          double* __restrict__ detJ) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  double a1[3], a2[3];
  for (int k = 0; k < 3; ++k) { a1[k] = fld(A1, 3, cell, k, nv, r); a2[k] = fld(A2, 3, cell, k, nv, r); }
  const double a11 = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
  const double a12 = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
  const double a22 = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
  const double detA = a11 * a22 - a12 * a12, idet = 1. / detA;
  const double r11 = idet * a22, r12 = -idet * a12, r22 = idet * a11;
  fldw(Ga, 4, cell, 0, nv, r) = a11; fldw(Ga, 4, cell, 1, nv, r) = a12;
  fldw(Ga, 4, cell, 2, nv, r) = a12; fldw(Ga, 4, cell, 3, nv, r) = a22;
  fldw(Gar, 4, cell, 0, nv, r) = r11; fldw(Gar, 4, cell, 1, nv, r) = r12;
  fldw(Gar, 4, cell, 2, nv, r) = r12; fldw(Gar, 4, cell, 3, nv, r) = r22;
  double n[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
  const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int k = 0; k < 3; ++k) {
    fldw(A1r, 3, cell, k, nv, r) = r11 * a1[k] + r12 * a2[k];
    fldw(A2r, 3, cell, k, nv, r) = r12 * a1[k] + r22 * a2[k];
    fldw(A3, 3, cell, k, nv, r) = n[k] / nn;
  }
  detJ[t] = sqrt(detA) / sinth[r % nlat];
}

// curvature tensor b_ij = -(a_i . d a3 / d theta_j) (:457-474)
__global__ void k_mb_curv(int ncell, int nv, const double* __restrict__ A1, const double* __restrict__ A2,
                          const double* __restrict__ A31, const double* __restrict__ A32, double* __restrict__ Gb) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  double b11 = 0, b12 = 0, b21 = 0, b22 = 0;
  for (int k = 0; k < 3; ++k) {
    const double a1 = fld(A1, 3, cell, k, nv, r), a2 = fld(A2, 3, cell, k, nv, r);
    const double d1 = fld(A31, 3, cell, k, nv, r), d2 = fld(A32, 3, cell, k, nv, r);
    b11 -= a1 * d1; b12 -= a1 * d2; b21 -= a2 * d1; b22 -= a2 * d2;
  }
  fldw(Gb, 4, cell, 0, nv, r) = b11; fldw(Gb, 4, cell, 1, nv, r) = b12;
  fldw(Gb, 4, cell, 2, nv, r) = b21; fldw(Gb, 4, cell, 3, nv, r) = b22;
}

__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double s = 0;
  for (int k = 0; k < nw; ++k) s += red[k];
  return s;
}

// The part of RBC_ComputeGeometry the surface sources need, on the point
// layout [comp][cell][r]: unit normal a3 = a1 x a2 / |a1 x a2| and detJ =
// sqrt(det a_ij) / sin(theta) (:425-454, as k_mb_geom) from the tangents
// a1 = dx/dtheta, a2 = dx/dphi.
__global__ void k_geom_point(long long n, int nv, int nlat, const double* __restrict__ sinth,
                             const double* __restrict__ A1, const double* __restrict__ A2, double* __restrict__ a3,
                             double* __restrict__ detJ) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int r = (int)(t % nv);
  double a1[3], a2[3];
  for (int k = 0; k < 3; ++k) { a1[k] = A1[t + k * n]; a2[k] = A2[t + k * n]; }
  const double a11 = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
  const double a12 = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
  const double a22 = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
  const double detA = a11 * a22 - a12 * a12;
  double nrm[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
  const double nn = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  for (int k = 0; k < 3; ++k) a3[t + k * n] = nrm[k] / nn;
  detJ[t] = sqrt(detA) / sinth[r % nlat];
}

// area of each cell (:476-480), the reduction of k_mb_sums; one CTA per cell
__global__ void k_cell_area(int nv, int nlat, const double* __restrict__ w, const double* __restrict__ detJ,
                            double* __restrict__ area) {
  __shared__ double red[32];
  const int cell = blockIdx.x;
  double s = 0;
  for (int r = threadIdx.x; r < nv; r += blockDim.x) s += detJ[(size_t)cell * nv + r] * w[r % nlat];
  const double A = block_sum(s, red);
  if (threadIdx.x == 0) area[cell] = A;
}

// area, centroid and volume of each cell (:476-501); one CTA per cell
__global__ void k_mb_sums(int nv, int nlat, const double* __restrict__ w, const double* __restrict__ X,
                          const double* __restrict__ A3, const double* __restrict__ detJ, double* __restrict__ area,
                          double* __restrict__ vol) {
  __shared__ double red[32];
  const int cell = blockIdx.x;
  double s = 0, sx[3] = {0, 0, 0};
  for (int r = threadIdx.x; r < nv; r += blockDim.x) {
    const double ds = detJ[(size_t)cell * nv + r] * w[r % nlat];
    s += ds;
    for (int k = 0; k < 3; ++k) sx[k] += ds * fld(X, 3, cell, k, nv, r);
  }
  const double A = block_sum(s, red);
  double xc[3];
  for (int k = 0; k < 3; ++k) xc[k] = block_sum(sx[k], red) / A;
  double v = 0;
  for (int r = threadIdx.x; r < nv; r += blockDim.x) {
    const double ds = detJ[(size_t)cell * nv + r] * w[r % nlat];
    double d = 0;
    for (int k = 0; k < 3; ++k) d += fld(A3, 3, cell, k, nv, r) * (fld(X, 3, cell, k, nv, r) - xc[k]);
    v += ds * d;
  }
  const double V = block_sum(v, red);
  if (threadIdx.x == 0) {
    area[cell] = A;
    vol[cell] = V / 3.0;
  }
}

__device__ __forceinline__ void mm2(const double* A, const double* B, double* C) {
  C[0] = A[0] * B[0] + A[1] * B[2]; C[1] = A[0] * B[1] + A[1] * B[3];
  C[2] = A[2] * B[0] + A[3] * B[2]; C[3] = A[2] * B[1] + A[3] * B[3];
}

// Shell_ElasStrs (Skalak) and Shell_Bend per point: tau, bnd contravariant
__global__ void k_mb_stress(int ncell, int nv, const int* __restrict__ ctype, const double* __restrict__ mod,
                            const double* __restrict__ Ga, const double* __restrict__ Gar, const double* __restrict__ Gb,
                            const double* __restrict__ ref_ar, const double* __restrict__ ref_b,
                            double* __restrict__ tau, double* __restrict__ bnd) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv), ty = ctype[cell];
  const double ES = mod[3 * ty], ED = mod[3 * ty + 1], EB = mod[3 * ty + 2];
  double a[4], ar[4], arr[4], b[4], brf[4], V2[4];
  for (int q = 0; q < 4; ++q) {
    a[q] = fld(Ga, 4, cell, q, nv, r); ar[q] = fld(Gar, 4, cell, q, nv, r); b[q] = fld(Gb, 4, cell, q, nv, r);
    arr[q] = ref_ar[((size_t)ty * 4 + q) * nv + r]; brf[q] = ref_b[((size_t)ty * 4 + q) * nv + r];
  }
  mm2(a, arr, V2);
  const double lbd1 = V2[0] + V2[3] - 2.0;
  const double lbd2 = V2[0] * V2[3] - V2[1] * V2[2] - 1.0;
  const double JS = sqrt(V2[0] * V2[3] - V2[1] * V2[2]);
  for (int q = 0; q < 4; ++q) fldw(tau, 4, cell, q, nv, r) = 0.5 * ES / JS * (lbd1 + 1.0) * arr[q] + 0.5 * JS * (ED * lbd2 - ES) * ar[q];
  double bm[4], bmr[4], d[4], o[4];
  mm2(ar, b, bm);
  mm2(arr, brf, bmr);
  for (int q = 0; q < 4; ++q) d[q] = bm[q] - bmr[q];
  mm2(d, ar, o);
  for (int q = 0; q < 4; ++q) fldw(bnd, 4, cell, q, nv, r) = -EB * o[q];
}

// RBC_CovarGrad_Tensor, first half: tc_ij = t^{11} a1_i a1_j + t^{12} a1_i a2_j + t^{21} a2_i a1_j + t^{22} a2_i a2_j
__global__ void k_mb_tcart(int ncell, int nv, const double* __restrict__ T, const double* __restrict__ A1,
                           const double* __restrict__ A2, double* __restrict__ TC) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  double a1[3], a2[3], tt[4];
  for (int k = 0; k < 3; ++k) { a1[k] = fld(A1, 3, cell, k, nv, r); a2[k] = fld(A2, 3, cell, k, nv, r); }
  for (int q = 0; q < 4; ++q) tt[q] = fld(T, 4, cell, q, nv, r);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      fldw(TC, 9, cell, 3 * i + j, nv, r) = tt[0] * a1[i] * a1[j] + tt[1] * a1[i] * a2[j] + tt[2] * a2[i] * a1[j] + tt[3] * a2[i] * a2[j];
}

// second half: dt(al, be, kd) = a_al^rcp . (d tc / d theta_kd) a_be^rcp
__global__ void k_mb_tproj(int ncell, int nv, const double* __restrict__ TC1, const double* __restrict__ TC2,
                           const double* __restrict__ A1r, const double* __restrict__ A2r, double* __restrict__ DT) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  double u[2][3];
  for (int k = 0; k < 3; ++k) { u[0][k] = fld(A1r, 3, cell, k, nv, r); u[1][k] = fld(A2r, 3, cell, k, nv, r); }
  for (int kd = 0; kd < 2; ++kd) {
    const double* td = kd == 0 ? TC1 : TC2;
    double m[9];
    for (int q = 0; q < 9; ++q) m[q] = fld(td, 9, cell, q, nv, r);
    for (int al = 0; al < 2; ++al)
      for (int be = 0; be < 2; ++be) {
        double s = 0;
        for (int i = 0; i < 3; ++i) {
          double mv = 0;
          for (int j = 0; j < 3; ++j) mv += m[3 * i + j] * u[be][j];
          s += u[al][i] * mv;
        }
        fldw(DT, 8, cell, (2 * al + be) * 2 + kd, nv, r) = s;
      }
  }
}

// tau_n (Shell_ResForce :842-848) and its Cartesian form for RBC_CovarGrad_Vec
__global__ void k_mb_taun(int ncell, int nv, const double* __restrict__ DB, const double* __restrict__ A1,
                          const double* __restrict__ A2, double* __restrict__ TN, double* __restrict__ VC) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  // dbnd(i, j, k): field (2i + j) * 2 + k
  const double n1 = fld(DB, 8, cell, 0, nv, r) + fld(DB, 8, cell, 5, nv, r);  // (1,1,1) + (2,1,2)
  const double n2 = fld(DB, 8, cell, 2, nv, r) + fld(DB, 8, cell, 7, nv, r);  // (1,2,1) + (2,2,2)
  fldw(TN, 2, cell, 0, nv, r) = n1;
  fldw(TN, 2, cell, 1, nv, r) = n2;
  for (int k = 0; k < 3; ++k) fldw(VC, 3, cell, k, nv, r) = n1 * fld(A1, 3, cell, k, nv, r) + n2 * fld(A2, 3, cell, k, nv, r);
}

// tangential residual force (:851-864) and the normal one (:867-876)
__global__ void k_mb_force(int ncell, int nv, const double* __restrict__ DTAU, const double* __restrict__ TN,
                           const double* __restrict__ Gar, const double* __restrict__ Gb, const double* __restrict__ tau,
                           const double* __restrict__ V1, const double* __restrict__ V2, const double* __restrict__ A1r,
                           const double* __restrict__ A2r, double* __restrict__ FL) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nv) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  double f1 = -fld(DTAU, 8, cell, 0, nv, r) - fld(DTAU, 8, cell, 5, nv, r);
  double f2 = -fld(DTAU, 8, cell, 2, nv, r) - fld(DTAU, 8, cell, 7, nv, r);
  double b[4], ar[4];
  for (int q = 0; q < 4; ++q) { b[q] = fld(Gb, 4, cell, q, nv, r); ar[q] = fld(Gar, 4, cell, q, nv, r); }
  const double n1 = fld(TN, 2, cell, 0, nv, r), n2 = fld(TN, 2, cell, 1, nv, r);
  const double bt1 = b[0] * n1 + b[1] * n2, bt2 = b[2] * n1 + b[3] * n2;
  f1 += ar[0] * bt1 + ar[1] * bt2;
  f2 += ar[2] * bt1 + ar[3] * bt2;
  // RBC_CovarGrad_Vec projection: dv(1,1) = a1^rcp . v_1, dv(2,2) = a2^rcp . v_2
  double dv11 = 0, dv22 = 0;
  for (int k = 0; k < 3; ++k) {
    dv11 += fld(A1r, 3, cell, k, nv, r) * fld(V1, 3, cell, k, nv, r);
    dv22 += fld(A2r, 3, cell, k, nv, r) * fld(V2, 3, cell, k, nv, r);
  }
  double tb = 0;
  for (int q = 0; q < 4; ++q) tb += fld(tau, 4, cell, q, nv, r) * b[q];
  fldw(FL, 3, cell, 0, nv, r) = f1;
  fldw(FL, 3, cell, 1, nv, r) = f2;
  fldw(FL, 3, cell, 2, nv, r) = -dv11 - dv22 - tb;
}

// average normal force removed (:879-885), Cartesian force to the SoA point layout (:888-894)
__global__ void k_mb_final(int nv, int nlat, long long n, const double* __restrict__ w, const double* __restrict__ FL,
                           const double* __restrict__ detJ, const double* __restrict__ area, const double* __restrict__ A1,
                           const double* __restrict__ A2, const double* __restrict__ A3, double* __restrict__ f) {
  __shared__ double red[32];
  const int cell = blockIdx.x;
  double s = 0;
  for (int r = threadIdx.x; r < nv; r += blockDim.x) s += fld(FL, 3, cell, 2, nv, r) * detJ[(size_t)cell * nv + r] * w[r % nlat];
  const double fn = block_sum(s, red) / area[cell];
  for (int r = threadIdx.x; r < nv; r += blockDim.x) {
    const double f1 = fld(FL, 3, cell, 0, nv, r), f2 = fld(FL, 3, cell, 1, nv, r), f3 = fld(FL, 3, cell, 2, nv, r) - fn;
    for (int k = 0; k < 3; ++k)
      f[(size_t)cell * nv + r + k * n] = f1 * fld(A1, 3, cell, k, nv, r) + f2 * fld(A2, 3, cell, k, nv, r) +
                                         f3 * fld(A3, 3, cell, k, nv, r);
  }
}

// per-cell fields -> SoA point layout (3 x n)
__global__ void k_mb_scatter(int ncell, int nv, const double* __restrict__ X, double* __restrict__ x) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x, n = (long long)ncell * nv;
  if (t >= n) return;
  const int cell = (int)(t / nv), r = (int)(t % nv);
  for (int k = 0; k < 3; ++k) x[t + k * n] = X[((size_t)cell * 3 + k) * nv + r];
}

// AddIntraCellRepulsionForce per point: the nearest admissible point of the
// same cell (excl: grid pairs closer than the patch radius on the reference
// sphere, DistOnSphere tabulated per (ri, rj))
__global__ void k_mb_repulsion(int ncell, int nv, int nlat, long long n, const double* __restrict__ x,
                               const double* __restrict__ a3, const double* __restrict__ area,
                               const unsigned char* __restrict__ excl, double force_coef, double* __restrict__ f,
                               unsigned long long* __restrict__ cnt) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int cell = (int)(p / nv), ri = (int)(p % nv);
  const double epsDist = 2.0 * sqrt(area[cell]) / nlat, eps2 = epsDist * epsDist;
  const double xi0 = x[p], xi1 = x[p + n], xi2 = x[p + 2 * n];
  const size_t b = (size_t)cell * nv;
  const unsigned char* row = excl + (size_t)ri * nv;
  double dist = 1e300;
  for (int rj = 0; rj < nv; ++rj) {
    if (row[rj]) continue;
    const size_t q = b + rj;
    const double d0 = xi0 - x[q], d1 = xi1 - x[q + n], d2 = xi2 - x[q + 2 * n];
    const double rr2 = d0 * d0 + d1 * d1 + d2 * d2;
    if (rr2 > eps2) continue;  // rr > epsDist
    const double rr = sqrt(rr2);
    const double xxn = -(d0 * a3[q] + d1 * a3[q + n] + d2 * a3[q + 2 * n]);
    if (xxn / rr < 0.707) continue;
    dist = fmin(dist, rr);
  }
  if (dist < epsDist) {
    const double FF = force_coef * exp(1.0 - dist / epsDist);
    for (int k = 0; k < 3; ++k) f[p + k * n] += FF * a3[p + k * n];
    atomicAdd(cnt, 1ull);
  }
}

// d pbar(m, n, theta) / d theta from P (sin(theta) > 0 on the Gauss rows)
void dpbar_table(int L, double theta, const double* P, double* dP) {
  const double x = std::cos(theta), s = std::sin(theta);
  for (int i = 0; i < L * L; ++i) dP[i] = 0.;
  for (int m = 0; m < L; ++m)
    for (int n = m; n < L; ++n) {
      const double q = n > m ? std::sqrt((2.0 * n + 1.0) * (n + m) * (n - m) / (2.0 * n - 1.0)) * P[m * L + n - 1] : 0.0;
      dP[m * L + n] = (n * x * P[m * L + n] - q) / s;
    }
}

size_t grad_smem(int L, int nlat, int nv) { return sizeof(double) * (size_t)(nv + 2 * L * nlat + 2 * L * L + 4 * nlat * L); }

rbc3d_status mb_tables(rbc3d_ctx* ctx) {
  auto& M = ctx->mb;
  const int nlat = ctx->nlat, nlon = ctx->nlon, L = nlat;
  if (M.L == L && M.P.p) return RBC3D_OK;
  std::vector<double> P((size_t)nlat * L * L), DP((size_t)nlat * L * L), wf(nlat), cs((size_t)L * nlon),
      sn((size_t)L * nlon), st(nlat);
  for (int i = 0; i < nlat; ++i) {
    pbar_table(L, ctx->h_th[i], &P[(size_t)i * L * L]);
    dpbar_table(L, ctx->h_th[i], &P[(size_t)i * L * L], &DP[(size_t)i * L * L]);
    wf[i] = ctx->h_w[i] / RBC3D_PI;  // Gauss weight x 2 / nlon (w = Gauss weight x 2 pi / nlon)
    st[i] = std::sin(ctx->h_th[i]);
  }
  for (int m = 0; m < L; ++m)
    for (int j = 0; j < nlon; ++j) {
      cs[(size_t)m * nlon + j] = std::cos(m * ctx->h_phi[j]);
      sn[(size_t)m * nlon + j] = std::sin(m * ctx->h_phi[j]);
    }
  CUDA_TRY(M.P.upload(P.data(), P.size(), ctx->st)); CUDA_TRY(M.DP.upload(DP.data(), DP.size(), ctx->st));
  CUDA_TRY(M.wf.upload(wf.data(), wf.size(), ctx->st)); CUDA_TRY(M.cs.upload(cs.data(), cs.size(), ctx->st));
  CUDA_TRY(M.sn.upload(sn.data(), sn.size(), ctx->st)); CUDA_TRY(M.sinth.upload(st.data(), st.size(), ctx->st));
  const size_t sm = grad_smem(L, nlat, nlat * nlon);
  if (sm > 48 * 1024) CUDA_TRY(cudaFuncSetAttribute(k_mb_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  M.L = L;
  return RBC3D_OK;
}

MbArgs mb_args(const rbc3d_ctx* ctx) {
  const auto& M = ctx->mb;
  return MbArgs{M.L, ctx->nlat, ctx->nlon, ctx->nlat * ctx->nlon, M.P.p, M.DP.p, M.wf.p, M.cs.p, M.sn.p};
}

void grad(rbc3d_ctx* ctx, int nf, const double* F, double* Vt, double* Vp) {
  const MbArgs a = mb_args(ctx);
  k_mb_grad<<<nf, 256, grad_smem(a.L, a.nlat, a.nv), ctx->st>>>(a, F, Vt, Vp);
  ++ctx->launches;
}

// device geometry of ncell cells (per-cell field layout)
struct Geom {
  DBuf<double> X, A1, A2, Ga, Gar, A1r, A2r, A3, detJ, Gb, area, vol;
};

rbc3d_status mb_geometry_dev(rbc3d_ctx* ctx, int ncell, const double* x_dev, Geom& G);

rbc3d_status mb_geometry(rbc3d_ctx* ctx, int ncell, const double* x_host, Geom& G) {
  DBuf<double> xs;
  CUDA_TRY(xs.upload(x_host, 3 * (size_t)ncell * ctx->nlat * ctx->nlon, ctx->st));
  return mb_geometry_dev(ctx, ncell, xs.p, G);  // synchronises before xs is freed
}

rbc3d_status mb_geometry_dev(rbc3d_ctx* ctx, int ncell, const double* x_dev, Geom& G) {
  const int nv = ctx->nlat * ctx->nlon;
  const size_t n = (size_t)ncell * nv;
  DBuf<double> A31, A32;
  CUDA_TRY(G.X.alloc(3 * n)); CUDA_TRY(G.A1.alloc(3 * n)); CUDA_TRY(G.A2.alloc(3 * n));
  CUDA_TRY(G.Ga.alloc(4 * n)); CUDA_TRY(G.Gar.alloc(4 * n)); CUDA_TRY(G.A1r.alloc(3 * n)); CUDA_TRY(G.A2r.alloc(3 * n));
  CUDA_TRY(G.A3.alloc(3 * n)); CUDA_TRY(G.detJ.alloc(n)); CUDA_TRY(G.Gb.alloc(4 * n));
  CUDA_TRY(G.area.alloc(ncell)); CUDA_TRY(G.vol.alloc(ncell));
  CUDA_TRY(A31.alloc(3 * n)); CUDA_TRY(A32.alloc(3 * n));
  const int nb = mb_nblk((long long)n, 256);
  { k_mb_gather<<<nb, 256, 0, ctx->st>>>(ncell, nv, x_dev, G.X.p); ++ctx->launches; }
  grad(ctx, 3 * ncell, G.X.p, G.A1.p, G.A2.p);
  { k_mb_geom<<<nb, 256, 0, ctx->st>>>(ncell, nv, ctx->nlat, ctx->mb.sinth.p, G.A1.p, G.A2.p, G.Ga.p, G.Gar.p, G.A1r.p,
                                        G.A2r.p, G.A3.p, G.detJ.p); ++ctx->launches; }
  grad(ctx, 3 * ncell, G.A3.p, A31.p, A32.p);
  { k_mb_curv<<<nb, 256, 0, ctx->st>>>(ncell, nv, G.A1.p, G.A2.p, A31.p, A32.p, G.Gb.p); ++ctx->launches; }
  { k_mb_sums<<<ncell, 256, 0, ctx->st>>>(nv, ctx->nlat, ctx->w.p, G.X.p, G.A3.p, G.detJ.p, G.area.p, G.vol.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));  // A31, A32 (and the caller's staging) are freed on return
  return RBC3D_OK;
}

}  // namespace

rbc3d_status cells_geometry_dev(rbc3d_ctx* ctx) {
  rbc3d_status s;
  if ((s = mb_tables(ctx))) return s;
  const int nv = ctx->nlat * ctx->nlon;
  const size_t n = (size_t)ctx->ncell * nv;
  // the point layout [comp][cell][r] is 3 ncell fields of nv points: ShGradGau
  // of each, no reordering, into tangent buffers kept across calls
  CUDA_TRY(ctx->tan1.alloc(3 * n)); CUDA_TRY(ctx->tan2.alloc(3 * n));
  grad(ctx, 3 * ctx->ncell, ctx->x.p, ctx->tan1.p, ctx->tan2.p);
  { k_geom_point<<<mb_nblk((long long)n, 256), 256, 0, ctx->st>>>((long long)n, nv, ctx->nlat, ctx->mb.sinth.p,
                                                                   ctx->tan1.p, ctx->tan2.p, ctx->a3.p, ctx->detJ.p);
    ++ctx->launches; }
  { k_cell_area<<<ctx->ncell, 256, 0, ctx->st>>>(nv, ctx->nlat, ctx->w.p, ctx->detJ.p, ctx->area.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

extern "C" {

rbc3d_status rbc3d_set_ref_cells(rbc3d_ctx* ctx, int ntypes, const double* xref, const double* ES, const double* ED,
                                 const double* EB) {
  if (!ctx || ntypes < 1 || ntypes > RBC3D_MAX_CELLTYPES || !xref || !ES || !ED || !EB)
    return ctx_fail(ctx, RBC3D_ERR_ARG, "set_ref_cells: bad arguments");
  if (ctx->h_th.empty()) return ctx_fail(ctx, RBC3D_ERR_STATE, "cell grid not set");
  rbc3d_status s;
  if ((s = mb_tables(ctx))) return s;
  const int nv = ctx->nlat * ctx->nlon;
  Geom G;
  if ((s = mb_geometry(ctx, ntypes, xref, G))) return s;
  auto& M = ctx->mb;
  CUDA_TRY(M.ref_ar.alloc((size_t)ntypes * 4 * nv)); CUDA_TRY(M.ref_b.alloc((size_t)ntypes * 4 * nv));
  CUDA_TRY(cudaMemcpyAsync(M.ref_ar.p, G.Gar.p, sizeof(double) * ntypes * 4 * nv, cudaMemcpyDeviceToDevice, ctx->st));
  CUDA_TRY(cudaMemcpyAsync(M.ref_b.p, G.Gb.p, sizeof(double) * ntypes * 4 * nv, cudaMemcpyDeviceToDevice, ctx->st));
  M.ES.assign(ES, ES + ntypes); M.ED.assign(ED, ED + ntypes); M.EB.assign(EB, EB + ntypes);
  M.nref = ntypes;
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status rbc3d_cell_geometry(rbc3d_ctx* ctx, int ncell, const double* x, double* a3, double* detJ, double* area,
                                 double* vol) {
  if (!ctx || ncell < 0 || (ncell > 0 && !x)) return ctx_fail(ctx, RBC3D_ERR_ARG, "cell_geometry: bad arguments");
  if (ctx->h_th.empty()) return ctx_fail(ctx, RBC3D_ERR_STATE, "cell grid not set");
  if (ncell == 0) return RBC3D_OK;
  rbc3d_status s;
  if ((s = mb_tables(ctx))) return s;
  const int nv = ctx->nlat * ctx->nlon;
  const size_t n = (size_t)ncell * nv;
  Geom G;
  if ((s = mb_geometry(ctx, ncell, x, G))) return s;
  if (a3) {
    DBuf<double> o;
    CUDA_TRY(o.alloc(3 * n));
    { k_mb_scatter<<<mb_nblk((long long)n, 256), 256, 0, ctx->st>>>(ncell, nv, G.A3.p, o.p); ++ctx->launches; }
    CUDA_TRY(cudaMemcpyAsync(a3, o.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
  }
  if (detJ) CUDA_TRY(cudaMemcpyAsync(detJ, G.detJ.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st));
  if (area) CUDA_TRY(cudaMemcpyAsync(area, G.area.p, sizeof(double) * ncell, cudaMemcpyDeviceToHost, ctx->st));
  if (vol) CUDA_TRY(cudaMemcpyAsync(vol, G.vol.p, sizeof(double) * ncell, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status rbc3d_intra_cell_repulsion(rbc3d_ctx* ctx, int ncell, const double* x, const double* a3,
                                        const double* area, double force_coef, double* f, int* count) {
  if (!ctx || ncell < 0 || (ncell > 0 && (!x || !a3 || !area || !f)))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "intra_cell_repulsion: bad arguments");
  if (ctx->h_th.empty() || ctx->radius <= 0) return ctx_fail(ctx, RBC3D_ERR_STATE, "cell grid not set");
  if (count) *count = 0;
  if (ncell == 0) return RBC3D_OK;
  const int nlat = ctx->nlat, nlon = ctx->nlon, nv = nlat * nlon;
  const size_t n = (size_t)ncell * nv;
  auto& M = ctx->mb;
  if (M.excl_nv != nv) {
    // DistOnSphere (ModPolarPatch.F90:249-257) of every grid pair < patch radius
    std::vector<unsigned char> ex((size_t)nv * nv);
    for (int ri = 0; ri < nv; ++ri)
      for (int rj = 0; rj < nv; ++rj) {
        const double t0 = ctx->h_th[ri % nlat], p0 = ctx->h_phi[ri / nlat];
        const double t1 = ctx->h_th[rj % nlat], p1 = ctx->h_phi[rj / nlat];
        double d = std::cos(t0 - t1) - std::sin(t0) * std::sin(t1) * (1. - std::cos(p0 - p1));
        d = std::acos(std::min(1.0, std::max(-1.0, d)));
        ex[(size_t)ri * nv + rj] = d < ctx->radius ? 1 : 0;
      }
    CUDA_TRY(M.excl.upload(ex.data(), ex.size(), ctx->st));
    M.excl_nv = nv;
  }
  DBuf<double> dx, da, dar, df;
  DBuf<unsigned long long> dc;
  CUDA_TRY(dx.upload(x, 3 * n, ctx->st)); CUDA_TRY(da.upload(a3, 3 * n, ctx->st));
  CUDA_TRY(dar.upload(area, ncell, ctx->st)); CUDA_TRY(df.upload(f, 3 * n, ctx->st));
  CUDA_TRY(dc.alloc(1)); CUDA_TRY(cudaMemsetAsync(dc.p, 0, sizeof(unsigned long long), ctx->st));
  { k_mb_repulsion<<<mb_nblk((long long)n, 128), 128, 0, ctx->st>>>(ncell, nv, nlat, (long long)n, dx.p, da.p, dar.p,
                                                                       M.excl.p, force_coef, df.p, dc.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  unsigned long long c = 0;
  CUDA_TRY(cudaMemcpyAsync(f, df.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaMemcpyAsync(&c, dc.p, sizeof(c), cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  if (count) *count = (int)c;
  return RBC3D_OK;
}

rbc3d_status rbc3d_shell_res_force(rbc3d_ctx* ctx, int ncell, const int* celltype, const double* x, double* f) {
  if (!ctx || ncell < 0 || (ncell > 0 && (!celltype || !x || !f)))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "shell_res_force: bad arguments");
  auto& M = ctx->mb;
  if (M.nref == 0) return ctx_fail(ctx, RBC3D_ERR_STATE, "reference cells not set");
  for (int c = 0; c < ncell; ++c)
    if (celltype[c] < 0 || celltype[c] >= M.nref) return ctx_fail(ctx, RBC3D_ERR_ARG, "shell_res_force: bad celltype");
  if (ncell == 0) return RBC3D_OK;
  rbc3d_status s;
  const int nv = ctx->nlat * ctx->nlon;
  const size_t n = (size_t)ncell * nv;
  Geom G;
  if ((s = mb_geometry(ctx, ncell, x, G))) return s;
  std::vector<double> mod(3 * (size_t)M.nref);
  for (int t = 0; t < M.nref; ++t) { mod[3 * t] = M.ES[t]; mod[3 * t + 1] = M.ED[t]; mod[3 * t + 2] = M.EB[t]; }
  DBuf<int> ct;
  DBuf<double> dmod, tau, bnd, TC, TC1, TC2, DB, DTAU, TN, VC, V1, V2, FL, out;
  CUDA_TRY(ct.upload(celltype, ncell, ctx->st)); CUDA_TRY(dmod.upload(mod.data(), mod.size(), ctx->st));
  CUDA_TRY(tau.alloc(4 * n)); CUDA_TRY(bnd.alloc(4 * n)); CUDA_TRY(TC.alloc(9 * n)); CUDA_TRY(TC1.alloc(9 * n));
  CUDA_TRY(TC2.alloc(9 * n)); CUDA_TRY(DB.alloc(8 * n)); CUDA_TRY(DTAU.alloc(8 * n)); CUDA_TRY(TN.alloc(2 * n));
  CUDA_TRY(VC.alloc(3 * n)); CUDA_TRY(V1.alloc(3 * n)); CUDA_TRY(V2.alloc(3 * n)); CUDA_TRY(FL.alloc(3 * n));
  CUDA_TRY(out.alloc(3 * n));
  const int nb = mb_nblk((long long)n, 256);
  { k_mb_stress<<<nb, 256, 0, ctx->st>>>(ncell, nv, ct.p, dmod.p, G.Ga.p, G.Gar.p, G.Gb.p, M.ref_ar.p, M.ref_b.p, tau.p,
                                          bnd.p); ++ctx->launches; }
  // RBC_CovarGrad_Tensor(bnd) -> tau_n
  { k_mb_tcart<<<nb, 256, 0, ctx->st>>>(ncell, nv, bnd.p, G.A1.p, G.A2.p, TC.p); ++ctx->launches; }
  grad(ctx, 9 * ncell, TC.p, TC1.p, TC2.p);
  { k_mb_tproj<<<nb, 256, 0, ctx->st>>>(ncell, nv, TC1.p, TC2.p, G.A1r.p, G.A2r.p, DB.p); ++ctx->launches; }
  { k_mb_taun<<<nb, 256, 0, ctx->st>>>(ncell, nv, DB.p, G.A1.p, G.A2.p, TN.p, VC.p); ++ctx->launches; }
  // RBC_CovarGrad_Tensor(tau_t)
  { k_mb_tcart<<<nb, 256, 0, ctx->st>>>(ncell, nv, tau.p, G.A1.p, G.A2.p, TC.p); ++ctx->launches; }
  grad(ctx, 9 * ncell, TC.p, TC1.p, TC2.p);
  { k_mb_tproj<<<nb, 256, 0, ctx->st>>>(ncell, nv, TC1.p, TC2.p, G.A1r.p, G.A2r.p, DTAU.p); ++ctx->launches; }
  // RBC_CovarGrad_Vec(tau_n)
  grad(ctx, 3 * ncell, VC.p, V1.p, V2.p);
  { k_mb_force<<<nb, 256, 0, ctx->st>>>(ncell, nv, DTAU.p, TN.p, G.Gar.p, G.Gb.p, tau.p, V1.p, V2.p, G.A1r.p, G.A2r.p,
                                         FL.p); ++ctx->launches; }
  { k_mb_final<<<ncell, 256, 0, ctx->st>>>(nv, ctx->nlat, (long long)n, ctx->w.p, FL.p, G.detJ.p, G.area.p, G.A1.p,
                                            G.A2.p, G.A3.p, out.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(f, out.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

}  // extern "C"
