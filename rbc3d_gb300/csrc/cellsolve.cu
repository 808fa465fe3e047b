// cellsolve.cu -- the cell velocity solve of Solve_RBC_Vel
// (ModVelSolver.F90:44-132) on the device, FP64 throughout (rtol 1e-11).
//
// Unknowns are the spherical-harmonic coefficients of the cell surface
// velocities in the layout of Glob_Sph_Trans (ModVelSolver.F90:641-719): per
// cell a(m, n) for m < nlat0, n >= m, then b(m, n) for 1 <= m < nlat0, three
// components each.  The transforms are Spherepack's shags / shsgs / shses
// restricted to degree < nlat0, from their documented definitions:
//   g(theta, phi) = 1/2 sum_n a(0,n) pbar(0,n) + sum_{m>=1} sum_n pbar(m,n)
//                   (a(m,n) cos(m phi) - b(m,n) sin(m phi))
//   a(m,n) = 2/nlon sum_i wG_i pbar(m,n,theta_i) sum_j g_ij cos(m phi_j),
//   b(m,n) = -2/nlon sum_i wG_i pbar(m,n,theta_i) sum_j g_ij sin(m phi_j),
// with pbar normalised to unit L2 norm on [-1, 1] (no Condon-Shortley phase)
// and wG the Gauss weights.  One CTA per (cell, component): the longitude
// sums for all m, then the Legendre sums, through shared memory.
//
// MyMatMult (ModVelSolver.F90:523-601): coefficients -> g on the Gauss grid
// -> Rbc_BuildSurfaceSource(gFlag) (ModRbc.F90:716-807: g detJ analysed,
// ShFilter to degree < nlat0, synthesised on the equiangular grid with both
// poles, Spline_Build_On_Sphere with FFT_Diff derivatives as 2 nlat x 2 nlat
// and nlon x nlon differentiation matrices) -> the double-layer matvec
// (c1 = 0, c2 = -1/(4 pi), real space + corrections + PME on the cells) + g
// -> coefficients.  Compute_Rhs (:455-515): the single-layer matvec with walls
// (c1 = 1/(4 pi)) + 2 vBkg / Acoef -> coefficients.  GMRES as NoSlipWall's
// (gmres.cuh), warm-started from the caller's solution vector.
#include <chrono>
#include <cmath>
#include <vector>

#include "ctx.hpp"
#include "gmres.cuh"

// Spherepack pbar(m, n, theta) for 0 <= m <= n < L, P[m*L + n]: the standard
// recurrences for orthonormal associated Legendre functions.
void pbar_table(int L, double theta, double* P) {
  const double x = std::cos(theta), sn = std::sin(theta);
  for (int i = 0; i < L * L; ++i) P[i] = 0.;
  double pmm = std::sqrt(0.5);
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

namespace {

inline int cs_nblk(long long n, int b) { return (int)((n + b - 1) / b); }

// FFT_Diff (ModFFT.F90:25-93) on a periodic axis of M points as a matrix:
// modes k < M/2 times i k (domain 2 pi), mode M/2 zeroed, so
// D[j][l] = -(2/M) sum_{k=1}^{M/2-1} k sin(2 pi k (j - l) / M).
std::vector<double> diff_matrix(int M) {
  std::vector<double> D((size_t)M * M, 0.);
  const int K = M / 2 - 1;
  for (int j = 0; j < M; ++j)
    for (int l = 0; l < M; ++l) {
      double s = 0;
      for (int k = 1; k <= K; ++k) s += k * std::sin(2.0 * RBC3D_PI * k * (double)(j - l) / M);
      D[(size_t)j * M + l] = -2.0 / M * s;
    }
  return D;
}

struct ShArgs {
  int L, nlat, nlon, nrow, ncell, npt;
  int nvar;           // components of the field (1 or 3); coefficient and staging layouts keep stride 3
  const double* P;    // [row][m][n]
  const double* wf;   // analysis weight per Gauss row: wG_i * 2 / nlon
  const double* cs;   // cos(m phi_j) [m][j]
  const double* sn;   // sin(m phi_j)
};

// index of a(m, n) / b(m, n) of component k in one cell's packed vector
__device__ __forceinline__ int pack_a(int L, int m, int n, int k) {
  // a: rows m' < m hold L - m' entries each
  return 3 * (m * L - (m * (m - 1)) / 2 + (n - m)) + k;
}
__device__ __forceinline__ int pack_b(int L, int m, int n, int k) {
  const int na = L * (L + 1) / 2;  // number of a(m, n)
  // b: m' from 1 to m-1 hold L - m' entries each
  return 3 * (na + (m - 1) * L - ((m - 1) * m) / 2 + (n - m)) + k;
}

// analysis: grid (point layout, comps stride npt) x optional per-point factor
// -> packed coefficients (cell stride 3 L^2); one CTA per (cell, comp)
__global__ void k_sh_anal(ShArgs a, const double* __restrict__ v, const double* __restrict__ fac,
                          double* __restrict__ cvec) {
  extern __shared__ double sm[];
  const int cell = blockIdx.x / a.nvar, comp = blockIdx.x % a.nvar;
  const int nlat = a.nlat, nlon = a.nlon, L = a.L, nv = nlat * nlon;
  double* g = sm;               // nv
  double* C = g + nv;           // [m][i]
  double* S = C + L * nlat;
  const size_t base = (size_t)cell * nv;
  for (int r = threadIdx.x; r < nv; r += blockDim.x)
    g[r] = v[base + r + (size_t)comp * a.npt] * (fac ? fac[base + r] : 1.0);
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
  double* out = cvec + (size_t)cell * 3 * L * L;
  for (int t = threadIdx.x; t < L * L; t += blockDim.x) {
    const int m = t / L, n = t % L;
    if (n < m) continue;
    double sa = 0, sb = 0;
    for (int i = 0; i < nlat; ++i) {
      const double p = a.P[((size_t)i * L + m) * L + n] * a.wf[i];
      sa += p * C[m * nlat + i];
      sb -= p * S[m * nlat + i];
    }
    out[pack_a(L, m, n, comp)] = sa;
    if (m > 0) out[pack_b(L, m, n, comp)] = sb;
  }
}

// synthesis on the rows of a.P: packed coefficients -> out[cell][comp] rows
// x nlon; point layout (Gauss rows) when equi == 0, else the equiangular
// staging layout f[((cell*3 + comp) * nlon + j) * nrow + i]
__global__ void k_sh_synth(ShArgs a, const double* __restrict__ cvec, double* __restrict__ out, int equi) {
  extern __shared__ double sm[];
  const int cell = blockIdx.x / a.nvar, comp = blockIdx.x % a.nvar;
  const int L = a.L, nrow = a.nrow, nlon = a.nlon;
  double* A = sm;           // [m][n]
  double* Bc = A + L * L;
  double* Gm = Bc + L * L;  // [m][i]
  double* Hm = Gm + L * nrow;
  const double* cc = cvec + (size_t)cell * 3 * L * L;
  for (int t = threadIdx.x; t < L * L; t += blockDim.x) {
    const int m = t / L, n = t % L;
    A[t] = n >= m ? cc[pack_a(L, m, n, comp)] : 0.;
    Bc[t] = (n >= m && m > 0) ? cc[pack_b(L, m, n, comp)] : 0.;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < L * nrow; t += blockDim.x) {
    const int m = t / nrow, i = t % nrow;
    double g = 0, h = 0;
    for (int n = m; n < L; ++n) {
      const double p = a.P[((size_t)i * L + m) * L + n];
      g += p * A[m * L + n];
      h += p * Bc[m * L + n];
    }
    Gm[t] = g;
    Hm[t] = h;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nrow * nlon; t += blockDim.x) {
    const int i = t % nrow, j = t / nrow;
    double s = 0.5 * Gm[i];
    for (int m = 1; m < L; ++m) s += Gm[m * nrow + i] * a.cs[m * nlon + j] - Hm[m * nrow + i] * a.sn[m * nlon + j];
    if (equi) out[((size_t)(cell * 3 + comp) * nlon + j) * nrow + i] = s;
    else out[(size_t)cell * nrow * nlon + i + (size_t)nrow * j + (size_t)comp * a.npt] = s;
  }
}

// Rbc_BuildSurfaceSource for one (cell, comp) in one pass (ModRbc.F90:716-807):
// ShAnalGau of v (times fac) on the Gauss rows, ShFilter to degree < L, then
// the node values of Spline_Build_On_Sphere (ModSpline.F90:121-143) on the
// doubled meridian grid (M = 2 nlat rows, N = nlon columns): u, its FFT_Diff
// along the meridian great circle (u_th), along the longitude (u_ph) and both
// (u_thph).  The filtered field restricted to a meridian great circle or to a
// latitude circle is a trigonometric polynomial of degree < L <= M/2, on
// which FFT_Diff is exact, so the derivatives are taken from the expansion
// itself: u_ph from m times the sine and cosine parts, u_th from dPE, the
// FFT_Diff of the pbar samples continued around the great circle (built on
// the host).  The two halves of the grid hold the same points: node (i >= nlat,
// j) is the point (M - i, j + N/2) with u_th and u_thph negated, and the
// columns j and j + N/2 of a row differ only in the sign of the odd-m terms,
// so the block evaluates the (nlat + 1) x N/2 column pairs once.  Needs an
// equispaced, even longitude grid (the FFT_Diff axis).
struct SplArgs {
  int L, nlat, nlon, npt, nvar, set;
  const double* PG;   // pbar at the Gauss rows [i][m][n]
  const double* PE;   // pbar at the equiangular rows i pi / nlat, i <= nlat
  const double* dPE;  // FFT_Diff of pbar along the meridian great circle, same rows
  const double* wf;   // analysis weight per Gauss row
  const double* cs;   // cos(m phi_j) [m][j]
  const double* sn;
};

__global__ void __launch_bounds__(256) k_sh_spline(SplArgs a, const double* __restrict__ v,
                                                   const double* __restrict__ fac, double* __restrict__ spl) {
  extern __shared__ double sm[];
  const int cell = blockIdx.x / a.nvar, comp = blockIdx.x % a.nvar;
  const int L = a.L, nlat = a.nlat, nlon = a.nlon, nv = nlat * nlon, R = nlat + 1, N2 = nlon / 2;
  double* A = sm;               // [m][n]
  double* B = A + L * L;
  double* Gt = B + L * L;       // [m][r], r <= nlat: G, H, G', H'
  double* Ht = Gt + L * R;
  double* Gd = Ht + L * R;
  double* Hd = Gd + L * R;
  double* g = Hd + L * R;       // [i + nlat j]
  double* C = g + nv;           // [m][i]
  double* S = C + L * nlat;
  const size_t base = (size_t)cell * nv;
  for (int r = threadIdx.x; r < nv; r += blockDim.x)
    g[r] = v[base + r + (size_t)comp * a.npt] * (fac ? fac[base + r] : 1.0);
  __syncthreads();
  // ShAnalGau, longitude part: columns j and j + N/2 paired (cos and sin of
  // m (phi + pi) are (-1)^m those of m phi)
  for (int t = threadIdx.x; t < L * nlat; t += blockDim.x) {
    const int m = t / nlat, i = t % nlat;
    const double sgn = (m & 1) ? -1.0 : 1.0;
    double c = 0, s = 0;
    for (int j = 0; j < N2; ++j) {
      const double x = g[i + nlat * j] + sgn * g[i + nlat * (j + N2)];
      c += x * a.cs[m * nlon + j];
      s += x * a.sn[m * nlon + j];
    }
    C[t] = c;
    S[t] = s;
  }
  __syncthreads();
  // Legendre part and ShFilter (n < L)
  for (int t = threadIdx.x; t < L * L; t += blockDim.x) {
    const int m = t / L, n = t % L;
    double sa = 0, sb = 0;
    if (n >= m)
      for (int i = 0; i < nlat; ++i) {
        const double p = a.PG[((size_t)i * L + m) * L + n] * a.wf[i];
        sa += p * C[m * nlat + i];
        sb -= p * S[m * nlat + i];
      }
    A[t] = sa;
    B[t] = m > 0 ? sb : 0.0;
  }
  __syncthreads();
  // G_m, H_m and their theta derivatives on the equiangular rows (the m = 0
  // term of the synthesis carries a factor 1/2)
  for (int t = threadIdx.x; t < L * R; t += blockDim.x) {
    const int m = t / R, r = t % R;
    double gs = 0, hs = 0, gd = 0, hd = 0;
    for (int n = m; n < L; ++n) {
      const size_t q = ((size_t)r * L + m) * L + n;
      const double p = a.PE[q], dp = a.dPE[q];
      gs += p * A[m * L + n]; hs += p * B[m * L + n];
      gd += dp * A[m * L + n]; hd += dp * B[m * L + n];
    }
    const double h = m == 0 ? 0.5 : 1.0;
    Gt[t] = h * gs; Ht[t] = h * hs; Gd[t] = h * gd; Hd[t] = h * hd;
  }
  __syncthreads();
  const int M = 2 * nlat;
  double* dst = spl + ((size_t)cell * SPL_NSET + a.set) * (size_t)M * nlon * SPL_NODE;
  for (int t = threadIdx.x; t < R * N2; t += blockDim.x) {
    const int r = t % R, j = t / R;
    double e[4] = {0, 0, 0, 0}, o[4] = {0, 0, 0, 0};  // u, u_th, u_ph, u_thph: even and odd m
    for (int m = 0; m < L; ++m) {
      const double c = a.cs[m * nlon + j], s = a.sn[m * nlon + j];
      const double gm = Gt[m * R + r], hm = Ht[m * R + r], gdm = Gd[m * R + r], hdm = Hd[m * R + r];
      const double w[4] = {gm * c - hm * s, gdm * c - hdm * s, -m * (gm * s + hm * c), -m * (gdm * s + hdm * c)};
      double* acc = (m & 1) ? o : e;
      for (int k = 0; k < 4; ++k) acc[k] += w[k];
    }
    double p1[4], p2[4];  // the points (r, j) and (r, j + N/2)
    for (int k = 0; k < 4; ++k) { p1[k] = e[k] + o[k]; p2[k] = e[k] - o[k]; }
    auto put = [&](int i, int jj, const double* val, double sg) {
      double* d = dst + ((size_t)jj * M + i) * SPL_NODE;
      d[0 * 3 + comp] = val[0];
      d[1 * 3 + comp] = sg * val[1];
      d[2 * 3 + comp] = val[2];
      d[3 * 3 + comp] = sg * val[3];
      if (a.nvar == 1)
        for (int kind = 0; kind < 4; ++kind) d[kind * 3 + 1] = d[kind * 3 + 2] = 0.0;
    };
    if (r < nlat) {
      put(r, j, p1, 1.0);
      put(r, j + N2, p2, 1.0);
    }
    if (r >= 1) {
      put(M - r, j + N2, p1, -1.0);
      put(M - r, j, p2, -1.0);
    }
  }
}

__global__ void k_add_vbkg(int n, const double* __restrict__ A, double b0, double b1, double b2, double* __restrict__ v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double iA = 2.0 / A[i];
  v[i] += b0 * iA;
  v[i + n] += b1 * iA;
  v[i + 2 * (size_t)n] += b2 * iA;
}

using CellSolveTabs = ShTabs;

rbc3d_status cell_tabs(rbc3d_ctx* ctx, int L, CellSolveTabs& T) {
  if (T.L == L && T.PG.p) return RBC3D_OK;  // tables of this grid and degree are current
  const int nlat = ctx->nlat, nlon = ctx->nlon;
  std::vector<double> th(nlat), phi(nlon), w(nlat);
  CUDA_TRY(cudaMemcpyAsync(th.data(), ctx->th.p, sizeof(double) * nlat, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaMemcpyAsync(phi.data(), ctx->phi.p, sizeof(double) * nlon, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaMemcpyAsync(w.data(), ctx->w.p, sizeof(double) * nlat, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  std::vector<double> PG((size_t)nlat * L * L), PE((size_t)(nlat + 1) * L * L), wf(nlat), cs((size_t)L * nlon),
      sn((size_t)L * nlon);
  for (int i = 0; i < nlat; ++i) pbar_table(L, th[i], &PG[(size_t)i * L * L]);
  for (int i = 0; i <= nlat; ++i) pbar_table(L, i * RBC3D_PI / nlat, &PE[(size_t)i * L * L]);
  // the grid's w is the Gauss weight x 2 pi / nlon (RBC_Create, ModRbc.F90:94)
  for (int i = 0; i < nlat; ++i) wf[i] = w[i] / RBC3D_PI;
  for (int m = 0; m < L; ++m)
    for (int j = 0; j < nlon; ++j) { cs[(size_t)m * nlon + j] = std::cos(m * phi[j]); sn[(size_t)m * nlon + j] = std::sin(m * phi[j]); }
  // dPE: FFT_Diff along the meridian great circle (M = 2 nlat points
  // theta_l = l pi / nlat, pbar continued past the pole by its own formula,
  // sin^m theta times a polynomial in cos theta) of pbar, at the rows l <= nlat
  const int M = 2 * nlat;
  std::vector<double> Dm = diff_matrix(M), Pext((size_t)M * L * L), dPE((size_t)(nlat + 1) * L * L, 0.0);
  for (int l = 0; l < M; ++l) pbar_table(L, l * RBC3D_PI / nlat, &Pext[(size_t)l * L * L]);
  for (int r = 0; r <= nlat; ++r)
    for (int l = 0; l < M; ++l) {
      const double d = Dm[(size_t)r * M + l];
      for (int q = 0; q < L * L; ++q) dPE[(size_t)r * L * L + q] += d * Pext[(size_t)l * L * L + q];
    }
  // the spline tables' derivatives assume FFT_Diff's axis: phi_j = phi_0 + 2 pi j / nlon, nlon even
  T.equi_lon = nlon % 2 == 0;
  for (int j = 0; j < nlon && T.equi_lon; ++j)
    T.equi_lon = std::fabs(phi[j] - phi[0] - 2.0 * RBC3D_PI * j / nlon) <= 1e-12;
  CUDA_TRY(T.PG.upload(PG.data(), PG.size(), ctx->st)); CUDA_TRY(T.PE.upload(PE.data(), PE.size(), ctx->st));
  CUDA_TRY(T.wf.upload(wf.data(), wf.size(), ctx->st));
  CUDA_TRY(T.cs.upload(cs.data(), cs.size(), ctx->st)); CUDA_TRY(T.sn.upload(sn.data(), sn.size(), ctx->st));
  CUDA_TRY(T.dPE.upload(dPE.data(), dPE.size(), ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  T.L = L;
  return RBC3D_OK;
}

ShArgs sh_args(const rbc3d_ctx* ctx, const CellSolveTabs& T, bool equi, int nvar = 3) {
  ShArgs a;
  a.L = T.L; a.nlat = ctx->nlat; a.nlon = ctx->nlon; a.ncell = ctx->ncell; a.npt = ctx->npt;
  a.nvar = nvar;
  a.nrow = equi ? ctx->nlat + 1 : ctx->nlat;
  a.P = equi ? T.PE.p : T.PG.p;
  a.wf = T.wf.p; a.cs = T.cs.p; a.sn = T.sn.p;
  return a;
}

// Glob_Sph_Trans PHYS_TO_FOUR of a point-layout field (times fac when given)
rbc3d_status sh_anal(rbc3d_ctx* ctx, const CellSolveTabs& T, const double* v, const double* fac, double* c,
                     int nvar = 3) {
  ShArgs a = sh_args(ctx, T, false, nvar);
  const size_t sm = sizeof(double) * ((size_t)a.nlat * a.nlon + 2 * (size_t)T.L * a.nlat);
  if (sm > 227 * 1024) return ctx_fail(ctx, RBC3D_ERR_ARG, "sh_anal: cell grid too large for one block");
  if (sm > 48 * 1024) CUDA_TRY(cudaFuncSetAttribute(k_sh_anal, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  { k_sh_anal<<<nvar * ctx->ncell, 128, sm, ctx->st>>>(a, v, fac, c); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}
rbc3d_status sh_synth(rbc3d_ctx* ctx, const CellSolveTabs& T, const double* c, double* out, bool equi, int nvar = 3) {
  ShArgs a = sh_args(ctx, T, equi, nvar);
  const size_t sm = sizeof(double) * (2 * (size_t)T.L * T.L + 2 * (size_t)T.L * a.nrow);
  if (sm > 227 * 1024) return ctx_fail(ctx, RBC3D_ERR_ARG, "sh_synth: degree too large for one block");
  if (sm > 48 * 1024) CUDA_TRY(cudaFuncSetAttribute(k_sh_synth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  { k_sh_synth<<<nvar * ctx->ncell, 128, sm, ctx->st>>>(a, c, out, equi ? 1 : 0); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// Rbc_BuildSurfaceSource for one field (ModRbc.F90:716-807) into spline set
// `set`: one k_sh_spline block per (cell, component).
rbc3d_status build_spline_set(rbc3d_ctx* ctx, const CellSolveTabs& T, const double* v, const double* fac, int nvar,
                              int set) {
  if (!T.equi_lon) return ctx_fail(ctx, RBC3D_ERR_ARG, "spline tables need an equispaced longitude grid of even size");
  spl_wait(ctx);  // on the main stream: no other build of the tables still in flight
  SplArgs a;
  a.L = T.L; a.nlat = ctx->nlat; a.nlon = ctx->nlon; a.npt = (int)ctx->npt; a.nvar = nvar; a.set = set;
  a.PG = T.PG.p; a.PE = T.PE.p; a.dPE = T.dPE.p; a.wf = T.wf.p; a.cs = T.cs.p; a.sn = T.sn.p;
  const size_t L = T.L, R = ctx->nlat + 1;
  const size_t sm = sizeof(double) * (2 * L * L + 4 * L * R + (size_t)ctx->nlat * ctx->nlon + 2 * L * ctx->nlat);
  if (sm > 227 * 1024) return ctx_fail(ctx, RBC3D_ERR_ARG, "spline build: cell grid too large for one block");
  if (sm > 48 * 1024) CUDA_TRY(cudaFuncSetAttribute(k_sh_spline, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  { k_sh_spline<<<nvar * ctx->ncell, 256, sm, ctx->st>>>(a, v, fac, ctx->spl.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// rbc%g <- g (device, point layout), Rbc_BuildSurfaceSource(gFlag) and
// SourceList_UpdateDensity(updateG)
rbc3d_status set_g_device(rbc3d_ctx* ctx, const CellSolveTabs& T, const double* g) {
  const size_t N = ctx->npt;
  rbc3d_status s;
  CUDA_TRY(ctx->g.alloc(3 * N));
  CUDA_TRY(cudaMemcpyAsync(ctx->g.p, g, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, ctx->st));
  if ((s = build_spline_set(ctx, T, g, ctx->detJ.p, 3, SPL_G))) return s;  // Rbc_BuildSurfaceSource(gFlag)
  ctx->has_g = true;
  if ((s = self_mixed_density(ctx, false, true))) return s;
  return build_source_density(ctx);
}

}  // namespace

rbc3d_status surface_sources_dev(rbc3d_ctx* ctx, int nlat0, bool geom, bool f, bool g) {
  if (nlat0 < 1 || nlat0 > ctx->nlat || 2 * (nlat0 - 1) >= ctx->nlon)
    return ctx_fail(ctx, RBC3D_ERR_ARG, "surface sources: need 1 <= nlat0 <= nlat, 2 (nlat0 - 1) < nlon");
  CellSolveTabs& T = ctx->shtab;
  rbc3d_status s;
  if ((s = cell_tabs(ctx, nlat0, T))) return s;
  if (geom) {
    if ((s = build_spline_set(ctx, T, ctx->x.p, nullptr, 3, SPL_X))) return s;
    if ((s = build_spline_set(ctx, T, ctx->a3.p, nullptr, 3, SPL_A3))) return s;
    if ((s = build_spline_set(ctx, T, ctx->detJ.p, nullptr, 1, SPL_DJ))) return s;
  }
  if (f && (s = build_spline_set(ctx, T, ctx->f.p, ctx->detJ.p, 3, SPL_F))) return s;
  if (g && (s = build_spline_set(ctx, T, ctx->g.p, ctx->detJ.p, 3, SPL_G))) return s;
  return RBC3D_OK;
}

extern "C" int rbc3d_cell_dof(const rbc3d_ctx* ctx, int nlat0) { return ctx ? 3 * nlat0 * nlat0 * ctx->ncell : 0; }

// Solve_RBC_Vel, ModVelSolver.F90:44-132 (Deflate off)
extern "C" rbc3d_status rbc3d_solve_rbc_vel(rbc3d_ctx* ctx, const rbc3d_solve_opts* o, int nlat0, double* sol,
                                            double* v, rbc3d_solve_stats* st) {
  if (!ctx || !o || !v) return RBC3D_ERR_ARG;
  if (nlat0 < 1 || nlat0 > ctx->nlat || 2 * (nlat0 - 1) >= ctx->nlon || (ctx->nlon % 2) != 0)
    return ctx_fail(ctx, RBC3D_ERR_ARG, "solve_rbc_vel: need 1 <= nlat0 <= nlat, 2 (nlat0 - 1) < nlon, even nlon");
  if (o->rtol < 0 || o->max_it < 0 || (o->guess && !sol) || !valid_prec(o->prec))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "solve_rbc_vel: bad options");
  const bool mixed = o->prec != RBC3D_FP64;  // FP32 operator inside an FP64 refinement loop
  if (ctx->npt == 0) return RBC3D_OK;
  auto t0 = std::chrono::steady_clock::now();
  rbc3d_solve_stats S{};
  CellSolveTabs& T = ctx->shtab;
  rbc3d_status s;
  if ((s = cell_tabs(ctx, nlat0, T))) return s;
  const size_t N = ctx->npt;
  const int n = 3 * nlat0 * nlat0 * ctx->ncell, R = o->restart > 0 ? o->restart : 30;
  const double ip4 = 1.0 / (4.0 * RBC3D_PI);
  TargetSet& t = ctx->tl[RBC3D_TLIST_RBC];
  DBuf<double> b, x, r, g, tmp;
  CUDA_TRY(b.alloc(n)); CUDA_TRY(x.alloc(n)); CUDA_TRY(r.alloc(n)); CUDA_TRY(g.alloc(3 * N));
  CUDA_TRY(tmp.alloc(8));
  // Compute_Rhs (:455-515): single layer of the cells and walls, PME, background flow
  const unsigned all = RBC3D_TERM_REAL | RBC3D_TERM_CORR | RBC3D_TERM_LINEAR | RBC3D_TERM_WALLS | RBC3D_TERM_PME;
  if ((s = matvec_dev(ctx, RBC3D_TLIST_RBC, ip4, 0.0, all, RBC3D_FP64))) return s;
  { k_add_vbkg<<<cs_nblk(N, 256), 256, 0, ctx->st>>>((int)N, t.Acoef.p, ctx->prm.vBkg[0], ctx->prm.vBkg[1],
                                                      ctx->prm.vBkg[2], t.v.p); ++ctx->launches; }
  if ((s = sh_anal(ctx, T, t.v.p, nullptr, b.p))) return s;
  bool all_one = true;
  for (int l = 0; l < ctx->prm.ncelltypes; ++l) all_one = all_one && ctx->prm.viscRat[l] == 1.0;
  if (all_one) {
    CUDA_TRY(cudaMemcpyAsync(x.p, b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    S.converged = 1;
  } else {
    if (o->guess && sol) CUDA_TRY(cudaMemcpyAsync(x.p, sol, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
    else CUDA_TRY(cudaMemsetAsync(x.p, 0, sizeof(double) * n, ctx->st));
    // MyMatMult (:523-601)
    const unsigned dl_terms = RBC3D_TERM_REAL | RBC3D_TERM_CORR | RBC3D_TERM_LINEAR | RBC3D_TERM_PME;
    auto matvec_p = [&](const double* u, double* y, int prec) -> rbc3d_status {
      S.matvecs++;
      rbc3d_status e;
      if ((e = sh_synth(ctx, T, u, g.p, false))) return e;
      if ((e = set_g_device(ctx, T, g.p))) return e;
      if ((e = matvec_dev(ctx, RBC3D_TLIST_RBC, 0.0, -ip4, dl_terms, prec))) return e;
      { k_axpby<<<cs_nblk(3 * N, 256), 256, 0, ctx->st>>>((int)(3 * N), 1.0, g.p, 1.0, t.v.p); ++ctx->launches; }
      return sh_anal(ctx, T, t.v.p, nullptr, y);
    };
    auto matvec = [&](const double* u, double* y) { return matvec_p(u, y, RBC3D_FP64); };
    auto matvec32 = [&](const double* u, double* y) { return matvec_p(u, y, o->prec); };
    DBuf<double> w;
    CUDA_TRY(w.alloc(n));
    if ((s = matvec(x.p, w.p))) return s;
    CUDA_TRY(cudaMemcpyAsync(r.p, b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    { k_axpby<<<cs_nblk(n, 256), 256, 0, ctx->st>>>(n, -1.0, w.p, 1.0, r.p); ++ctx->launches; }
    const double beta = dev_norm(ctx, n, r.p, tmp.p);
    S.rnorm0 = beta;
    S.bnorm = dev_norm(ctx, n, b.p, tmp.p);
    const double ttol = std::max(o->rtol * S.bnorm, 1e-50);
    if (mixed) {
      if ((s = gmres_ir(ctx, n, matvec, matvec32, b.p, x.p, r.p, beta, ttol, o->max_it, R, RBC3D_IR_ETA, S))) return s;
    } else if ((s = gmres_cycles(ctx, n, matvec, b.p, x.p, r.p, beta, ttol, o->max_it, R, S))) {
      return s;
    }
  }
  // the surface velocities; rbc%g and its spline are left at the solution
  if ((s = sh_synth(ctx, T, x.p, g.p, false))) return s;
  if (!all_one && (s = set_g_device(ctx, T, g.p))) return s;
  CUDA_TRY(cudaMemcpyAsync(v, g.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, ctx->st));
  if (sol) CUDA_TRY(cudaMemcpyAsync(sol, x.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  S.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = S;
  return S.converged ? RBC3D_OK : ctx_fail(ctx, RBC3D_ERR_NOCONV, "GMRES reached max_it");
}
