// walls.cu -- wall quadrature, the self-wall operator and the NoSlipWall GMRES.
//
//   AddIntOnWalls (ModIntOnWalls.F90:37-128): cell / raw targets against every
//     wall triangle whose centroid lies in the 27 neighbour cells, translated
//     to the nearest image, MinDistToTri (Eberly) <= rc, 7-point gqTri7 rule
//     or Duffy's 3 x 4 x 4 rule when closer than sqrt(area).
//   PrepareSingIntOnWall (ModIntOnWalls.F90:181-308): assembled once on the
//     GPU: (vertex, triangle) pair list -> per-pair 3x3x3 influence blocks ->
//     radix sort by (row vertex, column vertex) -> segmented sums -> block-CSR
//     with 3x3 blocks (rows and columns component-major as the PETSc matrix).
//   NoSlipWall (ModNoSlip.F90:45-150): restarted GMRES on the wall-density
//     increment, FP64 Arnoldi (classical Gram-Schmidt as PETSc's default) and
//     FP64 Givens / Hessenberg least squares, all on the device.
#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "ctx.hpp"
#include "gmres.cuh"

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

struct TriRules {
  double r7[7], s7[7], w7[7];  // gqTri7, ModQuadRule.F90:69-94
  double rg[4], wg[4];         // GauLeg(0,1,4) for Duffy, ModIntOnWalls.F90:400
};
__constant__ TriRules c_rules;

__host__ __device__ __forceinline__ double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// One quadrature point: rhs += K(xt - xg) (ds*fg); lhs[l] += wv[l] * ds * K
template <bool LHS>
__device__ __forceinline__ void quad_point(const Tables& T, const double* xt, const double* xg, const double* fg, double ds,
                                           const double* wv, double* rhs, double (*lhs)[9]) {
  double xx[3] = {xt[0] - xg[0], xt[1] - xg[1], xt[2] - xg[2]};
  double rr = sqrt(dot3(xx, xx)), EA, EB;
  ewald_sl64(T, rr, EA, EB);
  double f3[3] = {ds * fg[0], ds * fg[1], ds * fg[2]};
  double xf = dot3(xx, f3);
  for (int c = 0; c < 3; ++c) rhs[c] += EA * xx[c] * xf + EB * f3[c];
  if (LHS) {
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        double Lrc = ds * (EA * xx[r] * xx[c] + (r == c ? EB : 0.));
        for (int l = 0; l < 3; ++l) lhs[l][r * 3 + c] += wv[l] * Lrc;
      }
  }
}

// Tri_Int_Regular, ModIntOnWalls.F90:319-363
template <bool LHS>
__device__ void tri_int_regular(const Tables& T, const double xv[3][3], const double fv[3][3], const double* xt,
                                double* rhs, double (*lhs)[9]) {
  double a[3], b[3];
  for (int c = 0; c < 3; ++c) { a[c] = xv[1][c] - xv[0][c]; b[c] = xv[2][c] - xv[0][c]; }
  double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  double detJ = 2 * (0.5 * sqrt(dot3(cr, cr)));
  for (int q = 0; q < 7; ++q) {
    double s = c_rules.r7[q], t = c_rules.s7[q];
    double xg[3], fg[3];
    for (int c = 0; c < 3; ++c) {
      xg[c] = (1. - s - t) * xv[0][c] + s * xv[1][c] + t * xv[2][c];
      fg[c] = (1. - s - t) * fv[0][c] + s * fv[1][c] + t * fv[2][c];
    }
    double wv[3] = {1 - s - t, s, t};
    quad_point<LHS>(T, xt, xg, fg, c_rules.w7[q] * detJ, wv, rhs, lhs);
  }
}

// Tri_Int_Duffy, ModIntOnWalls.F90:373-465
template <bool LHS>
__device__ void tri_int_duffy(const Tables& T, const double xv[3][3], const double fv[3][3], const double* xt,
                              double s0, double t0, double* rhs, double (*lhs)[9]) {
  double x0[3], f0[3];
  for (int c = 0; c < 3; ++c) {
    x0[c] = (1 - s0 - t0) * xv[0][c] + s0 * xv[1][c] + t0 * xv[2][c];
    f0[c] = (1 - s0 - t0) * fv[0][c] + s0 * fv[1][c] + t0 * fv[2][c];
  }
  const double S1[3] = {0., 1., 0.}, T1[3] = {0., 0., 1.}, S2[3] = {1., 0., 0.}, T2[3] = {0., 1., 0.};
  for (int n = 0; n < 3; ++n) {
    const double* x1 = xv[n];
    const double* x2 = xv[(n + 1) % 3];
    const double* f1 = fv[n];
    const double* f2 = fv[(n + 1) % 3];
    double a[3], b[3];
    for (int c = 0; c < 3; ++c) { a[c] = x1[c] - x0[c]; b[c] = x2[c] - x0[c]; }
    double nr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    double detJ = sqrt(dot3(nr, nr));
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        double s = c_rules.rg[i], t = s * c_rules.rg[j];
        double xg[3], fg[3];
        for (int c = 0; c < 3; ++c) {
          xg[c] = (1. - s) * x0[c] + (s - t) * x1[c] + t * x2[c];
          fg[c] = (1. - s) * f0[c] + (s - t) * f1[c] + t * f2[c];
        }
        double ds = c_rules.wg[i] * c_rules.wg[j] * detJ * s;
        double wv[3] = {0, 0, 0};
        if (LHS) {
          double sG = (1. - s) * s0 + (s - t) * S1[n] + t * S2[n];
          double tG = (1. - s) * t0 + (s - t) * T1[n] + t * T2[n];
          wv[0] = 1. - sG - tG; wv[1] = sG; wv[2] = tG;
        }
        quad_point<LHS>(T, xt, xg, fg, ds, wv, rhs, lhs);
      }
  }
}

struct WallArgs {
  int nvert, nele;
  const double* x;
  const double* f;
  const int* e2v;
  const double* eps;
  const int* cs;
  const int* ce;
  const int* order;
  int Nc[3];
  double h[3], L[3], iL[3];
  double rc;
  Tables T;
};

__device__ __forceinline__ void load_tri(const WallArgs& a, int e, double xv[3][3], double fv[3][3], bool wf) {
  for (int l = 0; l < 3; ++l) {
    int iv = a.e2v[e + (size_t)l * a.nele];
    for (int c = 0; c < 3; ++c) {
      xv[l][c] = a.x[iv + (size_t)c * a.nvert];
      fv[l][c] = wf ? a.f[iv + (size_t)c * a.nvert] : 0.;
    }
  }
}
__device__ __forceinline__ void translate_tri(const WallArgs& a, const double* xi, double xv[3][3]) {
  for (int c = 0; c < 3; ++c) {
    double sh = round((xi[c] - xv[0][c]) * a.iL[c]) * a.L[c];
    for (int l = 0; l < 3; ++l) xv[l][c] += sh;
  }
}
__device__ __forceinline__ int home_cell(const WallArgs& a, const double* xi, int& ci, int& cj, int& ck) {
  ci = imod((int)floor(xi[0] * a.Nc[0] * a.iL[0]), a.Nc[0]);
  cj = imod((int)floor(xi[1] * a.Nc[1] * a.iL[1]), a.Nc[1]);
  ck = imod((int)floor(xi[2] * a.Nc[2] * a.iL[2]), a.Nc[2]);
  return 0;
}

// AddIntOnWalls for cell / raw targets (one thread per target, cell-list order)
__global__ void k_wall_quad(WallArgs a, int nt, const double* __restrict__ tx, const double* __restrict__ tA,
                            const int* __restrict__ torder, double c1, double* __restrict__ v,
                            unsigned long long* cnt) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nt) return;
  int i = torder[q];
  double xi[3] = {tx[i], tx[i + nt], tx[i + 2 * (size_t)nt]};
  int ci, cj, ck;
  home_cell(a, xi, ci, cj, ck);
  double acc[3] = {0, 0, 0};
  unsigned long long np = 0, nd = 0;
  for (int nb = 0; nb < 27; ++nb) {
    int nc = imod(ci + nb % 3 - 1, a.Nc[0]) + a.Nc[0] * (imod(cj + (nb / 3) % 3 - 1, a.Nc[1]) + a.Nc[1] * imod(ck + nb / 9 - 1, a.Nc[2]));
    for (int p = a.cs[nc]; p < a.ce[nc]; ++p) {
      int e = a.order[p];
      double xv[3][3], fv[3][3];
      load_tri(a, e, xv, fv, true);
      translate_tri(a, xi, xv);
      double s0, t0;
      double rr = min_dist_to_tri(xi, xv, s0, t0);
      if (rr > a.rc) continue;
      ++np;
      double dv[3] = {0, 0, 0};
      if (rr < a.eps[e]) { tri_int_duffy<false>(a.T, xv, fv, xi, s0, t0, dv, nullptr); ++nd; }
      else tri_int_regular<false>(a.T, xv, fv, xi, dv, nullptr);
      for (int c = 0; c < 3; ++c) acc[c] += c1 * dv[c] / tA[i];
    }
  }
  for (int c = 0; c < 3; ++c) v[i + (size_t)c * nt] += acc[c];
  if (np) { atomicAdd(cnt + 4, np); if (nd) atomicAdd(cnt + 5, nd); }
}

// Self-wall assembly, pass 1/2: count (mode 0) or list (mode 1) the
// (vertex, triangle) pairs within rc.
__global__ void k_self_pairs(WallArgs a, int mode, int* __restrict__ count, const int* __restrict__ off,
                             int2* __restrict__ pairs) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nvert) return;
  double xi[3] = {a.x[i], a.x[i + a.nvert], a.x[i + 2 * (size_t)a.nvert]};
  int ci, cj, ck;
  home_cell(a, xi, ci, cj, ck);
  int n = 0, base = mode ? off[i] : 0;
  for (int nb = 0; nb < 27; ++nb) {
    int nc = imod(ci + nb % 3 - 1, a.Nc[0]) + a.Nc[0] * (imod(cj + (nb / 3) % 3 - 1, a.Nc[1]) + a.Nc[1] * imod(ck + nb / 9 - 1, a.Nc[2]));
    for (int p = a.cs[nc]; p < a.ce[nc]; ++p) {
      int e = a.order[p];
      double xv[3][3], fv[3][3];
      load_tri(a, e, xv, fv, false);
      translate_tri(a, xi, xv);
      double s0, t0;
      if (min_dist_to_tri(xi, xv, s0, t0) > a.rc) continue;
      if (mode) pairs[base + n] = make_int2(i, e);
      ++n;
    }
  }
  if (!mode) count[i] = n;
}

// pass 3: one 3x3x3 influence block per pair -> three keyed 3x3 blocks
__global__ void k_self_blocks(WallArgs a, long long npair, const int2* __restrict__ pairs,
                              unsigned long long* __restrict__ keys, int* __restrict__ idx, double* __restrict__ blk) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  int i = pairs[p].x, e = pairs[p].y;
  double xi[3] = {a.x[i], a.x[i + a.nvert], a.x[i + 2 * (size_t)a.nvert]};
  double xv[3][3], fv[3][3];
  load_tri(a, e, xv, fv, false);
  translate_tri(a, xi, xv);
  double s0, t0;
  double rr = min_dist_to_tri(xi, xv, s0, t0);
  double rhs[3] = {0, 0, 0}, lhs[3][9];
  for (int l = 0; l < 3; ++l)
    for (int k = 0; k < 9; ++k) lhs[l][k] = 0.;
  if (rr > a.eps[e]) tri_int_regular<true>(a.T, xv, fv, xi, rhs, lhs);
  else tri_int_duffy<true>(a.T, xv, fv, xi, s0, t0, rhs, lhs);
  for (int l = 0; l < 3; ++l) {
    int iv = a.e2v[e + (size_t)l * a.nele];
    long long slot = 3 * p + l;
    keys[slot] = (unsigned long long)i * (unsigned long long)a.nvert + (unsigned long long)iv;
    idx[slot] = (int)slot;
    for (int k = 0; k < 9; ++k) blk[slot * 9 + k] = lhs[l][k];
  }
}

__global__ void k_uniq_flags(long long n, const unsigned long long* __restrict__ k, int* __restrict__ flag) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  flag[p] = (p == 0 || k[p] != k[p - 1]) ? 1 : 0;
}
// pass 4: segmented sums into block-CSR entries
__global__ void k_self_reduce(long long n, int nvert, const unsigned long long* __restrict__ k, const int* __restrict__ perm,
                              const int* __restrict__ seg, const double* __restrict__ blk, int* __restrict__ bcol,
                              int* __restrict__ brow, double* __restrict__ bval) {
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (p > 0 && k[p] == k[p - 1]) return;  // only segment heads
  int u = seg[p] - 1;  // inclusive scan of head flags: 1-based segment ids
  double s[9];
  for (int c = 0; c < 9; ++c) s[c] = 0.;
  for (long long q = p; q < n && k[q] == k[p]; ++q)
    for (int c = 0; c < 9; ++c) s[c] += blk[(size_t)perm[q] * 9 + c];
  for (int c = 0; c < 9; ++c) bval[(size_t)u * 9 + c] = s[c];
  bcol[u] = (int)(k[p] % (unsigned long long)nvert);
  brow[u] = (int)(k[p] / (unsigned long long)nvert);
}
__global__ void k_row_ptr(int nb, int nvert, const int* __restrict__ brow, int* __restrict__ rowptr) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nb) return;
  int r = brow[u];
  if (u == 0) for (int q = 0; q <= r; ++q) rowptr[q] = 0;
  if (u == nb - 1) for (int q = r + 1; q <= nvert; ++q) rowptr[q] = nb;
  if (u > 0 && brow[u - 1] != r)
    for (int q = brow[u - 1] + 1; q <= r; ++q) rowptr[q] = u;
}

// SingIntOnWall (ModIntOnWalls.F90:136-172): v += c1 * (M f) / Acoef, block-CSR
__global__ void k_self_spmv(int nvert, const int* __restrict__ rowptr, const int* __restrict__ bcol,
                            const double* __restrict__ bval, const double* __restrict__ f, const double* __restrict__ tA,
                            double c1, double* __restrict__ v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  double y[3] = {0, 0, 0};
  for (int b = rowptr[i]; b < rowptr[i + 1]; ++b) {
    int j = bcol[b];
    const double* B = bval + (size_t)b * 9;
    double fj[3] = {f[j], f[j + nvert], f[j + 2 * (size_t)nvert]};
    for (int r = 0; r < 3; ++r) y[r] += B[r * 3 + 0] * fj[0] + B[r * 3 + 1] * fj[1] + B[r * 3 + 2] * fj[2];
  }
  for (int r = 0; r < 3; ++r) v[i + (size_t)r * nvert] += c1 * y[r] / tA[i];
}

__global__ void k_wall_geom(int nele, int nvert, const int* __restrict__ e2v, const double* __restrict__ x,
                            double* __restrict__ area, double* __restrict__ eps, double* __restrict__ cen) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  double xv[3][3];
  for (int l = 0; l < 3; ++l) {
    int iv = e2v[e + (size_t)l * nele];
    for (int c = 0; c < 3; ++c) xv[l][c] = x[iv + (size_t)c * nvert];
  }
  double a[3], b[3];
  for (int c = 0; c < 3; ++c) { a[c] = xv[1][c] - xv[0][c]; b[c] = xv[2][c] - xv[0][c]; }
  double nr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  double an = sqrt(dot3(nr, nr));
  area[e] = 0.5 * an;             // Wall_ComputeGeometry, ModWall.F90:118-145
  eps[e] = sqrt(area[e]);
  for (int c = 0; c < 3; ++c) cen[e + (size_t)c * nele] = (1.0 / 3) * (xv[0][c] + xv[1][c] + xv[2][c]);
}

// AssembleArray (ModNoSlip.F90:361-384)
__global__ void k_expand(int nvert, const int* __restrict__ glb, const double* __restrict__ u, double* __restrict__ f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  int g = glb[i];
  for (int c = 0; c < 3; ++c) f[i + (size_t)c * nvert] = u[3 * (size_t)g + c];
}
__global__ void k_assemble(int nvert, const int* __restrict__ glb, const int* __restrict__ writer,
                           const double* __restrict__ v, double scale, double* __restrict__ u) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert || !writer[i]) return;  // the last duplicate wins, as the sequential loop
  int g = glb[i];
  for (int c = 0; c < 3; ++c) u[3 * (size_t)g + c] = scale * v[i + (size_t)c * nvert];
}
__global__ void k_add_const(int n, double a0, double a1, double a2, double* v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  v[i] += a0; v[i + n] += a1; v[i + 2 * (size_t)n] += a2;
}

WallArgs wall_args(rbc3d_ctx* ctx) {
  WallState& W = ctx->wall;
  WallArgs a;
  a.nvert = W.nvert; a.nele = W.nele; a.x = W.x.p; a.f = W.f.p; a.e2v = W.e2v.p; a.eps = W.eps.p;
  a.cs = W.cstart.p; a.ce = W.cend.p; a.order = W.order.p;
  for (int d = 0; d < 3; ++d) { a.Nc[d] = ctx->hg.Nc[d]; a.h[d] = ctx->hg.h[d]; a.L[d] = ctx->hg.L[d]; a.iL[d] = ctx->iLb[d]; }
  a.rc = ctx->prm.rc;
  a.T = ctx->T;
  return a;
}


}  // namespace

static rbc3d_status writer_flags(rbc3d_ctx* ctx, DBuf<int>& wr) {
  WallState& W = ctx->wall;
  std::vector<int> last(W.ndof / 3, -1), flag(W.nvert, 0);
  for (int i = 0; i < W.nvert; ++i) last[W.hglb[i]] = i;
  for (int i = 0; i < W.nvert; ++i) flag[i] = last[W.hglb[i]] == i;
  CUDA_TRY(wr.upload(flag.data(), flag.size(), ctx->st));
  return RBC3D_OK;
}

rbc3d_status wall_setup(rbc3d_ctx* ctx) {
  WallState& W = ctx->wall;
  if (W.nvert == 0) return RBC3D_OK;
  static bool rules_set = false;
  if (!rules_set) {
    TriRules R;
    double r = (6. - std::sqrt(15.)) / 21., s = r, t = 1 - r - s;
    double rr[7] = {r, s, t, 0, 0, 0, 1. / 3.}, ss[7] = {s, t, r, 0, 0, 0, 1. / 3.};
    double w1 = (155. - std::sqrt(15.)) / 2400.;
    r = (6. + std::sqrt(15.)) / 21.; s = r; t = 1 - r - s;
    rr[3] = r; rr[4] = s; rr[5] = t; ss[3] = s; ss[4] = t; ss[5] = r;
    double w2 = (155. + std::sqrt(15.)) / 2400.;
    for (int i = 0; i < 7; ++i) { R.r7[i] = rr[i]; R.s7[i] = ss[i]; }
    for (int i = 0; i < 3; ++i) { R.w7[i] = w1; R.w7[i + 3] = w2; }
    R.w7[6] = 9. / 80.;
    host_gauleg(0., 1., 4, R.rg, R.wg);
    CUDA_TRY(cudaMemcpyToSymbol(c_rules, &R, sizeof(R)));
    rules_set = true;
  }
  CUDA_TRY(W.x.upload(W.hx.data(), W.hx.size(), ctx->st));
  CUDA_TRY(W.f.upload(W.hf.data(), W.hf.size(), ctx->st));
  CUDA_TRY(W.e2v.upload(W.he2v.data(), W.he2v.size(), ctx->st));
  CUDA_TRY(W.glb.upload(W.hglb.data(), W.hglb.size(), ctx->st));
  CUDA_TRY(W.area.alloc(W.nele)); CUDA_TRY(W.eps.alloc(W.nele)); CUDA_TRY(W.cen.alloc(3 * (size_t)W.nele));
  { k_wall_geom<<<nblk(W.nele, 256), 256, 0, ctx->st>>>(W.nele, W.nvert, W.e2v.p, W.x.p, W.area.p, W.eps.p, W.cen.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  rbc3d_status s = writer_flags(ctx, W.writer);
  if (s) return s;
  return sort_points_by_cell(ctx, W.nele, W.cen.p, W.order, W.cstart, W.cend);
}

rbc3d_status wall_prepare_self(rbc3d_ctx* ctx) {
  WallState& W = ctx->wall;
  if (W.nvert == 0) return RBC3D_OK;
  WallArgs a = wall_args(ctx);
  DBuf<int> count, off;
  CUDA_TRY(count.alloc(W.nvert + 1)); CUDA_TRY(off.alloc(W.nvert + 1));
  CUDA_TRY(cudaMemsetAsync(count.p, 0, sizeof(int) * (W.nvert + 1), ctx->st));
  { k_self_pairs<<<nblk(W.nvert, 128), 128, 0, ctx->st>>>(a, 0, count.p, nullptr, nullptr); ++ctx->launches; }
  size_t tmp = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp, count.p, off.p, W.nvert + 1, ctx->st);
  DBuf<char> tb;
  CUDA_TRY(tb.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceScan::ExclusiveSum(tb.p, tmp, count.p, off.p, W.nvert + 1, ctx->st));
  int npair = 0;
  CUDA_TRY(cudaMemcpyAsync(&npair, off.p + W.nvert, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  if (npair == 0) {
    CUDA_TRY(W.rowptr.alloc(W.nvert + 1));
    CUDA_TRY(cudaMemsetAsync(W.rowptr.p, 0, sizeof(int) * (W.nvert + 1), ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
    W.nnz = 0;
    W.prepared = true;
    return RBC3D_OK;
  }
  DBuf<int2> pairs;
  CUDA_TRY(pairs.alloc(npair));
  { k_self_pairs<<<nblk(W.nvert, 128), 128, 0, ctx->st>>>(a, 1, nullptr, off.p, pairs.p); ++ctx->launches; }
  long long ne = 3LL * npair;
  DBuf<unsigned long long> k1, k2;
  DBuf<int> i1, i2, flag, seg;
  DBuf<double> blk;
  CUDA_TRY(k1.alloc(ne)); CUDA_TRY(k2.alloc(ne)); CUDA_TRY(i1.alloc(ne)); CUDA_TRY(i2.alloc(ne));
  CUDA_TRY(flag.alloc(ne)); CUDA_TRY(seg.alloc(ne)); CUDA_TRY(blk.alloc(9 * ne));
  { k_self_blocks<<<nblk(npair, 128), 128, 0, ctx->st>>>(a, npair, pairs.p, k1.p, i1.p, blk.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, k1.p, k2.p, i1.p, i2.p, (int)ne, 0, 64, ctx->st);
  DBuf<char> tb2;
  CUDA_TRY(tb2.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceRadixSort::SortPairs(tb2.p, tmp, k1.p, k2.p, i1.p, i2.p, (int)ne, 0, 64, ctx->st));
  { k_uniq_flags<<<nblk(ne, 256), 256, 0, ctx->st>>>(ne, k2.p, flag.p); ++ctx->launches; }
  tmp = 0;
  cub::DeviceScan::InclusiveSum(nullptr, tmp, flag.p, seg.p, (int)ne, ctx->st);
  DBuf<char> tb3;
  CUDA_TRY(tb3.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceScan::InclusiveSum(tb3.p, tmp, flag.p, seg.p, (int)ne, ctx->st));
  int nb = 0;
  CUDA_TRY(cudaMemcpyAsync(&nb, seg.p + ne - 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  DBuf<int> brow;
  CUDA_TRY(W.col.alloc(nb)); CUDA_TRY(brow.alloc(nb)); CUDA_TRY(W.val.alloc(9 * (size_t)nb));
  CUDA_TRY(W.rowptr.alloc(W.nvert + 1));
  { k_self_reduce<<<nblk(ne, 256), 256, 0, ctx->st>>>(ne, W.nvert, k2.p, i2.p, seg.p, blk.p, W.col.p, brow.p, W.val.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  if (nb > 0) { k_row_ptr<<<nblk(nb, 256), 256, 0, ctx->st>>>(nb, W.nvert, brow.p, W.rowptr.p); ++ctx->launches; }
  else CUDA_TRY(cudaMemsetAsync(W.rowptr.p, 0, sizeof(int) * (W.nvert + 1), ctx->st));
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  W.nnz = 9LL * nb;
  W.prepared = true;
  return RBC3D_OK;
}

rbc3d_status run_wall_quad(rbc3d_ctx* ctx, int tlist, double c1, int prec) {
  (void)prec;
  WallState& W = ctx->wall;
  TargetSet& t = ctx->tl[tlist];
  if (W.nele == 0 || t.n == 0 || tlist == RBC3D_TLIST_WALL) return RBC3D_OK;
  rbc3d_status s = sort_targets(ctx, tlist);
  if (s) return s;
  WallArgs a = wall_args(ctx);
  CUDA_TRY(cudaMemsetAsync(ctx->dcnt.p + 4, 0, 2 * sizeof(unsigned long long), ctx->st));
  { k_wall_quad<<<nblk(t.n, 128), 128, 0, ctx->st>>>(a, t.n, t.x.p, t.Acoef.p, t.order.p, c1, t.v.p, ctx->dcnt.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  unsigned long long h[2];
  CUDA_TRY(cudaMemcpyAsync(h, ctx->dcnt.p + 4, sizeof(h), cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->counts.wall_pairs = (long long)h[0];
  ctx->counts.wall_duffy = (long long)h[1];
  return RBC3D_OK;
}

rbc3d_status run_wall_self(rbc3d_ctx* ctx, double c1) {
  WallState& W = ctx->wall;
  if (W.nvert == 0) return RBC3D_OK;
  if (!W.prepared) return ctx_fail(ctx, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
  TargetSet& t = ctx->tl[RBC3D_TLIST_WALL];
  { k_self_spmv<<<nblk(W.nvert, 128), 128, 0, ctx->st>>>(W.nvert, W.rowptr.p, W.col.p, W.val.p, W.f.p, t.Acoef.p, c1,
                                                        t.v.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// Compute_Wall_Residual_Vel (ModNoSlip.F90:153-193) into tl[WALL].v
rbc3d_status wall_residual_dev(rbc3d_ctx* ctx, int prec) {
  double c = 1. / (4. * RBC3D_PI);
  rbc3d_status s = matvec_dev(ctx, RBC3D_TLIST_WALL, c, c, RBC3D_TERM_ALL, prec);
  if (s) return s;
  TargetSet& t = ctx->tl[RBC3D_TLIST_WALL];
  { k_add_const<<<nblk(t.n, 256), 256, 0, ctx->st>>>(t.n, ctx->prm.vBkg[0], ctx->prm.vBkg[1], ctx->prm.vBkg[2], t.v.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}


// MyMatMult (ModNoSlip.F90:255-308): y = assemble(SingIntOnWall + PME(walls)) of expand(u)
rbc3d_status wall_matmult_dev(rbc3d_ctx* ctx, int prec, const double* u_dev, double* y_dev) {
  WallState& W = ctx->wall;
  TargetSet& t = ctx->tl[RBC3D_TLIST_WALL];
  if (!W.prepared) return ctx_fail(ctx, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
  { k_expand<<<nblk(W.nvert, 256), 256, 0, ctx->st>>>(W.nvert, W.glb.p, u_dev, W.f.p); ++ctx->launches; }
  CUDA_TRY(t.v.alloc(3 * (size_t)t.n));
  CUDA_TRY(cudaMemsetAsync(t.v.p, 0, sizeof(double) * 3 * t.n, ctx->st));
  double c1 = 1. / (4. * RBC3D_PI);
  rbc3d_status s;
  if ((s = run_wall_self(ctx, c1))) return s;
  if ((s = pme_spread(ctx, c1, 0., 0, 1, prec))) return s;
  if ((s = pme_transform(ctx))) return s;
  if ((s = pme_gather(ctx, RBC3D_TLIST_WALL))) return s;
  { k_assemble<<<nblk(W.nvert, 256), 256, 0, ctx->st>>>(W.nvert, W.glb.p, W.writer.p, t.v.p, 1.0, y_dev); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// NoSlipWall (ModNoSlip.F90:45-150)
// The learned spectral operator as the solve's right preconditioner (guess
// mode 5; wallspec.cu).
struct SpecPrec {
  rbc3d_ctx* ctx;
  bool on;
  bool active() const { return on; }
  rbc3d_status operator()(const double* in, double* out) const { return wall_spec_apply_dev(ctx, in, out); }
};

rbc3d_status wall_solve(rbc3d_ctx* ctx, const rbc3d_solve_opts* o, const double* guess, rbc3d_solve_stats* st) {
  WallState& W = ctx->wall;
  if (W.nvert == 0) return RBC3D_OK;
  if (!W.prepared) return ctx_fail(ctx, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
  auto t0 = std::chrono::steady_clock::now();
  rbc3d_solve_stats S{};
  const int n = W.ndof, R = o->restart > 0 ? o->restart : 30;
  const int prec = o->prec;
  if (!valid_prec(prec)) return ctx_fail(ctx, RBC3D_ERR_ARG, "no_slip_wall: bad precision mode");
  const bool mixed = prec != RBC3D_FP64;  // FP32 operator inside an FP64 refinement loop
  DBuf<double> b, x, r, w, f0, tmp;
  CUDA_TRY(b.alloc(n)); CUDA_TRY(x.alloc(n)); CUDA_TRY(r.alloc(n)); CUDA_TRY(w.alloc(n));
  CUDA_TRY(f0.alloc(3 * (size_t)W.nvert)); CUDA_TRY(tmp.alloc(8));
  CUDA_TRY(cudaMemcpyAsync(f0.p, W.f.p, sizeof(double) * 3 * W.nvert, cudaMemcpyDeviceToDevice, ctx->st));
  rbc3d_status s;
  // rhs = -assemble(residual velocity), FP64 in the mixed-precision solve
  if ((s = wall_residual_dev(ctx, mixed ? RBC3D_FP64 : prec))) return s;
  { k_assemble<<<nblk(W.nvert, 256), 256, 0, ctx->st>>>(W.nvert, W.glb.p, W.writer.p, ctx->tl[RBC3D_TLIST_WALL].v.p, -1.0,
                                                       b.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  if (o->guess == 4) {  // the learned spectral operator's prediction (wallspec.cu)
    if ((s = wall_spec_predict_dev(ctx, b.p, x.p, nullptr))) return s;
  } else if (o->guess == 5) {  // the same prediction, and the operator as the right preconditioner
    if ((s = wall_spec_predict_dev(ctx, b.p, x.p, nullptr))) return s;
  } else if (o->guess && guess) {
    CUDA_TRY(cudaMemcpyAsync(x.p, guess, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
  } else {
    CUDA_TRY(cudaMemsetAsync(x.p, 0, sizeof(double) * n, ctx->st));
  }
  DBuf<double> x2, w2;  // guess mode 3: second guess vector and its image
  if (o->guess == 3 && guess) {
    CUDA_TRY(x2.alloc(n)); CUDA_TRY(w2.alloc(n));
    CUDA_TRY(cudaMemcpyAsync(x2.p, guess + n, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
  }
  auto matvec = [&](const double* in, double* out) -> rbc3d_status {
    S.matvecs++;
    return wall_matmult_dev(ctx, prec, in, out);
  };
  // r = b - A x
  if ((s = matvec(x.p, w.p))) return s;
  CUDA_TRY(cudaMemcpyAsync(r.p, b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
  { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, -1.0, w.p, 1.0, r.p); ++ctx->launches; }
  if (o->guess == 2 && guess) {
    // minimum-residual scaling of the guess: x0 <- a x0, a = <b, A x0> / ||A x0||^2,
    // so that ||b - A x0|| <= ||b|| whatever the guess (w holds A x0)
    { k_dots<<<1, 512, 0, ctx->st>>>(n, 1, w.p, 0, b.p, tmp.p); ++ctx->launches; }
    { k_dots<<<1, 512, 0, ctx->st>>>(n, 1, w.p, 0, w.p, tmp.p + 1); ++ctx->launches; }
    double bw[2] = {0, 0};
    CUDA_TRY(cudaMemcpyAsync(bw, tmp.p, sizeof(double) * 2, cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
    const double a = bw[1] > 0 ? bw[0] / bw[1] : 0.0;
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, 0.0, w.p, a, x.p); ++ctx->launches; }
    CUDA_TRY(cudaMemcpyAsync(r.p, b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, -a, w.p, 1.0, r.p); ++ctx->launches; }
  }
  if (o->guess == 3 && guess) {
    // x0 = p x1 + q x2 minimising ||b - p A x1 - q A x2|| (2x2 normal equations;
    // w holds A x1), so the initial residual is no larger than either vector's
    if ((s = matvec(x2.p, w2.p))) return s;
    const double* pa[5] = {w.p, w.p, w2.p, w.p, w2.p};
    const double* pb[5] = {w.p, w2.p, w2.p, b.p, b.p};
    for (int i = 0; i < 5; ++i) { k_dots<<<1, 512, 0, ctx->st>>>(n, 1, pa[i], 0, pb[i], tmp.p + i); ++ctx->launches; }
    double m[5] = {0, 0, 0, 0, 0};
    CUDA_TRY(cudaMemcpyAsync(m, tmp.p, sizeof(double) * 5, cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
    double p = 0, q = 0;
    const double det = m[0] * m[2] - m[1] * m[1];
    if (det > 1e-14 * m[0] * m[2] && det > 0) {
      p = (m[3] * m[2] - m[4] * m[1]) / det;
      q = (m[4] * m[0] - m[3] * m[1]) / det;
    } else if (m[0] >= m[2] && m[0] > 0) {
      p = m[3] / m[0];
    } else if (m[2] > 0) {
      q = m[4] / m[2];
    }
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, q, x2.p, p, x.p); ++ctx->launches; }
    CUDA_TRY(cudaMemcpyAsync(r.p, b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, -p, w.p, 1.0, r.p); ++ctx->launches; }
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, -q, w2.p, 1.0, r.p); ++ctx->launches; }
  }
  auto matvec64 = [&](const double* in, double* out) -> rbc3d_status {
    S.matvecs++;
    return wall_matmult_dev(ctx, RBC3D_FP64, in, out);
  };
  if (mixed) {  // the initial residual of the guess with the FP64 operator
    if ((s = matvec64(x.p, w.p))) return s;
    CUDA_TRY(cudaMemcpyAsync(r.p, b.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, -1.0, w.p, 1.0, r.p); ++ctx->launches; }
  }
  const double beta = dev_norm(ctx, n, r.p, tmp.p);
  S.rnorm0 = beta;
  S.bnorm = dev_norm(ctx, n, b.p, tmp.p);
  // KSPConvergedDefault: ||r|| < max(rtol * ||b||, abstol), ||b|| of the right-hand side
  const double ttol = std::max(o->rtol * S.bnorm, 1e-50);
  SpecPrec pc{ctx, o->guess == 5};
  if (mixed) {
    if ((s = gmres_ir(ctx, n, matvec64, matvec, b.p, x.p, r.p, beta, ttol, o->max_it, R, RBC3D_IR_ETA, S, pc)))
      return s;
  } else if ((s = gmres_cycles(ctx, n, matvec, b.p, x.p, r.p, beta, ttol, o->max_it, R, S, pc))) {
    return s;
  }
  // every converged solve teaches the spectral model the pair (A x, x) =
  // (b - r, x), r the true residual the solve ended on: exact whatever the
  // tolerance the solve stopped at
  if (S.converged && ctx->wspec.ready && ctx->wspec.record) {
    { k_axpby<<<nblk(n, 256), 256, 0, ctx->st>>>(n, -1.0, r.p, 1.0, b.p); ++ctx->launches; }
    if ((s = wall_spec_add_dev(ctx, b.p, x.p))) return s;
  }
  // wall f = f0 + expand(x)
  { k_expand<<<nblk(W.nvert, 256), 256, 0, ctx->st>>>(W.nvert, W.glb.p, x.p, W.f.p); ++ctx->launches; }
  { k_axpby<<<nblk(3 * W.nvert, 256), 256, 0, ctx->st>>>(3 * W.nvert, 1.0, f0.p, 1.0, W.f.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  S.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = S;
  return S.converged ? RBC3D_OK : ctx_fail(ctx, RBC3D_ERR_NOCONV, "GMRES reached max_it");
}

// b = -AssembleArray(Compute_Wall_Residual_Vel) (ModNoSlip.F90:110-113), host copy
extern "C" rbc3d_status rbc3d_wall_rhs(rbc3d_ctx* ctx, int prec, double* b) {
  if (!ctx || !b || !valid_prec(prec)) return RBC3D_ERR_ARG;
  WallState& W = ctx->wall;
  if (W.nvert == 0) return RBC3D_OK;
  if (!W.prepared) return ctx_fail(ctx, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
  rbc3d_status s = wall_residual_dev(ctx, prec);
  if (s) return s;
  DBuf<double> db;
  CUDA_TRY(db.alloc(W.ndof));
  { k_assemble<<<nblk(W.nvert, 256), 256, 0, ctx->st>>>(W.nvert, W.glb.p, W.writer.p, ctx->tl[RBC3D_TLIST_WALL].v.p, -1.0, db.p); ++ctx->launches; }
  CUDA_TRY(cudaMemcpyAsync(b, db.p, sizeof(double) * W.ndof, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

// MinDistToTri on the host (ModIntOnWalls.F90:480-577), for host callers of
// the reference's repulsion routines (ModRepulsion.F90:600).  x: x(3,3)
// column-major as the reference (x(l,:) = vertex l); any output may be NULL.
extern "C" rbc3d_status rbc3d_min_dist_to_tri(const double xtar[3], const double x[9], double* s0, double* t0,
                                              double x0[3], double* dist) {
  if (!xtar || !x) return RBC3D_ERR_ARG;
  double xv[3][3];
  for (int l = 0; l < 3; ++l)
    for (int c = 0; c < 3; ++c) xv[l][c] = x[l + 3 * c];
  double s = 0, t = 0;
  const double d = min_dist_to_tri(xtar, xv, s, t);
  if (s0) *s0 = s;
  if (t0) *t0 = t;
  if (x0)
    for (int c = 0; c < 3; ++c) x0[c] = (1 - s - t) * xv[0][c] + s * xv[1][c] + t * xv[2][c];
  if (dist) *dist = d;
  return RBC3D_OK;
}
