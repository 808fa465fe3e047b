// gmres.cuh -- restarted GMRES on the device (FP64), the KSPGMRES defaults
// the reference configures in NoSlipWall (ModNoSlip.F90:69-87) and
// Solve_RBC_Vel (ModVelSolver.F90:74-90): classical Gram-Schmidt without
// refinement, Givens rotations, PCNONE, converged when the true residual
// ||b - A x|| < rtol ||b|| (KSPConvergedDefault); a cycle ends on the Givens
// estimate and the true residual after the update decides.  The Krylov basis,
// Hessenberg matrix and rotations stay on the device; one scalar per
// iteration is read back for the convergence test.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.hpp"

namespace {

// ---- GMRES kernels (FP64)
__global__ void k_dots(int n, int nv, const double* __restrict__ V, size_t ld, const double* __restrict__ w,
                       double* __restrict__ out) {
  // block j computes V_j . w
  int j = blockIdx.x;
  if (j >= nv) return;
  const double* vj = V + (size_t)j * ld;
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += vj[i] * w[i];
  __shared__ double red[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.;
    t = warp_sum(t);
    if (threadIdx.x == 0) out[j] = t;
  }
}
// Sliced dot products for the Arnoldi step: block (slice, j) sums V_j . w
// over rows [slice*kDotRows, (slice+1)*kDotRows); k_dots_sum then adds the
// slices of each j in slice order.  Fixed summation order (deterministic), and
// (j, slice) blocks fill the GPU where one block per basis vector would not.
constexpr int kDotRows = 2048;
constexpr int kDotThreads = 256;
__global__ void __launch_bounds__(kDotThreads) k_dots_part(int n, const double* __restrict__ V, size_t ld,
                                                           const double* __restrict__ w, double* __restrict__ part,
                                                           int nslice) {
  const int sl = blockIdx.x, j = blockIdx.y;
  const double* vj = V + (size_t)j * ld;
  const int i1 = min(n, (sl + 1) * kDotRows);
  double s = 0;
  for (int i = sl * kDotRows + threadIdx.x; i < i1; i += kDotThreads) s += vj[i] * w[i];
  __shared__ double red[kDotThreads / 32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < kDotThreads / 32; ++k) t += red[k];
    part[(size_t)j * nslice + sl] = t;
  }
}
__global__ void k_dots_sum(int nv, int nslice, const double* __restrict__ part, double* __restrict__ out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  double s = 0;
  for (int k = 0; k < nslice; ++k) s += part[(size_t)j * nslice + k];
  out[j] = s;
}
__global__ void k_orth(int n, int nv, const double* __restrict__ V, size_t ld, const double* __restrict__ h,
                       double* __restrict__ w) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = w[i];
  for (int j = 0; j < nv; ++j) s -= h[j] * V[(size_t)j * ld + i];
  w[i] = s;
}
__global__ void k_axpby(int n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}
// Givens / Hessenberg step for column k (single thread).  H column-major with
// leading dimension ldh = restart+1.  Writes |g_{k+1}| to res.
__global__ void k_givens(int k, int ldh, double* H, const double* hcol, double hn, double* cs, double* sn,
                         double* g, double* res) {
  if (threadIdx.x || blockIdx.x) return;
  double* c = H + (size_t)ldh * k;
  for (int j = 0; j <= k; ++j) c[j] = hcol[j];
  c[k + 1] = hn;
  for (int j = 0; j < k; ++j) {
    double a = c[j], b = c[j + 1];
    c[j] = cs[j] * a + sn[j] * b;
    c[j + 1] = -sn[j] * a + cs[j] * b;
  }
  double a = c[k], b = c[k + 1];
  double den = sqrt(a * a + b * b);
  cs[k] = den > 0 ? a / den : 1.;
  sn[k] = den > 0 ? b / den : 0.;
  c[k] = den;
  c[k + 1] = 0.;
  g[k + 1] = -sn[k] * g[k];
  g[k] = cs[k] * g[k];
  *res = fabs(g[k + 1]);
}
__global__ void k_backsolve(int k, int ldh, const double* H, const double* g, double* y) {
  if (threadIdx.x || blockIdx.x) return;
  for (int i = k - 1; i >= 0; --i) {
    double s = g[i];
    for (int j = i + 1; j < k; ++j) s -= H[i + (size_t)ldh * j] * y[j];
    y[i] = s / H[i + (size_t)ldh * i];
  }
}
__global__ void k_xupdate(int n, int k, const double* __restrict__ V, size_t ld, const double* __restrict__ y,
                          double* __restrict__ x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = x[i];
  for (int j = 0; j < k; ++j) s += y[j] * V[(size_t)j * ld + i];
  x[i] = s;
}


inline int gm_nblk(long long n, int b) { return (int)((n + b - 1) / b); }

// out[j] = V_j . w for j < nv (device), on the context stream.  Partial sums
// go to ctx->dotpart; without room for them one block per j does the sum.
inline void dev_dots(rbc3d_ctx* ctx, int n, int nv, const double* V, size_t ld, const double* w, double* out) {
  const int nslice = gm_nblk(n, kDotRows);
  if (nslice <= 1 || ctx->dotpart.alloc((size_t)nv * nslice) != cudaSuccess) {
    k_dots<<<nv, 512, 0, ctx->st>>>(n, nv, V, ld, w, out);
    ++ctx->launches;
    return;
  }
  k_dots_part<<<dim3(nslice, nv), kDotThreads, 0, ctx->st>>>(n, V, ld, w, ctx->dotpart.p, nslice);
  k_dots_sum<<<gm_nblk(nv, 128), 128, 0, ctx->st>>>(nv, nslice, ctx->dotpart.p, out);
  ctx->launches += 2;
}

inline double dev_norm(rbc3d_ctx* ctx, int n, const double* v, double* tmp) {
  dev_dots(ctx, n, 1, v, 0, v, tmp);
  double h = 0;
  cudaMemcpyAsync(&h, tmp, sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
  cudaStreamSynchronize(ctx->st);
  return std::sqrt(h);
}

// No preconditioner (the reference's PCNONE).
struct NoPrec {
  bool active() const { return false; }
  rbc3d_status operator()(const double*, double*) const { return RBC3D_OK; }
};

// GMRES cycles from x (device, in/out) for A x = b (device).  On entry r must
// hold b - A x and beta its norm; ttol is the absolute tolerance.  Counts go
// to S (iterations, converged, rnorm; matvecs through the functor).  With an
// active preconditioner M (pc(in, out): out = M in) the cycles run on A M
// (right preconditioning: the Arnoldi vectors are z = M v, the update is
// x += M V y), so the residual they minimise and the convergence test are
// still those of b - A x.
template <class MV, class PC = NoPrec>
rbc3d_status gmres_cycles(rbc3d_ctx* ctx, int n, MV&& matvec, const double* b, double* x, double* r, double beta,
                          double ttol, int max_it, int R, rbc3d_solve_stats& S, PC&& pc = PC()) {
  const size_t ld = (size_t)n;
  DBuf<double> V, w, H, cs, sn, g, hcol, yv, tmp, z, u;
  if (pc.active()) { CUDA_TRY(z.alloc(n)); CUDA_TRY(u.alloc(n)); }
  CUDA_TRY(V.alloc((size_t)(R + 1) * ld)); CUDA_TRY(w.alloc(n));
  CUDA_TRY(H.alloc((size_t)(R + 1) * R)); CUDA_TRY(cs.alloc(R)); CUDA_TRY(sn.alloc(R)); CUDA_TRY(g.alloc(R + 1));
  CUDA_TRY(hcol.alloc(R + 1)); CUDA_TRY(yv.alloc(R)); CUDA_TRY(tmp.alloc(R + 2));
  rbc3d_status s;
  auto residual = [&]() -> rbc3d_status {  // r = b - A x
    rbc3d_status e = matvec(x, w.p);
    if (e) return e;
    CUDA_TRY(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    { k_axpby<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, -1.0, w.p, 1.0, r); ++ctx->launches; }
    return RBC3D_OK;
  };
  int its = 0;
  bool conv = beta <= ttol;
  while (!conv && its < max_it) {
    { k_axpby<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, 1.0 / beta, r, 0.0, V.p); ++ctx->launches; }
    std::vector<double> gh(R + 1, 0.);
    gh[0] = beta;
    CUDA_TRY(cudaMemcpyAsync(g.p, gh.data(), sizeof(double) * (R + 1), cudaMemcpyHostToDevice, ctx->st));
    int k;
    for (k = 0; k < R && its < max_it; ++k) {
      if (pc.active()) {
        if ((s = pc(V.p + k * ld, z.p)) || (s = matvec(z.p, w.p))) return s;
      } else if ((s = matvec(V.p + k * ld, w.p))) {
        return s;
      }
      dev_dots(ctx, n, k + 1, V.p, ld, w.p, hcol.p);
      { k_orth<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, k + 1, V.p, ld, hcol.p, w.p); ++ctx->launches; }
      double hn = dev_norm(ctx, n, w.p, tmp.p);
      if (hn > 0) { k_axpby<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, 1.0 / hn, w.p, 0.0, V.p + (k + 1) * ld); ++ctx->launches; }
      { k_givens<<<1, 1, 0, ctx->st>>>(k, R + 1, H.p, hcol.p, hn, cs.p, sn.p, g.p, tmp.p + R + 1); ++ctx->launches; }
      double res = 0;
      CUDA_TRY(cudaMemcpyAsync(&res, tmp.p + R + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
      CUDA_TRY(cudaStreamSynchronize(ctx->st));
      ++its;
      if (res <= ttol || hn == 0) { ++k; conv = true; break; }
    }
    { k_backsolve<<<1, 1, 0, ctx->st>>>(k, R + 1, H.p, g.p, yv.p); ++ctx->launches; }
    if (pc.active()) {  // x += M (V y)
      CUDA_TRY(cudaMemsetAsync(u.p, 0, sizeof(double) * n, ctx->st));
      { k_xupdate<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, k, V.p, ld, yv.p, u.p); ++ctx->launches; }
      if ((s = pc(u.p, z.p))) return s;
      { k_axpby<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, 1.0, z.p, 1.0, x); ++ctx->launches; }
    } else {
      k_xupdate<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, k, V.p, ld, yv.p, x);
      ++ctx->launches;
    }
    if ((s = residual())) return s;
    beta = dev_norm(ctx, n, r, tmp.p);
    conv = beta <= ttol;  // the true residual decides, not the Givens estimate
  }
  S.iterations = its;
  S.converged = conv ? 1 : 0;
  S.rnorm = beta;
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// Mixed-precision solve (GMRES with iterative refinement): the residual
// r = b - A x is formed with the FP64 operator (mv64) and the correction
// A d = r is solved by inner GMRES cycles on the FP32 operator (mv32, FP64
// Arnoldi and Hessenberg) to a relative reduction eta, then x += d.  Each
// refinement lowers the FP64 residual by about max(eta, the FP32 operator's
// relative error), so the solve reaches the same ||b - A x|| < ttol as the FP64
// solve, judged by the FP64 residual.  On entry r and beta hold the FP64
// residual of x.  S.iterations counts the inner iterations, S.refinements the
// corrections.  An active preconditioner pc acts in the inner cycles.
template <class MV64, class MV32, class PC = NoPrec>
rbc3d_status gmres_ir(rbc3d_ctx* ctx, int n, MV64&& mv64, MV32&& mv32, const double* b, double* x, double* r,
                      double beta, double ttol, int max_it, int R, double eta, rbc3d_solve_stats& S,
                      PC&& pc = PC()) {
  DBuf<double> rhs, d, ri, w;
  CUDA_TRY(rhs.alloc(n)); CUDA_TRY(d.alloc(n)); CUDA_TRY(ri.alloc(n)); CUDA_TRY(w.alloc(n));
  rbc3d_status s;
  int its = 0, refinements = 0;
  const int max_refine = 32;
  bool conv = beta <= ttol;
  while (!conv && its < max_it && refinements < max_refine) {
    // inner: A32 d = r from d = 0, to max(eta ||r||, ttol / 2)
    CUDA_TRY(cudaMemcpyAsync(rhs.p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    CUDA_TRY(cudaMemcpyAsync(ri.p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    CUDA_TRY(cudaMemsetAsync(d.p, 0, sizeof(double) * n, ctx->st));
    rbc3d_solve_stats Si{};
    if ((s = gmres_cycles(ctx, n, mv32, rhs.p, d.p, ri.p, beta, std::max(eta * beta, 0.5 * ttol), max_it - its, R, Si, pc)))
      return s;
    its += Si.iterations;
    ++refinements;
    { k_axpby<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, 1.0, d.p, 1.0, x); ++ctx->launches; }
    // FP64 residual of the corrected x
    if ((s = mv64(x, w.p))) return s;
    CUDA_TRY(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    { k_axpby<<<gm_nblk(n, 256), 256, 0, ctx->st>>>(n, -1.0, w.p, 1.0, r); ++ctx->launches; }
    const double nb = dev_norm(ctx, n, r, w.p);
    if (!(nb < beta) && Si.iterations == 0) { beta = nb; break; }  // no progress possible
    beta = nb;
    conv = beta <= ttol;
  }
  S.iterations = its;
  S.refinements = refinements;
  S.converged = conv ? 1 : 0;
  S.rnorm = beta;
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

}  // namespace
