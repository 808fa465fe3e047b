// wallspec.cu -- learned spectral operator for the wall no-slip solve (no
// counterpart in the reference; NoSlipWall, ModNoSlip.F90:45-150, starts
// every solve from a zero increment).
//
// The wall operator A of NoSlipWall (the self-wall quadrature plus the wall
// PME, MyMatMult ModNoSlip.F90:255-308) commutes with the translations of a
// tube meshed as a uniform stack of rings along the periodic z axis (up to
// the PME mesh error), so in the basis of axial Fourier modes it is block
// diagonal: one dim x dim block A_m per mode, dim = 3 vertices per ring.
// Every solved step gives a pair (b, x) with A x = b; transformed along z it
// gives one pair (b_m, x_m) per mode, and because A_m does not depend on
// where along the tube a pattern sits, a pair seen at one position teaches
// the operator at every position.  The model keeps per mode an orthonormal
// basis Q_m of the transformed right-hand sides seen so far (classical
// Gram-Schmidt, twice) and the matching solutions Z_m (the same
// combinations of the x_m, so A_m Z_m = Q_m); a new right-hand side is
// predicted as x_m = Z_m Q_m^H b_m, the least-squares fit of the solution
// on the pairs' span (exact once Q_m spans the whole block).  A direction is
// added only when its part orthogonal to Q_m exceeds tau times the mode's
// norm, so repeated or near-repeated pairs do not add noise.  The pairs are
// exact: b is A x formed with the FP64 operator (or the solve's right-hand
// side minus its true final residual), not the solve's right-hand side,
// whose mismatch at the solve tolerance Gram-Schmidt would amplify.
//
// As a right preconditioner of the solve (guess mode 5) a mode whose basis
// spans its block acts as M_m = Z_m Q_m^H, the block's inverse (A M = I up to
// the PME mesh's translation error); a mode with a partial basis is left
// alone (M_m = I).  Two completions of a partial basis measured slower than
// the plain solve on the tube (126 iterations, 10 pairs): the per-mode scalar
// c_m = sum Re<x_m, b_m> / sum ||b_m||^2 on the whole mode (234), and the
// same scalar on the basis' orthogonal complement, M_m = Z_m Q_m^H + c_m (I -
// Q_m Q_m^H) (209; the coupling block c_m Q^H A Q_perp of A M is large).
//
// Transforms: cuFFT D2Z / Z2D along the rings of the unique-vertex
// unknowns (index k*dim + j, k the ring, j = 3 * vertex-in-ring + component);
// the per-mode work is one CTA per mode in FP64.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <set>
#include <tuple>
#include <vector>

#include "ctx.hpp"

namespace {

constexpr int SPEC_THREADS = 256;
constexpr int SPEC_MAXDIM = 510;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {  // conj(a) b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// ||v||^2 of the block's shared vector (fixed summation order)
__device__ double block_norm2(const double2* v, int dim, double* red) {
  double s = 0;
  for (int e = threadIdx.x; e < dim; e += blockDim.x) s += v[e].x * v[e].x + v[e].y * v[e].y;
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  double t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  return t;
}

// h_j = <q_j, v> for j < n (one warp per j)
__device__ void block_dots(const double2* __restrict__ Qm, int dim, int n, const double2* v, double2* h) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = wid; j < n; j += nw) {
    const double2* q = Qm + (size_t)j * dim;
    double2 s = make_double2(0, 0);
    for (int e = lane; e < dim; e += 32) {
      const double2 t = cconjmul(q[e], v[e]);
      s.x += t.x; s.y += t.y;
    }
    s = warp_sum2(s);
    if (lane == 0) h[j] = s;
  }
  __syncthreads();
}

// One CTA per mode: Gram-Schmidt (two passes) of the pair (b_m, x_m) against
// the mode's basis; the orthogonal part is appended when large enough.
__global__ void __launch_bounds__(SPEC_THREADS) k_spec_add(int dim, int kmax, double tau,
                                                           const double2* __restrict__ bh,
                                                           const double2* __restrict__ xh, double2* __restrict__ Q,
                                                           double2* __restrict__ Z, int* __restrict__ nb,
                                                           int* __restrict__ added) {
  __shared__ double2 v[SPEC_MAXDIM], z[SPEC_MAXDIM], h[SPEC_MAXDIM];
  __shared__ double red[SPEC_THREADS / 32];
  const int m = blockIdx.x;
  const int n = nb[m];
  double2* Qm = Q + (size_t)m * kmax * dim;
  double2* Zm = Z + (size_t)m * kmax * dim;
  for (int e = threadIdx.x; e < dim; e += blockDim.x) {
    v[e] = bh[(size_t)m * dim + e];
    z[e] = xh[(size_t)m * dim + e];
  }
  __syncthreads();
  const double n0 = sqrt(block_norm2(v, dim, red));
  for (int pass = 0; pass < 2 && n > 0; ++pass) {
    block_dots(Qm, dim, n, v, h);
    for (int e = threadIdx.x; e < dim; e += blockDim.x) {
      double2 av = v[e], az = z[e];
      for (int j = 0; j < n; ++j) {
        const double2 hq = cmul(h[j], Qm[(size_t)j * dim + e]), hz = cmul(h[j], Zm[(size_t)j * dim + e]);
        av.x -= hq.x; av.y -= hq.y;
        az.x -= hz.x; az.y -= hz.y;
      }
      v[e] = av;
      z[e] = az;
    }
    __syncthreads();
  }
  const double r = sqrt(block_norm2(v, dim, red));
  const bool grow = n0 > 0 && r > tau * n0 && n < kmax;
  if (grow) {
    const double ir = 1.0 / r;
    for (int e = threadIdx.x; e < dim; e += blockDim.x) {
      Qm[(size_t)n * dim + e] = make_double2(v[e].x * ir, v[e].y * ir);
      Zm[(size_t)n * dim + e] = make_double2(z[e].x * ir, z[e].y * ir);
    }
  }
  if (threadIdx.x == 0) {
    if (grow) nb[m] = n + 1;
    added[m] = grow ? 1 : 0;
  }
}

// One CTA per mode: x_m = Z_m Q_m^H b_m, and (ro not null) the part of b_m
// outside the basis, rem_m = b_m - Q_m Q_m^H b_m.
__global__ void __launch_bounds__(SPEC_THREADS) k_spec_predict(int dim, int kmax, const double2* __restrict__ bh,
                                                               const double2* __restrict__ Q,
                                                               const double2* __restrict__ Z,
                                                               const int* __restrict__ nb, double2* __restrict__ xo,
                                                               double2* __restrict__ ro) {
  __shared__ double2 v[SPEC_MAXDIM], h[SPEC_MAXDIM];
  const int m = blockIdx.x;
  const int n = nb[m];
  const double2* Qm = Q + (size_t)m * kmax * dim;
  const double2* Zm = Z + (size_t)m * kmax * dim;
  for (int e = threadIdx.x; e < dim; e += blockDim.x) v[e] = bh[(size_t)m * dim + e];
  __syncthreads();
  block_dots(Qm, dim, n, v, h);
  for (int e = threadIdx.x; e < dim; e += blockDim.x) {
    double2 ax = make_double2(0, 0), ar = v[e];
    for (int j = 0; j < n; ++j) {
      const double2 hz = cmul(h[j], Zm[(size_t)j * dim + e]), hq = cmul(h[j], Qm[(size_t)j * dim + e]);
      ax.x += hz.x; ax.y += hz.y;
      ar.x -= hq.x; ar.y -= hq.y;
    }
    xo[(size_t)m * dim + e] = ax;
    if (ro) ro[(size_t)m * dim + e] = ar;
  }
}

// One CTA per mode: the preconditioner, M_m v_m = Z_m Q_m^H v_m for a mode
// whose basis spans the block, else v_m.
__global__ void __launch_bounds__(SPEC_THREADS) k_spec_apply(int dim, int kmax, const double2* __restrict__ vh,
                                                             const double2* __restrict__ Q,
                                                             const double2* __restrict__ Z,
                                                             const int* __restrict__ nb,
                                                             double2* __restrict__ xo) {
  __shared__ double2 v[SPEC_MAXDIM], h[SPEC_MAXDIM];
  const int m = blockIdx.x;
  const int n = nb[m];
  if (n < dim) {  // partial basis: identity
    for (int e = threadIdx.x; e < dim; e += blockDim.x) xo[(size_t)m * dim + e] = vh[(size_t)m * dim + e];
    return;
  }
  const double2* Qm = Q + (size_t)m * kmax * dim;
  const double2* Zm = Z + (size_t)m * kmax * dim;
  for (int e = threadIdx.x; e < dim; e += blockDim.x) v[e] = vh[(size_t)m * dim + e];
  __syncthreads();
  block_dots(Qm, dim, n, v, h);
  for (int e = threadIdx.x; e < dim; e += blockDim.x) {
    double2 ax = make_double2(0, 0);
    for (int j = 0; j < n; ++j) {
      const double2 hz = cmul(h[j], Zm[(size_t)j * dim + e]);
      ax.x += hz.x; ax.y += hz.y;
    }
    xo[(size_t)m * dim + e] = ax;
  }
}

__global__ void k_scale(int n, double a, double* __restrict__ x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= a;
}

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

// The wall is a uniform stack of nring rings along z: unique vertex
// g = k * nper + i sits at the position of vertex i shifted by k Lz / nring,
// and shifting every element by one ring maps the triangulation onto itself.
bool ring_stack(const rbc3d_ctx* ctx, int nring, int nper) {
  const WallState& W = ctx->wall;
  const int nu = nring * nper;
  std::vector<double> px(3 * (size_t)nu, 0.0);
  std::vector<char> seen(nu, 0);
  for (int v = 0; v < W.nvert; ++v) {
    const int g = W.hglb[v];
    if (g < 0 || g >= nu) return false;
    if (!seen[g]) {
      seen[g] = 1;
      for (int c = 0; c < 3; ++c) px[3 * (size_t)g + c] = W.hx[v + (size_t)c * W.nvert];
    }
  }
  for (char s : seen)
    if (!s) return false;
  const double Lz = ctx->prm.Lb[2], dz = Lz / nring;
  const double tol = 1e-9 * std::max({ctx->prm.Lb[0], ctx->prm.Lb[1], Lz});
  for (int k = 0; k < nring; ++k)
    for (int i = 0; i < nper; ++i) {
      const size_t g = (size_t)k * nper + i;
      const double ddz = px[3 * g + 2] - px[3 * (size_t)i + 2] - k * dz;
      if (std::fabs(px[3 * g] - px[3 * (size_t)i]) > tol || std::fabs(px[3 * g + 1] - px[3 * (size_t)i + 1]) > tol ||
          std::fabs(ddz - std::round(ddz / Lz) * Lz) > tol)
        return false;
    }
  std::set<std::tuple<int, int, int>> tri;
  auto key = [](int a, int b, int c) {
    int t[3] = {a, b, c};
    std::sort(t, t + 3);
    return std::make_tuple(t[0], t[1], t[2]);
  };
  for (int e = 0; e < W.nele; ++e)
    tri.insert(key(W.hglb[W.he2v[e]], W.hglb[W.he2v[e + W.nele]], W.hglb[W.he2v[e + 2 * (size_t)W.nele]]));
  auto shift = [&](int g) { return (g + nper) % nu; };
  for (const auto& t : tri)
    if (!tri.count(key(shift(std::get<0>(t)), shift(std::get<1>(t)), shift(std::get<2>(t))))) return false;
  return true;
}

// forward transform of x_dev (left unchanged: the transform reads a copy)
rbc3d_status forward(rbc3d_ctx* ctx, const double* x_dev, double2* out) {
  WallSpec& S = ctx->wspec;
  CUDA_TRY(cudaMemcpyAsync(S.fin.p, x_dev, sizeof(double) * S.nring * S.dim, cudaMemcpyDeviceToDevice, ctx->st));
  if (cufftSetStream(S.d2z, ctx->st) != CUFFT_SUCCESS ||
      cufftExecD2Z(S.d2z, S.fin.p, reinterpret_cast<cufftDoubleComplex*>(out)) != CUFFT_SUCCESS)
    return ctx_fail(ctx, RBC3D_ERR_CUDA, "wall spectral model: cufftExecD2Z");
  return RBC3D_OK;
}

// inverse transform of in (overwritten) to out, normalised
rbc3d_status inverse(rbc3d_ctx* ctx, double2* in, double* out) {
  WallSpec& S = ctx->wspec;
  if (cufftSetStream(S.z2d, ctx->st) != CUFFT_SUCCESS ||
      cufftExecZ2D(S.z2d, reinterpret_cast<cufftDoubleComplex*>(in), out) != CUFFT_SUCCESS)
    return ctx_fail(ctx, RBC3D_ERR_CUDA, "wall spectral model: cufftExecZ2D");
  const int n = S.nring * S.dim;
  k_scale<<<nblk(n, 256), 256, 0, ctx->st>>>(n, 1.0 / S.nring, out);
  ++ctx->launches;
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

}  // namespace

void wall_spec_release(rbc3d_ctx* ctx) {
  WallSpec& S = ctx->wspec;
  if (S.d2z) cufftDestroy(S.d2z);
  if (S.z2d) cufftDestroy(S.z2d);
  S.d2z = S.z2d = 0;
  S.Q.release(); S.Z.release(); S.nb.release(); S.bh.release(); S.xh.release(); S.rh.release();
  S.tmp.release(); S.fin.release(); S.added.release();
  S.ready = false;
  S.record = false;
  S.pairs = 0;
}

rbc3d_status wall_spec_add_dev(rbc3d_ctx* ctx, const double* b_dev, const double* x_dev) {
  WallSpec& S = ctx->wspec;
  if (!S.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model not initialised");
  rbc3d_status s;
  if ((s = forward(ctx, b_dev, S.bh.p)) || (s = forward(ctx, x_dev, S.xh.p))) return s;
  k_spec_add<<<S.nm, SPEC_THREADS, 0, ctx->st>>>(S.dim, S.kmax, S.tau, S.bh.p, S.xh.p, S.Q.p, S.Z.p, S.nb.p,
                                                 S.added.p);
  ++ctx->launches;
  CUDA_TRY(cudaGetLastError());
  ++S.pairs;
  return RBC3D_OK;
}

rbc3d_status wall_spec_predict_dev(rbc3d_ctx* ctx, const double* b_dev, double* x0_dev, double* rem_dev) {
  WallSpec& S = ctx->wspec;
  if (!S.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model not initialised");
  rbc3d_status s;
  if ((s = forward(ctx, b_dev, S.bh.p))) return s;
  k_spec_predict<<<S.nm, SPEC_THREADS, 0, ctx->st>>>(S.dim, S.kmax, S.bh.p, S.Q.p, S.Z.p, S.nb.p, S.xh.p,
                                                     rem_dev ? S.rh.p : nullptr);
  ++ctx->launches;
  CUDA_TRY(cudaGetLastError());
  if ((s = inverse(ctx, S.xh.p, x0_dev))) return s;
  if (rem_dev && (s = inverse(ctx, S.rh.p, rem_dev))) return s;
  return RBC3D_OK;
}

// out = M v (the preconditioner above); v_dev is left unchanged
rbc3d_status wall_spec_apply_dev(rbc3d_ctx* ctx, const double* v_dev, double* out_dev) {
  WallSpec& S = ctx->wspec;
  if (!S.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model not initialised");
  rbc3d_status s;
  if ((s = forward(ctx, v_dev, S.bh.p))) return s;
  k_spec_apply<<<S.nm, SPEC_THREADS, 0, ctx->st>>>(S.dim, S.kmax, S.bh.p, S.Q.p, S.Z.p, S.nb.p, S.xh.p);
  ++ctx->launches;
  CUDA_TRY(cudaGetLastError());
  return inverse(ctx, S.xh.p, out_dev);
}

extern "C" rbc3d_status rbc3d_wall_spectral_init(rbc3d_ctx* ctx, int nring, double tau, int record) {
  if (!ctx) return RBC3D_ERR_ARG;
  WallState& W = ctx->wall;
  if (W.nvert == 0) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model: no wall set");
  if (nring < 2 || W.ndof % (3 * nring) != 0 || !(tau > 0 && tau < 1))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "wall spectral model: bad ring count or tau");
  const int nper = W.ndof / (3 * nring);
  if (3 * nper > SPEC_MAXDIM) return ctx_fail(ctx, RBC3D_ERR_ARG, "wall spectral model: more than 170 vertices per ring");
  if (!ring_stack(ctx, nring, nper))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "wall spectral model: the wall is not a uniform ring stack along z");
  wall_spec_release(ctx);
  WallSpec& S = ctx->wspec;
  S.nring = nring;
  S.dim = 3 * nper;
  S.nm = nring / 2 + 1;
  S.kmax = S.dim;
  S.tau = tau;
  S.record = record != 0;
  const size_t nb = (size_t)S.nm * S.kmax * S.dim;
  CUDA_TRY(S.Q.alloc(nb)); CUDA_TRY(S.Z.alloc(nb));
  CUDA_TRY(S.nb.alloc(S.nm)); CUDA_TRY(S.added.alloc(S.nm));
  CUDA_TRY(S.bh.alloc((size_t)S.nm * S.dim)); CUDA_TRY(S.xh.alloc((size_t)S.nm * S.dim));
  CUDA_TRY(S.rh.alloc((size_t)S.nm * S.dim));
  CUDA_TRY(S.tmp.alloc(2 * (size_t)W.ndof)); CUDA_TRY(S.fin.alloc(W.ndof));
  CUDA_TRY(cudaMemsetAsync(S.nb.p, 0, sizeof(int) * S.nm, ctx->st));
  int n[1] = {nring}, inr[1] = {nring}, onm[1] = {S.nm};
  if (cufftPlanMany(&S.d2z, 1, n, inr, S.dim, 1, onm, S.dim, 1, CUFFT_D2Z, S.dim) != CUFFT_SUCCESS ||
      cufftPlanMany(&S.z2d, 1, n, onm, S.dim, 1, inr, S.dim, 1, CUFFT_Z2D, S.dim) != CUFFT_SUCCESS) {
    wall_spec_release(ctx);
    return ctx_fail(ctx, RBC3D_ERR_CUDA, "wall spectral model: cufftPlanMany");
  }
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  S.ready = true;
  return RBC3D_OK;
}

extern "C" rbc3d_status rbc3d_wall_spectral_add(rbc3d_ctx* ctx, const double* x, int* added) {
  if (!ctx || !x) return RBC3D_ERR_ARG;
  WallSpec& S = ctx->wspec;
  if (!S.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model not initialised");
  if (!ctx->wall.prepared) return ctx_fail(ctx, RBC3D_ERR_STATE, "PrepareSingIntOnWall not called");
  const int n = ctx->wall.ndof;
  // the pair (A x, x) with the FP64 wall operator (MyMatMult): exact, whatever
  // tolerance the solve that produced x stopped at
  CUDA_TRY(cudaMemcpyAsync(S.tmp.p + n, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
  // MyMatMult overwrites the wall density; the caller's density is kept
  const size_t nf = 3 * (size_t)ctx->wall.nvert;
  DBuf<double> fsave;
  CUDA_TRY(fsave.alloc(nf));
  CUDA_TRY(cudaMemcpyAsync(fsave.p, ctx->wall.f.p, sizeof(double) * nf, cudaMemcpyDeviceToDevice, ctx->st));
  rbc3d_status s = wall_matmult_dev(ctx, RBC3D_FP64, S.tmp.p + n, S.tmp.p);
  CUDA_TRY(cudaMemcpyAsync(ctx->wall.f.p, fsave.p, sizeof(double) * nf, cudaMemcpyDeviceToDevice, ctx->st));
  if (s) return s;
  if ((s = wall_spec_add_dev(ctx, S.tmp.p, S.tmp.p + n))) return s;
  if (added) {
    std::vector<int> a(S.nm);
    CUDA_TRY(cudaMemcpyAsync(a.data(), S.added.p, sizeof(int) * S.nm, cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
    int t = 0;
    for (int v : a) t += v;
    *added = t;
  }
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

extern "C" rbc3d_status rbc3d_wall_spectral_predict(rbc3d_ctx* ctx, const double* b, double* x0, double* rem) {
  if (!ctx || !b || !x0) return RBC3D_ERR_ARG;
  WallSpec& S = ctx->wspec;
  if (!S.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model not initialised");
  const int n = ctx->wall.ndof;
  CUDA_TRY(cudaMemcpyAsync(S.tmp.p, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
  DBuf<double> out;
  CUDA_TRY(out.alloc(2 * (size_t)n));
  rbc3d_status s = wall_spec_predict_dev(ctx, S.tmp.p, out.p, rem ? out.p + n : nullptr);
  if (s) return s;
  CUDA_TRY(cudaMemcpyAsync(x0, out.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st));
  if (rem) CUDA_TRY(cudaMemcpyAsync(rem, out.p + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

extern "C" rbc3d_status rbc3d_wall_spectral_size(rbc3d_ctx* ctx, int* nmodes, int* nbasis, long long* pairs) {
  if (!ctx) return RBC3D_ERR_ARG;
  WallSpec& S = ctx->wspec;
  if (nmodes) *nmodes = S.ready ? S.nm : 0;
  if (pairs) *pairs = S.pairs;
  if (nbasis && S.ready) {
    CUDA_TRY(cudaMemcpyAsync(nbasis, S.nb.p, sizeof(int) * S.nm, cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
  }
  return RBC3D_OK;
}
