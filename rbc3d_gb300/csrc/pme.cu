// pme.cu -- smooth-particle-mesh Ewald of ModPME.F90 on one GPU.
//
//   PME_Distrib_Source (ModPME.F90:58-133, 405-443): B-spline spreading of
//     c1*f (3 grids) and c2*g (x) Bcoef*a3 (9 grids) with global atomics;
//     walls spread one centroid source per triangle.
//   PME_Transform (ModPME.F90:137-222): batched 3-D R2C FFTs (cuFFT), one
//     fused kernel for the Stokeslet / stresslet influence and the B-spline
//     factor bb, 3 C2R FFTs.  Unnormalised, as Get_That / Get_R.
//   PME_Add_Interp_Vel (ModPME.F90:228-248, 450-489): B-spline gather.
//
// FFT conventions.  The reference transforms z with sign +1 forward and -1
// backward (ModPFFTW.F90:110-111) and compensates by negating kz in the wave
// numbers (ModPME.F90:303).  Here all three axes use the standard -1 forward
// transform, so index m along z carries qz = m/Lz for m <= Nz/2 and
// (m-Nz)/Lz above (the reference's Nyquist z plane keeps +Nz/(2Lz)).  FFTW's
// c2r ignores the imaginary parts of the kx = 0 and kx = Nx/2 planes after
// the y and z passes; that equals replacing those planes by their Hermitian
// part, which the influence kernel does explicitly so any C2R algorithm
// reproduces the reference.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.hpp"

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

template <typename R> struct C2;
template <> struct C2<float> { typedef float2 T; };
template <> struct C2<double> { typedef double2 T; };

struct SpreadArgs {
  int n;               // sources
  const double* x;     // 3n
  const double* f;     // 3n (already f*dS)  or null
  const double* g;     // 3n (g*dS*Bcoef)    or null
  const double* a3;    // 3n
  int N[3];
  double ih[3];
  int P;
  double c1, c2;
  int sl, dl;
  size_t G;
};

// x*ih in FP64, then the B-spline recursion in R (all its values are O(1)).
template <typename R>
__device__ __forceinline__ void weights(double x, double ih, int P, int& imin, R* w) {
  double xc = x * ih;
  imin = (int)floor(xc) - (P - 1);
  R u0 = (R)((double)imin - (xc - (double)P));
  R u[8];
  u[0] = u0;
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

template <typename R>
__global__ void k_spread(SpreadArgs a, R* __restrict__ grid) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  R wx[8], wy[8], wz[8];
  int imin, jmin, kmin;
  weights<R>(a.x[p], a.ih[0], a.P, imin, wx);
  weights<R>(a.x[p + a.n], a.ih[1], a.P, jmin, wy);
  weights<R>(a.x[p + 2 * (size_t)a.n], a.ih[2], a.P, kmin, wz);
  R fv[3] = {0, 0, 0}, tv[9];
  if (a.sl)
    for (int k = 0; k < 3; ++k) fv[k] = (R)(a.c1 * a.f[p + (size_t)k * a.n]);
  if (a.dl) {
    double gg[3], aa[3];
    for (int k = 0; k < 3; ++k) { gg[k] = a.g[p + (size_t)k * a.n]; aa[k] = a.a3[p + (size_t)k * a.n]; }
    for (int ii = 0; ii < 3; ++ii)
      for (int jj = 0; jj < 3; ++jj) tv[ii + 3 * jj] = (R)(a.c2 * (gg[ii] * aa[jj]));
  }
  for (int k0 = 0; k0 < a.P; ++k0) {
    int k = imod(kmin + k0, a.N[2]);
    for (int j0 = 0; j0 < a.P; ++j0) {
      int j = imod(jmin + j0, a.N[1]);
      R wyz = wy[j0] * wz[k0];
      size_t row = (size_t)a.N[0] * (j + (size_t)a.N[1] * k);
      for (int i0 = 0; i0 < a.P; ++i0) {
        int i = imod(imin + i0, a.N[0]);
        R wxyz = wx[i0] * wyz;
        size_t q = row + i;
        if (a.sl)
          for (int c = 0; c < 3; ++c) atomicAdd(grid + q + c * a.G, wxyz * fv[c]);
        if (a.dl)
          for (int c = 0; c < 9; ++c) atomicAdd(grid + (3 + c) * a.G + q, wxyz * tv[c]);
      }
    }
  }
}

// Wall centroid sources (ModPME.F90:104-131): x = mean of the vertices,
// f = mean vertex density * element area.
__global__ void k_wall_sources(int nele, int nvert, const int* __restrict__ e2v, const double* __restrict__ x,
                               const double* __restrict__ f, const double* __restrict__ area,
                               double* __restrict__ xs, double* __restrict__ fs) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  int v0 = e2v[e], v1 = e2v[e + nele], v2 = e2v[e + 2 * (size_t)nele];
  for (int k = 0; k < 3; ++k) {
    size_t o = (size_t)k * nvert;
    xs[e + (size_t)k * nele] = (1.0 / 3) * (x[v0 + o] + x[v1 + o] + x[v2 + o]);
    fs[e + (size_t)k * nele] = (1.0 / 3) * (f[v0 + o] + f[v1 + o] + f[v2 + o]) * area[e];
  }
}

struct InflArgs {
  int N1, N2, N3, NH;
  size_t GC;
  double iL[3];
  double alpha, vol;
  int sl, dl;
  const double* bbx;
  const double* bby;
  const double* bbz;
};

template <typename R, typename CT>
__device__ __forceinline__ void influence(const InflArgs& a, const CT* __restrict__ F, int i, int j, int k, CT* out) {
  size_t q = (size_t)i + (size_t)a.NH * (j + (size_t)a.N2 * k);
  if (i == 0 && j == 0 && k == 0) {
    for (int d = 0; d < 3; ++d) { out[d].x = 0; out[d].y = 0; }
    return;
  }
  R qv[3];
  qv[0] = (R)(i * a.iL[0]);
  qv[1] = (R)((j < a.N2 / 2) ? j * a.iL[1] : (j - a.N2) * a.iL[1]);
  qv[2] = (R)((2 * k <= a.N3) ? k * a.iL[2] : (k - a.N3) * a.iL[2]);
  const R PI_ = (R)RBC3D_PI;
  const R alpha = (R)a.alpha;
  R sq = (R)sqrt(RBC3D_PI * a.alpha);
  R qt[3] = {sq * qv[0], sq * qv[1], sq * qv[2]};
  R q2 = qv[0] * qv[0] + qv[1] * qv[1] + qv[2] * qv[2];
  R q2t = PI_ * alpha * q2;
  R e = exp(-q2t);
  R phi0 = e / q2t, phi1 = (e + phi0) / q2t;
  R vr[3] = {0, 0, 0}, vi[3] = {0, 0, 0};
  if (a.sl) {
    CT Fv[3] = {F[q], F[q + a.GC], F[q + 2 * a.GC]};
    R qfr = qt[0] * Fv[0].x + qt[1] * Fv[1].x + qt[2] * Fv[2].x;
    R qfi = qt[0] * Fv[0].y + qt[1] * Fv[1].y + qt[2] * Fv[2].y;
    R s = (R)2 * alpha / (R)a.vol * phi1;
    for (int d = 0; d < 3; ++d) {
      vr[d] += s * (q2t * Fv[d].x - qt[d] * qfr);
      vi[d] += s * (q2t * Fv[d].y - qt[d] * qfi);
    }
  }
  if (a.dl) {
    CT T[3][3];
    for (int aa = 0; aa < 3; ++aa)
      for (int bb = 0; bb < 3; ++bb) T[aa][bb] = F[q + (size_t)(3 + aa + 3 * bb) * a.GC];
    R trr = T[0][0].x + T[1][1].x + T[2][2].x, tri = T[0][0].y + T[1][1].y + T[2][2].y;
    R qTqr = 0, qTqi = 0;
    for (int aa = 0; aa < 3; ++aa) {
      R tr_ = T[aa][0].x * qv[0] + T[aa][1].x * qv[1] + T[aa][2].x * qv[2];
      R ti_ = T[aa][0].y * qv[0] + T[aa][1].y * qv[1] + T[aa][2].y * qv[2];
      qTqr += qv[aa] * tr_;
      qTqi += qv[aa] * ti_;
    }
    R s0 = (R)4 * PI_ * alpha / (R)a.vol * phi0;
    R s1 = (R)8 * PI_ * PI_ * alpha * alpha / (R)a.vol * phi1;
    for (int d = 0; d < 3; ++d) {
      R wr = qv[d] * trr + (qv[0] * T[0][d].x + qv[1] * T[1][d].x + qv[2] * T[2][d].x) +
             (T[d][0].x * qv[0] + T[d][1].x * qv[1] + T[d][2].x * qv[2]);
      R wi = qv[d] * tri + (qv[0] * T[0][d].y + qv[1] * T[1][d].y + qv[2] * T[2][d].y) +
             (T[d][0].y * qv[0] + T[d][1].y * qv[1] + T[d][2].y * qv[2]);
      // tmp = i*s0*w - i*s1*(qTq)*q ;  v -= tmp   (i*(a+ib) = -b + ia)
      R tr_ = -s0 * wi + s1 * qTqi * qv[d];
      R ti_ = s0 * wr - s1 * qTqr * qv[d];
      vr[d] -= tr_;
      vi[d] -= ti_;
    }
  }
  R bb = (R)(a.bbx[i] * a.bby[j] * a.bbz[k]);
  for (int d = 0; d < 3; ++d) { out[d].x = bb * vr[d]; out[d].y = bb * vi[d]; }
}

template <typename R, typename CT>
__global__ void k_influence(InflArgs a, const CT* __restrict__ F, CT* __restrict__ V) {
  size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= a.GC) return;
  int i = (int)(idx % a.NH);
  int j = (int)((idx / a.NH) % a.N2);
  int k = (int)(idx / ((size_t)a.NH * a.N2));
  CT out[3];
  influence<R, CT>(a, F, i, j, k, out);
  if (i == 0 || 2 * i == a.N1) {
    // Hermitian part of the kx = 0 / Nx/2 planes
    CT op[3];
    int jp = (a.N2 - j) % a.N2, kp = (a.N3 - k) % a.N3;
    influence<R, CT>(a, F, i, jp, kp, op);
    for (int d = 0; d < 3; ++d) {
      out[d].x = (R)0.5 * (out[d].x + op[d].x);
      out[d].y = (R)0.5 * (out[d].y - op[d].y);
    }
  }
  for (int d = 0; d < 3; ++d) V[idx + d * a.GC] = out[d];
}

struct GatherArgs {
  int n;
  const double* x;
  const double* A;
  double* v;
  int N[3];
  double ih[3];
  int P;
  size_t G;
};

template <typename R>
__global__ void k_gather(GatherArgs a, const R* __restrict__ vel) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  R wx[8], wy[8], wz[8];
  int imin, jmin, kmin;
  weights<R>(a.x[p + 2 * (size_t)a.n], a.ih[2], a.P, kmin, wz);
  weights<R>(a.x[p + (size_t)a.n], a.ih[1], a.P, jmin, wy);
  weights<R>(a.x[p], a.ih[0], a.P, imin, wx);
  R dv[3] = {0, 0, 0};
  for (int k0 = 0; k0 < a.P; ++k0) {
    int k = imod(kmin + k0, a.N[2]);
    for (int j0 = 0; j0 < a.P; ++j0) {
      int j = imod(jmin + j0, a.N[1]);
      R wyz = wy[j0] * wz[k0];
      size_t row = (size_t)a.N[0] * (j + (size_t)a.N[1] * k);
      for (int i0 = 0; i0 < a.P; ++i0) {
        int i = imod(imin + i0, a.N[0]);
        R wxyz = wx[i0] * wyz;
        size_t q = row + i;
        dv[0] += wxyz * __ldg(vel + q);
        dv[1] += wxyz * __ldg(vel + q + a.G);
        dv[2] += wxyz * __ldg(vel + q + 2 * a.G);
      }
    }
  }
  double iA = 1.0 / a.A[p];
  for (int d = 0; d < 3; ++d) a.v[p + (size_t)d * a.n] += (double)dv[d] * iA;
}

rbc3d_status make_plans(rbc3d_ctx* ctx, int prec) {
  PmeState& P = ctx->pme;
  int n[3] = {P.N3, P.N2, P.N1};
  int idist = (int)P.G, odist = (int)P.GC;
  auto mk = [&](cufftHandle* h, cufftType t, int batch, bool fwd) -> cufftResult {
    return cufftPlanMany(h, 3, n, nullptr, 1, fwd ? idist : odist, nullptr, 1, fwd ? odist : idist, t, batch);
  };
  if (prec == RBC3D_FP32C && !P.planned32) {
    if (mk(&P.r2c32_3, CUFFT_R2C, 3, true) || mk(&P.r2c32_12, CUFFT_R2C, 12, true) || mk(&P.c2r32_3, CUFFT_C2R, 3, false))
      return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftPlanMany (FP32) failed");
    cufftSetStream(P.r2c32_3, ctx->st); cufftSetStream(P.r2c32_12, ctx->st); cufftSetStream(P.c2r32_3, ctx->st);
    P.planned32 = true;
  }
  if (prec == RBC3D_FP64 && !P.planned64) {
    if (mk(&P.r2c64_3, CUFFT_D2Z, 3, true) || mk(&P.r2c64_12, CUFFT_D2Z, 12, true) || mk(&P.c2r64_3, CUFFT_Z2D, 3, false))
      return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftPlanMany (FP64) failed");
    cufftSetStream(P.r2c64_3, ctx->st); cufftSetStream(P.r2c64_12, ctx->st); cufftSetStream(P.c2r64_3, ctx->st);
    P.planned64 = true;
  }
  return RBC3D_OK;
}

}  // namespace

// PME_Init (ModPME.F90:252-338): B-spline factors bb
rbc3d_status pme_setup(rbc3d_ctx* ctx) {
  PmeState& P = ctx->pme;
  P.N1 = ctx->prm.Nb[0]; P.N2 = ctx->prm.Nb[1]; P.N3 = ctx->prm.Nb[2];
  P.NH = P.N1 / 2 + 1;
  P.G = (size_t)P.N1 * P.N2 * P.N3;
  P.GC = (size_t)P.NH * P.N2 * P.N3;
  const int p = ctx->prm.P;
  // MP(1..P) = BsplineFunc(P + epsilon, P) (ModPME.F90:313)
  std::vector<double> MP(p), u(p);
  double xc = (double)p + 2.220446049250313e-16;
  int imin = (int)std::floor(xc) - (p - 1);
  u[0] = imin - (xc - p);
  for (int j = 1; j < p; ++j) u[j] = u[j - 1] + 1;
  MP[0] = 1.;
  for (int j = 1; j < p; ++j) MP[j] = 0.;
  for (int pp = 2; pp <= p; ++pp) {
    for (int j = pp; j >= 2; --j) MP[j - 1] = u[j - 1] / (pp - 1.) * MP[j - 1] + (pp - u[j - 1]) / (pp - 1.) * MP[j - 2];
    MP[0] = u[0] / (pp - 1.) * MP[0];
  }
  auto bfac = [&](int N, int kmax, std::vector<double>& out) {
    out.resize(kmax + 1);
    for (int k = 0; k <= kmax; ++k) {
      double br = 0, bi = 0;
      for (int m = 0; m <= p - 2; ++m) {
        double ang = RBC3D_TWO_PI * k * m / (double)N;
        br += MP[m] * std::cos(ang);
        bi += MP[m] * std::sin(ang);
      }
      out[k] = 1.0 / (br * br + bi * bi);  // |exp(i*theta)/b|^2
    }
  };
  std::vector<double> bx, by, bz;
  bfac(P.N1, P.N1 / 2, bx);
  bfac(P.N2, P.N2 - 1, by);
  bfac(P.N3, P.N3 - 1, bz);
  CUDA_TRY(P.bbx.upload(bx.data(), bx.size(), ctx->st));
  CUDA_TRY(P.bby.upload(by.data(), by.size(), ctx->st));
  CUDA_TRY(P.bbz.upload(bz.data(), bz.size(), ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status pme_release(rbc3d_ctx* ctx) {
  PmeState& P = ctx->pme;
  if (P.planned32) { cufftDestroy(P.r2c32_3); cufftDestroy(P.r2c32_12); cufftDestroy(P.c2r32_3); }
  if (P.planned64) { cufftDestroy(P.r2c64_3); cufftDestroy(P.r2c64_12); cufftDestroy(P.c2r64_3); }
  P.planned32 = P.planned64 = false;
  return RBC3D_OK;
}

rbc3d_status pme_spread(rbc3d_ctx* ctx, double c1, double c2, int cells, int walls, int prec) {
  PmeState& P = ctx->pme;
  if (prec != RBC3D_FP64) prec = RBC3D_FP32C;  // FP32C and FP32M share the FP32 PME
  P.sl = std::fabs(c1) > 1.e-10;  // flag_sing_lay, ModPME.F90:74
  P.dl = std::fabs(c2) > 1.e-10;  // flag_doub_lay
  P.prec = prec;
  P.ready = false;
  int ncomp = P.dl ? 12 : 3;
  SpreadArgs a;
  for (int d = 0; d < 3; ++d) { a.N[d] = ctx->prm.Nb[d]; a.ih[d] = ctx->prm.Nb[d] / ctx->prm.Lb[d]; }
  a.P = ctx->prm.P; a.G = P.G; a.c1 = c1; a.c2 = c2;
  if (prec == RBC3D_FP32C) {
    CUDA_TRY(P.grid32.alloc(12 * P.G));
    CUDA_TRY(cudaMemsetAsync(P.grid32.p, 0, sizeof(float) * ncomp * P.G, ctx->st));
  } else {
    CUDA_TRY(P.grid64.alloc(12 * P.G));
    CUDA_TRY(cudaMemsetAsync(P.grid64.p, 0, sizeof(double) * ncomp * P.G, ctx->st));
  }
  if (cells && ctx->npt > 0) {
    // a density that was never set is zero
    a.n = ctx->npt; a.x = ctx->s_x.p; a.f = ctx->s_f.p; a.g = ctx->s_g.p; a.a3 = ctx->s_a3.p;
    a.sl = P.sl && ctx->has_f; a.dl = P.dl && ctx->has_g;
    if (a.sl || a.dl) {
      if (prec == RBC3D_FP32C) { k_spread<float><<<nblk(a.n, 128), 128, 0, ctx->st>>>(a, P.grid32.p); ++ctx->launches; }
      else { k_spread<double><<<nblk(a.n, 128), 128, 0, ctx->st>>>(a, P.grid64.p); ++ctx->launches; }
      CUDA_TRY(cudaGetLastError());
    }
  }
  if (walls && ctx->wall.nele > 0 && P.sl) {
    WallState& W = ctx->wall;
    CUDA_TRY(W.src_x.alloc(3 * (size_t)W.nele));
    CUDA_TRY(W.src_f.alloc(3 * (size_t)W.nele));
    { k_wall_sources<<<nblk(W.nele, 256), 256, 0, ctx->st>>>(W.nele, W.nvert, W.e2v.p, W.x.p, W.f.p, W.area.p, W.src_x.p, W.src_f.p); ++ctx->launches; }
    a.n = W.nele; a.x = W.src_x.p; a.f = W.src_f.p; a.g = nullptr; a.a3 = nullptr; a.sl = 1; a.dl = 0;
    if (prec == RBC3D_FP32C) { k_spread<float><<<nblk(a.n, 128), 128, 0, ctx->st>>>(a, P.grid32.p); ++ctx->launches; }
    else { k_spread<double><<<nblk(a.n, 128), 128, 0, ctx->st>>>(a, P.grid64.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
  }
  return RBC3D_OK;
}

rbc3d_status pme_transform(rbc3d_ctx* ctx) {
  PmeState& P = ctx->pme;
  rbc3d_status s = make_plans(ctx, P.prec);
  if (s) return s;
  InflArgs a;
  a.N1 = P.N1; a.N2 = P.N2; a.N3 = P.N3; a.NH = P.NH; a.GC = P.GC;
  for (int d = 0; d < 3; ++d) a.iL[d] = ctx->iLb[d];
  a.alpha = ctx->prm.alpha; a.vol = ctx->prm.Lb[0] * ctx->prm.Lb[1] * ctx->prm.Lb[2];
  a.sl = P.sl; a.dl = P.dl;
  a.bbx = P.bbx.p; a.bby = P.bby.p; a.bbz = P.bbz.p;
  if (P.prec == RBC3D_FP32C) {
    CUDA_TRY(P.spec32.alloc(12 * P.GC)); CUDA_TRY(P.vspec32.alloc(3 * P.GC)); CUDA_TRY(P.vel32.alloc(3 * P.G));
    if (P.dl) { if (cufftExecR2C(P.r2c32_12, P.grid32.p, (cufftComplex*)P.spec32.p)) return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftExecR2C"); }
    else if (cufftExecR2C(P.r2c32_3, P.grid32.p, (cufftComplex*)P.spec32.p)) return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftExecR2C");
    { k_influence<float, float2><<<nblk(P.GC, 256), 256, 0, ctx->st>>>(a, P.spec32.p, P.vspec32.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
    if (cufftExecC2R(P.c2r32_3, (cufftComplex*)P.vspec32.p, P.vel32.p)) return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftExecC2R");
  } else {
    CUDA_TRY(P.spec64.alloc(12 * P.GC)); CUDA_TRY(P.vspec64.alloc(3 * P.GC)); CUDA_TRY(P.vel64.alloc(3 * P.G));
    if (P.dl) { if (cufftExecD2Z(P.r2c64_12, P.grid64.p, (cufftDoubleComplex*)P.spec64.p)) return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftExecD2Z"); }
    else if (cufftExecD2Z(P.r2c64_3, P.grid64.p, (cufftDoubleComplex*)P.spec64.p)) return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftExecD2Z");
    { k_influence<double, double2><<<nblk(P.GC, 256), 256, 0, ctx->st>>>(a, P.spec64.p, P.vspec64.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
    if (cufftExecZ2D(P.c2r64_3, (cufftDoubleComplex*)P.vspec64.p, P.vel64.p)) return ctx_fail(ctx, RBC3D_ERR_CUDA, "cufftExecZ2D");
  }
  P.ready = true;
  return RBC3D_OK;
}

rbc3d_status pme_gather(rbc3d_ctx* ctx, int tlist) {
  PmeState& P = ctx->pme;
  if (!P.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "PME_Transform not called");
  TargetSet& t = ctx->tl[tlist];
  if (t.n == 0) return RBC3D_OK;
  GatherArgs a;
  a.n = t.n; a.x = t.x.p; a.A = t.Acoef.p; a.v = t.v.p;
  for (int d = 0; d < 3; ++d) { a.N[d] = ctx->prm.Nb[d]; a.ih[d] = ctx->prm.Nb[d] / ctx->prm.Lb[d]; }
  a.P = ctx->prm.P; a.G = P.G;
  if (P.prec == RBC3D_FP32C) { k_gather<float><<<nblk(a.n, 128), 128, 0, ctx->st>>>(a, P.vel32.p); ++ctx->launches; }
  else { k_gather<double><<<nblk(a.n, 128), 128, 0, ctx->st>>>(a, P.vel64.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}
