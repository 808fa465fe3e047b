// pme.cu -- smooth-particle-mesh Ewald of ModPME.F90 on one GPU.
//
//   PME_Distrib_Source (ModPME.F90:58-133, 405-443): B-spline spreading of
//     c1*f (3 grids) and c2*g (x) Bcoef*a3 (9 grids); walls spread one
//     centroid source per triangle.  Sources are binned by 8^3 grid tiles
//     (once per position update); a CTA accumulates one tile's sources into
//     a (8+P-1)^3 box in shared memory and adds the box to the grids with
//     one global atomic per touched node.
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
#include <cub/cub.cuh>
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
  // fixed trip counts (guarded by P) keep w[] in registers
#pragma unroll
  for (int pp = 2; pp <= 8; ++pp) {
    if (pp > P) break;
    R inv = (R)1 / (R)(pp - 1);
#pragma unroll
    for (int j = pp; j >= 2; --j) w[j - 1] = u[j - 1] * inv * w[j - 1] + ((R)pp - u[j - 1]) * inv * w[j - 2];
    w[0] = u[0] * inv * w[0];
  }
}

constexpr int SPREAD_TILE = 8;     // grid nodes per tile edge
constexpr int SPREAD_CHUNK = 256;  // sources per CTA at most

struct TileArgs {
  int ntile[3];        // tiles per axis
  int B;               // box edge, SPREAD_TILE + P - 1
  int cg;              // grid planes per warp (3)
  const int2* sched;   // [rounds][32] stencil-node schedule
  int c0;              // first grid plane of the launch (3 per warp from there)
};

// Tile of each source's stencil origin (the stencil is x*ih - (P-1) .. x*ih).
__global__ void k_tile_keys(int n, const double* __restrict__ x, SpreadArgs a, TileArgs t, int* __restrict__ key,
                            int* __restrict__ idx) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int tc[3];
  for (int d = 0; d < 3; ++d) {
    int m = (int)floor(x[p + (size_t)d * n] * a.ih[d]) - (a.P - 1);
    tc[d] = imod(m, a.N[d]) / SPREAD_TILE;
  }
  key[p] = tc[0] + t.ntile[0] * (tc[1] + t.ntile[1] * tc[2]);
  idx[p] = p;
}

// Stencil-node schedule of the spread: lane l handles, in round r, the r-th
// stencil node whose box offset i0 + B j0 + B^2 k0 falls in shared-memory
// bank l, so the 32 lanes of one round never share a bank.  The number of
// rounds is the largest count of nodes per bank (7 for P = 6, B = 13: the
// 216 nodes in 7 conflict-free rounds).
__host__ __device__ constexpr int spread_rounds(int P) {
  int B = SPREAD_TILE + P - 1, cnt[32] = {}, mx = 0;
  for (int k = 0; k < P; ++k)
    for (int j = 0; j < P; ++j)
      for (int i = 0; i < P; ++i) {
        int b = (i + B * j + B * B * k) % 32;
        if (++cnt[b] > mx) mx = cnt[b];
      }
  return mx;
}

// Shared-memory bytes of k_spread_tile: the box (3 planes per warp) and one
// batch of 32 staged sources (24 weights, 3 values per warp, box offset).
inline size_t spread_smem_bytes(int B, int nw, size_t elem) {
  return (size_t)3 * nw * B * B * B * elem + 32 * ((24 + 3 * nw) * elem + sizeof(int));
}

// One CTA per chunk of a tile, warp w owning grid planes c0+3w..+2 (one
// vector quantity: c1 f, or one column of c2 g (x) a3).  Sources are staged
// 32 at a time (weights, values, box offset); then every warp adds them one
// after another into its planes of a shared-memory box, lanes over the
// stencil nodes in the bank-conflict-free schedule.  A warp alone owns its
// planes, so plain read-modify-writes suffice.  Finally the box goes to the
// grids with one global atomic per nonzero node and plane.
template <typename R, int PT>  // PT: the B-spline order, 2..8
__global__ void __launch_bounds__(128) k_spread_tile(SpreadArgs a, TileArgs t, const int* __restrict__ perm,
                                                     const int4* __restrict__ chunk, R* __restrict__ grid) {
  constexpr int P = PT, NR = spread_rounds(PT);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int4 ch = chunk[blockIdx.x];
  if (ch.y >= ch.z) return;  // an empty entry past the end of the chunk list
  const int nw = blockDim.x >> 5;
  const int B = t.B, B2 = B * B, B3 = B2 * B;
  R* box = reinterpret_cast<R*>(smem_raw);  // [3 nw][B3]
  R* sw = box + (size_t)3 * nw * B3;         // [32][24]
  R* sv = sw + 32 * 24;                      // [32][3 nw]
  int* sb = reinterpret_cast<int*>(sv + 32 * 3 * nw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int tx = ch.x % t.ntile[0], ty = (ch.x / t.ntile[0]) % t.ntile[1], tz = ch.x / (t.ntile[0] * t.ntile[1]);
  const int o[3] = {tx * SPREAD_TILE, ty * SPREAD_TILE, tz * SPREAD_TILE};
  const int cfirst = t.c0;
  // this lane's nodes: box offset and (i0, j0, k0) packed, offset -1 if none
  int noff[NR], nidx[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const int2 e = t.sched[q * 32 + lane];
    noff[q] = e.x;
    nidx[q] = e.y;
  }
  for (int i = threadIdx.x; i < 3 * nw * B3; i += blockDim.x) box[i] = (R)0;
  const int nsrc = ch.z - ch.y;
  for (int s0 = 0; s0 < nsrc; s0 += 32) {
    const int nb = min(32, nsrc - s0);
    __syncthreads();
    if (lane < nb) {
      const int p = perm[ch.y + s0 + lane];
      if (wid == 0) {
        R w[8];
        int m[3];
        for (int d = 0; d < 3; ++d) {
          weights<R>(a.x[p + (size_t)d * a.n], a.ih[d], P, m[d], w);
#pragma unroll
          for (int q = 0; q < 8; ++q) sw[lane * 24 + d * 8 + q] = w[q];
        }
        sb[lane] = imod(m[0] - o[0], a.N[0]) + B * (imod(m[1] - o[1], a.N[1]) + B * imod(m[2] - o[2], a.N[2]));
      }
      for (int c = 0; c < 3; ++c) {
        const int gc = cfirst + 3 * wid + c;
        R v;
        if (gc < 3) v = (R)(a.c1 * a.f[p + (size_t)gc * a.n]);
        else {
          const int ii = (gc - 3) % 3, jj = (gc - 3) / 3;
          v = (R)(a.c2 * (a.g[p + (size_t)ii * a.n] * a.a3[p + (size_t)jj * a.n]));
        }
        sv[lane * 3 * nw + 3 * wid + c] = v;
      }
    }
    __syncthreads();
    R* wbox = box + (size_t)3 * wid * B3;
    for (int s = 0; s < nb; ++s) {
      const R* ws = sw + s * 24;
      const R v0 = sv[s * 3 * nw + 3 * wid], v1 = sv[s * 3 * nw + 3 * wid + 1], v2 = sv[s * 3 * nw + 3 * wid + 2];
      R* bs = wbox + sb[s];
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        if (noff[r] >= 0) {
          const R w = ws[nidx[r] & 15] * ws[8 + ((nidx[r] >> 4) & 15)] * ws[16 + (nidx[r] >> 8)];
          R* q = bs + noff[r];
          const R o0 = q[0], o1 = q[B3], o2 = q[2 * B3];
          q[0] = o0 + w * v0;
          q[B3] = o1 + w * v1;
          q[2 * B3] = o2 + w * v2;
        }
      }
      __syncwarp();  // the next source may touch the same nodes
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < B3; i += blockDim.x) {
    const int bx = i % B, by = (i / B) % B, bz = i / B2;
    const int gx = (o[0] + bx) % a.N[0], gy = (o[1] + by) % a.N[1], gz = (o[2] + bz) % a.N[2];
    const size_t q = gx + (size_t)a.N[0] * (gy + (size_t)a.N[1] * gz);
    for (int c = 0; c < 3 * nw; ++c) {
      const R v = box[i + (size_t)c * B3];
      if (v != (R)0) atomicAdd(grid + q + (size_t)(cfirst + c) * a.G, v);
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

TileArgs tile_args(const rbc3d_ctx* ctx, size_t elem) {
  TileArgs t;
  for (int d = 0; d < 3; ++d) t.ntile[d] = (ctx->prm.Nb[d] + SPREAD_TILE - 1) / SPREAD_TILE;
  t.B = SPREAD_TILE + ctx->prm.P - 1;
  t.cg = 3;
  return t;
}

__global__ void k_key_ranges(int n, const int* __restrict__ key, int* __restrict__ ts, int* __restrict__ te) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int k = key[p];
  if (p == 0 || key[p - 1] != k) ts[k] = p;
  if (p == n - 1 || key[p + 1] != k) te[k] = p + 1;
}
__global__ void k_chunk_counts(int nt, const int* __restrict__ ts, const int* __restrict__ te, int* __restrict__ cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > nt) return;
  cnt[k] = k < nt ? (te[k] - ts[k] + SPREAD_CHUNK - 1) / SPREAD_CHUNK : 0;
}
__global__ void k_fill_chunks(int nt, const int* __restrict__ ts, const int* __restrict__ te, const int* __restrict__ off,
                              int cap, int4* __restrict__ chunk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nt) {
    int o = off[k];
    for (int c = ts[k]; c < te[k]; c += SPREAD_CHUNK) chunk[o++] = make_int4(k, c, min(te[k], c + SPREAD_CHUNK), 0);
  }
  for (int i = off[nt] + k; i < cap; i += gridDim.x * blockDim.x) chunk[i] = make_int4(0, 0, 0, 0);
}

// Bin n sources (SoA positions on the device) by tile; chunks built on the device.
rbc3d_status build_spread_plan(rbc3d_ctx* ctx, int n, const double* x, SpreadArgs a, SpreadPlan& pl) {
  pl.n = n;
  pl.nchunk = 0;
  pl.valid = true;
  if (n == 0) return RBC3D_OK;
  TileArgs t = tile_args(ctx, 4);
  DBuf<int>&key = ctx->plan_key, &key2 = ctx->plan_key2, &idx = ctx->plan_idx;
  CUDA_TRY(key.alloc(n)); CUDA_TRY(key2.alloc(n)); CUDA_TRY(idx.alloc(n)); CUDA_TRY(pl.perm.alloc(n));
  { k_tile_keys<<<nblk(n, 256), 256, 0, ctx->st>>>(n, x, a, t, key.p, idx.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  const int ntiles = t.ntile[0] * t.ntile[1] * t.ntile[2];
  int bits = 1;
  while ((1 << bits) < ntiles) ++bits;
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, key.p, key2.p, idx.p, pl.perm.p, n, 0, bits, ctx->st);
  DBuf<char>& tb = ctx->plan_tmp;
  CUDA_TRY(tb.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceRadixSort::SortPairs(tb.p, tmp, key.p, key2.p, idx.p, pl.perm.p, n, 0, bits, ctx->st));
  // chunks of at most SPREAD_CHUNK sources of one tile, in tile order, built
  // on the device: the tiles' ranges in the sorted keys, their chunk counts,
  // the counts' scan, the chunks; the list has a fixed capacity and its empty
  // tail entries are skipped by the spread
  DBuf<int>&ts = ctx->plan_ts, &te = ctx->plan_te, &cnt = ctx->plan_cnt, &off = ctx->plan_off;
  CUDA_TRY(ts.alloc(ntiles)); CUDA_TRY(te.alloc(ntiles)); CUDA_TRY(cnt.alloc(ntiles + 1)); CUDA_TRY(off.alloc(ntiles + 1));
  CUDA_TRY(cudaMemsetAsync(ts.p, 0, sizeof(int) * ntiles, ctx->st));
  CUDA_TRY(cudaMemsetAsync(te.p, 0, sizeof(int) * ntiles, ctx->st));
  { k_key_ranges<<<nblk(n, 256), 256, 0, ctx->st>>>(n, key2.p, ts.p, te.p); ++ctx->launches; }
  { k_chunk_counts<<<nblk(ntiles + 1, 256), 256, 0, ctx->st>>>(ntiles, ts.p, te.p, cnt.p); ++ctx->launches; }
  size_t stmp = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, stmp, cnt.p, off.p, ntiles + 1, ctx->st);
  DBuf<char>& sb = ctx->plan_scan;
  CUDA_TRY(sb.alloc(stmp + 1));
  CUDA_TRY(cub::DeviceScan::ExclusiveSum(sb.p, stmp, cnt.p, off.p, ntiles + 1, ctx->st));
  const int cap = ntiles + (n + SPREAD_CHUNK - 1) / SPREAD_CHUNK;
  CUDA_TRY(pl.chunk.alloc(cap));
  { k_fill_chunks<<<nblk(ntiles + 1, 256), 256, 0, ctx->st>>>(ntiles, ts.p, te.p, off.p, cap, pl.chunk.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  pl.nchunk = cap;
  return RBC3D_OK;
}

// The node schedule of k_spread_tile for order P (see spread_rounds).
rbc3d_status spread_schedule(rbc3d_ctx* ctx, int P, TileArgs& t) {
  PmeState& S = ctx->pme;
  if (S.sched_P != P) {
    const int B = SPREAD_TILE + P - 1, NR = spread_rounds(P);
    std::vector<int2> tab((size_t)NR * 32, make_int2(-1, 0));
    std::vector<int> cnt(32, 0);
    for (int k = 0; k < P; ++k)
      for (int j = 0; j < P; ++j)
        for (int i = 0; i < P; ++i) {
          const int off = i + B * j + B * B * k, b = off % 32;
          tab[(size_t)cnt[b]++ * 32 + b] = make_int2(off, i | (j << 4) | (k << 8));
        }
    CUDA_TRY(S.sched.upload(tab.data(), tab.size(), ctx->st));
    S.sched_P = P;
  }
  t.sched = S.sched.p;
  return RBC3D_OK;
}

template <typename R, int PT>
rbc3d_status launch_spread_p(rbc3d_ctx* ctx, const SpreadArgs& a, const SpreadPlan& pl, R* grid) {
  TileArgs t = tile_args(ctx, sizeof(R));
  rbc3d_status st = spread_schedule(ctx, PT, t);
  if (st) return st;
  // warps (3-plane groups) per launch: as many as the 227 KB of shared memory hold
  const int gfirst = a.sl ? 0 : 1, glast = a.dl ? 4 : 1;
  int per = glast - gfirst;
  while (per > 1 && spread_smem_bytes(t.B, per, sizeof(R)) > 227 * 1024) --per;
  for (int g = gfirst; g < glast; g += per) {
    const int nw = std::min(per, glast - g);
    t.c0 = 3 * g;
    const size_t bytes = spread_smem_bytes(t.B, nw, sizeof(R));
    CUDA_TRY(cudaFuncSetAttribute(k_spread_tile<R, PT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    { k_spread_tile<R, PT><<<pl.nchunk, 32 * nw, bytes, ctx->st>>>(a, t, pl.perm.p, pl.chunk.p, grid); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
  }
  return RBC3D_OK;
}
template <typename R>
rbc3d_status launch_spread(rbc3d_ctx* ctx, const SpreadArgs& a, const SpreadPlan& pl, R* grid) {
  if (pl.nchunk == 0) return RBC3D_OK;
  switch (a.P) {
    case 2: return launch_spread_p<R, 2>(ctx, a, pl, grid);
    case 3: return launch_spread_p<R, 3>(ctx, a, pl, grid);
    case 4: return launch_spread_p<R, 4>(ctx, a, pl, grid);
    case 5: return launch_spread_p<R, 5>(ctx, a, pl, grid);
    case 6: return launch_spread_p<R, 6>(ctx, a, pl, grid);
    case 7: return launch_spread_p<R, 7>(ctx, a, pl, grid);
    default: return launch_spread_p<R, 8>(ctx, a, pl, grid);  // P <= 8 checked at rbc3d_create
  }
}

// The cell sources' spread plan (tile binning of the sorted positions), built
// when the positions change rather than in the first spread after them.
rbc3d_status pme_prepare_cells(rbc3d_ctx* ctx) {
  PmeState& P = ctx->pme;
  if (P.cplan.valid || ctx->npt == 0 || !ctx->s_x.p) return RBC3D_OK;
  SpreadArgs a{};
  for (int d = 0; d < 3; ++d) { a.N[d] = ctx->prm.Nb[d]; a.ih[d] = ctx->prm.Nb[d] / ctx->prm.Lb[d]; }
  a.P = ctx->prm.P; a.G = P.G;
  a.n = ctx->npt; a.x = ctx->s_x.p;
  return build_spread_plan(ctx, a.n, a.x, a, P.cplan);
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
      rbc3d_status s;
      if (!P.cplan.valid && (s = build_spread_plan(ctx, a.n, a.x, a, P.cplan))) return s;
      s = prec == RBC3D_FP32C ? launch_spread<float>(ctx, a, P.cplan, P.grid32.p)
                              : launch_spread<double>(ctx, a, P.cplan, P.grid64.p);
      if (s) return s;
    }
  }
  if (walls && ctx->wall.nele > 0 && P.sl) {
    WallState& W = ctx->wall;
    CUDA_TRY(W.src_x.alloc(3 * (size_t)W.nele));
    CUDA_TRY(W.src_f.alloc(3 * (size_t)W.nele));
    { k_wall_sources<<<nblk(W.nele, 256), 256, 0, ctx->st>>>(W.nele, W.nvert, W.e2v.p, W.x.p, W.f.p, W.area.p, W.src_x.p, W.src_f.p); ++ctx->launches; }
    a.n = W.nele; a.x = W.src_x.p; a.f = W.src_f.p; a.g = nullptr; a.a3 = nullptr; a.sl = 1; a.dl = 0;
    rbc3d_status s;
    if (!P.wplan.valid && (s = build_spread_plan(ctx, a.n, a.x, a, P.wplan))) return s;
    s = prec == RBC3D_FP32C ? launch_spread<float>(ctx, a, P.wplan, P.grid32.p)
                            : launch_spread<double>(ctx, a, P.wplan, P.grid64.p);
    if (s) return s;
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
  // the transforms run on the context's current stream (the matvec may put PME on its side stream)
  if (P.prec == RBC3D_FP32C) {
    cufftSetStream(P.r2c32_3, ctx->st); cufftSetStream(P.r2c32_12, ctx->st); cufftSetStream(P.c2r32_3, ctx->st);
  } else {
    cufftSetStream(P.r2c64_3, ctx->st); cufftSetStream(P.r2c64_12, ctx->st); cufftSetStream(P.c2r64_3, ctx->st);
  }
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
