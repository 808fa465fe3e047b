// selfmix.cu -- RBC_SingInt (ModRbcSingInt.F90:29-90) for the FP32M mode:
// the own-cell polar-patch quadrature with FP64-accurate geometry and FP32
// arithmetic.
//
// The only cancellation-prone quantity of the patch quadrature is the
// separation xx = x(patch point) - x(target), as small as 1e-2 for the first
// radial ring.  Positions are stored relative to each cell's centre as FP32
// (hi, lo) pairs computed in FP64, and each stencil node's offset from the
// target, (X_hi - t_hi) + (X_lo - t_lo), is formed before the bicubic
// weights are applied, so xx carries ~1e-7 relative error instead of the
// ~1e-5 of plain FP32 positions.  Densities, normals, weights and the Ewald
// kernel are FP32 (erfc as exp(-x^2) t Q(t), the fit of fit_erfcx),
// accumulated with Kahan compensation per target.  Node records are read
// as float4.  erfc is exp(-x^2) t Q(t) with the fitted
// polynomial of fit_erfcx (pair.cu).
//
// Patch geometry: the bicubic weights of patch point q of a target at
// latitude ilat0 depend only on (ilat0, q); longitudes shift the stencil by
// whole grid columns (phiG = atan2(...) + phi0 with phi0 on the grid), so they
// are tabulated once per grid.
#include <cmath>
#include <vector>

#include "ctx.hpp"

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

// Node record (52 floats = 13 float4): x hi(3) lo(3) u1(3) u2(3) u12(3) |
// a3 u u1 u2 u12 (12) | FdetJ (12) | GdetJ (12) | pad(1)
constexpr int REC = 52;
constexpr int OFF_X = 0, OFF_A3 = 15, OFF_F = 27, OFF_G = 39;

struct SelfW {
  int i1, j1b;
  float cx[4], cy[4];
};

// mean of each cell's grid points (x SoA, 3 x npt)
__global__ void k_cell_mean(int nv, long long npt, const double* __restrict__ x, double* __restrict__ xc) {
  __shared__ double red[3][32];
  const int cell = blockIdx.x;
  double s[3] = {0, 0, 0};
  for (int r = threadIdx.x; r < nv; r += blockDim.x)
    for (int k = 0; k < 3; ++k) s[k] += x[(size_t)cell * nv + r + k * npt];
  for (int k = 0; k < 3; ++k) {
    double v = warp_sum(s[k]);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    xc[3 * cell + threadIdx.x] = t / nv;
  }
}

__global__ void k_mix_geom(int ncell, int m, int n, const double* __restrict__ spl, const double* __restrict__ xc,
                           float* __restrict__ out) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)m * n;
  if (idx >= (long long)ncell * per) return;
  int cell = (int)(idx / per);
  int node = (int)(idx - (long long)cell * per);
  const double* sx = spl + (((size_t)cell * SPL_NSET + SPL_X) * per + node) * SPL_NODE;
  const double* sa = spl + (((size_t)cell * SPL_NSET + SPL_A3) * per + node) * SPL_NODE;
  float* o = out + ((size_t)cell * per + node) * REC;
  for (int k = 0; k < 3; ++k) {
    double r = sx[k] - xc[3 * cell + k];
    float h = (float)r;
    o[OFF_X + k] = h;
    o[OFF_X + 3 + k] = (float)(r - (double)h);
    o[OFF_X + 6 + k] = (float)sx[3 + k];   // u1
    o[OFF_X + 9 + k] = (float)sx[6 + k];   // u2
    o[OFF_X + 12 + k] = (float)sx[9 + k];  // u12
  }
  for (int k = 0; k < 12; ++k) o[OFF_A3 + k] = (float)sa[k];
  o[REC - 1] = 0.f;
}

__global__ void k_mix_dens(int ncell, int m, int n, const double* __restrict__ spl, float* __restrict__ out, int do_f,
                           int do_g) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)m * n;
  if (idx >= (long long)ncell * per) return;
  int cell = (int)(idx / per);
  int node = (int)(idx - (long long)cell * per);
  float* o = out + ((size_t)cell * per + node) * REC;
  if (do_f) {
    const double* s = spl + (((size_t)cell * SPL_NSET + SPL_F) * per + node) * SPL_NODE;
    for (int k = 0; k < 12; ++k) o[OFF_F + k] = (float)s[k];
  }
  if (do_g) {
    const double* s = spl + (((size_t)cell * SPL_NSET + SPL_G) * per + node) * SPL_NODE;
    for (int k = 0; k < 12; ++k) o[OFF_G + k] = (float)s[k];
  }
}

// Interpolated own position of every cell point (Spline_Interp at the grid
// point, as RBC_SingInt does), relative to the cell centre, as hi/lo.
__global__ void k_mix_targets(int npt, int nlat, int nlon, int m, const double* __restrict__ th,
                              const double* __restrict__ phi, const double* __restrict__ spl,
                              const double* __restrict__ xc, float4* __restrict__ thi, float4* __restrict__ tlo) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npt) return;
  int nv = nlat * nlon, cell = p / nv, r = p - cell * nv;
  int ilat = r % nlat, ilon = r / nlat;
  SplW W;
  spline_weights(th[ilat], phi[ilon], m, nlon, W);
  double x[3];
  spline_eval(spl + ((size_t)cell * SPL_NSET + SPL_X) * (size_t)m * nlon * SPL_NODE, W, 3, x);
  float h[3], l[3];
  for (int k = 0; k < 3; ++k) {
    double d = x[k] - xc[3 * cell + k];
    h[k] = (float)d;
    l[k] = (float)(d - (double)h[k]);
  }
  thi[p] = make_float4(h[0], h[1], h[2], 0.f);
  tlo[p] = make_float4(l[0], l[1], l[2], 0.f);
}

struct MixArgs {
  int nt, ncell, nlat, nlon, m, NQ, nrad;
  const double* tA;
  double* v;
  const float* rec;
  const SelfW* W;
  const float* pw;
  const float4* thi;
  const float4* tlo;
  const int* celltype;
  double B[RBC3D_MAX_CELLTYPES];
  float c1, c2;
  float rc2, sqpa, two_isqa, m8_ispi, q75_spi;
  float erfcx_q[ERFCX_DEG + 1];
};

// The 13 float4 of a node record in registers (only those the terms need).
template <bool DL>
__device__ __forceinline__ void load_rec(const float* r, float* v) {
  const float4* r4 = reinterpret_cast<const float4*>(r);
#pragma unroll
  for (int i = 0; i < REC / 4; ++i) {
    // SL needs x (floats 0-14) and F (27-38): float4 0-3 and 6-9
    if (!DL && (i == 4 || i == 5 || i >= 10)) continue;
    const float4 q = __ldg(r4 + i);
    v[4 * i] = q.x; v[4 * i + 1] = q.y; v[4 * i + 2] = q.z; v[4 * i + 3] = q.w;
  }
}

// one warp per target; warps of a block walk one latitude ring so that
// neighbouring warps share most stencil nodes in L1
template <bool DL>
__global__ void __launch_bounds__(256) k_self_mix(MixArgs a) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nv = a.nlat * a.nlon;
  if (w >= a.ncell * nv) return;
  const int cell = w / nv, rr = w - cell * nv;
  const int ilon0 = rr % a.nlon, ilat0 = rr / a.nlon;
  const int p = cell * nv + ilon0 * a.nlat + ilat0;
  const float c1 = a.c1;
  const float c2m = DL ? (float)(a.c2 * a.B[a.celltype[cell]]) : 0.f;
  const float4 th4 = a.thi[p], tl4 = a.tlo[p];
  const float th_[3] = {th4.x, th4.y, th4.z}, tl_[3] = {tl4.x, tl4.y, tl4.z};
  const float* base = a.rec + (size_t)cell * a.m * a.nlon * REC;
  Kahan3 acc;
  acc.zero();
  for (int q = lane; q < a.NQ; q += 32) {
    const SelfW e = a.W[ilat0 * a.NQ + q];
    const int irad = q % a.nrad;
    int j1 = e.j1b + ilon0;
    j1 = imod(j1, a.nlon);
    const int j2 = (j1 + 1 == a.nlon) ? 0 : j1 + 1;
    const int i1 = e.i1, i2 = (i1 + 1 == a.m) ? 0 : i1 + 1;
    const int nodes[4] = {i1 + a.m * j1, i1 + a.m * j2, i2 + a.m * j1, i2 + a.m * j2};
    // weights of (u, u1, u2, u12) per node (Spline_Interp, ModSpline.F90:172-185)
    const float wu[4] = {e.cx[0] * e.cy[0], e.cx[0] * e.cy[1], e.cx[1] * e.cy[0], e.cx[1] * e.cy[1]};
    const float w1[4] = {e.cx[2] * e.cy[0], e.cx[2] * e.cy[1], e.cx[3] * e.cy[0], e.cx[3] * e.cy[1]};
    const float w2[4] = {e.cx[0] * e.cy[2], e.cx[0] * e.cy[3], e.cx[1] * e.cy[2], e.cx[1] * e.cy[3]};
    const float w12[4] = {e.cx[2] * e.cy[2], e.cx[2] * e.cy[3], e.cx[3] * e.cy[2], e.cx[3] * e.cy[3]};
    float xx[3] = {0, 0, 0}, F[3] = {0, 0, 0}, G[3] = {0, 0, 0}, A3[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float v[REC];
      load_rec<DL>(base + (size_t)nodes[k] * REC, v);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float d = __fadd_rn(__fsub_rn(v[OFF_X + c], th_[c]), __fsub_rn(v[OFF_X + 3 + c], tl_[c]));
        xx[c] += wu[k] * d + w1[k] * v[OFF_X + 6 + c] + w2[k] * v[OFF_X + 9 + c] + w12[k] * v[OFF_X + 12 + c];
        F[c] += wu[k] * v[OFF_F + c] + w1[k] * v[OFF_F + 3 + c] + w2[k] * v[OFF_F + 6 + c] + w12[k] * v[OFF_F + 9 + c];
        if (DL) {
          G[c] += wu[k] * v[OFF_G + c] + w1[k] * v[OFF_G + 3 + c] + w2[k] * v[OFF_G + 6 + c] +
                  w12[k] * v[OFF_G + 9 + c];
          A3[c] += wu[k] * v[OFF_A3 + c] + w1[k] * v[OFF_A3 + 3 + c] + w2[k] * v[OFF_A3 + 6 + c] +
                   w12[k] * v[OFF_A3 + 9 + c];
        }
      }
    }
    const float r2 = xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2];
    if (r2 >= a.rc2) continue;  // rr >= rc (ModRbcSingInt.F90:65)
    const float rinv = rsqrtf(r2), rv = r2 * rinv, ir2 = rinv * rinv;
    const float st = rv * a.sqpa, ex = __expf(-st * st);
    // erfc(st) = exp(-st^2) t Q(t), t = 1/(1 + st/2) (fit_erfcx)
    const float tq = __fdividef(1.f, fmaf(0.5f, st, 1.f));
    float Qp = a.erfcx_q[ERFCX_DEG];
#pragma unroll
    for (int k = ERFCX_DEG - 1; k >= 0; --k) Qp = fmaf(Qp, tq, a.erfcx_q[k]);
    const float e1 = ex * (tq * Qp), e2 = a.two_isqa * ex;
    const float wq = a.pw[irad];
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    if (c1 != 0.f) {
      const float A = (e1 * rinv + e2) * ir2, Bc = e1 * rinv - e2;
      const float f0 = wq * F[0], f1 = wq * F[1], f2 = wq * F[2];
      const float d = xx[0] * f0 + xx[1] * f1 + xx[2] * f2;
      v0 = c1 * (A * xx[0] * d + Bc * f0);
      v1 = c1 * (A * xx[1] * d + Bc * f1);
      v2 = c1 * (A * xx[2] * d + Bc * f2);
    }
    if (DL) {
      const float cdl = a.m8_ispi * (ex * (st * (1.5f + st * st)) + a.q75_spi * e1);
      const float Ad = cdl * ir2 * ir2 * rinv;
      const float dg = wq * (xx[0] * G[0] + xx[1] * G[1] + xx[2] * G[2]);
      const float da = xx[0] * A3[0] + xx[1] * A3[1] + xx[2] * A3[2];
      const float t = c2m * Ad * dg * da;
      v0 += t * xx[0]; v1 += t * xx[1]; v2 += t * xx[2];
    }
    acc.add(0, v0);
    acc.add(1, v1);
    acc.add(2, v2);
  }
  double dv[3];
  for (int k = 0; k < 3; ++k) dv[k] = warp_sum((double)acc.s[k] - (double)acc.c[k]);
  if (lane == 0) {
    double iA = 1.0 / a.tA[p];
    for (int k = 0; k < 3; ++k) a.v[p + (size_t)k * a.nt] += dv[k] * iA;
  }
}

}  // namespace

// Patch weights per (target latitude, patch point): from thG and the atan2
// part of phiG of RbcPolarPatch_Create.
rbc3d_status self_mixed_grid(rbc3d_ctx* ctx, const std::vector<double>& thG, const std::vector<double>& phiA,
                             const std::vector<double>& pw) {
  const int NQ = ctx->nrad * ctx->nazm, m = ctx->m, n = ctx->nlon;
  const double ihx = m / RBC3D_TWO_PI, ihy = n / RBC3D_TWO_PI;
  const double hx = RBC3D_TWO_PI / m, hy = RBC3D_TWO_PI / n;
  std::vector<SelfW> W((size_t)ctx->nlat * NQ);
  for (size_t i = 0; i < W.size(); ++i) {
    double x = thG[i] * ihx, y = phiA[i] * ihy;
    int i1 = (int)std::floor(x), j1 = (int)std::floor(y);
    double s = x - i1, t = y - j1;
    SelfW e;
    e.i1 = ((i1 % m) + m) % m;
    e.j1b = j1;
    e.cx[0] = (float)(1 + s * s * (-3. + 2. * s)); e.cx[1] = (float)(s * s * (3. - 2. * s));
    e.cx[2] = (float)(hx * s * (1. + s * (-2. + s))); e.cx[3] = (float)(hx * s * s * (-1. + s));
    e.cy[0] = (float)(1 + t * t * (-3. + 2. * t)); e.cy[1] = (float)(t * t * (3. - 2. * t));
    e.cy[2] = (float)(hy * t * (1. + t * (-2. + t))); e.cy[3] = (float)(hy * t * t * (-1. + t));
    W[i] = e;
  }
  std::vector<float> pwf(pw.begin(), pw.end());
  CUDA_TRY(ctx->mix_w.upload((const char*)W.data(), W.size() * sizeof(SelfW), ctx->st));
  CUDA_TRY(ctx->mix_pw.upload(pwf.data(), pwf.size(), ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

// FP32 node records and target positions for the current geometry.
rbc3d_status self_mixed_geom(rbc3d_ctx* ctx) {
  self_ff_invalidate(ctx, true, false, false);
  ctx->rep_valid = false;  // the near pass's FP32 replay records follow the geometry
  const int nv = ctx->nlat * ctx->nlon;
  // cell centres (mean of the grid points) from the uploaded positions
  CUDA_TRY(ctx->mix_xc.alloc(3 * (size_t)ctx->ncell));
  { k_cell_mean<<<ctx->ncell, 256, 0, ctx->st>>>(nv, ctx->npt, ctx->x.p, ctx->mix_xc.p); ++ctx->launches; }
  // the node records are built on first use (run_self_mixed); the target
  // positions serve the float-float patch too
  ctx->mix_sets = 0;
  CUDA_TRY(ctx->mix_thi.alloc(ctx->npt));
  CUDA_TRY(ctx->mix_tlo.alloc(ctx->npt));
  { k_mix_targets<<<nblk(ctx->npt, 128), 128, 0, ctx->st>>>(ctx->npt, ctx->nlat, ctx->nlon, ctx->m, ctx->th.p,
                                                             ctx->phi.p, ctx->spl.p, ctx->mix_xc.p, ctx->mix_thi.p,
                                                             ctx->mix_tlo.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

rbc3d_status self_mixed_density(rbc3d_ctx* ctx, bool f, bool g) {
  self_ff_invalidate(ctx, false, f, g);
  if (f) ctx->mix_sets &= ~2;
  if (g) ctx->mix_sets &= ~4;
  return RBC3D_OK;
}

rbc3d_status run_self_mixed(rbc3d_ctx* ctx, int tlist, double c1, double c2) {
  TargetSet& t = ctx->tl[tlist];
  if (tlist != RBC3D_TLIST_RBC || t.n == 0 || ctx->ncell == 0) return RBC3D_OK;
  // FP32 node records of the current geometry and densities (bit 0 geometry, 1 f, 2 g)
  const long long per = (long long)ctx->m * ctx->nlon;
  if (!ctx->mix_rec.p || ctx->mix_rec.n < (size_t)ctx->ncell * per * REC) {
    CUDA_TRY(ctx->mix_rec.alloc((size_t)ctx->ncell * per * REC));
    ctx->mix_sets = 0;
  }
  if (!(ctx->mix_sets & 1)) {
    { k_mix_geom<<<nblk(ctx->ncell * per, 256), 256, 0, ctx->st>>>(ctx->ncell, ctx->m, ctx->nlon, ctx->spl.p,
                                                                    ctx->mix_xc.p, ctx->mix_rec.p); ++ctx->launches; }
    ctx->mix_sets |= 1;
  }
  const bool df = ctx->has_f && !(ctx->mix_sets & 2), dg = ctx->has_g && !(ctx->mix_sets & 4);
  if (df || dg) {
    { k_mix_dens<<<nblk(ctx->ncell * per, 256), 256, 0, ctx->st>>>(ctx->ncell, ctx->m, ctx->nlon, ctx->spl.p,
                                                                    ctx->mix_rec.p, df, dg); ++ctx->launches; }
    ctx->mix_sets |= (df ? 2 : 0) | (dg ? 4 : 0);
  }
  CUDA_TRY(cudaGetLastError());
  MixArgs a;
  a.nt = t.n; a.ncell = ctx->ncell; a.nlat = ctx->nlat; a.nlon = ctx->nlon; a.m = ctx->m;
  a.NQ = ctx->nrad * ctx->nazm; a.nrad = ctx->nrad;
  a.tA = t.Acoef.p; a.v = t.v.p; a.rec = ctx->mix_rec.p; a.W = (const SelfW*)ctx->mix_w.p; a.pw = ctx->mix_pw.p;
  a.thi = ctx->mix_thi.p; a.tlo = ctx->mix_tlo.p; a.celltype = ctx->celltype.p;
  for (int l = 0; l < RBC3D_MAX_CELLTYPES; ++l) a.B[l] = ctx->Bcoef[l];
  a.c1 = (float)((c1 != 0 && ctx->has_f) ? c1 : 0.0);
  a.c2 = (float)((c2 != 0 && ctx->has_g) ? c2 : 0.0);
  a.rc2 = (float)(ctx->prm.rc * ctx->prm.rc);
  a.sqpa = (float)std::sqrt(RBC3D_PI / ctx->prm.alpha);
  a.two_isqa = (float)(2.0 / std::sqrt(ctx->prm.alpha));
  a.m8_ispi = (float)(-8.0 / std::sqrt(RBC3D_PI));
  a.q75_spi = (float)(0.75 * std::sqrt(RBC3D_PI));
  erfcx_coeffs(ctx);
  for (int k = 0; k <= ERFCX_DEG; ++k) a.erfcx_q[k] = ctx->erfcx_q[k];
  long long threads = (long long)t.n * 32;
  if (a.c2 != 0.f) { k_self_mix<true><<<(int)((threads + 255) / 256), 256, 0, ctx->st>>>(a); ++ctx->launches; }
  else { k_self_mix<false><<<(int)((threads + 255) / 256), 256, 0, ctx->st>>>(a); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}
