// selfff.cu -- RBC_SingInt (ModRbcSingInt.F90:29-90) for the FP32D mode: the
// own-cell polar-patch quadrature in float-float arithmetic on the FP32 pipe.
//
// GB300 issues FP64 at about 1/76 of its FP32 FMA rate (1.06 against 78
// TFLOP/s measured), and the FP64 patch kernel is bound by that pipe.  Here
// every quantity is an unevaluated sum hi + lo of two FP32 numbers (48
// significant bits):
//   * the Spline_Interp sums are compensated dot products (Ogita, Rump and
//     Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005):
//     each product w v split exactly by the FMA form of TwoProduct, the high
//     parts summed error-free, the rounding errors and the lo-part cross
//     terms summed in FP32.  The sums start from a power of two `off` at
//     least twice a bound on their sum of |w v| (the per-cell maxima of the
//     node values times the weight-sum bounds 1, h/4 and h^2/16), so every
//     partial sum stays above every product in magnitude and Dekker's
//     FastTwoSum (3 operations) is exact where Knuth's TwoSum takes 6; off
//     is subtracted exactly at the end.  The FP32 correction term is rounded
//     on the scale of off, so for the position x, whose interpolant is
//     differenced against the target, the bound covers the 12 derivative
//     terms only: off is subtracted before the 4 value terms, which are
//     added with TwoSum (all 16 from the larger offset: the corrections
//     move from 2.3e-12 to 2.3e-11 of the FP64 patch);
//   * the Ewald kernel (EwaldCoeff_SL / _DL, ModEwaldFunc.F90:86-180, the
//     same tables as hi/lo) is evaluated with Dekker's float-float product
//     and sum, and 1/r by rsqrtf, an FP32 Newton step and a float-float
//     Newton step.
// The patch corrections agree with the FP64 kernel to a few 1e-12 relative
// (rel-L2, 256-cell workload); the interpolation sums carry errors of a few
// 1e-12 of sum |w v| (x) or of the cell's maxima (f, g, a3).
//
// Data layout.  Per node and slot d (u, u_th, u_ph, u_thph) the 12 values x
// (relative to the cell centre), f and g density sets and a3 (three
// components each) are stored as three quads; a quad's hi and lo parts form
// one 32-byte entry, read with one 256-bit load, in its own plane
// [cell][d*3 + quad][node tile]: the lanes of a warp interpolate at
// neighbouring patch points, and with 2 x 2 node tiles per 128-byte line
// their stencil nodes share lines (a record per node put each lane's load
// in its own line and kept the L1 data pipe 95% busy; separate hi and lo
// planes of 16-byte entries took two loads and two lines per quad).
// Consecutive values share one bicubic weight, so they run in pairs as
// packed FP32x2 operations.  Patch weights per (target latitude,
// patch point) are the 16 Spline_Interp products as hi/lo planes (coalesced
// across the lanes, which walk consecutive patch points); target positions
// are the FP32M hi/lo records relative to the same cell centre.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.hpp"

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

constexpr int FF_PLANES = 24;  // float4 per node: 4 slots x 3 quads x (hi, lo)

// Position of spline node (i, j) in a plane: tiles of 2^ti (latitude rows) x
// 2^tj (longitude columns), one 128-byte line of 32-byte entries per plane.
// With 16-byte entries (8 per line) 2 x 4 tiles measured best for the
// 25 x 50 grid (k_self_ff at 256 cells: 6.81 ms; 4 x 2 7.02, 8 x 1 7.07,
// 1 x 8 7.65); 32-byte entries in 2 x 2 tiles: 6.68 ms in the matvec.
struct NodeMap {
  int ti, tj, nti;  // log2 tile sizes, tiles along i
  long long per;    // padded nodes per plane
  __device__ __forceinline__ int pos(int i, int j) const {
    return (((j >> tj) * nti + (i >> ti)) << (ti + tj)) + (i & ((1 << ti) - 1)) + ((j & ((1 << tj) - 1)) << ti);
  }
};
inline NodeMap node_map(int m, int n) {
  NodeMap M;
  M.ti = 1; M.tj = 1;
  M.nti = (m + (1 << M.ti) - 1) >> M.ti;
  const int ntj = (n + (1 << M.tj) - 1) >> M.tj;
  M.per = (long long)M.nti * ntj << (M.ti + M.tj);
  return M;
}

// ---------------------------------------------------------------------------
// float-float arithmetic
struct ff {
  float h, l;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_norm(ff a) { return fast_two_sum(a.h, a.l); }
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ ff ff_sub(ff a, ff b) {
  ff s = two_sum(a.h, -b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fsub_rn(a.l, b.l)));
}
// product without the final renormalisation: |l| stays ~2^-23 |h|
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return {p, e};
}
__device__ __forceinline__ bool ff_ge(ff a, ff b) { return a.h > b.h || (a.h == b.h && a.l >= b.l); }

// lazy accumulator: hi parts summed exactly, errors and lo parts in FP32
struct ffacc {
  float s, c;
  __device__ __forceinline__ void add(ff v) {
    const ff t = two_sum(s, v.h);
    s = t.h;
    c = __fadd_rn(c, __fadd_rn(t.l, v.l));
  }
};

// one 32-byte read-only load (hi quad, lo quad of one node)
__device__ __forceinline__ void ld8(const float4* p, float4& h, float4& l) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(h.x), "=f"(h.y), "=f"(h.z), "=f"(h.w), "=f"(l.x), "=f"(l.y), "=f"(l.z), "=f"(l.w)
      : "l"(p));
}

// packed FP32x2 helpers (round to nearest, as the scalar forms)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(d)
      : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)));
  return *reinterpret_cast<float2*>(&d);
}

// Compensated dot-product accumulator for two values sharing a weight.
struct Dot2 {
  float2 s, c;
  // s + c += w * v with w = (wh, wl), v = (vh, vl) per half; nwh = -wh.
  // FAST: s has been kept above every product in magnitude (FastTwoSum)
  template <bool FAST>
  __device__ __forceinline__ void add(float2 wh, float2 nwh, float2 wl, float2 vh, float2 vl) {
    const float2 p = __fmul2_rn(wh, vh);
    const float2 ne = __ffma2_rn(nwh, vh, p);  // p - wh vh: minus the product's rounding error
    const float2 t = __fadd2_rn(s, p);
    float2 err;
    if (FAST) {
      err = sub2(p, sub2(t, s));
    } else {
      const float2 bb = sub2(t, s);
      err = __fadd2_rn(sub2(s, sub2(t, bb)), sub2(p, bb));
    }
    s = t;
    c = __ffma2_rn(wh, vl, c);
    c = __ffma2_rn(wl, vh, c);
    c = __fadd2_rn(c, sub2(err, ne));
  }
  __device__ __forceinline__ ff x() const { return two_sum(s.x, c.x); }
  __device__ __forceinline__ ff y() const { return two_sum(s.y, c.y); }
};

struct FFArgs {
  int nt, ncell, nlat, nlon, m, NQ, nrad;
  const double* tA;
  double* v;
  const float4* rec;    // [cell][slot x quad][node tile][hi, lo]
  const int2* widx;     // (i1, j1b) per (latitude, patch point)
  const float4* w;      // 8 planes of nlat*NQ: hi of slot d of nodes 0..3 (d = 0..3), then lo
  const float2* pw;     // patch weights, hi/lo
  const float4* thi;    // target positions relative to the cell centre, hi
  const float4* tlo;    // and lo
  const float4* tab;    // [3][EWALD_NTAB]: {T_i hi, T_i lo, (T_i+1 - T_i) hi, lo}
  const uint4* bnd;     // [set x f g a3][cell]: max |u|, |u_th|, |u_ph|, |u_thph| (float bits)
  NodeMap map;
  float hq1, hq2, hq12; // derivative weight-sum bounds: h_th / 4, h_ph / 4, h_th h_ph / 16
  const int* celltype;
  const short* perm;    // [latitude][k]: the patch point lane k of the warp's pass takes
  ff c1;                // c1
  ff c2B[RBC3D_MAX_CELLTYPES];  // c2 Bcoef per cell type
  ff rc2, r_eps, ntab_over_rc;
};

__device__ __forceinline__ ff ld_ff(float2 v) { return {v.x, v.y}; }

// T + D f1 for table t at index it
__device__ __forceinline__ ff tab_lerp(const float4* tab, int t, int it, ff f1) {
  const float4 e = __ldg(tab + (size_t)t * EWALD_NTAB + it);
  return ff_add({e.x, e.y}, ff_mul({e.z, e.w}, f1));
}

__device__ __forceinline__ ff dot3(const ff* a, const ff* b) {
  return ff_add(ff_add(ff_mul(a[0], b[0]), ff_mul(a[1], b[1])), ff_mul(a[2], b[2]));
}

// One target of the own-cell patch: warp index w (cell, latitude ring,
// longitude), its grid point p, position, DL factor, record base and the
// starting offsets of its cell's sums (x: the derivative terms'; f, g, a3:
// all 16 terms').
struct Tgt {
  int p, cell, ilat0, ilon0;
  ff xi[3];
  ff c2m;
  const float4* base;
  float2 offs[6];
};

template <bool DL>
__device__ __forceinline__ Tgt target(const FFArgs& a, int w) {
  Tgt T;
  const int nv = a.nlat * a.nlon;
  T.cell = w / nv;
  const int rr = w - T.cell * nv;
  T.ilon0 = rr % a.nlon;
  T.ilat0 = rr / a.nlon;
  T.p = T.cell * nv + T.ilon0 * a.nlat + T.ilat0;
  const float4 th4 = a.thi[T.p], tl4 = a.tlo[T.p];
  T.xi[0] = {th4.x, tl4.x}; T.xi[1] = {th4.y, tl4.y}; T.xi[2] = {th4.z, tl4.z};
  T.c2m = DL ? a.c2B[a.celltype[T.cell]] : ff{0.f, 0.f};
  T.base = a.rec + (size_t)T.cell * FF_PLANES * a.map.per;
  float off[4], offd[2];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const uint4 b = __ldg(a.bnd + (size_t)s * a.ncell + T.cell);
    const float Bd = a.hq1 * __uint_as_float(b.y) + a.hq2 * __uint_as_float(b.z) + a.hq12 * __uint_as_float(b.w);
    int e;
    frexpf(2.f * 1.01f * (__uint_as_float(b.x) + Bd), &e);  // 2 B < 2^e
    off[s] = ldexpf(1.f, e);
    if (s < 2) {  // x, and f where it shares a pair with x
      frexpf(2.f * 1.01f * Bd, &e);
      offd[s] = ldexpf(1.f, e);
    }
  }
  T.offs[0] = make_float2(offd[0], offd[0]); T.offs[1] = make_float2(offd[0], offd[1]);
  T.offs[2] = make_float2(off[1], off[1]); T.offs[3] = make_float2(off[2], off[2]);
  T.offs[4] = make_float2(off[2], off[3]); T.offs[5] = make_float2(off[3], off[3]);
  return T;
}

// Patch point q of target T added to acc (RBC_SingInt's loop body).
template <bool SL, bool DL>
__device__ __forceinline__ void patch_point(const FFArgs& a, const Tgt& T, int q, ffacc* acc) {
  constexpr int NP = DL ? 6 : 3;  // value pairs per slot: (x.x x.y) (x.z f.x) (f.y f.z) | (g.x g.y) (g.z a.x) (a.y a.z)
  constexpr int NX = 2;           // the pairs that hold x: value terms by TwoSum
  const size_t per = (size_t)a.map.per;
  const size_t plane = (size_t)a.nlat * a.NQ;
  const size_t wi = (size_t)T.ilat0 * a.NQ + q;
  const int2 ix = __ldg(a.widx + wi);
  const int j1 = imod(ix.y + T.ilon0, a.nlon), j2 = (j1 + 1 == a.nlon) ? 0 : j1 + 1;
  const int i1 = ix.x, i2 = (i1 + 1 == a.m) ? 0 : i1 + 1;
  const int nodes[4] = {a.map.pos(i1, j1), a.map.pos(i1, j2), a.map.pos(i2, j1), a.map.pos(i2, j2)};
  Dot2 d2[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) { d2[k].s = T.offs[k]; d2[k].c = make_float2(0.f, 0.f); }
  // slots u_th, u_ph, u_thph first (FastTwoSum from off), then u (the x
  // pairs: off subtracted, TwoSum; the others: FastTwoSum, off subtracted after)
#pragma unroll
  for (int dd = 0; dd < 4; ++dd) {
    const int d = (dd + 1) & 3;
    if (d == 0) {
#pragma unroll
      for (int k = 0; k < NX; ++k) d2[k].s = sub2(d2[k].s, T.offs[k]);  // exact: off/2 <= s <= 3 off/2
    }
    const float4 wh4 = __ldg(a.w + d * plane + wi), wl4 = __ldg(a.w + (4 + d) * plane + wi);
    const float whs[4] = {wh4.x, wh4.y, wh4.z, wh4.w}, wls[4] = {wl4.x, wl4.y, wl4.z, wl4.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 wh = make_float2(whs[k], whs[k]), nwh = make_float2(-whs[k], -whs[k]);
      const float2 wl = make_float2(wls[k], wls[k]);
      const float4* r = T.base + 2 * ((size_t)(3 * d) * per + nodes[k]);
      float2 vh[DL ? 6 : 4], vl[DL ? 6 : 4];
#pragma unroll
      for (int i = 0; i < (DL ? 3 : 2); ++i) {  // SL: quads (x.x x.y x.z f.x) (f.y f.z . .)
        float4 h, l;
        ld8(r + 2 * (size_t)i * per, h, l);
        vh[2 * i] = make_float2(h.x, h.y); vh[2 * i + 1] = make_float2(h.z, h.w);
        vl[2 * i] = make_float2(l.x, l.y); vl[2 * i + 1] = make_float2(l.z, l.w);
      }
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        if (d == 0 && i < NX) d2[i].add<false>(wh, nwh, wl, vh[i], vl[i]);
        else d2[i].add<true>(wh, nwh, wl, vh[i], vl[i]);
      }
    }
  }
#pragma unroll
  for (int k = NX; k < NP; ++k) d2[k].s = sub2(d2[k].s, T.offs[k]);
  // interpolated x (relative to the cell centre), f, g, a3
  ff xx[3], F[3], G[3], A[3];
  xx[0] = ff_sub(d2[0].x(), T.xi[0]);
  xx[1] = ff_sub(d2[0].y(), T.xi[1]);
  xx[2] = ff_sub(d2[1].x(), T.xi[2]);
  F[0] = d2[1].y(); F[1] = d2[2].x(); F[2] = d2[2].y();
  if (DL) {
    G[0] = d2[3].x(); G[1] = d2[3].y(); G[2] = d2[4].x();
    A[0] = d2[4].y(); A[1] = d2[5].x(); A[2] = d2[5].y();
  }
  const ff r2 = ff_add(ff_add(ff_mul(xx[0], xx[0]), ff_mul(xx[1], xx[1])), ff_mul(xx[2], xx[2]));
  if (ff_ge(r2, a.rc2)) return;  // rr >= rc (ModRbcSingInt.F90:65)
  if (!(r2.h > 0.f)) return;
  // 1/r: rsqrtf, an FP32 Newton step, a float-float Newton step
  float y = rsqrtf(r2.h);
  y = y * fmaf(-0.5f * r2.h, y * y, 1.5f);
  const float y2 = __fmul_rn(y, y), y2e = fmaf(y, y, -y2);
  const float t0 = __fmul_rn(r2.h, y2);
  const float t1 = fmaf(r2.h, y2, -t0) + fmaf(r2.h, y2e, r2.l * y2);
  const float eps = __fsub_rn(__fsub_rn(1.f, t0), t1);  // 1 - r2 y^2
  const ff ir = fast_two_sum(y, 0.5f * y * eps);
  const ff rv = ff_norm(ff_mul(r2, ir));
  // EwaldCoeff_SL / _DL share the table position; below r_eps or beyond
  // the table both are zero
  if (!ff_ge(rv, a.r_eps)) return;
  const ff sp = ff_norm(ff_mul(rv, a.ntab_over_rc));
  float fi = floorf(sp.h);
  if (sp.h == fi && sp.l < 0.f) fi -= 1.f;
  const int it = (int)fi;
  if (it < 0 || it >= EWALD_NTAB) return;
  const ff f1 = two_sum(__fsub_rn(sp.h, fi), sp.l);
  const ff ir2 = ff_mul(ir, ir);
  const int irad = q % a.nrad;
  const ff wq = ld_ff(__ldg(a.pw + irad));
  ff cx = {0.f, 0.f}, cf = {0.f, 0.f};  // dv += cx xx + cf f
  if (SL) {
    const ff cs1 = tab_lerp(a.tab, 0, it, f1), cs2 = tab_lerp(a.tab, 1, it, f1);
    const ff c1ir = ff_mul(cs1, ir);
    const ff EA = ff_mul(ff_add(c1ir, cs2), ir2), EB = ff_sub(c1ir, cs2);
    // c1 wq (EA xx (xx . f) + EB f)
    const ff sw = ff_mul(a.c1, wq);
    cx = ff_mul(sw, ff_mul(EA, dot3(xx, F)));
    cf = ff_mul(sw, EB);
  }
  if (DL) {
    // c2 Bcoef wq EA xx (xx . g)(xx . a3), EA = cd / r^5
    const ff cd = tab_lerp(a.tab, 2, it, f1);
    const ff EA = ff_mul(cd, ff_mul(ir2, ff_mul(ir2, ir)));
    const ff t = ff_mul(ff_mul(ff_mul(T.c2m, wq), EA), ff_mul(dot3(xx, G), dot3(xx, A)));
    cx = SL ? ff_add(cx, t) : t;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    acc[k].add(ff_mul(cx, xx[k]));
    if (SL) acc[k].add(ff_mul(cf, F[k]));
  }
}

// One warp per target; the 8 warps of a block take 8 consecutive targets of
// a latitude ring, so that they share weight entries and most stencil nodes
// in L1.  The lanes of one pass take patch points in the order of their
// stencil cells' 2 x 2 node tiles (a per-latitude permutation), so that they
// read fewer distinct lines (6.71 -> 6.60 ms at 256 cells against the
// radial-ray order; raster order of the stencil cells: 7.25 ms).  (Packing the 8-point tails of 4 targets into one full pass saved
// 15% of the instructions but not time: the kernel is bound by the L1 data
// pipe, 7.08 against 6.81 ms at 256 cells.)
template <bool SL, bool DL>
__global__ void __launch_bounds__(256, 2) k_self_ff(FFArgs a) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= a.ncell * a.nlat * a.nlon) return;
  const Tgt T = target<DL>(a, w);
  ffacc acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  const short* pr = a.perm + (size_t)T.ilat0 * a.NQ;
  for (int k = lane; k < a.NQ; k += 32) patch_point<SL, DL>(a, T, pr[k], acc);
  double dv[3];
  for (int k = 0; k < 3; ++k) dv[k] = warp_sum((double)acc[k].s + (double)acc[k].c);
  if (lane == 0) {
    const double iA = 1.0 / a.tA[T.p];
    for (int k = 0; k < 3; ++k) a.v[T.p + (size_t)k * a.nt] += dv[k] * iA;
  }
}

// hi/lo split of an FP64 value
__device__ __forceinline__ void split(double v, float* h, float* l) {
  const float hv = (float)v;
  *h = hv;
  *l = (float)(v - (double)hv);
}

// node records of the spline sets named in `sets` (bit 0 x, 1 f, 2 g, 3 a3):
// value 3 s + c of slot d goes to component (3 s + c) % 4 of quad (3 s + c) / 4.
// bnd[s][cell] collects max |value| per slot (float bits, rounded up; a warp
// spanning two cells gives both the larger maximum).
__global__ void k_ff_rec(int ncell, int m, long long per, NodeMap map, const double* __restrict__ spl,
                         const double* __restrict__ xc, float4* __restrict__ out, unsigned* __restrict__ bnd, int sets) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = idx < (long long)ncell * per;
  const int cell = valid ? (int)(idx / per) : ncell - 1;
  const long long node = idx - (long long)cell * per;  // i + m j
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(0xffffffffu, cell, 1);
  const bool lead = lane == 0 || prev != cell;
  const int ni = valid ? (int)(node % m) : 0, nj = valid ? (int)(node / m) : 0;
  float* o = reinterpret_cast<float*>(out + (size_t)cell * FF_PLANES * map.per) + 8 * (size_t)map.pos(ni, nj);
  const size_t pstride = 8 * (size_t)map.per;  // floats between planes of 32-byte entries
  const int src[4] = {SPL_X, SPL_F, SPL_G, SPL_A3};
  for (int s = 0; s < 4; ++s) {
    if (!(sets & (1 << s))) continue;
    const double* sp = spl + (((size_t)cell * SPL_NSET + src[s]) * per + node) * SPL_NODE;
    for (int d = 0; d < 4; ++d) {
      unsigned mx = 0;
      if (valid)
        for (int c = 0; c < 3; ++c) {
          double v = sp[3 * d + c];
          if (s == 0 && d == 0) v -= xc[3 * cell + c];
          const int q = (3 * s + c) >> 2, e = (3 * s + c) & 3;
          split(v, o + (3 * d + q) * pstride + e, o + (3 * d + q) * pstride + 4 + e);
          mx = max(mx, __float_as_uint(__double2float_ru(fabs(v))));
        }
      mx = __reduce_max_sync(0xffffffffu, mx);
      if (valid && lead) atomicMax(bnd + ((size_t)s * ncell + cell) * 4 + d, mx);
    }
  }
}

inline ff hsplit(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

}  // namespace

// Ewald tables as {T_i, T_i+1 - T_i} hi/lo (ModEwaldFunc.F90:96-104, 151-162).
rbc3d_status self_ff_tables(rbc3d_ctx* ctx, const std::vector<double>& c1, const std::vector<double>& c2,
                            const std::vector<double>& dl) {
  const int N = EWALD_NTAB;
  std::vector<float4> t(3 * (size_t)N);
  const std::vector<double>* src[3] = {&c1, &c2, &dl};
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < N; ++i) {
      const double v = (*src[k])[i], d = (*src[k])[i + 1] - v;
      const ff a = hsplit(v), b = hsplit(d);
      t[(size_t)k * N + i] = make_float4(a.h, a.l, b.h, b.l);
    }
  CUDA_TRY(ctx->ff_tab.upload(t.data(), t.size(), ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

// Patch weights per (latitude, patch point) as hi/lo planes, from the FP64
// table of k_self, and the patch weights pw as hi/lo.
rbc3d_status self_ff_grid(rbc3d_ctx* ctx, const std::vector<SelfW64>& W, const std::vector<double>& pw) {
  const size_t n = W.size();
  std::vector<int2> idx(n);
  std::vector<float4> w(8 * n);
  for (size_t i = 0; i < n; ++i) {
    idx[i] = make_int2(W[i].i1, W[i].j1b);
    for (int d = 0; d < 4; ++d) {
      ff e[4];
      for (int k = 0; k < 4; ++k) e[k] = hsplit(W[i].w[4 * k + d]);
      w[(size_t)d * n + i] = make_float4(e[0].h, e[1].h, e[2].h, e[3].h);
      w[(size_t)(4 + d) * n + i] = make_float4(e[0].l, e[1].l, e[2].l, e[3].l);
    }
  }
  std::vector<float2> p(pw.size());
  for (size_t i = 0; i < pw.size(); ++i) {
    const ff e = hsplit(pw[i]);
    p[i] = make_float2(e.h, e.l);
  }
  // lane order of the patch points per latitude: by the 2 x 2 tile of their
  // stencil cell (i1, j1b), then by the cell inside the tile
  {
    const int nlat = ctx->nlat, NQ = (int)(n / nlat);
    std::vector<short> perm(n);
    std::vector<int> q(NQ);
    for (int l = 0; l < nlat; ++l) {
      for (int k = 0; k < NQ; ++k) q[k] = k;
      auto key = [&](int k) {
        const int2 t = idx[(size_t)l * NQ + k];
        const int i = t.x, j = t.y + 4096;  // j1b may be negative
        return ((long long)(i >> 1) * 100000 + (j >> 1)) * 4 + (i & 1) * 2 + (j & 1);
      };
      std::stable_sort(q.begin(), q.end(), [&](int a2, int b2) { return key(a2) < key(b2); });
      for (int k = 0; k < NQ; ++k) perm[(size_t)l * NQ + k] = (short)q[k];
    }
    CUDA_TRY(ctx->ff_perm.upload(perm.data(), perm.size(), ctx->st));
  }
  CUDA_TRY(ctx->ff_widx.upload(idx.data(), idx.size(), ctx->st));
  CUDA_TRY(ctx->ff_w.upload(w.data(), w.size(), ctx->st));
  CUDA_TRY(ctx->ff_pw.upload(p.data(), p.size(), ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

// Node records are rebuilt on first use after the positions or densities change.
void self_ff_invalidate(rbc3d_ctx* ctx, bool geom, bool f, bool g) {
  if (geom) ctx->ff_sets &= ~(1 | 8);
  if (f) ctx->ff_sets &= ~2;
  if (g) ctx->ff_sets &= ~4;
}

// The float-float node records of the sets in `need` (bit 0 x, 1 f, 2 g,
// 3 a3) that are out of date, on the current stream.
rbc3d_status self_ff_records(rbc3d_ctx* ctx, int need) {
  const long long per = (long long)ctx->m * ctx->nlon;
  const NodeMap map = node_map(ctx->m, ctx->nlon);
  if (!ctx->ff_rec.p || ctx->ff_rec.n < (size_t)ctx->ncell * map.per * FF_PLANES) {
    CUDA_TRY(ctx->ff_rec.alloc((size_t)ctx->ncell * map.per * FF_PLANES));
    ctx->ff_sets = 0;
  }
  CUDA_TRY(ctx->ff_bnd.alloc(16 * (size_t)ctx->ncell));
  const int build = need & ~ctx->ff_sets;
  if (build) {
    for (int k = 0; k < 4; ++k)
      if (build & (1 << k))
        CUDA_TRY(cudaMemsetAsync(ctx->ff_bnd.p + 4 * (size_t)k * ctx->ncell, 0, 16 * (size_t)ctx->ncell, ctx->st));
    { k_ff_rec<<<nblk(ctx->ncell * per, 256), 256, 0, ctx->st>>>(ctx->ncell, ctx->m, per, map, ctx->spl.p,
                                                                  ctx->mix_xc.p, ctx->ff_rec.p, ctx->ff_bnd.p, build);
      ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
    ctx->ff_sets |= build;
  }
  return RBC3D_OK;
}

rbc3d_status run_self_ff(rbc3d_ctx* ctx, int tlist, double c1, double c2) {
  TargetSet& t = ctx->tl[tlist];
  if (tlist != RBC3D_TLIST_RBC || t.n == 0 || ctx->ncell == 0) return RBC3D_OK;
  if (!ctx->phi_uniform) return ctx_fail(ctx, RBC3D_ERR_ARG, "FP32D needs phi(j) = j*2*pi/nlon");
  const bool sl = c1 != 0 && ctx->has_f, dl = c2 != 0 && ctx->has_g;
  if (!sl && !dl) return RBC3D_OK;
  const NodeMap map = node_map(ctx->m, ctx->nlon);
  // records this call reads: x always, f for SL, g and a3 for DL
  rbc3d_status s = self_ff_records(ctx, 1 | (sl ? 2 : 0) | (dl ? 4 | 8 : 0));
  if (s) return s;
  FFArgs a;
  a.nt = t.n; a.ncell = ctx->ncell; a.nlat = ctx->nlat; a.nlon = ctx->nlon; a.m = ctx->m;
  a.NQ = ctx->nrad * ctx->nazm; a.nrad = ctx->nrad;
  a.tA = t.Acoef.p; a.v = t.v.p; a.rec = ctx->ff_rec.p;
  a.widx = ctx->ff_widx.p; a.w = ctx->ff_w.p; a.pw = ctx->ff_pw.p;
  a.thi = ctx->mix_thi.p; a.tlo = ctx->mix_tlo.p; a.tab = ctx->ff_tab.p; a.celltype = ctx->celltype.p;
  a.perm = ctx->ff_perm.p;
  a.bnd = reinterpret_cast<const uint4*>(ctx->ff_bnd.p);
  a.map = map;
  const double hx = RBC3D_TWO_PI / ctx->m, hy = RBC3D_TWO_PI / ctx->nlon;
  a.hq1 = (float)(hx / 4); a.hq2 = (float)(hy / 4); a.hq12 = (float)(hx * hy / 16);
  const ff z = {0.f, 0.f};
  a.c1 = sl ? hsplit(c1) : z;
  for (int l = 0; l < RBC3D_MAX_CELLTYPES; ++l) a.c2B[l] = dl ? hsplit(c2 * ctx->Bcoef[l]) : z;
  a.rc2 = hsplit(ctx->prm.rc * ctx->prm.rc);
  a.r_eps = hsplit(ctx->T.r_eps);
  a.ntab_over_rc = hsplit(ctx->T.ntab_over_rc);
  const int grid = (int)((t.n + 7ll) / 8);  // blocks of 8 warps, one target each
  if (sl && dl) { k_self_ff<true, true><<<grid, 256, 0, ctx->st>>>(a); ++ctx->launches; }
  else if (sl) { k_self_ff<true, false><<<grid, 256, 0, ctx->st>>>(a); ++ctx->launches; }
  else { k_self_ff<false, true><<<grid, 256, 0, ctx->st>>>(a); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}
