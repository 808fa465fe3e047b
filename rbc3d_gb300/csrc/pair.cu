// pair.cu -- cell lists and the real-space Stokeslet / stresslet pair sums of
// AddIntOnRbcs (ModIntOnRbcs.F90:47-112) on the GPU.
//
// Cell list: the linked lists hoc/next of HashTable_Build (ModHashTable.F90:
// 23-62) become a stable radix sort of the points by cell id plus
// [start, end) ranges per cell.  The same Nc = max(floor(L/rc), 3) cells are
// used, so a target visits its 27 neighbour cells exactly as the reference.
//
// Pair kernels: work units of one target cell's targets (a cell's units
// equal-sized, heaviest units launched first), each thread owning one
// target; the 27 neighbour cells are streamed through shared memory.  FP64:
// one CTA per unit of <= 128 targets, tiles of 128 sources shared by the
// CTA.  FP32: one warp per unit of <= 32 targets, each warp staging its own
// 32-source chunks, so the four warps of a CTA may serve different cells
// (CTA-sized units left 18% of the CTAs' thread slots idle on the 256-cell
// workload, warp units 5%).  Tiles whose bounding box lies farther than rc
// from the CTA's (or a warp's) targets are skipped.  FP32 with cell targets:
// the own-cell pairs (79% of the pairs on the 256-cell workload) go to a
// dense per-cell pass (k_pair_own32), and k_pair32 skips the target's own
// surface (whole tiles and chunks when a warp's targets share one surface).
// FP32: sources carry hi/lo FP32
// coordinates relative to their own cell centre (from FP64, once per
// position update) and the targets are shifted into each neighbour cell's
// frame with an error-free difference, so x_j - x_i keeps full FP32 accuracy
// regardless of the box size; each target accumulates with Kahan
// compensation.  FP64 (the plain form): positions relative to the target
// cell centre, reference table arithmetic.
#include <cub/cub.cuh>

#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "ctx.hpp"

namespace {

constexpr int TILE = 128;

__global__ void k_hash_keys(int n, const double* __restrict__ x, int Nc0, int Nc1, int Nc2, double s0, double s1,
                            double s2, int* __restrict__ key, int* __restrict__ idx) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  // HashTable_Index, ModHashTable.F90:67-94 (single node): modulo(floor(x*Nc/L), Nc)
  int i1 = imod((int)floor(x[p] * s0), Nc0);
  int i2 = imod((int)floor(x[p + n] * s1), Nc1);
  int i3 = imod((int)floor(x[p + 2 * (size_t)n] * s2), Nc2);
  key[p] = i1 + Nc0 * (i2 + Nc1 * i3);
  idx[p] = p;
}

__global__ void k_cell_ranges(int n, const int* __restrict__ key, int* __restrict__ cs, int* __restrict__ ce) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int k = key[p];
  if (p == 0 || key[p - 1] != k) cs[k] = p;
  if (p == n - 1 || key[p + 1] != k) ce[k] = p + 1;
}

// Lists built on the device from sorted cell ranges (no host round trip).
// Every list has a fixed capacity (an upper bound on its length); the
// entries past its true length are empty (zero counts) and their consumers
// skip them.

// pieces[c] = ceil(count of cell c / P); pieces[nc] = 0 (the scan's total)
__global__ void k_piece_counts(int nc, const int* __restrict__ cs, const int* __restrict__ ce, int P,
                               int* __restrict__ pieces) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > nc) return;
  pieces[c] = c < nc ? (ce[c] - cs[c] + P - 1) / P : 0;
}

// (first, count) of the P-sized pieces of every cell, at off[c] (exclusive
// scan of the piece counts); entries [off[nc], cap) are cleared
__global__ void k_fill_pieces(int nc, const int* __restrict__ cs, const int* __restrict__ ce, int P,
                              const int* __restrict__ off, int cap, int2* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nc) {
    const int b0 = cs[c], e = ce[c];
    int k = off[c];
    for (int b = b0; b < e; b += P) out[k++] = make_int2(b, min(P, e - b));
  }
  for (int i = off[nc] + c; i < cap; i += gridDim.x * blockDim.x) out[i] = make_int2(0, 0);
}

// Work units of the pair sums (the cells' targets in equal-sized units of at
// most `tile`), keyed by their work: targets x the sources of the 27
// neighbour cells.  Unit counts first, then the units at the scanned offsets.
__global__ void k_unit_counts(int nc, int tile, const int* __restrict__ cs, const int* __restrict__ ce,
                              int* __restrict__ cnt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > nc) return;
  cnt[c] = c < nc ? (ce[c] - cs[c] + tile - 1) / tile : 0;
}
__global__ void k_fill_units(int nc, int tile, int Nc0, int Nc1, int Nc2, const int* __restrict__ cs, const int* __restrict__ ce,
                             const int* __restrict__ ss, const int* __restrict__ se, const int* __restrict__ off,
                             int cap, int4* __restrict__ units, long long* __restrict__ key, int* __restrict__ idx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nc) {
    const int cnt = ce[c] - cs[c];
    if (cnt > 0) {
      const int ci = c % Nc0, cj = (c / Nc0) % Nc1, ck = c / (Nc0 * Nc1);
      long long nsrc = 0;
      for (int nb = 0; nb < 27; ++nb) {
        const int ni = (ci + nb % 3 - 1 + Nc0) % Nc0, nj = (cj + (nb / 3) % 3 - 1 + Nc1) % Nc1;
        const int nk = (ck + nb / 9 - 1 + Nc2) % Nc2;
        const int q = ni + Nc0 * (nj + Nc1 * nk);
        nsrc += se[q] - ss[q];
      }
      const int k = (cnt + tile - 1) / tile, per = (cnt + k - 1) / k;
      int u = off[c];
      for (int b = 0; b < cnt; b += per, ++u) {
        const int m = min(per, cnt - b);
        units[u] = make_int4(c, cs[c] + b, m, 0);
        key[u] = nsrc * m;
        idx[u] = u;
      }
    }
  }
  for (int i = off[nc] + c; i < cap; i += gridDim.x * blockDim.x) {
    units[i] = make_int4(0, 0, 0, 0);
    key[i] = -1;
    idx[i] = i;
  }
}
__global__ void k_gather_units(int cap, const int* __restrict__ idx, const int4* __restrict__ in,
                               int4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cap) out[i] = in[idx[i]];
}

// Gather cell-point geometry into cell-list order.
__global__ void k_gather_src(int n, int nlat, int nv, const int* __restrict__ order, const double* __restrict__ x,
                             double* __restrict__ sx, int4* __restrict__ meta) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int p = order[q];
  for (int k = 0; k < 3; ++k) sx[q + (size_t)k * n] = x[p + (size_t)k * n];
  int cell = p / nv, r = p - cell * nv;
  meta[q] = make_int4(cell + 1, r % nlat, r / nlat, p);
}

// The sources' normals, sorted (FP64) and as FP32 records.
__global__ void k_gather_a3(int n, const int* __restrict__ order, const double* __restrict__ a3,
                            double* __restrict__ sa3, float4* __restrict__ a4) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int p = order[q];
  double v[3];
  for (int k = 0; k < 3; ++k) {
    v[k] = a3[p + (size_t)k * n];
    sa3[q + (size_t)k * n] = v[k];
  }
  a4[q] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
}

__device__ __forceinline__ double min_image(double d, double L, double iL) { return d - round(d * iL) * L; }

// FP32 pair-sum records of the sorted sources (see PairArgs); the normals'
// records come from k_gather_a3.
__global__ void k_src_records(int n, const double* __restrict__ sx, const int4* __restrict__ meta,
                              const float4* __restrict__ usph, int nlat, int Nc0, int Nc1, int Nc2, double h0,
                              double h1, double h2, double L0, double L1, double L2, float4* __restrict__ p0,
                              float4* __restrict__ p1, float4* __restrict__ u4) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int Nc[3] = {Nc0, Nc1, Nc2};
  const double h[3] = {h0, h1, h2}, L[3] = {L0, L1, L2};
  float hi[3], lo[3];
  for (int k = 0; k < 3; ++k) {
    const double x = sx[q + (size_t)k * n];
    const int c = imod((int)floor(x * (Nc[k] / L[k])), Nc[k]);  // HashTable_Index
    const double r = min_image(x - (c + 0.5) * h[k], L[k], 1.0 / L[k]);
    hi[k] = (float)r;
    lo[k] = (float)(r - (double)hi[k]);
  }
  const int4 m = meta[q];
  p0[q] = make_float4(hi[0], hi[1], hi[2], __int_as_float(m.x));
  p1[q] = make_float4(lo[0], lo[1], lo[2], __int_as_float(m.y | (m.z << 16)));
  u4[q] = usph[m.y + nlat * m.z];
}

// Bounding box of each tile (TILE consecutive sources of one cell), from the
// hi coordinates, with the range of the sources' surfaces in w (int bits);
// tiles listed as (first source, count).
__global__ void k_tile_boxes(const int2* __restrict__ tiles, const float4* __restrict__ p0, float4* __restrict__ box) {
  const int2 t = tiles[blockIdx.x];
  const float big = 3.0e38f;
  float3 lo = make_float3(big, big, big), hi = make_float3(-big, -big, -big);
  int smin = INT_MAX, smax = INT_MIN;
  for (int i = threadIdx.x; i < t.y; i += blockDim.x) {
    const float4 p = p0[t.x + i];
    lo.x = fminf(lo.x, p.x); lo.y = fminf(lo.y, p.y); lo.z = fminf(lo.z, p.z);
    hi.x = fmaxf(hi.x, p.x); hi.y = fmaxf(hi.y, p.y); hi.z = fmaxf(hi.z, p.z);
    smin = min(smin, __float_as_int(p.w)); smax = max(smax, __float_as_int(p.w));
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo.x = fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
    lo.y = fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
    lo.z = fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
    hi.x = fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
    hi.y = fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
    hi.z = fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
    smin = min(smin, __shfl_xor_sync(0xffffffffu, smin, o));
    smax = max(smax, __shfl_xor_sync(0xffffffffu, smax, o));
  }
  __shared__ float3 red[32][2];
  __shared__ int sred[32][2];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[w][0] = lo; red[w][1] = hi; sred[w][0] = smin; sred[w][1] = smax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      lo.x = fminf(lo.x, red[k][0].x); lo.y = fminf(lo.y, red[k][0].y); lo.z = fminf(lo.z, red[k][0].z);
      hi.x = fmaxf(hi.x, red[k][1].x); hi.y = fmaxf(hi.y, red[k][1].y); hi.z = fmaxf(hi.z, red[k][1].z);
      smin = min(smin, sred[k][0]); smax = max(smax, sred[k][1]);
    }
    box[2 * blockIdx.x] = make_float4(lo.x, lo.y, lo.z, __int_as_float(smin));
    box[2 * blockIdx.x + 1] = make_float4(hi.x, hi.y, hi.z, __int_as_float(smax));
  }
}

// Point-order records of the own-cell pair sums: hi/lo FP32 of the position
// relative to the cell's first point (minimum image: a cell spans less than
// half the box), the grid indices, and the point's sorted source position.
__global__ void k_own_records(int n, int nlat, int nv, const double* __restrict__ x, const int* __restrict__ order,
                              double L0, double L1, double L2, float4* __restrict__ op0, float4* __restrict__ op1,
                              int* __restrict__ sinv) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) sinv[order[q]] = q;
  const int p = q;
  if (p >= n) return;
  const int cell = p / nv, r = p - cell * nv;
  const double L[3] = {L0, L1, L2};
  float hi[3], lo[3];
  for (int k = 0; k < 3; ++k) {
    const double d = min_image(x[p + (size_t)k * n] - x[(size_t)cell * nv + (size_t)k * n], L[k], 1.0 / L[k]);
    hi[k] = (float)d;
    lo[k] = (float)(d - (double)hi[k]);
  }
  op0[p] = make_float4(hi[0], hi[1], hi[2], __int_as_float((r % nlat) | ((r / nlat) << 16)));
  op1[p] = make_float4(lo[0], lo[1], lo[2], 0.f);
}

// c1 f dS and c2 g dS Bcoef of the sorted sources in FP32 (per call).
__global__ void k_src_dens4(int n, double c1, double c2, const double* __restrict__ sf, const double* __restrict__ sg,
                            int do_g, float4* __restrict__ F, float4* __restrict__ Gv) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  F[q] = make_float4((float)(c1 * sf[q]), (float)(c1 * sf[q + n]), (float)(c1 * sf[q + 2 * (size_t)n]), 0.f);
  if (do_g)
    Gv[q] = make_float4((float)(c2 * sg[q]), (float)(c2 * sg[q + n]), (float)(c2 * sg[q + 2 * (size_t)n]), 0.f);
}

// SourceList_UpdateDensity (ModSourceList.F90:160-189): f*dS, g*dS with
// dS = detJ*w(ilat); the sorted copy of g also carries Bcoef of the cell type.
__global__ void k_density(int n, int nlat, int nv, const double* __restrict__ f, const double* __restrict__ detJ,
                          const double* __restrict__ w, double* __restrict__ sf) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int ilat = (p % nv) % nlat;
  double ds = detJ[p] * w[ilat];
  for (int k = 0; k < 3; ++k) sf[p + (size_t)k * n] = f[p + (size_t)k * n] * ds;
}
__global__ void k_gather_density(int n, int nv, const int* __restrict__ order, const double* __restrict__ sf,
                                 const double* __restrict__ sg, const int* __restrict__ celltype,
                                 const double* __restrict__ Bc, double* __restrict__ ssf, double* __restrict__ ssg,
                                 int do_f, int do_g) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int p = order[q];
  double B = Bc[celltype[p / nv]];
  for (int k = 0; k < 3; ++k) {
    if (do_f) ssf[q + (size_t)k * n] = sf[p + (size_t)k * n];
    if (do_g) ssg[q + (size_t)k * n] = sg[p + (size_t)k * n] * B;
  }
}

struct PairArgs {
  // targets
  int nt;
  const double* tx;
  const double* tA;
  const int4* tmeta;
  const int* torder;
  const int4* units;
  int nunits;  // k_pair32: warp units
  double* v;  // 3*nt accumulator
  // sources (sorted)
  int ns;
  const double* sx;
  const double* sf;
  const double* sg;
  const double* sa3;
  const int4* smeta;
  const int* cs;
  const int* ce;
  // FP32 source records (sorted order) and tile boxes
  const float4* sp0;   // (x, y, z) hi relative to the source's hash-cell centre, surf bits
  const float4* sp1;   // (x, y, z) lo, id bits (ilat | ilon << 16)
  const float4* su;    // unit-sphere coordinates of the grid point
  const float4* sa4;   // a3
  const float4* sF4;   // c1 f dS
  const float4* sG4;   // c2 g dS Bcoef
  const int* toff;     // per hash cell: first tile (TILE consecutive sources per tile)
  const float4* tbox;  // per tile: lo, hi (relative to the cell centre)
  const int* coff;     // per hash cell: first 32-source chunk
  const float4* cbox;  // per chunk: lo, hi
  // grid
  int Nc[3];
  double h[3], L[3], iL[3];
  const double* th;
  const double* phi;
  const float4* usph;
  int nlat, nlon, nhalf;
  const double* mtab64;  // MaskFunc of same-cell grid pairs, (ilat_i, ilat_j, |dlon|), or null
  const float* mtab32;   // 1 - mask in FP32
  double radius, inv_radius;
  float inv_radius_f, chord2_max;
  double c1, c2;
  float c1f, c2f;
  double rc2;
  float rc2_f, reps2_f;
  float rc2_loose;  // (rc + 1e-3)^2: hi-part reject threshold of the FP32 pair kernel
  float rthr2_f;  // FP32 path: cross-surface pairs closer than this are left to the FP64 near-singular pass
  float sqpa_f, two_isqa_f, m8_ispi_f, q75_spi_f;  // sqrt(pi/alpha), 2/sqrt(alpha), -8/sqrt(pi), 0.75 sqrt(pi)
  float erfcx_q[ERFCX_DEG + 1];  // erfc(x) exp(x^2) = t Q(t), t = 1/(1 + x/2), on [0, rc sqrt(pi/alpha)]
  Tables T;
  // near-singular work list
  int collect;
  int4* items;
  int cap;
  unsigned long long* cnt;  // [0] items, [1] pairs, [2] overflow
  // own-cell pairs of the FP32 modes (cell targets, same-cell weight table):
  // k_pair_own32 takes them and k_pair32 skips same-surface sources
  int own_split;
  const float4* op0;  // per point (point order): (x, y, z) hi relative to its cell's first point, id bits
  const float4* op1;  // lo
  const int* sinv;    // point -> sorted source position
};


struct NbrList {
  int n;
  int surf[RBC3D_NBR_MAX];
  int idx[RBC3D_NBR_MAX];  // ilat | ilon << 16
  float d2[RBC3D_NBR_MAX];
  int overflow;
  __device__ __forceinline__ void insert(int s, int id, float d) {
    for (int e = 0; e < n; ++e)
      if (surf[e] == s) {
        if (d < d2[e]) { d2[e] = d; idx[e] = id; }
        return;
      }
    if (n < RBC3D_NBR_MAX) { surf[n] = s; idx[n] = id; d2[n] = d; ++n; }
    else overflow = 1;
  }
};

// Shared-memory source tile of the FP64 pair kernel
struct TileD {
  double x[TILE], y[TILE], z[TILE];
  double fx[TILE], fy[TILE], fz[TILE], gx[TILE], gy[TILE], gz[TILE];
  double ax[TILE], ay[TILE], az[TILE];
  int surf[TILE], ilat[TILE], ilon[TILE];
};

// Box-to-box distance test of the tile culling: true if every point of box
// [alo, ahi] is farther than sqrt(rc2) from every point of [blo, bhi].  The
// boxes hold FP32 coordinates; the margin absorbs their rounding.
__device__ __forceinline__ bool boxes_apart(float3 alo, float3 ahi, float3 blo, float3 bhi, float rc2) {
  float gx = fmaxf(0.f, fmaxf(alo.x - bhi.x, blo.x - ahi.x));
  float gy = fmaxf(0.f, fmaxf(alo.y - bhi.y, blo.y - ahi.y));
  float gz = fmaxf(0.f, fmaxf(alo.z - bhi.z, blo.z - ahi.z));
  float g = sqrtf(gx * gx + gy * gy + gz * gz) - 1e-3f;
  return g > 0.f && g * g > rc2;
}

__device__ __forceinline__ void warp_minmax(float3& lo, float3& hi) {
  for (int o = 16; o > 0; o >>= 1) {
    lo.x = fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
    lo.y = fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
    lo.z = fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
    hi.x = fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
    hi.y = fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
    hi.z = fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
  }
}

// Error-free a - b = s + e (Knuth TwoSum).
__device__ __forceinline__ void two_diff(float a, float b, float& s, float& e) {
  s = a - b;
  float bb = a - s;
  e = (a - (s + bb)) + (bb - b);
}

// Target and tile bounding boxes of the culling, shared by both precisions.
struct CullBoxes {
  float3 wlo, whi;  // this warp's targets
  float3 clo, chi;  // the CTA's targets
};

__device__ __forceinline__ CullBoxes cull_boxes(bool active, float tx, float ty, float tz, float3 (*wb)[2]) {
  const float big = 3.0e38f;
  CullBoxes b;
  b.wlo = active ? make_float3(tx, ty, tz) : make_float3(big, big, big);
  b.whi = active ? make_float3(tx, ty, tz) : make_float3(-big, -big, -big);
  warp_minmax(b.wlo, b.whi);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) { wb[w][0] = b.wlo; wb[w][1] = b.whi; }
  __syncthreads();
  b.clo = wb[0][0]; b.chi = wb[0][1];
  for (int k = 1; k < nw; ++k) {
    b.clo.x = fminf(b.clo.x, wb[k][0].x); b.clo.y = fminf(b.clo.y, wb[k][0].y); b.clo.z = fminf(b.clo.z, wb[k][0].z);
    b.chi.x = fmaxf(b.chi.x, wb[k][1].x); b.chi.y = fmaxf(b.chi.y, wb[k][1].y); b.chi.z = fmaxf(b.chi.z, wb[k][1].z);
  }
  return b;
}

__device__ __forceinline__ float3 f3sub(float3 a, float3 d) { return make_float3(a.x - d.x, a.y - d.y, a.z - d.z); }

// Per-warp source chunk in structure-of-arrays form, so that two consecutive
// sources' components load as one float2 for the packed FP32x2 arithmetic.
template <bool DL>
struct ChunkX2 {
  float hx[32], hy[32], hz[32], lx[32], ly[32], lz[32];
  float fx[32], fy[32], fz[32];
  float gx[DL ? 32 : 2], gy[DL ? 32 : 2], gz[DL ? 32 : 2];
  float ax[DL ? 32 : 2], ay[DL ? 32 : 2], az[DL ? 32 : 2];
  int surf[32], id[32];
};

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 ld2(const float* p, int j) { return *reinterpret_cast<const float2*>(p + j); }

// The coefficients of the Ewald real-space kernels (EwaldCoeff_SL /
// EwaldCoeff_DL, ModEwaldFunc.F90:86-180) at two pair distances at once, in
// packed FP32x2 arithmetic: the Stokeslet term A (x.f) x + B f and the
// stresslet factor Adl of (x.g)(x.n) x, for squared distances r2 (a pair of
// weight 0 enters with r^2 = 1, harmless).
template <bool DL>
__device__ __forceinline__ void ewald_coef2(const PairArgs& a, float2 r2, float wa, float wb, float2& A, float2& B,
                                            float2& Adl) {
  const float2 sqpa2 = f2(a.sqpa_f, a.sqpa_f), half2 = f2(0.5f, 0.5f), one2 = f2(1.f, 1.f);
  const float2 tisqa2 = f2(a.two_isqa_f, a.two_isqa_f);
  const float2 rs = f2(wa != 0.f ? r2.x : 1.f, wb != 0.f ? r2.y : 1.f);
  const float2 rinv = f2(rsqrtf(rs.x), rsqrtf(rs.y));
  const float2 r = __fmul2_rn(rs, rinv);
  const float2 st = __fmul2_rn(r, sqpa2);
  const float2 ex = f2(__expf(-st.x * st.x), __expf(-st.y * st.y));
  const float2 den = __ffma2_rn(half2, st, one2);
  const float2 tq = f2(__fdividef(1.f, den.x), __fdividef(1.f, den.y));
  float2 Q = f2(a.erfcx_q[ERFCX_DEG], a.erfcx_q[ERFCX_DEG]);
#pragma unroll
  for (int k = ERFCX_DEG - 1; k >= 0; --k) Q = __ffma2_rn(Q, tq, f2(a.erfcx_q[k], a.erfcx_q[k]));
  const float2 c1 = __fmul2_rn(ex, __fmul2_rn(tq, Q)), c2 = __fmul2_rn(tisqa2, ex);
  const float2 ir2 = __fmul2_rn(rinv, rinv);
  const float2 c1r = __fmul2_rn(c1, rinv);
  A = __fmul2_rn(__fadd2_rn(c1r, c2), ir2);
  B = __fadd2_rn(c1r, f2(-c2.x, -c2.y));
  if (DL) {
    const float2 st2 = __fmul2_rn(st, st);
    const float2 cdl = __fmul2_rn(f2(a.m8_ispi_f, a.m8_ispi_f),
                                  __ffma2_rn(ex, __fmul2_rn(st, __fadd2_rn(f2(1.5f, 1.5f), st2)),
                                             __fmul2_rn(f2(a.q75_spi_f, a.q75_spi_f), c1)));
    Adl = __fmul2_rn(__fmul2_rn(cdl, __fmul2_rn(ir2, ir2)), rinv);
  }
}

// A (x.f) x + B f + Adl (x.g)(x.n) x for two pairs (DL: the last term)
template <bool DL>
__device__ __forceinline__ void ewald_apply2(float2 xx, float2 yy, float2 zz, float2 A, float2 B, float2 Adl,
                                             float2 fx, float2 fy, float2 fz, float2 gx, float2 gy, float2 gz,
                                             float2 nx, float2 ny, float2 nz, float2& vx, float2& vy, float2& vz) {
  const float2 Ad = __fmul2_rn(A, __ffma2_rn(xx, fx, __ffma2_rn(yy, fy, __fmul2_rn(zz, fz))));
  vx = __ffma2_rn(Ad, xx, __fmul2_rn(B, fx));
  vy = __ffma2_rn(Ad, yy, __fmul2_rn(B, fy));
  vz = __ffma2_rn(Ad, zz, __fmul2_rn(B, fz));
  if (DL) {
    const float2 dg = __ffma2_rn(xx, gx, __ffma2_rn(yy, gy, __fmul2_rn(zz, gz)));
    const float2 da = __ffma2_rn(xx, nx, __ffma2_rn(yy, ny, __fmul2_rn(zz, nz)));
    const float2 t = __fmul2_rn(__fmul2_rn(Adl, dg), da);
    vx = __ffma2_rn(t, xx, vx);
    vy = __ffma2_rn(t, yy, vy);
    vz = __ffma2_rn(t, zz, vz);
  }
}

// The Ewald real-space kernels of two sources at once added to (cx, cy, cz)
// with the weights wa, wb: pair vectors (xx, yy, zz) with squares r2, the
// sources' c1 f dS (f*), c2 g dS Bcoef (g*) and normals (n*).
template <bool DL>
__device__ __forceinline__ void ewald_pair2(const PairArgs& a, float2 xx, float2 yy, float2 zz, float2 r2, float wa,
                                            float wb, float2 fx, float2 fy, float2 fz, float2 gx, float2 gy, float2 gz,
                                            float2 nx, float2 ny, float2 nz, float& cx, float& cy, float& cz) {
  float2 A, B, Adl, vx, vy, vz;
  ewald_coef2<DL>(a, r2, wa, wb, A, B, Adl);
  ewald_apply2<DL>(xx, yy, zz, A, B, Adl, fx, fy, fz, gx, gy, gz, nx, ny, nz, vx, vy, vz);
  cx = fmaf(wb, vx.y, fmaf(wa, vx.x, cx));
  cy = fmaf(wb, vy.y, fmaf(wa, vy.x, cy));
  cz = fmaf(wb, vz.y, fmaf(wa, vz.x, cz));
}

// FP32 real-space pair sums (EwaldCoeff_SL / EwaldCoeff_DL of ModEwaldFunc
// over the 27 neighbour hash cells, AddIntOnRbcs ModIntOnRbcs.F90:25-160).
// One CTA per (hash cell, up to TILE targets).  Sources carry FP32 hi/lo
// coordinates relative to their own cell centre; per neighbour cell the
// targets are shifted into that frame with an error-free difference, so the
// pair vector keeps full FP32 accuracy however far from the origin the cells
// are.  Source tiles (TILE consecutive sources of a cell) whose bounding box
// is farther than rc from the CTA's targets are not loaded, and a warp skips
// a loaded tile that is out of its own targets' reach.
// Each warp stages its own 32-source chunks (no block barrier).  The inner
// loop runs over pairs of sources: the geometric tests, weights and
// neighbour bookkeeping stay per source and in source order; the Ewald
// kernels of both sources run in packed FP32x2 arithmetic (__ffma2_rn /
// __fmul2_rn / __fadd2_rn, round-to-nearest like the scalar operations), a
// source that does not contribute entering with weight 0 and a harmless
// r^2 = 1 (4.20 -> 3.96 ms against the one-source loop on the 256-cell
// workload).  Eight 128-thread blocks per SM (64 registers a thread, 132
// bytes of spills): with the own-cell pairs taken by k_pair_own32 this
// kernel runs a little longer than at six blocks (80 registers), but the
// PME spread beside it gets its SMs sooner (the FP32D matvec 10.62 -> 10.52
// ms on the 256-cell workload; four, five and seven blocks: 10.65, 10.61,
// 10.58).  Before the own-cell split, six blocks against the unbounded 96
// registers: 3.58 against 3.76 ms alone; Estrin's scheme for the fitted erfc
// polynomial measured slower.
template <bool DL>
__global__ void __launch_bounds__(TILE, 8) k_pair32(PairArgs a) {
  __shared__ __align__(16) ChunkX2<DL> s_ch[TILE / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int wu = blockIdx.x * (TILE / 32) + wid;  // this warp's unit
  if (wu >= a.nunits) return;
  const int4 unit = a.units[wu];
  if (unit.z == 0) return;  // the empty tail
  const int cell = unit.x;
  const bool active = lane < unit.z;
  const int ci = cell % a.Nc[0], cj = (cell / a.Nc[0]) % a.Nc[1], ck = cell / (a.Nc[0] * a.Nc[1]);
  const double c0[3] = {(ci + 0.5) * a.h[0], (cj + 0.5) * a.h[1], (ck + 0.5) * a.h[2]};
  int ti = active ? a.torder[unit.y + lane] : 0;
  float th_[3] = {0, 0, 0}, tl_[3] = {0, 0, 0};
  float4 ui = make_float4(0, 0, 0, 0);
  int surf_i = -2, tlat = 0, tlon = 0;
  if (active) {
    for (int k = 0; k < 3; ++k) {
      double r = min_image(a.tx[ti + (size_t)k * a.nt] - c0[k], a.L[k], a.iL[k]);
      th_[k] = (float)r;
      tl_[k] = (float)(r - (double)th_[k]);
    }
    int4 m = a.tmeta[ti];
    surf_i = m.x;
    if (m.y >= 0) { ui = a.usph[m.y + a.nlat * m.z]; tlat = m.y; tlon = m.z; }
  }
  const float* mrow = a.mtab32 ? a.mtab32 + (size_t)tlat * a.nlat * a.nhalf : nullptr;
  float3 wlo0, whi0;
  {
    const float big = 3.0e38f;
    wlo0 = active ? make_float3(th_[0], th_[1], th_[2]) : make_float3(big, big, big);
    whi0 = active ? make_float3(th_[0], th_[1], th_[2]) : make_float3(-big, -big, -big);
    warp_minmax(wlo0, whi0);
  }
  ChunkX2<DL>& C = s_ch[wid];
  Kahan3 acc;
  acc.zero();
  NbrList L;
  L.n = 0; L.overflow = 0;
  int run_surf = -3, run_id = -1;
  float run_d2 = 3.4e38f;
  unsigned npairs = 0;  // < 2^32 pairs per target
  // own-cell pairs left to k_pair_own32: the warp's surface when all its
  // targets share one (whole tiles and chunks of it are skipped), else -7
  int wsurf = -7;
  if (a.own_split) {
    const int s0 = __shfl_sync(0xffffffffu, surf_i, 0);
    wsurf = __all_sync(0xffffffffu, !active || surf_i == s0) ? s0 : -7;
  }

  // per-source bookkeeping in source order: neighbour-surface runs, the pair
  // count, the weight (0 when the pair does not contribute here)
  // (the closest point per other surface: runs of accepted pairs of one
  // surface, each run's minimum merged into L by surface, so sources that
  // are out of reach need no bookkeeping)
  auto weight = [&](int sj, int idj, float r2, bool ok, int qglob) -> float {
    if (!ok) return 0.f;
    ++npairs;
    float wgt = 1.f;
    if (sj == surf_i && mrow) {
      int dl = abs((idj >> 16) - tlon);
      dl = min(dl, a.nlon - dl);
      wgt = __ldg(mrow + (idj & 0xffff) * a.nhalf + dl);
    } else if (sj == surf_i) {
      const float4 u = a.su[qglob];
      const float ex = ui.x - u.x, ey = ui.y - u.y, ez = ui.z - u.z;
      const float ch2 = ex * ex + ey * ey + ez * ez;
      if (ch2 < a.chord2_max) {
        const float t = 2.f * asinf(0.5f * sqrtf(ch2)) * a.inv_radius_f;
        const float sx = t * (float)MASK_NTAB;
        const int i = (int)sx;
        if (i < MASK_NTAB) {
          const float2 e = __ldg(a.T.mask32 + i);
          wgt = 1.f - (e.x + (sx - (float)i) * e.y);
        }
      }
    } else if (a.collect) {
      if (sj != run_surf) {
        if (run_id >= 0) L.insert(run_surf, run_id, run_d2);
        run_surf = sj; run_id = -1; run_d2 = 3.4e38f;
      }
      if (r2 < run_d2) { run_d2 = r2; run_id = idj; }
      if (r2 < a.rthr2_f) return 0.f;
    }
    if (r2 < a.reps2_f) return 0.f;
    return wgt;
  };

  for (int nb = 0; nb < 27; ++nb) {
    const int dx = nb % 3 - 1, dy = (nb / 3) % 3 - 1, dz = nb / 9 - 1;
    const int ni = imod(ci + dx, a.Nc[0]), nj = imod(cj + dy, a.Nc[1]), nk = imod(ck + dz, a.Nc[2]);
    const int ncell = ni + a.Nc[0] * (nj + a.Nc[1] * nk);
    const int sbeg = a.cs[ncell], send = a.ce[ncell];
    if (sbeg >= send) continue;
    const double d64[3] = {dx * a.h[0], dy * a.h[1], dz * a.h[2]};
    const float3 dh = make_float3((float)d64[0], (float)d64[1], (float)d64[2]);
    const float3 dl = make_float3((float)(d64[0] - (double)dh.x), (float)(d64[1] - (double)dh.y),
                                  (float)(d64[2] - (double)dh.z));
    float tsh[3], tsl[3];
    {
      float e;
      two_diff(th_[0], dh.x, tsh[0], e); tsl[0] = (tl_[0] - dl.x) + e;
      two_diff(th_[1], dh.y, tsh[1], e); tsl[1] = (tl_[1] - dl.y) + e;
      two_diff(th_[2], dh.z, tsh[2], e); tsl[2] = (tl_[2] - dl.z) + e;
    }
    const float2 nth0 = f2(-tsh[0], -tsh[0]), nth1 = f2(-tsh[1], -tsh[1]), nth2 = f2(-tsh[2], -tsh[2]);
    const float2 ntl0 = f2(-tsl[0], -tsl[0]), ntl1 = f2(-tsl[1], -tsl[1]), ntl2 = f2(-tsl[2], -tsl[2]);
    const float3 wlo = f3sub(wlo0, dh), whi = f3sub(whi0, dh);
    const int t0 = a.toff[ncell];
    for (int base = sbeg, tt = t0; base < send; base += TILE, ++tt) {
      const float4 blo = a.tbox[2 * tt], bhi = a.tbox[2 * tt + 1];
      if (boxes_apart(wlo, whi, make_float3(blo.x, blo.y, blo.z), make_float3(bhi.x, bhi.y, bhi.z), a.rc2_f)) continue;
      if (__float_as_int(blo.w) == wsurf && __float_as_int(bhi.w) == wsurf) continue;  // own cell only
      const int tend = min(base + TILE, send);
      for (int cb = base, cc = a.coff[ncell] + (base - sbeg) / 32; cb < tend; cb += 32, ++cc) {
        {
          const float4 clo4 = a.cbox[2 * cc], chi4 = a.cbox[2 * cc + 1];
          if (boxes_apart(wlo, whi, make_float3(clo4.x, clo4.y, clo4.z), make_float3(chi4.x, chi4.y, chi4.z), a.rc2_f))
            continue;  // uniform over the warp
          if (__float_as_int(clo4.w) == wsurf && __float_as_int(chi4.w) == wsurf) continue;  // own cell only
        }
        const int cnt = min(32, tend - cb);
        __syncwarp();
        if (lane < cnt) {
          const int q = cb + lane;
          const float4 p0 = a.sp0[q], p1 = a.sp1[q], f = a.sF4[q];
          C.hx[lane] = p0.x; C.hy[lane] = p0.y; C.hz[lane] = p0.z; C.surf[lane] = __float_as_int(p0.w);
          C.lx[lane] = p1.x; C.ly[lane] = p1.y; C.lz[lane] = p1.z; C.id[lane] = __float_as_int(p1.w);
          C.fx[lane] = f.x; C.fy[lane] = f.y; C.fz[lane] = f.z;
          if (DL) {
            const float4 g = a.sG4[q], an = a.sa4[q];
            C.gx[lane] = g.x; C.gy[lane] = g.y; C.gz[lane] = g.z;
            C.ax[lane] = an.x; C.ay[lane] = an.y; C.az[lane] = an.z;
          }
        }
        __syncwarp();
        if (!active) continue;
        float cx = 0.f, cy = 0.f, cz = 0.f;
        int j = 0;
        for (; j + 2 <= cnt; j += 2) {
          // hi parts of both sources, reject when both are out of reach
          const float2 hx = __fadd2_rn(ld2(C.hx, j), nth0), hy = __fadd2_rn(ld2(C.hy, j), nth1),
                       hz = __fadd2_rn(ld2(C.hz, j), nth2);
          const float2 h2 = __ffma2_rn(hx, hx, __ffma2_rn(hy, hy, __fmul2_rn(hz, hz)));
          const int sa = C.surf[j], sb = C.surf[j + 1];
          bool oka = h2.x <= a.rc2_loose && !(a.own_split && sa == surf_i);
          bool okb = h2.y <= a.rc2_loose && !(a.own_split && sb == surf_i);
          if (!(oka || okb)) continue;
          const float2 xx = __fadd2_rn(hx, __fadd2_rn(ld2(C.lx, j), ntl0));
          const float2 yy = __fadd2_rn(hy, __fadd2_rn(ld2(C.ly, j), ntl1));
          const float2 zz = __fadd2_rn(hz, __fadd2_rn(ld2(C.lz, j), ntl2));
          const float2 r2 = __ffma2_rn(xx, xx, __ffma2_rn(yy, yy, __fmul2_rn(zz, zz)));
          oka = oka && r2.x <= a.rc2_f;
          okb = okb && r2.y <= a.rc2_f;
          const float wa = weight(sa, C.id[j], r2.x, oka, cb + j);
          const float wb = weight(sb, C.id[j + 1], r2.y, okb, cb + j + 1);
          if (wa == 0.f && wb == 0.f) continue;
          const float2 z2 = f2(0.f, 0.f);
          ewald_pair2<DL>(a, xx, yy, zz, r2, wa, wb, ld2(C.fx, j), ld2(C.fy, j), ld2(C.fz, j),
                          DL ? ld2(C.gx, j) : z2, DL ? ld2(C.gy, j) : z2, DL ? ld2(C.gz, j) : z2,
                          DL ? ld2(C.ax, j) : z2, DL ? ld2(C.ay, j) : z2, DL ? ld2(C.az, j) : z2, cx, cy, cz);
        }
        if (j < cnt) {  // the odd last source
          const float hx = C.hx[j] - tsh[0], hy = C.hy[j] - tsh[1], hz = C.hz[j] - tsh[2];
          bool ok = hx * hx + hy * hy + hz * hz <= a.rc2_loose && !(a.own_split && C.surf[j] == surf_i);
          float xx = 0.f, yy = 0.f, zz = 0.f, r2 = 0.f;
          if (ok) {
            xx = __fadd_rn(hx, C.lx[j] - tsl[0]);
            yy = __fadd_rn(hy, C.ly[j] - tsl[1]);
            zz = __fadd_rn(hz, C.lz[j] - tsl[2]);
            r2 = xx * xx + yy * yy + zz * zz;
            ok = r2 <= a.rc2_f;
          }
          const float w = weight(C.surf[j], C.id[j], r2, ok, cb + j);
          if (w != 0.f) {
            const float rinv = rsqrtf(r2);
            const float r = r2 * rinv;
            const float st = r * a.sqpa_f;
            const float ex = __expf(-st * st);
            const float tq = __fdividef(1.f, fmaf(0.5f, st, 1.f));
            float Q = a.erfcx_q[ERFCX_DEG];
#pragma unroll
            for (int k = ERFCX_DEG - 1; k >= 0; --k) Q = fmaf(Q, tq, a.erfcx_q[k]);
            const float c1 = ex * (tq * Q), c2 = a.two_isqa_f * ex;
            const float ir2 = rinv * rinv;
            const float A = (c1 * rinv + c2) * ir2;
            const float B = c1 * rinv - c2;
            const float fx = C.fx[j], fy = C.fy[j], fz = C.fz[j];
            const float Ad = A * (xx * fx + yy * fy + zz * fz);
            float vx = Ad * xx + B * fx, vy = Ad * yy + B * fy, vz = Ad * zz + B * fz;
            if (DL) {
              const float cdl = a.m8_ispi_f * (ex * (st * (1.5f + st * st)) + a.q75_spi_f * c1);
              const float Adl = cdl * ir2 * ir2 * rinv;
              const float t = Adl * (xx * C.gx[j] + yy * C.gy[j] + zz * C.gz[j]) *
                              (xx * C.ax[j] + yy * C.ay[j] + zz * C.az[j]);
              vx += t * xx; vy += t * yy; vz += t * zz;
            }
            cx = fmaf(w, vx, cx);
            cy = fmaf(w, vy, cy);
            cz = fmaf(w, vz, cz);
          }
        }
        acc.add(0, cx);
        acc.add(1, cy);
        acc.add(2, cz);
        if (a.collect && run_id >= 0) { L.insert(run_surf, run_id, run_d2); }
        run_surf = -3; run_id = -1; run_d2 = 3.4e38f;
      }
    }
  }
  if (active) {
    double iA = 1.0 / a.tA[ti];
    for (int k = 0; k < 3; ++k) a.v[ti + (size_t)k * a.nt] += ((double)acc.s[k] - (double)acc.c[k]) * iA;
    if (a.collect) {
      if (L.overflow) atomicAdd(a.cnt + 2, 1ull);
      for (int e = 0; e < L.n; ++e) {
        unsigned long long pos = atomicAdd(a.cnt + 0, 1ull);
        if (pos < (unsigned long long)a.cap) a.items[pos] = make_int4(ti, L.surf[e], L.idx[e] & 0xffff, L.idx[e] >> 16);
      }
    }
  }
  unsigned long long np = npairs;
  for (int o = 16; o > 0; o >>= 1) np += __shfl_xor_sync(0xffffffffu, np, o);
  if ((tid & 31) == 0 && np) atomicAdd(a.cnt + 1, np);
}

// Own-cell pairs of the FP32 modes: the pairs of AddIntOnRbcs whose source
// lies on the target's own cell with the weight 1 - MaskFunc of the same-cell
// table (ModIntOnRbcs.F90:77-80).  Every point of a biconcave cell lies
// within rc of every other (79% of the pairs within rc on the 256-cell
// workload), so per cell this is a dense all-pairs pass over tiles of
// OWN_TILE points in ring-major order, one CTA per (target tile T, source
// tile S >= T).  Pair (i, j) and pair (j, i) share the distance, the weight
// (the table is symmetric) and the kernel coefficients, so off the diagonal
// a CTA evaluates them once and adds both: to its target i (registers) and
// to its source j (per-warp sums in shared memory; at step s lane l takes
// the source pair (l + s) mod OWN_TILE/2, so the lanes of a warp touch
// distinct sources and read consecutive ones).  A diagonal CTA (S = T) takes
// every ordered pair of its tile one way.  The pair arithmetic is k_pair32's
// (ewald_coef2 / ewald_apply2), positions hi/lo FP32 relative to the cell's
// first point, FP32 sums per 32 sources (Kahan-compensated across them) and
// per warp, added to the accumulator in FP64 atomically, after k_pair32 on
// the same stream.  The target tile's at most (OWN_TILE - 1) / nlon + 2
// latitude rings' rows of the weight table sit in shared memory.
constexpr int OWN_TILE = 128;
template <bool DL>
__global__ void __launch_bounds__(OWN_TILE) k_pair_own32(PairArgs a) {
  __shared__ __align__(16) float s_src[15][OWN_TILE];  // hi xyz, lo xyz, f xyz, g xyz, normal xyz
  __shared__ __align__(16) int s_id[OWN_TILE];
  __shared__ __align__(16) float s_rev[OWN_TILE / 32][3][OWN_TILE];  // per warp: the sources' sums
  extern __shared__ float s_mask[];  // rows lat0.. of the table, nlat * nhalf each
  const int nlat = a.nlat, nlon = a.nlon, nv = nlat * nlon, rowlen = nlat * a.nhalf;
  const int ntile = (nv + OWN_TILE - 1) / OWN_TILE, npt = ntile * (ntile + 1) / 2;
  const int cell = blockIdx.x / npt;
  int r = blockIdx.x - cell * npt, T = 0;
  while (r >= ntile - T) { r -= ntile - T; ++T; }
  const int S = T + r;
  const bool diag = S == T;
  const int tid = threadIdx.x, wid = tid >> 5;
  const int k = T * OWN_TILE + tid;  // ring-major index of the target in its cell
  const bool active = k < nv;
  const int tlat = active ? k / nlon : 0, tlon = active ? k - tlat * nlon : 0;
  const int lat0 = T * OWN_TILE / nlon;
  const int nrow = min(nlat - 1, (T * OWN_TILE + OWN_TILE - 1) / nlon) - lat0 + 1;
  for (int i = tid; i < nrow * rowlen; i += OWN_TILE) s_mask[i] = a.mtab32[(size_t)lat0 * rowlen + i];
  const int p = cell * nv + tlon * nlat + tlat;  // the target's point index (= its target index)
  // the source tile, and the per-warp sums cleared
  const int js = S * OWN_TILE + tid;
  int ps = 0;
  if (js < nv) {
    const int sl = js / nlon;
    ps = cell * nv + (js - sl * nlon) * nlat + sl;
    const int q = a.sinv[ps];
    const float4 q0 = a.op0[ps], q1 = a.op1[ps], f = a.sF4[q];
    s_src[0][tid] = q0.x; s_src[1][tid] = q0.y; s_src[2][tid] = q0.z;
    s_src[3][tid] = q1.x; s_src[4][tid] = q1.y; s_src[5][tid] = q1.z;
    s_src[6][tid] = f.x; s_src[7][tid] = f.y; s_src[8][tid] = f.z;
    s_id[tid] = __float_as_int(q0.w);
    if (DL) {
      const float4 g = a.sG4[q], an = a.sa4[q];
      s_src[9][tid] = g.x; s_src[10][tid] = g.y; s_src[11][tid] = g.z;
      s_src[12][tid] = an.x; s_src[13][tid] = an.y; s_src[14][tid] = an.z;
    }
  } else {  // padding: a source beyond rc of every target
    for (int c = 0; c < 15; ++c) s_src[c][tid] = 0.f;
    s_src[0][tid] = 1.0e18f;
    s_id[tid] = 0;
  }
  for (int w = 0; w < OWN_TILE / 32; ++w)
    for (int c = 0; c < 3; ++c) s_rev[w][c][tid] = 0.f;
  // the target: position, and off the diagonal its densities for the reverse terms
  float4 t0 = make_float4(0.f, 0.f, 0.f, 0.f), t1 = t0, tf = t0, tg = t0, tn = t0;
  if (active) {
    t0 = a.op0[p];
    t1 = a.op1[p];
    if (!diag) {
      const int q = a.sinv[p];
      tf = a.sF4[q];
      if (DL) { tg = a.sG4[q]; tn = a.sa4[q]; }
    }
  }
  __syncthreads();
  const float2 nth0 = f2(-t0.x, -t0.x), nth1 = f2(-t0.y, -t0.y), nth2 = f2(-t0.z, -t0.z);
  const float2 ntl0 = f2(-t1.x, -t1.x), ntl1 = f2(-t1.y, -t1.y), ntl2 = f2(-t1.z, -t1.z);
  const float2 tfx = f2(tf.x, tf.x), tfy = f2(tf.y, tf.y), tfz = f2(tf.z, tf.z);
  const float2 tgx = f2(tg.x, tg.x), tgy = f2(tg.y, tg.y), tgz = f2(tg.z, tg.z);
  const float2 tnx = f2(-tn.x, -tn.x), tny = f2(-tn.y, -tn.y), tnz = f2(-tn.z, -tn.z);  // (x.g)(-x.n) x: reverse sign
  const float* mrow = s_mask + (tlat - lat0) * rowlen;
  Kahan3 acc;
  acc.zero();
  unsigned npairs = 0;
  const float2 z2 = f2(0.f, 0.f);
  float cx = 0.f, cy = 0.f, cz = 0.f;
  for (int step = 0; step < OWN_TILE / 2; ++step) {
    if (active) {
      const int j = 2 * ((tid + step) & (OWN_TILE / 2 - 1));
      const float2 xx = __fadd2_rn(__fadd2_rn(ld2(s_src[0], j), nth0), __fadd2_rn(ld2(s_src[3], j), ntl0));
      const float2 yy = __fadd2_rn(__fadd2_rn(ld2(s_src[1], j), nth1), __fadd2_rn(ld2(s_src[4], j), ntl1));
      const float2 zz = __fadd2_rn(__fadd2_rn(ld2(s_src[2], j), nth2), __fadd2_rn(ld2(s_src[5], j), ntl2));
      const float2 r2 = __ffma2_rn(xx, xx, __ffma2_rn(yy, yy, __fmul2_rn(zz, zz)));
      const bool oka = r2.x <= a.rc2_f, okb = r2.y <= a.rc2_f;
      npairs += ((unsigned)oka + (unsigned)okb) * (diag ? 1u : 2u);
      const int2 id = *reinterpret_cast<const int2*>(s_id + j);
      float wa = 0.f, wb = 0.f;
      if (oka && !(r2.x < a.reps2_f)) {
        int dl = abs((id.x >> 16) - tlon);
        dl = min(dl, nlon - dl);
        wa = mrow[(id.x & 0xffff) * a.nhalf + dl];
      }
      if (okb && !(r2.y < a.reps2_f)) {
        int dl = abs((id.y >> 16) - tlon);
        dl = min(dl, nlon - dl);
        wb = mrow[(id.y & 0xffff) * a.nhalf + dl];
      }
      if (wa != 0.f || wb != 0.f) {
        float2 A, B, Adl, vx, vy, vz;
        ewald_coef2<DL>(a, r2, wa, wb, A, B, Adl);
        ewald_apply2<DL>(xx, yy, zz, A, B, Adl, ld2(s_src[6], j), ld2(s_src[7], j), ld2(s_src[8], j),
                         DL ? ld2(s_src[9], j) : z2, DL ? ld2(s_src[10], j) : z2, DL ? ld2(s_src[11], j) : z2,
                         DL ? ld2(s_src[12], j) : z2, DL ? ld2(s_src[13], j) : z2, DL ? ld2(s_src[14], j) : z2, vx,
                         vy, vz);
        cx = fmaf(wb, vx.y, fmaf(wa, vx.x, cx));
        cy = fmaf(wb, vy.y, fmaf(wa, vy.x, cy));
        cz = fmaf(wb, vz.y, fmaf(wa, vz.x, cz));
        if (!diag) {  // pair (j, i): the vector is -x, so only the stresslet term changes sign
          ewald_apply2<DL>(xx, yy, zz, A, B, Adl, tfx, tfy, tfz, tgx, tgy, tgz, tnx, tny, tnz, vx, vy, vz);
          const float2 w2 = f2(wa, wb);
          float2* rx = reinterpret_cast<float2*>(&s_rev[wid][0][j]);
          float2* ry = reinterpret_cast<float2*>(&s_rev[wid][1][j]);
          float2* rz = reinterpret_cast<float2*>(&s_rev[wid][2][j]);
          *rx = __ffma2_rn(w2, vx, *rx);
          *ry = __ffma2_rn(w2, vy, *ry);
          *rz = __ffma2_rn(w2, vz, *rz);
        }
      }
      if ((step & 15) == 15) {
        acc.add(0, cx);
        acc.add(1, cy);
        acc.add(2, cz);
        cx = cy = cz = 0.f;
      }
    }
    __syncwarp();  // the lanes' per-warp sums of this step are written before the next step's
  }
  __syncthreads();
  if (active) {
    const double iA = 1.0 / a.tA[p];
    for (int c = 0; c < 3; ++c) atomicAdd(a.v + p + (size_t)c * a.nt, ((double)acc.s[c] - (double)acc.c[c]) * iA);
  }
  if (!diag && js < nv) {
    const double iA = 1.0 / a.tA[ps];
    for (int c = 0; c < 3; ++c) {
      float sum = 0.f;
      for (int w = 0; w < OWN_TILE / 32; ++w) sum += s_rev[w][c][tid];
      atomicAdd(a.v + ps + (size_t)c * a.nt, (double)sum * iA);
    }
  }
  unsigned long long np = npairs;
  for (int o = 16; o > 0; o >>= 1) np += __shfl_xor_sync(0xffffffffu, np, o);
  if ((tid & 31) == 0 && np) atomicAdd(a.cnt + 1, np);
}

// FP64 plain form: the same traversal with the reference arithmetic.
template <bool DL>
__global__ void __launch_bounds__(TILE) k_pair64(PairArgs a) {
  __shared__ TileD sm;
  __shared__ float3 wb[TILE / 32][2];
  const int4 unit = a.units[blockIdx.x];
  if (unit.z == 0) return;  // an empty entry past the end of the unit list
  const int cell = unit.x;
  const int tid = threadIdx.x;
  const bool active = tid < unit.z;
  const int ci = cell % a.Nc[0], cj = (cell / a.Nc[0]) % a.Nc[1], ck = cell / (a.Nc[0] * a.Nc[1]);
  const double c0[3] = {(ci + 0.5) * a.h[0], (cj + 0.5) * a.h[1], (ck + 0.5) * a.h[2]};
  int ti = active ? a.torder[unit.y + tid] : 0;
  double t_[3] = {0, 0, 0};
  int surf_i = -2, tlat = 0, tlon = 0;
  double th_i = 0, phi_i = 0;
  if (active) {
    for (int k = 0; k < 3; ++k) t_[k] = min_image(a.tx[ti + (size_t)k * a.nt] - c0[k], a.L[k], a.iL[k]);
    int4 m = a.tmeta[ti];
    surf_i = m.x;
    if (m.y >= 0) { th_i = a.th[m.y]; phi_i = a.phi[m.z]; tlat = m.y; tlon = m.z; }
  }
  // the same tile culling as the FP32 form (boxes in FP32 with a margin)
  const CullBoxes cb = cull_boxes(active, (float)t_[0], (float)t_[1], (float)t_[2], wb);
  double acc[3] = {0, 0, 0};
  NbrList L;
  L.n = 0; L.overflow = 0;
  int run_surf = -3, run_id = -1;
  double run_d = 1e300;
  unsigned long long npairs = 0;

  for (int nb = 0; nb < 27; ++nb) {
    int dx = nb % 3 - 1, dy = (nb / 3) % 3 - 1, dz = nb / 9 - 1;
    int ni = imod(ci + dx, a.Nc[0]), nj = imod(cj + dy, a.Nc[1]), nk = imod(ck + dz, a.Nc[2]);
    int ncell = ni + a.Nc[0] * (nj + a.Nc[1] * nk);
    int sbeg = a.cs[ncell], send = a.ce[ncell];
    const float3 dh = make_float3((float)(dx * a.h[0]), (float)(dy * a.h[1]), (float)(dz * a.h[2]));
    const float3 wlo = f3sub(cb.wlo, dh), whi = f3sub(cb.whi, dh);
    const float3 clo = f3sub(cb.clo, dh), chi = f3sub(cb.chi, dh);
    for (int base = sbeg, tt = a.toff[ncell]; base < send; base += TILE, ++tt) {
      const float4 blo = a.tbox[2 * tt], bhi = a.tbox[2 * tt + 1];
      const float3 bl = make_float3(blo.x, blo.y, blo.z), bh = make_float3(bhi.x, bhi.y, bhi.z);
      if (boxes_apart(clo, chi, bl, bh, a.rc2_f)) continue;  // uniform over the CTA
      int cnt = min(TILE, send - base);
      __syncthreads();
      if (tid < cnt) {
        int q = base + tid;
        sm.x[tid] = min_image(a.sx[q] - c0[0], a.L[0], a.iL[0]);
        sm.y[tid] = min_image(a.sx[q + a.ns] - c0[1], a.L[1], a.iL[1]);
        sm.z[tid] = min_image(a.sx[q + 2 * (size_t)a.ns] - c0[2], a.L[2], a.iL[2]);
        sm.fx[tid] = a.sf[q]; sm.fy[tid] = a.sf[q + a.ns]; sm.fz[tid] = a.sf[q + 2 * (size_t)a.ns];
        if (DL) {
          sm.gx[tid] = a.sg[q]; sm.gy[tid] = a.sg[q + a.ns]; sm.gz[tid] = a.sg[q + 2 * (size_t)a.ns];
          sm.ax[tid] = a.sa3[q]; sm.ay[tid] = a.sa3[q + a.ns]; sm.az[tid] = a.sa3[q + 2 * (size_t)a.ns];
        }
        int4 m = a.smeta[q];
        sm.surf[tid] = m.x; sm.ilat[tid] = m.y; sm.ilon[tid] = m.z;
      }
      __syncthreads();
      if (active && !boxes_apart(wlo, whi, bl, bh, a.rc2_f)) {
        for (int j = 0; j < cnt; ++j) {
          const int sj = sm.surf[j];
          if (a.collect && sj != run_surf) {
            if (run_id >= 0) L.insert(run_surf, run_id, (float)run_d);
            run_surf = sj; run_id = -1; run_d = 1e300;
          }
          double xx = sm.x[j] - t_[0], yy = sm.y[j] - t_[1], zz = sm.z[j] - t_[2];
          const double r2 = xx * xx + yy * yy + zz * zz;
          if (r2 > a.rc2) continue;  // the square root only for pairs inside the cutoff
          const double ir = rsqrt(r2), rr = r2 > 0. ? r2 * ir : 0.;
          ++npairs;
          double mask = 0.;
          if (sj == surf_i && a.mtab64) {
            int dl = abs(sm.ilon[j] - tlon);
            dl = min(dl, a.nlon - dl);
            mask = __ldg(a.mtab64 + ((size_t)tlat * a.nlat + sm.ilat[j]) * a.nhalf + dl);
          } else if (sj == surf_i) {
            double dth = dist_on_sphere(th_i, phi_i, a.th[sm.ilat[j]], a.phi[sm.ilon[j]]);
            mask = mask64(a.T, dth * a.inv_radius);
          } else if (a.collect) {
            if (rr < run_d) { run_d = rr; run_id = sm.ilat[j] | (sm.ilon[j] << 16); }
          }
          double EA, EB;
          ewald_sl64r(a.T, rr, ir, EA, EB);
          double s1 = (1. - mask) * a.c1;
          double d = xx * sm.fx[j] + yy * sm.fy[j] + zz * sm.fz[j];
          acc[0] += s1 * (EA * xx * d + EB * sm.fx[j]);
          acc[1] += s1 * (EA * yy * d + EB * sm.fy[j]);
          acc[2] += s1 * (EA * zz * d + EB * sm.fz[j]);
          if (DL) {
            double EAd = ewald_dl64r(a.T, rr, ir);
            double dg = xx * sm.gx[j] + yy * sm.gy[j] + zz * sm.gz[j];
            double da = xx * sm.ax[j] + yy * sm.ay[j] + zz * sm.az[j];
            double s2 = (1. - mask) * a.c2;
            acc[0] += s2 * (EAd * xx * dg * da);
            acc[1] += s2 * (EAd * yy * dg * da);
            acc[2] += s2 * (EAd * zz * dg * da);
          }
        }
        if (a.collect && run_id >= 0) L.insert(run_surf, run_id, (float)run_d);
        run_surf = -3; run_id = -1; run_d = 1e300;
      }
    }
  }
  if (active) {
    double iA = 1.0 / a.tA[ti];
    for (int k = 0; k < 3; ++k) a.v[ti + (size_t)k * a.nt] += acc[k] * iA;
    if (a.collect) {
      if (L.overflow) atomicAdd(a.cnt + 2, 1ull);
      for (int e = 0; e < L.n; ++e) {
        unsigned long long pos = atomicAdd(a.cnt + 0, 1ull);
        if (pos < (unsigned long long)a.cap) a.items[pos] = make_int4(ti, L.surf[e], L.idx[e] & 0xffff, L.idx[e] >> 16);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) npairs += __shfl_xor_sync(0xffffffffu, npairs, o);
  if ((tid & 31) == 0 && npairs) atomicAdd(a.cnt + 1, npairs);
}

// AddLinearInt (ModIntOnRbcs.F90:162-201): xvint = sum Bcoef * x * (g.a3) dS
__global__ void k_linear_reduce(int n, int nv, const double* __restrict__ x, const double* __restrict__ sg,
                                const double* __restrict__ a3, const int* __restrict__ celltype,
                                const double* __restrict__ Bc, double* __restrict__ out) {
  double acc[3] = {0, 0, 0};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    double vn = sg[p] * a3[p] + sg[p + n] * a3[p + n] + sg[p + 2 * (size_t)n] * a3[p + 2 * (size_t)n];
    double B = Bc[celltype[p / nv]];
    for (int k = 0; k < 3; ++k) acc[k] += B * x[p + (size_t)k * n] * vn;
  }
  for (int k = 0; k < 3; ++k) {
    double s = warp_sum(acc[k]);
    if ((threadIdx.x & 31) == 0) atomicAdd(out + k, s);
  }
}
__global__ void k_linear_add(int nt, const double* __restrict__ tA, const double* __restrict__ xv, double scale,
                             double* __restrict__ v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  double iA = 1.0 / tA[i];
  for (int k = 0; k < 3; ++k) v[i + (size_t)k * nt] += scale * xv[k] * iA;
}

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

rbc3d_status sort_points(rbc3d_ctx* ctx, int n, const double* x_dev, DBuf<int>& order, DBuf<int>& cs, DBuf<int>& ce) {
  const HashGrid& hg = ctx->hg;
  DBuf<int>&key = ctx->sort_key, &key2 = ctx->sort_key2, &idx = ctx->sort_idx;
  CUDA_TRY(key.alloc(n)); CUDA_TRY(key2.alloc(n)); CUDA_TRY(idx.alloc(n)); CUDA_TRY(order.alloc(n));
  CUDA_TRY(cs.alloc(hg.ncells)); CUDA_TRY(ce.alloc(hg.ncells));
  { k_hash_keys<<<nblk(n, 256), 256, 0, ctx->st>>>(n, x_dev, hg.Nc[0], hg.Nc[1], hg.Nc[2], hg.Nc[0] / hg.L[0],
                                                  hg.Nc[1] / hg.L[1], hg.Nc[2] / hg.L[2], key.p, idx.p); ++ctx->launches; }
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, key.p, key2.p, idx.p, order.p, n, 0, 32, ctx->st);
  DBuf<char>& tbuf = ctx->sort_tmp;
  CUDA_TRY(tbuf.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceRadixSort::SortPairs(tbuf.p, tmp, key.p, key2.p, idx.p, order.p, n, 0, 32, ctx->st));
  CUDA_TRY(cudaMemsetAsync(cs.p, 0, sizeof(int) * hg.ncells, ctx->st));
  CUDA_TRY(cudaMemsetAsync(ce.p, 0, sizeof(int) * hg.ncells, ctx->st));
  { k_cell_ranges<<<nblk(n, 256), 256, 0, ctx->st>>>(n, key2.p, cs.p, ce.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

// off = exclusive scan of cnt[0..nc] (nc + 1 entries; off[nc] the total), on the context stream
rbc3d_status scan_counts(rbc3d_ctx* ctx, int nc, const int* cnt, int* off) {
  size_t tmp = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp, cnt, off, nc + 1, ctx->st);
  DBuf<char>& tb = ctx->scan_tmp;
  CUDA_TRY(tb.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceScan::ExclusiveSum(tb.p, tmp, cnt, off, nc + 1, ctx->st));
  return RBC3D_OK;
}

// The units of `tile` targets at most into `units` (cap entries, the empty
// tail last): per-cell counts, their scan, the units, a stable sort by work.
rbc3d_status fill_units(rbc3d_ctx* ctx, const DBuf<int>& cs, const DBuf<int>& ce, const int* ss, const int* se,
                        int tile, int cap, DBuf<int4>& units) {
  const int nc = ctx->hg.ncells;
  rbc3d_status s;
  DBuf<int>& cnt = ctx->unit_cnt;
  CUDA_TRY(cnt.alloc(nc + 1)); CUDA_TRY(ctx->unit_off.alloc(nc + 1));
  CUDA_TRY(ctx->unit_tmp.alloc(cap)); CUDA_TRY(units.alloc(cap));
  CUDA_TRY(ctx->unit_key.alloc(2 * (size_t)cap)); CUDA_TRY(ctx->unit_idx.alloc(2 * (size_t)cap));
  const int g1 = nblk(nc + 1, 256);
  { k_unit_counts<<<g1, 256, 0, ctx->st>>>(nc, tile, cs.p, ce.p, cnt.p); ++ctx->launches; }
  if ((s = scan_counts(ctx, nc, cnt.p, ctx->unit_off.p))) return s;
  long long* key = ctx->unit_key.p;
  int* idx = ctx->unit_idx.p;
  { k_fill_units<<<g1, 256, 0, ctx->st>>>(nc, tile, ctx->hg.Nc[0], ctx->hg.Nc[1], ctx->hg.Nc[2], cs.p, ce.p, ss, se,
                                          ctx->unit_off.p, cap, ctx->unit_tmp.p, key, idx); ++ctx->launches; }
  // heaviest units first, so the last wave holds the light ones; the radix
  // sort is stable, so equal work keeps cell order (as a stable host sort);
  // the empty tail (key -1) stays last
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairsDescending(nullptr, tmp, key, key + cap, idx, idx + cap, cap, 0, 64, ctx->st);
  DBuf<char>& tb = ctx->sort_tmp;
  CUDA_TRY(tb.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceRadixSort::SortPairsDescending(tb.p, tmp, key, key + cap, idx, idx + cap, cap, 0, 64, ctx->st));
  { k_gather_units<<<nblk(cap, 256), 256, 0, ctx->st>>>(cap, idx + cap, ctx->unit_tmp.p, units.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

rbc3d_status make_units(rbc3d_ctx* ctx, TargetSet& t, const DBuf<int>& cs, const DBuf<int>& ce) {
  const int nc = ctx->hg.ncells;
  // capacity: every non-empty cell gives at most count / tile + 1 units
  const int cap = nc + (t.n + TILE - 1) / TILE, wcap = nc + (t.n + 31) / 32;
  rbc3d_status s;
  // sources per cell: the source list's ranges (or the targets' own when
  // there is no source list)
  const bool src = ctx->npt > 0 && ctx->s_cstart.p;
  const int* ss = src ? ctx->s_cstart.p : cs.p;
  const int* se = src ? ctx->s_cend.p : ce.p;
  if (!src) {  // no sources: every unit weighs 0
    CUDA_TRY(ctx->unit_zero.alloc(nc));
    CUDA_TRY(cudaMemsetAsync(ctx->unit_zero.p, 0, sizeof(int) * nc, ctx->st));
    ss = se = ctx->unit_zero.p;
  }
  // block units (FP64 pair sums: the block shares its source tiles) and
  // warp units (FP32 pair sums: each warp stages its own chunks, so a block's
  // warps may come from different cells and none idles)
  if ((s = fill_units(ctx, cs, ce, ss, se, TILE, cap, t.units))) return s;
  if ((s = fill_units(ctx, cs, ce, ss, se, 32, wcap, t.wunits))) return s;
  t.nunits = cap;
  t.nwunits = wcap;
  return RBC3D_OK;
}

}  // namespace


// erfc(x) exp(x^2) on [0, X] as t Q(t) with t = 1/(1 + x/2) (the variable of
// the Chebyshev erfc fit of Press et al., Numerical Recipes, sec. 6.2) and Q
// a degree-ERFCX_DEG polynomial: the truncated Chebyshev series of Q over the
// t-interval (projection on 64 Chebyshev nodes, FP64 std::erfc), converted to
// monomial coefficients in t.  Max relative error ~3e-7 in FP32 Horner for
// X = 4.24 (eps = 1e-6 at rc = 3), against ~1e-9 of the series itself.
void fit_erfcx(double X, float* q) {  // declared in ctx.hpp
  const int N = 64, D = ERFCX_DEG;
  const double tlo = 1.0 / (1.0 + 0.5 * X);
  const double a = 2.0 / (1.0 - tlo), b = -(1.0 + tlo) / (1.0 - tlo);  // s = a t + b in [-1, 1]
  double c[D + 1] = {0};
  for (int j = 0; j < N; ++j) {
    const double th = RBC3D_PI * (j + 0.5) / N, sj = std::cos(th), t = (sj - b) / a, x = 2.0 * (1.0 / t - 1.0);
    const double g = std::erfc(x) * std::exp(x * x) / t;
    for (int k = 0; k <= D; ++k) c[k] += 2.0 / N * g * std::cos(k * th);
  }
  c[0] *= 0.5;
  // sum c_k T_k(s), s = a t + b, as a polynomial in t: T_{k+1} = 2 s T_k - T_{k-1}
  double Tm[D + 1] = {0}, Tk[D + 1] = {0}, out[D + 1] = {0};
  Tm[0] = 1.0;                  // T_0
  Tk[0] = b; Tk[1] = a;         // T_1 = s
  for (int i = 0; i <= D; ++i) out[i] += c[0] * Tm[i];
  for (int k = 1; k <= D; ++k) {
    for (int i = 0; i <= D; ++i) out[i] += c[k] * Tk[i];
    double Tn[D + 1] = {0};
    for (int i = 0; i <= D; ++i) {
      Tn[i] += 2.0 * b * Tk[i] - Tm[i];
      if (i + 1 <= D) Tn[i + 1] += 2.0 * a * Tk[i];
    }
    for (int i = 0; i <= D; ++i) { Tm[i] = Tk[i]; Tk[i] = Tn[i]; }
  }
  for (int i = 0; i <= D; ++i) q[i] = (float)out[i];
}


rbc3d_status sort_points_by_cell(rbc3d_ctx* ctx, int n, const double* x_dev, DBuf<int>& order, DBuf<int>& cs,
                                DBuf<int>& ce) {
  return sort_points(ctx, n, x_dev, order, cs, ce);
}

rbc3d_status build_source_list(rbc3d_ctx* ctx, bool with_normals) {
  int n = ctx->npt;
  rbc3d_status s = sort_points(ctx, n, ctx->x.p, ctx->s_order, ctx->s_cstart, ctx->s_cend);
  if (s) return s;
  CUDA_TRY(ctx->s_x.alloc(3 * (size_t)n)); CUDA_TRY(ctx->s_a3.alloc(3 * (size_t)n)); CUDA_TRY(ctx->s_meta.alloc(n));
  CUDA_TRY(ctx->s_f.alloc(3 * (size_t)n)); CUDA_TRY(ctx->s_g.alloc(3 * (size_t)n));
  { k_gather_src<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, ctx->nlat * ctx->nlon, ctx->s_order.p, ctx->x.p,
                                                   ctx->s_x.p, ctx->s_meta.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  // FP32 pair-sum records and tile boxes
  CUDA_TRY(ctx->s_p0.alloc(n)); CUDA_TRY(ctx->s_p1.alloc(n)); CUDA_TRY(ctx->s_u4.alloc(n)); CUDA_TRY(ctx->s_a4.alloc(n));
  if (with_normals && (s = source_normals(ctx))) return s;
  {
    const HashGrid& hg = ctx->hg;
    k_src_records<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->s_x.p, ctx->s_meta.p, ctx->usph.p, ctx->nlat,
                                                     hg.Nc[0], hg.Nc[1], hg.Nc[2], hg.h[0], hg.h[1], hg.h[2], hg.L[0],
                                                     hg.L[1], hg.L[2], ctx->s_p0.p, ctx->s_p1.p, ctx->s_u4.p);
    ++ctx->launches;
    CUDA_TRY(ctx->s_op0.alloc(n)); CUDA_TRY(ctx->s_op1.alloc(n)); CUDA_TRY(ctx->s_inv.alloc(n));
    { k_own_records<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, ctx->nlat * ctx->nlon, ctx->x.p, ctx->s_order.p,
                                                       hg.L[0], hg.L[1], hg.L[2], ctx->s_op0.p, ctx->s_op1.p,
                                                       ctx->s_inv.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
    const int nc = hg.ncells;
    // tiles of TILE and chunks of 32 consecutive sources of one cell, with
    // their offsets per cell and bounding boxes
    const int capt = nc + (n + TILE - 1) / TILE, capc = nc + (n + 31) / 32;
    CUDA_TRY(ctx->s_toff.alloc(nc + 1)); CUDA_TRY(ctx->s_coff.alloc(nc + 1));
    CUDA_TRY(ctx->unit_cnt.alloc(nc + 1));
    DBuf<int2>& lt = ctx->list_tmp;
    CUDA_TRY(lt.alloc((size_t)capc + capt));
    CUDA_TRY(ctx->s_cbox.alloc(2 * (size_t)capc + 2)); CUDA_TRY(ctx->s_tbox.alloc(2 * (size_t)capt + 2));
    const int g1 = nblk(nc + 1, 256);
    { k_piece_counts<<<g1, 256, 0, ctx->st>>>(nc, ctx->s_cstart.p, ctx->s_cend.p, 32, ctx->unit_cnt.p); ++ctx->launches; }
    if ((s = scan_counts(ctx, nc, ctx->unit_cnt.p, ctx->s_coff.p))) return s;
    { k_fill_pieces<<<g1, 256, 0, ctx->st>>>(nc, ctx->s_cstart.p, ctx->s_cend.p, 32, ctx->s_coff.p, capc, lt.p); ++ctx->launches; }
    { k_piece_counts<<<g1, 256, 0, ctx->st>>>(nc, ctx->s_cstart.p, ctx->s_cend.p, TILE, ctx->unit_cnt.p); ++ctx->launches; }
    if ((s = scan_counts(ctx, nc, ctx->unit_cnt.p, ctx->s_toff.p))) return s;
    { k_fill_pieces<<<g1, 256, 0, ctx->st>>>(nc, ctx->s_cstart.p, ctx->s_cend.p, TILE, ctx->s_toff.p, capt, lt.p + capc);
      ++ctx->launches; }
    { k_tile_boxes<<<capc, 32, 0, ctx->st>>>(lt.p, ctx->s_p0.p, ctx->s_cbox.p); ++ctx->launches; }
    { k_tile_boxes<<<capt, TILE, 0, ctx->st>>>(lt.p + capc, ctx->s_p0.p, ctx->s_tbox.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
    ctx->s_ntiles = capt;
  }
  ctx->src_sorted = true;
  ctx->pme.cplan.valid = false;  // the PME tiles follow the source positions
  // tlist_rbc shares the source order
  TargetSet& t = ctx->tl[RBC3D_TLIST_RBC];
  t.sorted = false;
  return RBC3D_OK;
}

// The sorted sources' normals (a3 in source order and the FP32 records),
// once a3 is on the device.
rbc3d_status source_normals(rbc3d_ctx* ctx) {
  const int n = ctx->npt;
  if (n == 0) return RBC3D_OK;
  { k_gather_a3<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->s_order.p, ctx->a3.p, ctx->s_a3.p, ctx->s_a4.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

rbc3d_status build_source_density(rbc3d_ctx* ctx) {
  int n = ctx->npt, nv = ctx->nlat * ctx->nlon;
  if (n == 0) return RBC3D_OK;
  const double* Bc = ctx->dBcoef.p;
  if (ctx->has_f) { k_density<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, nv, ctx->f.p, ctx->detJ.p, ctx->w.p, ctx->sf.p); ++ctx->launches; }
  if (ctx->has_g) { k_density<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, nv, ctx->g.p, ctx->detJ.p, ctx->w.p, ctx->sg.p); ++ctx->launches; }
  { k_gather_density<<<nblk(n, 256), 256, 0, ctx->st>>>(n, nv, ctx->s_order.p, ctx->sf.p, ctx->sg.p, ctx->celltype.p,
                                                       Bc, ctx->s_f.p, ctx->s_g.p, ctx->has_f, ctx->has_g); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  ctx->src_density = true;
  return RBC3D_OK;
}

rbc3d_status sort_targets(rbc3d_ctx* ctx, int tlist) {
  TargetSet& t = ctx->tl[tlist];
  if (t.sorted) return RBC3D_OK;
  rbc3d_status s;
  if (tlist == RBC3D_TLIST_RBC) {
    // same points in the same order as the sources
    CUDA_TRY(t.order.alloc(ctx->npt)); CUDA_TRY(t.cstart.alloc(ctx->hg.ncells)); CUDA_TRY(t.cend.alloc(ctx->hg.ncells));
    CUDA_TRY(cudaMemcpyAsync(t.order.p, ctx->s_order.p, sizeof(int) * ctx->npt, cudaMemcpyDeviceToDevice, ctx->st));
    CUDA_TRY(cudaMemcpyAsync(t.cstart.p, ctx->s_cstart.p, sizeof(int) * ctx->hg.ncells, cudaMemcpyDeviceToDevice, ctx->st));
    CUDA_TRY(cudaMemcpyAsync(t.cend.p, ctx->s_cend.p, sizeof(int) * ctx->hg.ncells, cudaMemcpyDeviceToDevice, ctx->st));
  } else {
    if ((s = sort_points(ctx, t.n, t.x.p, t.order, t.cstart, t.cend))) return s;
  }
  if ((s = make_units(ctx, t, t.cstart, t.cend))) return s;
  t.sorted = true;
  return RBC3D_OK;
}

rbc3d_status run_pair_sum(rbc3d_ctx* ctx, int tlist, double c1, double c2, int prec, bool collect_nbr) {
  if (ctx->npt == 0) return RBC3D_OK;
  TargetSet& t = ctx->tl[tlist];
  if (t.n == 0) return RBC3D_OK;
  rbc3d_status s = sort_targets(ctx, tlist);
  if (s) return s;
  PairArgs a;
  a.nt = t.n; a.tx = t.x.p; a.tA = t.Acoef.p; a.tmeta = t.meta.p; a.torder = t.order.p; a.units = t.units.p; a.v = t.v.p;
  a.ns = ctx->npt; a.sx = ctx->s_x.p; a.sf = ctx->s_f.p; a.sg = ctx->s_g.p; a.sa3 = ctx->s_a3.p; a.smeta = ctx->s_meta.p;
  a.cs = ctx->s_cstart.p; a.ce = ctx->s_cend.p;
  a.sp0 = ctx->s_p0.p; a.sp1 = ctx->s_p1.p; a.su = ctx->s_u4.p; a.sa4 = ctx->s_a4.p;
  a.sF4 = ctx->s_F4.p; a.sG4 = ctx->s_G4.p; a.toff = ctx->s_toff.p; a.tbox = ctx->s_tbox.p;
  a.coff = ctx->s_coff.p; a.cbox = ctx->s_cbox.p;
  for (int d = 0; d < 3; ++d) { a.Nc[d] = ctx->hg.Nc[d]; a.h[d] = ctx->hg.h[d]; a.L[d] = ctx->hg.L[d]; a.iL[d] = ctx->iLb[d]; }
  a.th = ctx->th.p; a.phi = ctx->phi.p; a.usph = ctx->usph.p; a.nlat = ctx->nlat;
  a.nlon = ctx->nlon; a.nhalf = ctx->nlon / 2 + 1;
  a.mtab64 = ctx->phi_uniform ? ctx->mtab64.p : nullptr;
  a.mtab32 = ctx->phi_uniform ? ctx->mtab32.p : nullptr;
  a.radius = ctx->radius; a.inv_radius = 1.0 / ctx->radius; a.inv_radius_f = (float)(1.0 / ctx->radius);
  double cm = 2.0 * sin(0.5 * ctx->radius) * (1.0 + 1e-6);
  a.chord2_max = (float)(cm * cm);
  a.c1 = c1; a.c2 = c2; a.c1f = (float)c1; a.c2f = (float)c2;
  a.rc2 = ctx->prm.rc * ctx->prm.rc; a.rc2_f = (float)a.rc2;
  a.rc2_loose = (float)((ctx->prm.rc + 1e-3) * (ctx->prm.rc + 1e-3)); a.reps2_f = (float)(ctx->T.r_eps * ctx->T.r_eps);
  const double rthr = near_rthr_now(ctx);
  a.rthr2_f = (float)(rthr * rthr);
  a.sqpa_f = (float)sqrt(RBC3D_PI / ctx->prm.alpha);
  a.two_isqa_f = (float)(2.0 / sqrt(ctx->prm.alpha));
  a.m8_ispi_f = (float)(-8.0 / sqrt(RBC3D_PI));
  a.q75_spi_f = (float)(0.75 * sqrt(RBC3D_PI));
  erfcx_coeffs(ctx);
  for (int k = 0; k <= ERFCX_DEG; ++k) a.erfcx_q[k] = ctx->erfcx_q[k];
  a.T = ctx->T;
  a.collect = collect_nbr ? 1 : 0;
  a.items = ctx->items.p; a.cap = ctx->items_cap; a.cnt = ctx->dcnt.p;
  bool dl = (c2 != 0.0) && ctx->has_g;
  if (prec != RBC3D_FP64) {
    CUDA_TRY(ctx->s_F4.alloc(ctx->npt));
    if (dl) CUDA_TRY(ctx->s_G4.alloc(ctx->npt));
    a.sF4 = ctx->s_F4.p; a.sG4 = ctx->s_G4.p;
    { k_src_dens4<<<nblk(ctx->npt, 256), 256, 0, ctx->st>>>(ctx->npt, c1, c2, ctx->s_f.p, ctx->s_g.p, dl ? 1 : 0,
                                                             ctx->s_F4.p, ctx->s_G4.p); ++ctx->launches; }
    a.units = t.wunits.p;
    a.nunits = t.nwunits;
    // own-cell pairs of the cell targets by the dense pass when the
    // same-cell weights come from the table (uniform longitudes)
    const int nrow = std::min(ctx->nlat, (OWN_TILE - 1) / std::max(ctx->nlon, 1) + 2);
    const size_t own_sm = sizeof(float) * (size_t)nrow * ctx->nlat * a.nhalf;
    const bool own = tlist == RBC3D_TLIST_RBC && a.mtab32 && t.n == ctx->npt && ctx->s_op0.p && own_sm <= 160 * 1024;
    a.own_split = own ? 1 : 0;
    a.op0 = ctx->s_op0.p; a.op1 = ctx->s_op1.p; a.sinv = ctx->s_inv.p;
    const int nb = (t.nwunits + TILE / 32 - 1) / (TILE / 32);
    if (dl) { k_pair32<true><<<nb, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
    else { k_pair32<false><<<nb, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
    if (own) {
      const int nv = ctx->nlat * ctx->nlon, nt = (nv + OWN_TILE - 1) / OWN_TILE, nbo = ctx->ncell * (nt * (nt + 1) / 2);
      if (dl) {
        if (own_sm > 48 * 1024)
          CUDA_TRY(cudaFuncSetAttribute(k_pair_own32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)own_sm));
        k_pair_own32<true><<<nbo, OWN_TILE, own_sm, ctx->st>>>(a);
      } else {
        if (own_sm > 48 * 1024)
          CUDA_TRY(cudaFuncSetAttribute(k_pair_own32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)own_sm));
        k_pair_own32<false><<<nbo, OWN_TILE, own_sm, ctx->st>>>(a);
      }
      ++ctx->launches;
    }
  } else {
    a.own_split = 0;
    if (dl) { k_pair64<true><<<t.nunits, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
    else { k_pair64<false><<<t.nunits, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
  }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

rbc3d_status run_linear(rbc3d_ctx* ctx, int tlist, double c2) {
  if (c2 == 0.0 || ctx->npt == 0 || !ctx->has_g) return RBC3D_OK;
  TargetSet& t = ctx->tl[tlist];
  const double* Bc = ctx->dBcoef.p;
  CUDA_TRY(ctx->xvint.alloc(3));
  CUDA_TRY(cudaMemsetAsync(ctx->xvint.p, 0, 3 * sizeof(double), ctx->st));
  { k_linear_reduce<<<304, 256, 0, ctx->st>>>(ctx->npt, ctx->nlat * ctx->nlon, ctx->x.p, ctx->sg.p, ctx->a3.p,
                                            ctx->celltype.p, Bc, ctx->xvint.p); ++ctx->launches; }
  double pil = ctx->iLb[0] * ctx->iLb[1] * ctx->iLb[2];
  if (t.n) { k_linear_add<<<nblk(t.n, 256), 256, 0, ctx->st>>>(t.n, t.Acoef.p, ctx->xvint.p, c2 * (-8 * RBC3D_PI * pil), t.v.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

void erfcx_coeffs(rbc3d_ctx* ctx) {
  const double X = ctx->prm.rc * std::sqrt(RBC3D_PI / ctx->prm.alpha);
  if (ctx->erfcx_X != X) {
    ctx->erfcx_X = X;
    fit_erfcx(X, ctx->erfcx_q);
  }
}
