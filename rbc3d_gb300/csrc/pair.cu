// pair.cu -- cell lists and the real-space Stokeslet / stresslet pair sums of
// AddIntOnRbcs (ModIntOnRbcs.F90:47-112) on the GPU.
//
// Cell list: the linked lists hoc/next of HashTable_Build (ModHashTable.F90:
// 23-62) become a stable radix sort of the points by cell id plus
// [start, end) ranges per cell.  The same Nc = max(floor(L/rc), 3) cells are
// used, so a target visits its 27 neighbour cells exactly as the reference.
//
// Pair kernel: one CTA per (target cell, chunk of <= 128 targets); the 27
// neighbour cells are streamed through shared memory in tiles of 128 sources;
// each thread owns one target.  Positions are taken relative to the centre of
// the target cell in FP64 and split into FP32 hi/lo parts, so the FP32
// difference x_j - x_i is exact to ~1e-14 regardless of the box size.  The
// FP32 variant accumulates each target with Kahan compensation.
#include <cub/cub.cuh>

#include <algorithm>
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

// Gather cell-point geometry into cell-list order.
__global__ void k_gather_src(int n, int nlat, int nv, const int* __restrict__ order, const double* __restrict__ x,
                             const double* __restrict__ a3, double* __restrict__ sx, double* __restrict__ sa3,
                             int4* __restrict__ meta) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int p = order[q];
  for (int k = 0; k < 3; ++k) {
    sx[q + (size_t)k * n] = x[p + (size_t)k * n];
    sa3[q + (size_t)k * n] = a3[p + (size_t)k * n];
  }
  int cell = p / nv, r = p - cell * nv;
  meta[q] = make_int4(cell + 1, r % nlat, r / nlat, p);
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
  // grid
  int Nc[3];
  double h[3], L[3], iL[3];
  const double* th;
  const double* phi;
  const float4* usph;
  int nlat;
  double radius, inv_radius;
  float inv_radius_f, chord2_max;
  double c1, c2;
  float c1f, c2f;
  double rc2;
  float rc2_f, reps2_f;
  float rthr2_f;  // FP32 path: cross-surface pairs closer than this are left to the FP64 near-singular pass
  float sqpa_f, two_isqa_f, m8_ispi_f, q75_spi_f;  // sqrt(pi/alpha), 2/sqrt(alpha), -8/sqrt(pi), 0.75 sqrt(pi)
  Tables T;
  // near-singular work list
  int collect;
  int4* items;
  int cap;
  unsigned long long* cnt;  // [0] items, [1] pairs, [2] overflow
};

__device__ __forceinline__ double min_image(double d, double L, double iL) { return d - round(d * iL) * L; }

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

// Shared-memory source tile
struct TileF {
  float hx[TILE], hy[TILE], hz[TILE], lx[TILE], ly[TILE], lz[TILE];
  float fx[TILE], fy[TILE], fz[TILE], gx[TILE], gy[TILE], gz[TILE];
  float ax[TILE], ay[TILE], az[TILE];
  float ux[TILE], uy[TILE], uz[TILE];
  int surf[TILE], id[TILE];
};
struct TileD {
  double x[TILE], y[TILE], z[TILE];
  double fx[TILE], fy[TILE], fz[TILE], gx[TILE], gy[TILE], gz[TILE];
  double ax[TILE], ay[TILE], az[TILE];
  int surf[TILE], ilat[TILE], ilon[TILE];
};

template <bool DL>
__global__ void __launch_bounds__(TILE) k_pair32(PairArgs a) {
  __shared__ TileF sm;
  const int4 unit = a.units[blockIdx.x];
  const int cell = unit.x;
  const int tid = threadIdx.x;
  const bool active = tid < unit.z;
  const int ci = cell % a.Nc[0], cj = (cell / a.Nc[0]) % a.Nc[1], ck = cell / (a.Nc[0] * a.Nc[1]);
  const double c0[3] = {(ci + 0.5) * a.h[0], (cj + 0.5) * a.h[1], (ck + 0.5) * a.h[2]};
  int ti = active ? a.torder[unit.y + tid] : 0;
  float th_[3] = {0, 0, 0}, tl_[3] = {0, 0, 0};
  float4 ui = make_float4(0, 0, 0, 0);
  int surf_i = -2;
  if (active) {
    for (int k = 0; k < 3; ++k) {
      double r = min_image(a.tx[ti + (size_t)k * a.nt] - c0[k], a.L[k], a.iL[k]);
      th_[k] = (float)r;
      tl_[k] = (float)(r - (double)th_[k]);
    }
    int4 m = a.tmeta[ti];
    surf_i = m.x;
    if (m.y >= 0) ui = a.usph[m.y + a.nlat * m.z];
  }
  Kahan3 acc;
  acc.zero();
  NbrList L;
  L.n = 0; L.overflow = 0;
  int run_surf = -3, run_id = -1;
  float run_d2 = 3.4e38f;
  unsigned long long npairs = 0;

  for (int nb = 0; nb < 27; ++nb) {
    int dx = nb % 3 - 1, dy = (nb / 3) % 3 - 1, dz = nb / 9 - 1;
    int ni = imod(ci + dx, a.Nc[0]), nj = imod(cj + dy, a.Nc[1]), nk = imod(ck + dz, a.Nc[2]);
    int ncell = ni + a.Nc[0] * (nj + a.Nc[1] * nk);
    int sbeg = a.cs[ncell], send = a.ce[ncell];
    for (int base = sbeg; base < send; base += TILE) {
      int cnt = min(TILE, send - base);
      __syncthreads();
      if (tid < cnt) {
        int q = base + tid;
        double r[3];
        for (int k = 0; k < 3; ++k) r[k] = min_image(a.sx[q + (size_t)k * a.ns] - c0[k], a.L[k], a.iL[k]);
        float hx = (float)r[0], hy = (float)r[1], hz = (float)r[2];
        sm.hx[tid] = hx; sm.hy[tid] = hy; sm.hz[tid] = hz;
        sm.lx[tid] = (float)(r[0] - (double)hx); sm.ly[tid] = (float)(r[1] - (double)hy); sm.lz[tid] = (float)(r[2] - (double)hz);
        sm.fx[tid] = (float)(a.c1 * a.sf[q]); sm.fy[tid] = (float)(a.c1 * a.sf[q + a.ns]); sm.fz[tid] = (float)(a.c1 * a.sf[q + 2 * (size_t)a.ns]);
        if (DL) {
          sm.gx[tid] = (float)(a.c2 * a.sg[q]); sm.gy[tid] = (float)(a.c2 * a.sg[q + a.ns]); sm.gz[tid] = (float)(a.c2 * a.sg[q + 2 * (size_t)a.ns]);
          sm.ax[tid] = (float)a.sa3[q]; sm.ay[tid] = (float)a.sa3[q + a.ns]; sm.az[tid] = (float)a.sa3[q + 2 * (size_t)a.ns];
        }
        int4 m = a.smeta[q];
        float4 u = a.usph[m.y + a.nlat * m.z];
        sm.ux[tid] = u.x; sm.uy[tid] = u.y; sm.uz[tid] = u.z;
        sm.surf[tid] = m.x;
        sm.id[tid] = m.y | (m.z << 16);
      }
      __syncthreads();
      if (active) {
        for (int j = 0; j < cnt; ++j) {
          const int sj = sm.surf[j];
          if (a.collect && sj != run_surf) {
            if (run_id >= 0) L.insert(run_surf, run_id, run_d2);
            run_surf = sj; run_id = -1; run_d2 = 3.4e38f;
          }
          float xx = __fadd_rn(sm.hx[j] - th_[0], sm.lx[j] - tl_[0]);
          float yy = __fadd_rn(sm.hy[j] - th_[1], sm.ly[j] - tl_[1]);
          float zz = __fadd_rn(sm.hz[j] - th_[2], sm.lz[j] - tl_[2]);
          float r2 = xx * xx + yy * yy + zz * zz;
          if (r2 > a.rc2_f) continue;
          ++npairs;
          float wgt = 1.f;
          if (sj == surf_i) {
            float ex = ui.x - sm.ux[j], ey = ui.y - sm.uy[j], ez = ui.z - sm.uz[j];
            float ch2 = ex * ex + ey * ey + ez * ez;
            if (ch2 < a.chord2_max) {
              // dth = 2 asin(chord/2); MaskFunc lerp on the reference table
              float t = 2.f * asinf(0.5f * sqrtf(ch2)) * a.inv_radius_f;
              float s = t * (float)MASK_NTAB;
              int i = (int)s;
              if (i < MASK_NTAB) {
                float2 e = __ldg(a.T.mask32 + i);
                wgt = 1.f - (e.x + (s - (float)i) * e.y);
              } else wgt = 1.f;
            }
          } else {
            if (a.collect && r2 < run_d2) { run_d2 = r2; run_id = sm.id[j]; }
            // A pair this close to another surface is re-evaluated in FP64 by
            // the near-singular pass (its FP32 rounding would survive the
            // cancellation with the FP64 subtraction).
            if (a.collect && r2 < a.rthr2_f) continue;
          }
          if (r2 < a.reps2_f) continue;
          float rinv = rsqrtf(r2);
          float r = r2 * rinv;
          // Ewald coefficients evaluated directly (erfc / exp in FP32) rather
          // than by per-lane gathers into the 8193-entry tables: the tables'
          // lerp differs from the exact functions by ~2e-8 relative, below
          // FP32 resolution (the FP64 plain form keeps the tables).
          float st = r * a.sqpa_f;  // r*sqrt(pi/alpha)
          float ex = expf(-st * st);
          float c1 = erfcf(st), c2 = a.two_isqa_f * ex;
          float ir2 = rinv * rinv;
          float A = (c1 * rinv + c2) * ir2;
          float B = c1 * rinv - c2;
          float dotf = xx * sm.fx[j] + yy * sm.fy[j] + zz * sm.fz[j];
          float Ad = A * dotf;
          float vx = Ad * xx + B * sm.fx[j];
          float vy = Ad * yy + B * sm.fy[j];
          float vz = Ad * zz + B * sm.fz[j];
          if (DL) {
            // -8/sqrt(pi) [exp(-t^2)(1.5 t + t^3) + 0.75 sqrt(pi) erfc(t)] / r^5
            float cdl = a.m8_ispi_f * (ex * (st * (1.5f + st * st)) + a.q75_spi_f * c1);
            float Adl = cdl * ir2 * ir2 * rinv;
            float dg = xx * sm.gx[j] + yy * sm.gy[j] + zz * sm.gz[j];
            float da = xx * sm.ax[j] + yy * sm.ay[j] + zz * sm.az[j];
            float t = Adl * dg * da;
            vx += t * xx; vy += t * yy; vz += t * zz;
          }
          acc.add(0, wgt * vx);
          acc.add(1, wgt * vy);
          acc.add(2, wgt * vz);
        }
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
  // pair count
  for (int o = 16; o > 0; o >>= 1) npairs += __shfl_xor_sync(0xffffffffu, npairs, o);
  if ((tid & 31) == 0 && npairs) atomicAdd(a.cnt + 1, npairs);
}

// FP64 plain form: the same traversal with the reference arithmetic.
template <bool DL>
__global__ void __launch_bounds__(TILE) k_pair64(PairArgs a) {
  __shared__ TileD sm;
  const int4 unit = a.units[blockIdx.x];
  const int cell = unit.x;
  const int tid = threadIdx.x;
  const bool active = tid < unit.z;
  const int ci = cell % a.Nc[0], cj = (cell / a.Nc[0]) % a.Nc[1], ck = cell / (a.Nc[0] * a.Nc[1]);
  const double c0[3] = {(ci + 0.5) * a.h[0], (cj + 0.5) * a.h[1], (ck + 0.5) * a.h[2]};
  int ti = active ? a.torder[unit.y + tid] : 0;
  double t_[3] = {0, 0, 0};
  int surf_i = -2;
  double th_i = 0, phi_i = 0;
  if (active) {
    for (int k = 0; k < 3; ++k) t_[k] = min_image(a.tx[ti + (size_t)k * a.nt] - c0[k], a.L[k], a.iL[k]);
    int4 m = a.tmeta[ti];
    surf_i = m.x;
    if (m.y >= 0) { th_i = a.th[m.y]; phi_i = a.phi[m.z]; }
  }
  double acc[3] = {0, 0, 0};
  NbrList L;
  L.n = 0; L.overflow = 0;
  int run_surf = -3, run_id = -1;
  double run_d = 1e300;
  unsigned long long npairs = 0;
  const double rc = a.T.rc;

  for (int nb = 0; nb < 27; ++nb) {
    int dx = nb % 3 - 1, dy = (nb / 3) % 3 - 1, dz = nb / 9 - 1;
    int ni = imod(ci + dx, a.Nc[0]), nj = imod(cj + dy, a.Nc[1]), nk = imod(ck + dz, a.Nc[2]);
    int ncell = ni + a.Nc[0] * (nj + a.Nc[1] * nk);
    int sbeg = a.cs[ncell], send = a.ce[ncell];
    for (int base = sbeg; base < send; base += TILE) {
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
      if (active) {
        for (int j = 0; j < cnt; ++j) {
          const int sj = sm.surf[j];
          if (a.collect && sj != run_surf) {
            if (run_id >= 0) L.insert(run_surf, run_id, (float)run_d);
            run_surf = sj; run_id = -1; run_d = 1e300;
          }
          double xx = sm.x[j] - t_[0], yy = sm.y[j] - t_[1], zz = sm.z[j] - t_[2];
          double rr = sqrt(xx * xx + yy * yy + zz * zz);
          if (rr > rc) continue;
          ++npairs;
          double mask = 0.;
          if (sj == surf_i) {
            double dth = dist_on_sphere(th_i, phi_i, a.th[sm.ilat[j]], a.phi[sm.ilon[j]]);
            mask = mask64(a.T, dth * a.inv_radius);
          } else if (a.collect) {
            if (rr < run_d) { run_d = rr; run_id = sm.ilat[j] | (sm.ilon[j] << 16); }
          }
          double EA, EB;
          ewald_sl64(a.T, rr, EA, EB);
          double s1 = (1. - mask) * a.c1;
          double d = xx * sm.fx[j] + yy * sm.fy[j] + zz * sm.fz[j];
          acc[0] += s1 * (EA * xx * d + EB * sm.fx[j]);
          acc[1] += s1 * (EA * yy * d + EB * sm.fy[j]);
          acc[2] += s1 * (EA * zz * d + EB * sm.fz[j]);
          if (DL) {
            double EAd = ewald_dl64(a.T, rr);
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
  DBuf<int> key, key2, idx;
  CUDA_TRY(key.alloc(n)); CUDA_TRY(key2.alloc(n)); CUDA_TRY(idx.alloc(n)); CUDA_TRY(order.alloc(n));
  CUDA_TRY(cs.alloc(hg.ncells)); CUDA_TRY(ce.alloc(hg.ncells));
  { k_hash_keys<<<nblk(n, 256), 256, 0, ctx->st>>>(n, x_dev, hg.Nc[0], hg.Nc[1], hg.Nc[2], hg.Nc[0] / hg.L[0],
                                                  hg.Nc[1] / hg.L[1], hg.Nc[2] / hg.L[2], key.p, idx.p); ++ctx->launches; }
  size_t tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp, key.p, key2.p, idx.p, order.p, n, 0, 32, ctx->st);
  DBuf<char> tbuf;
  CUDA_TRY(tbuf.alloc(tmp + 1));
  CUDA_TRY(cub::DeviceRadixSort::SortPairs(tbuf.p, tmp, key.p, key2.p, idx.p, order.p, n, 0, 32, ctx->st));
  CUDA_TRY(cudaMemsetAsync(cs.p, 0, sizeof(int) * hg.ncells, ctx->st));
  CUDA_TRY(cudaMemsetAsync(ce.p, 0, sizeof(int) * hg.ncells, ctx->st));
  { k_cell_ranges<<<nblk(n, 256), 256, 0, ctx->st>>>(n, key2.p, cs.p, ce.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status make_units(rbc3d_ctx* ctx, TargetSet& t, const DBuf<int>& cs, const DBuf<int>& ce) {
  int nc = ctx->hg.ncells;
  std::vector<int> hs(nc), he(nc);
  CUDA_TRY(cudaMemcpy(hs.data(), cs.p, sizeof(int) * nc, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(he.data(), ce.p, sizeof(int) * nc, cudaMemcpyDeviceToHost));
  std::vector<int4> u;
  for (int c = 0; c < nc; ++c)
    for (int b = hs[c]; b < he[c]; b += TILE) u.push_back(make_int4(c, b, std::min(TILE, he[c] - b), 0));
  // heaviest cells first: cells are visited in decreasing neighbourhood load
  t.nunits = (int)u.size();
  if (t.nunits) CUDA_TRY(t.units.upload(u.data(), u.size(), ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

}  // namespace

rbc3d_status sort_points_by_cell(rbc3d_ctx* ctx, int n, const double* x_dev, DBuf<int>& order, DBuf<int>& cs,
                                DBuf<int>& ce) {
  return sort_points(ctx, n, x_dev, order, cs, ce);
}

rbc3d_status build_source_list(rbc3d_ctx* ctx) {
  int n = ctx->npt;
  rbc3d_status s = sort_points(ctx, n, ctx->x.p, ctx->s_order, ctx->s_cstart, ctx->s_cend);
  if (s) return s;
  CUDA_TRY(ctx->s_x.alloc(3 * (size_t)n)); CUDA_TRY(ctx->s_a3.alloc(3 * (size_t)n)); CUDA_TRY(ctx->s_meta.alloc(n));
  CUDA_TRY(ctx->s_f.alloc(3 * (size_t)n)); CUDA_TRY(ctx->s_g.alloc(3 * (size_t)n));
  { k_gather_src<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, ctx->nlat * ctx->nlon, ctx->s_order.p, ctx->x.p,
                                                   ctx->a3.p, ctx->s_x.p, ctx->s_a3.p, ctx->s_meta.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  ctx->src_sorted = true;
  ctx->pme.cplan.valid = false;  // the PME tiles follow the source positions
  // tlist_rbc shares the source order
  TargetSet& t = ctx->tl[RBC3D_TLIST_RBC];
  t.sorted = false;
  return RBC3D_OK;
}

rbc3d_status build_source_density(rbc3d_ctx* ctx) {
  int n = ctx->npt, nv = ctx->nlat * ctx->nlon;
  if (n == 0) return RBC3D_OK;
  DBuf<double> Bc;
  CUDA_TRY(Bc.upload(ctx->Bcoef, RBC3D_MAX_CELLTYPES, ctx->st));
  if (ctx->has_f) { k_density<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, nv, ctx->f.p, ctx->detJ.p, ctx->w.p, ctx->sf.p); ++ctx->launches; }
  if (ctx->has_g) { k_density<<<nblk(n, 256), 256, 0, ctx->st>>>(n, ctx->nlat, nv, ctx->g.p, ctx->detJ.p, ctx->w.p, ctx->sg.p); ++ctx->launches; }
  { k_gather_density<<<nblk(n, 256), 256, 0, ctx->st>>>(n, nv, ctx->s_order.p, ctx->sf.p, ctx->sg.p, ctx->celltype.p,
                                                       Bc.p, ctx->s_f.p, ctx->s_g.p, ctx->has_f, ctx->has_g); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
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
  for (int d = 0; d < 3; ++d) { a.Nc[d] = ctx->hg.Nc[d]; a.h[d] = ctx->hg.h[d]; a.L[d] = ctx->hg.L[d]; a.iL[d] = ctx->iLb[d]; }
  a.th = ctx->th.p; a.phi = ctx->phi.p; a.usph = ctx->usph.p; a.nlat = ctx->nlat;
  a.radius = ctx->radius; a.inv_radius = 1.0 / ctx->radius; a.inv_radius_f = (float)(1.0 / ctx->radius);
  double cm = 2.0 * sin(0.5 * ctx->radius) * (1.0 + 1e-6);
  a.chord2_max = (float)(cm * cm);
  a.c1 = c1; a.c2 = c2; a.c1f = (float)c1; a.c2f = (float)c2;
  a.rc2 = ctx->prm.rc * ctx->prm.rc; a.rc2_f = (float)a.rc2; a.reps2_f = (float)(ctx->T.r_eps * ctx->T.r_eps);
  a.rthr2_f = (float)(ctx->near_rthr * ctx->near_rthr);
  a.sqpa_f = (float)sqrt(RBC3D_PI / ctx->prm.alpha);
  a.two_isqa_f = (float)(2.0 / sqrt(ctx->prm.alpha));
  a.m8_ispi_f = (float)(-8.0 / sqrt(RBC3D_PI));
  a.q75_spi_f = (float)(0.75 * sqrt(RBC3D_PI));
  a.T = ctx->T;
  a.collect = collect_nbr ? 1 : 0;
  a.items = ctx->items.p; a.cap = ctx->items_cap; a.cnt = ctx->dcnt.p;
  bool dl = (c2 != 0.0) && ctx->has_g;
  if (prec != RBC3D_FP64) {
    if (dl) { k_pair32<true><<<t.nunits, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
    else { k_pair32<false><<<t.nunits, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
  } else {
    if (dl) { k_pair64<true><<<t.nunits, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
    else { k_pair64<false><<<t.nunits, TILE, 0, ctx->st>>>(a); ++ctx->launches; }
  }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

rbc3d_status run_linear(rbc3d_ctx* ctx, int tlist, double c2) {
  if (c2 == 0.0 || ctx->npt == 0 || !ctx->has_g) return RBC3D_OK;
  TargetSet& t = ctx->tl[tlist];
  DBuf<double> Bc;
  CUDA_TRY(Bc.upload(ctx->Bcoef, RBC3D_MAX_CELLTYPES, ctx->st));
  CUDA_TRY(ctx->xvint.alloc(3));
  CUDA_TRY(cudaMemsetAsync(ctx->xvint.p, 0, 3 * sizeof(double), ctx->st));
  { k_linear_reduce<<<304, 256, 0, ctx->st>>>(ctx->npt, ctx->nlat * ctx->nlon, ctx->x.p, ctx->sg.p, ctx->a3.p,
                                            ctx->celltype.p, Bc.p, ctx->xvint.p); ++ctx->launches; }
  double pil = ctx->iLb[0] * ctx->iLb[1] * ctx->iLb[2];
  if (t.n) { k_linear_add<<<nblk(t.n, 256), 256, 0, ctx->st>>>(t.n, t.Acoef.p, ctx->xvint.p, c2 * (-8 * RBC3D_PI * pil), t.v.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}
