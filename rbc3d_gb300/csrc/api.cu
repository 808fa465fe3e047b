// api.cu -- C ABI of the GB300 Ewald-split boundary-integral matvec
// (include/rbc3d_gpu.h): context set-up, uploads and the entry points that
// replace RBC3D's module procedures.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.hpp"

rbc3d_status ctx_fail(rbc3d_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}
rbc3d_status ctx_fail_cuda(rbc3d_ctx* ctx, cudaError_t e, const char* what) {
  if (ctx) ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
  return RBC3D_ERR_CUDA;
}

// GauLeg (ModQuadRule.F90:135-214): Numerical Recipes Gauss-Legendre nodes by
// simultaneous Newton iteration, EPS = 3e-14.
void host_gauleg(double x1, double x2, int n, double* x, double* w) {
  const double EPS = 3.e-14;
  int m = (n + 1) / 2;
  double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
  std::vector<double> p1(m), p2(m), p3(m), pp(m), z(m), z1(m);
  std::vector<char> act(m, 1);
  for (int j = 0; j < m; ++j) z[j] = std::cos(RBC3D_PI * ((j + 1) - 0.25) / (n + 0.5));
  for (int its = 1; its <= 10; ++its) {
    for (int k = 0; k < m; ++k)
      if (act[k]) { p1[k] = 1.0; p2[k] = 0.0; }
    for (int j = 1; j <= n; ++j)
      for (int k = 0; k < m; ++k)
        if (act[k]) { p3[k] = p2[k]; p2[k] = p1[k]; p1[k] = ((2.0 * j - 1.0) * z[k] * p2[k] - (j - 1.0) * p3[k]) / j; }
    bool any = false;
    for (int k = 0; k < m; ++k)
      if (act[k]) {
        pp[k] = n * (z[k] * p1[k] - p2[k]) / (z[k] * z[k] - 1.0);
        z1[k] = z[k];
        z[k] = z1[k] - p1[k] / pp[k];
        act[k] = std::fabs(z[k] - z1[k]) > EPS;
        any = any || act[k];
      }
    if (!any) break;
  }
  for (int k = 0; k < m; ++k) {
    x[k] = xm - xl * z[k];
    x[n - 1 - k] = xm + xl * z[k];
    w[k] = 2.0 * xl / ((1.0 - z[k] * z[k]) * pp[k] * pp[k]);
    w[n - 1 - k] = w[k];
  }
}

StageScope::StageScope(rbc3d_ctx* ctx, int stage) : c(ctx), slot(-1) {
  if (!c->prof) return;
  if (2 * (c->nrec + 1) > c->evpool.size()) {
    size_t old = c->evpool.size();
    c->evpool.resize(old + 512);
    for (size_t i = old; i < c->evpool.size(); ++i) cudaEventCreate(&c->evpool[i]);
    c->rec_stage.resize(c->evpool.size() / 2);
  }
  slot = (int)c->nrec++;
  c->rec_stage[slot] = stage;
  cudaEventRecord(c->evpool[2 * slot], c->st);
}
StageScope::~StageScope() {
  if (slot >= 0) cudaEventRecord(c->evpool[2 * slot + 1], c->st);
}

// The current stream waits for spline tables (and the target positions
// derived from them) that set_cells_x / set_cell_density_x left in flight on
// the side stream; on the side stream itself the wait is already implied.
void spl_wait(rbc3d_ctx* ctx) {
  if (ctx->spl_pending && ctx->ev_spl) cudaStreamWaitEvent(ctx->st, ctx->ev_spl, 0);
}

// near_rthr, computed on the device by set_cells_x, is read on its first use.
double near_rthr_now(rbc3d_ctx* ctx) {
  if (ctx->rthr_pending) {
    cudaEventSynchronize(ctx->ev_rthr);
    ctx->near_rthr = *ctx->h_rthr;
    ctx->rthr_pending = false;
  }
  return ctx->near_rthr;
}

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

static double mask_exact(double x) {  // MaskFunc_Exact, ModBasicMath.F90:332-346
  double t = std::fabs(x);
  if (t < 0.01) return 1.;
  if (t > 0.99) return 0.;
  return std::exp(2 * (std::exp(-1. / t)) / (t - 1));
}

// Host copy of MaskFunc (table lerp) for the patch weights.
static double mask_lerp(const std::vector<double>& tab, double x) {
  double s = std::fabs(x) * MASK_NTAB;
  int i = (int)std::floor(s);
  if (i >= MASK_NTAB) return 0.;
  return tab[i] * (i + 1 - s) + tab[i + 1] * (s - i);
}

// Spline table repack: ABI layout per cell [kind][var][j][i] (nvar vars) ->
// device layout [cell][set][node=i+m*j][kind*3+var].
__global__ void k_repack(int ncell, int m, int n, int nvar, int set, const double* __restrict__ src,
                         double* __restrict__ dst) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = (long long)m * n;
  long long total = (long long)ncell * per;
  if (idx >= total) return;
  int cell = (int)(idx / per);
  int node = (int)(idx - cell * per);
  const double* s = src + (size_t)cell * 4 * per * nvar;
  double* d = dst + (((size_t)cell * SPL_NSET + set) * per + node) * SPL_NODE;
  for (int kind = 0; kind < 4; ++kind)
    for (int v = 0; v < 3; ++v) d[kind * 3 + v] = (v < nvar) ? s[(size_t)kind * per * nvar + node + per * v] : 0.0;
}

__global__ void k_fill_meta(int n, int nv, int nlat, int4* meta) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int cell = p / nv, r = p - cell * nv;
  meta[p] = make_int4(cell + 1, r % nlat, r / nlat, 0);
}
__global__ void k_fill_acoef(int n, int nv, const int* celltype, const double* Ac, double* A) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  A[p] = Ac[celltype[p / nv]];
}
__global__ void k_fill_const(int n, int4 mv, double av, int4* meta, double* A) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  meta[p] = mv;
  A[p] = av;
}

rbc3d_status upload_splines(rbc3d_ctx* ctx, const double* h, int nvar, int set) {
  if (!h) return RBC3D_OK;
  size_t per = (size_t)ctx->m * ctx->nlon;
  size_t cnt = (size_t)ctx->ncell * 4 * per * nvar;
  // persistent staging buffer, stream-ordered reuse; the caller's buffer is
  // released by the synchronisation at the end of the entry point
  DBuf<double>& tmp = ctx->stage;
  CUDA_TRY(tmp.alloc(cnt));
  CUDA_TRY(cudaMemcpyAsync(tmp.p, h, sizeof(double) * cnt, cudaMemcpyHostToDevice, ctx->st));
  long long total = (long long)ctx->ncell * per;
  { k_repack<<<nblk(total, 256), 256, 0, ctx->st>>>(ctx->ncell, ctx->m, ctx->nlon, nvar, set, tmp.p, ctx->spl.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  return RBC3D_OK;
}

TargetSet* tset(rbc3d_ctx* ctx, int which) {
  if (which < 0 || which > 2) return nullptr;
  return &ctx->tl[which];
}

rbc3d_status begin(rbc3d_ctx* ctx, TargetSet& t) {
  CUDA_TRY(t.v.alloc(3 * (size_t)std::max(t.n, 1)));
  CUDA_TRY(cudaMemsetAsync(t.v.p, 0, sizeof(double) * 3 * t.n, ctx->st));
  return RBC3D_OK;
}
__global__ void k_vadd2(long long n, const double* __restrict__ a, double* __restrict__ v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] += a[i];
}

// v (caller's host array) += the matvec result: the caller's values go up,
// are added on the device and come back (two copies of 3n doubles, no host loop)
rbc3d_status finish_add(rbc3d_ctx* ctx, TargetSet& t, double* v) {
  const size_t n3 = 3 * (size_t)t.n;
  if (n3 == 0) return RBC3D_OK;
  DBuf<double>& d = ctx->vadd;
  CUDA_TRY(d.alloc(n3));
  CUDA_TRY(cudaMemcpyAsync(d.p, v, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->st));
  { k_vadd2<<<(int)((n3 + 255) / 256), 256, 0, ctx->st>>>((long long)n3, t.v.p, d.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(v, d.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

// Real space + corrections + linear term of AddIntOnRbcs on device (no download).
rbc3d_status self_stage(rbc3d_ctx* ctx, int which, double c1, double c2, int prec) {
  StageScope sc(ctx, 1);
  spl_wait(ctx);  // the patch reads the spline tables and the records built from them
  if (prec == RBC3D_FP32M) {
    if (!ctx->phi_uniform) return ctx_fail(ctx, RBC3D_ERR_ARG, "FP32M needs phi(j) = j*2*pi/nlon");
    return run_self_mixed(ctx, which, c1, c2);
  }
  if (prec == RBC3D_FP32D) return run_self_ff(ctx, which, c1, c2);
  return run_self_corr(ctx, which, c1, c2);
}

rbc3d_status pme_stages(rbc3d_ctx* ctx, int which, double c1, double c2, unsigned terms, int prec) {
  rbc3d_status s;
  {
    StageScope sc(ctx, 5);
    if ((s = pme_spread(ctx, c1, c2, 1, (terms & RBC3D_TERM_WALLS) ? 1 : 0, prec))) return s;
  }
  {
    StageScope sc(ctx, 6);
    if ((s = pme_transform(ctx))) return s;
  }
  StageScope sc(ctx, 7);
  return pme_gather(ctx, which);
}

__global__ void k_vadd(long long n, const double* __restrict__ a, double* __restrict__ v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] += a[i];
}

// The own-cell patch correction (with_self) and PME (with_pme) on the side
// stream, into the side accumulator t.v2; the main stream joins at ev_join.
rbc3d_status fork_side(rbc3d_ctx* ctx, int which, double c1, double c2, unsigned terms, int prec, bool with_self,
                       bool with_pme) {
  TargetSet& t = ctx->tl[which];
  const double sc1 = ctx->has_f ? c1 : 0.0, sc2 = ctx->has_g ? c2 : 0.0;
  CUDA_TRY(t.v2.alloc(3 * (size_t)std::max(t.n, 1)));
  CUDA_TRY(cudaEventRecord(ctx->ev_fork, ctx->st));
  CUDA_TRY(cudaStreamWaitEvent(ctx->st2, ctx->ev_fork, 0));
  std::swap(ctx->st, ctx->st2);
  dbuf_swap(t.v, t.v2);
  rbc3d_status s = RBC3D_OK;
  if (cudaMemsetAsync(t.v.p, 0, sizeof(double) * 3 * t.n, ctx->st) != cudaSuccess) s = RBC3D_ERR_CUDA;
  if (!s && with_self) s = self_stage(ctx, which, sc1, sc2, prec);
  if (!s && with_pme) s = pme_stages(ctx, which, c1, c2, terms, prec);
  dbuf_swap(t.v, t.v2);
  std::swap(ctx->st, ctx->st2);
  CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->st2));
  return s;
}

// self_late: the patch correction forks to the (low-priority) side stream
// after the pair sums, into the side accumulator, while the near-singular
// pass runs on the main stream.
rbc3d_status rbcs_dev(rbc3d_ctx* ctx, int which, double c1, double c2, int prec, unsigned terms,
                      bool self_elsewhere = false, bool self_late = false) {
  if (ctx->npt == 0) return RBC3D_OK;
  // a density that was never set is zero (the reference's cells start with f = g = 0)
  if (!ctx->has_f) c1 = 0.0;
  if (!ctx->has_g) c2 = 0.0;
  TargetSet& t = ctx->tl[which];
  bool corr = (terms & RBC3D_TERM_CORR) != 0;
  rbc3d_status s;
  for (int attempt = 0; attempt < 2; ++attempt) {
    CUDA_TRY(cudaMemsetAsync(ctx->dcnt.p, 0, sizeof(unsigned long long) * 3, ctx->st));
    if (terms & RBC3D_TERM_REAL || corr) {
      StageScope sc(ctx, 0);
      if ((s = run_pair_sum(ctx, which, (terms & RBC3D_TERM_REAL) ? c1 : 0.0, (terms & RBC3D_TERM_REAL) ? c2 : 0.0,
                            prec, corr)))
        return s;
    }
    if (!corr) break;
    unsigned long long h[3];
    CUDA_TRY(cudaMemcpyAsync(h, ctx->dcnt.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
    if (h[2]) return ctx_fail(ctx, RBC3D_ERR_OVERFLOW, "neighbour-cell list above NMax=32 for some target");
    if (h[0] <= (unsigned long long)ctx->items_cap) break;
    // grow the work list and redo the pass
    ctx->items_cap = (int)std::min<unsigned long long>(h[0] + h[0] / 4 + 1024, 0x7fffffffull);
    CUDA_TRY(ctx->items.alloc(ctx->items_cap));
    CUDA_TRY(cudaMemsetAsync(t.v.p, 0, sizeof(double) * 3 * t.n, ctx->st));
  }
  if (corr) {
    CUDA_TRY(cudaMemsetAsync(ctx->dcnt.p + 3, 0, sizeof(unsigned long long), ctx->st));
    CUDA_TRY(cudaMemsetAsync(ctx->dcnt.p + 6, 0, sizeof(unsigned long long), ctx->st));
    CUDA_TRY(cudaMemsetAsync(ctx->dcnt.p + 8, 0, sizeof(unsigned long long) * 3, ctx->st));
    if (self_late) {  // after fork_side: t.v2 is zeroed and PME queued on the side stream
      CUDA_TRY(cudaEventRecord(ctx->ev_fork, ctx->st));
      CUDA_TRY(cudaStreamWaitEvent(ctx->st2, ctx->ev_fork, 0));
      std::swap(ctx->st, ctx->st2);
      dbuf_swap(t.v, t.v2);
      s = self_stage(ctx, which, c1, c2, prec);
      dbuf_swap(t.v, t.v2);
      std::swap(ctx->st, ctx->st2);
      CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->st2));
      if (s) return s;
    } else if (!self_elsewhere && (s = self_stage(ctx, which, c1, c2, prec))) {
      return s;
    }
    {
      StageScope sc(ctx, 2);
      if ((s = run_near_corr(ctx, which, c1, c2, prec))) return s;
    }
  }
  if (terms & RBC3D_TERM_LINEAR) {
    StageScope sc(ctx, 3);
    if ((s = run_linear(ctx, which, c2))) return s;
  }
  unsigned long long h[10];
  CUDA_TRY(cudaMemcpyAsync(h, ctx->dcnt.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->counts.pairs_within_rc = (long long)h[1];
  if (corr) {
    ctx->counts.nbr_items = (long long)h[0];
    ctx->counts.nearsing_items = (long long)h[3];
    ctx->counts.screen_misses = (long long)h[6];
    ctx->counts.near_replays = (long long)h[8];
    ctx->counts.near_projections = (long long)h[9];
    ctx->counts.self_items = (which == RBC3D_TLIST_RBC) ? t.n : 0;
  }
  ctx->counts.nbr_overflow = (int)h[2];
  return RBC3D_OK;
}

}  // namespace

// Composite device-resident matvec used by the ABI calls (defined here so the
// wall solver can call it too).
rbc3d_status matvec_dev(rbc3d_ctx* ctx, int which, double c1, double c2, unsigned terms, int prec) {
  TargetSet& t = ctx->tl[which];
  rbc3d_status s;
  if ((s = begin(ctx, t))) return s;
  // A full cell matvec runs the own-cell patch correction and PME on the side
  // stream, into their own accumulator, while the main stream does the pair
  // sums, the near-singular pass, the linear term and the walls; the pipes
  // they load differ (FP32 / L1 / FP64 / shared memory), so the kernels share
  // the SMs.  The side accumulator is added at the join.
  const bool side = ctx->st2 && which == RBC3D_TLIST_RBC && ctx->npt > 0 && (terms & RBC3D_TERM_CORR) &&
                    (terms & RBC3D_TERM_PME);
  // PME joins the shorter stream: the side one when the patch correction is
  // the short FP32 one (FP32M: 8.5 ms against 9.0 with PME on the main
  // stream), else the main one after the pair and near passes (FP32C: 52.7
  // against 53.1 ms)
  // The float-float patch (FP32D) loads the FP32 pipe and L1 like the pair
  // sums: next to them it took 15.6 ms against 6.9 alone.  So the side
  // stream runs PME next to the pair sums and then the patch, forked after
  // them, while the main stream runs the FP64 near-singular pass beside the
  // end of PME: 12.2 ms, against 13.7 with PME on the main stream, 13.4 with PME
  // on a third low-priority stream (the FFTs interleave with the patch) and
  // 13.5 with PME on a third stream of medium priority (it starves the
  // patch).
  const bool late = side && prec == RBC3D_FP32D;
  const bool pme_side = prec == RBC3D_FP32M || late;
  if (side && (s = fork_side(ctx, which, c1, c2, terms, prec, !late, pme_side))) return s;
  if (terms & (RBC3D_TERM_REAL | RBC3D_TERM_CORR | RBC3D_TERM_LINEAR))
    if ((s = rbcs_dev(ctx, which, c1, c2, prec, terms, side && !late, late))) return s;
  if (terms & RBC3D_TERM_WALLS) {
    StageScope sc(ctx, 4);
    if (which == RBC3D_TLIST_WALL) { if ((s = run_wall_self(ctx, c1))) return s; }
    else if ((s = run_wall_quad(ctx, which, c1, prec))) return s;
  }
  if (side && !pme_side && (s = pme_stages(ctx, which, c1, c2, terms, prec))) return s;
  if (side) {
    CUDA_TRY(cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0));
    const long long n3 = 3ll * t.n;
    { k_vadd<<<nblk(n3, 256), 256, 0, ctx->st>>>(n3, t.v2.p, t.v.p); ++ctx->launches; }
    CUDA_TRY(cudaGetLastError());
  } else if (terms & RBC3D_TERM_PME) {
    if ((s = pme_stages(ctx, which, c1, c2, terms, prec))) return s;
  }
  return RBC3D_OK;
}

extern "C" {

int rbc3d_abi_version(void) { return RBC3D_ABI_VERSION; }

// SetEwaldPrms (ModConf.F90:348-408), single rank
rbc3d_status rbc3d_ewald_prms(double alpha, double eps, const double Lb[3], int P, double* rc, int Nb[3]) {
  if (!(alpha > 0) || !(eps > 0) || !Lb || !rc || !Nb) return RBC3D_ERR_ARG;
  double s = 1.;
  for (int it = 0; it < 10; ++it) {
    s = 0.75 * std::sqrt(RBC3D_PI) * eps / (s * s * s + 1.5 * s + 0.75 / s);
    s = std::sqrt(-std::log(s));
  }
  double r = std::sqrt(alpha / RBC3D_PI) * s;
  r = std::min(std::min(Lb[0] / 3.001, Lb[1] / 3.001), std::min(Lb[2] / 3.001, r));
  *rc = r;
  for (int d = 0; d < 3; ++d) Nb[d] = 2 * (int)std::ceil(std::sqrt(-std::log(eps) / (RBC3D_PI * alpha)) * Lb[d]);
  Nb[2] = std::max(Nb[2], P);
  return RBC3D_OK;
}

rbc3d_status rbc3d_create(const rbc3d_params* prm, rbc3d_ctx** out) {
  if (!prm || !out) return RBC3D_ERR_ARG;
  *out = nullptr;
  if (prm->ncelltypes < 1 || prm->ncelltypes > RBC3D_MAX_CELLTYPES || prm->P < 2 || prm->P > 8 || !(prm->rc > 0) ||
      !(prm->alpha > 0) || prm->nlat < 2 || prm->nlon < 4 || prm->nlon % 2)
    return RBC3D_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (!(prm->Lb[d] > 0) || prm->Nb[d] < prm->P || prm->rc > prm->Lb[d] / 3.0) return RBC3D_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return RBC3D_ERR_CUDA;
  rbc3d_ctx* ctx = new rbc3d_ctx();
  ctx->prm = *prm;
  cudaGetDevice(&ctx->device);
  {
    const char* e = getenv("RBC3D_VERIFY_SCREEN");
    ctx->verify_screen = e && e[0] == '1';
    const char* c = getenv("RBC3D_NEAR_STAGE_CAP");  // a smaller capacity sends the rest through k_near
    if (c && *c) ctx->near_stage_cap = std::max(0, std::min(atoi(c), NEAR_STAGE_CAP));
  }
  for (int d = 0; d < 3; ++d) ctx->iLb[d] = 1. / prm->Lb[d];
  for (int l = 0; l < prm->ncelltypes; ++l) {  // initCOEFs, ModConf.F90:327-344
    if (prm->viscRat[l] > 0) { ctx->Acoef[l] = 1. + prm->viscRat[l]; ctx->Bcoef[l] = 1. - prm->viscRat[l]; }
    else { ctx->Acoef[l] = 1.; ctx->Bcoef[l] = -1.; }
  }
  rbc3d_status s = RBC3D_OK;
  auto bail = [&](rbc3d_status code) { rbc3d_destroy(ctx); return code; };
  {
    int lowest = 0, highest = 0;
    cudaDeviceGetStreamPriorityRange(&lowest, &highest);
    if (cudaStreamCreateWithPriority(&ctx->st, cudaStreamNonBlocking, highest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->st2, cudaStreamNonBlocking, lowest) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_spl, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_up, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_rthr, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_geom, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_dens, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost((void**)&ctx->h_rthr, sizeof(double)) != cudaSuccess)
      return bail(RBC3D_ERR_CUDA);
  }
  // Ewald tables, ModEwaldFunc.F90:96-104, 151-162
  const int N = EWALD_NTAB;
  const double alpha = prm->alpha, rc = prm->rc;
  std::vector<double> c1(N + 1), c2(N + 1), dl(N + 1), mk(MASK_NTAB + 1);
  for (int i = 0; i <= N; ++i) {
    double r_t = std::sqrt(RBC3D_PI / alpha) * ((double)i * rc / N);
    c1[i] = std::erfc(r_t);
    c2[i] = 2 / std::sqrt(alpha) * std::exp(-(r_t * r_t));
    dl[i] = -8 / std::sqrt(RBC3D_PI) * (std::exp(-(r_t * r_t)) * (1.5 * r_t + r_t * r_t * r_t) +
                                        0.75 * std::sqrt(RBC3D_PI) * std::erfc(r_t));
  }
  for (int i = 0; i <= MASK_NTAB; ++i) mk[i] = mask_exact((double)i / MASK_NTAB);
  std::vector<float4> sl32(N);
  std::vector<float2> dl32(N), mk32(MASK_NTAB);
  for (int i = 0; i < N; ++i) {
    sl32[i] = make_float4((float)c1[i], (float)(c1[i + 1] - c1[i]), (float)c2[i], (float)(c2[i + 1] - c2[i]));
    dl32[i] = make_float2((float)dl[i], (float)(dl[i + 1] - dl[i]));
  }
  for (int i = 0; i < MASK_NTAB; ++i) mk32[i] = make_float2((float)mk[i], (float)(mk[i + 1] - mk[i]));
  if (ctx->t_sl1.upload(c1.data(), c1.size(), ctx->st) || ctx->t_sl2.upload(c2.data(), c2.size(), ctx->st) ||
      ctx->t_dl.upload(dl.data(), dl.size(), ctx->st) || ctx->t_mask.upload(mk.data(), mk.size(), ctx->st) ||
      ctx->t_sl32.upload(sl32.data(), sl32.size(), ctx->st) || ctx->t_dl32.upload(dl32.data(), dl32.size(), ctx->st) ||
      ctx->t_mask32.upload(mk32.data(), mk32.size(), ctx->st) || ctx->dcnt.alloc(16) || ctx->xvint.alloc(3) ||
      ctx->dBcoef.upload(ctx->Bcoef, RBC3D_MAX_CELLTYPES, ctx->st))
    return bail(RBC3D_ERR_CUDA);
  if (self_ff_tables(ctx, c1, c2, dl)) return bail(RBC3D_ERR_CUDA);
  Tables& T = ctx->T;
  T.sl_c1 = ctx->t_sl1.p; T.sl_c2 = ctx->t_sl2.p; T.dl_c1 = ctx->t_dl.p; T.mask = ctx->t_mask.p;
  T.sl32 = ctx->t_sl32.p; T.dl32 = ctx->t_dl32.p; T.mask32 = ctx->t_mask32.p;
  T.rc = rc; T.r_eps = 1.e-3 * std::sqrt(alpha / RBC3D_PI); T.ntab_over_rc = N / rc;
  T.rc_f = (float)rc; T.r_eps_f = (float)T.r_eps; T.ntab_over_rc_f = (float)(N / rc);
  // cell list
  for (int d = 0; d < 3; ++d) {
    ctx->hg.Nc[d] = std::max((int)std::floor(prm->Lb[d] / prm->rc), 3);
    ctx->hg.L[d] = prm->Lb[d];
    ctx->hg.h[d] = prm->Lb[d] / ctx->hg.Nc[d];
  }
  ctx->hg.ncells = ctx->hg.Nc[0] * ctx->hg.Nc[1] * ctx->hg.Nc[2];
  ctx->nlat = prm->nlat; ctx->nlon = prm->nlon; ctx->m = 2 * prm->nlat;
  if ((s = pme_setup(ctx))) return bail(s);
  // ReAdd rules (ModRbcSingInt.F90:254-261): GauLeg(-1,1,16) for the sinh map
  std::vector<double> gs(16), gw(16);
  host_gauleg(-1., 1., 16, gs.data(), gw.data());
  if (ctx->rd_s.upload(gs.data(), 16, ctx->st) || ctx->rd_w.upload(gw.data(), 16, ctx->st)) return bail(RBC3D_ERR_CUDA);
  cudaStreamSynchronize(ctx->st);
  *out = ctx;
  return RBC3D_OK;
}

rbc3d_status rbc3d_destroy(rbc3d_ctx* ctx) {
  if (!ctx) return RBC3D_OK;
  pme_release(ctx);
  wall_spec_release(ctx);
  if (ctx->st2) cudaStreamSynchronize(ctx->st2);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  for (cudaEvent_t e : ctx->evpool) cudaEventDestroy(e);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->ev_spl) cudaEventDestroy(ctx->ev_spl);
  if (ctx->ev_up) cudaEventDestroy(ctx->ev_up);
  if (ctx->ev_rthr) cudaEventDestroy(ctx->ev_rthr);
  if (ctx->ev_geom) cudaEventDestroy(ctx->ev_geom);
  if (ctx->ev_dens) cudaEventDestroy(ctx->ev_dens);
  if (ctx->h_rthr) cudaFreeHost(ctx->h_rthr);
  if (ctx->st2) cudaStreamDestroy(ctx->st2);
  if (ctx->t0) { cudaEventDestroy(ctx->t0); cudaEventDestroy(ctx->t1); }
  cudaStream_t st = ctx->st;
  delete ctx;
  if (st) cudaStreamDestroy(st);
  return RBC3D_OK;
}

const char* rbc3d_last_error(const rbc3d_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

// RBC_Create grid (ModRbc.F90:92-94) + RbcPolarPatch_Create (ModPolarPatch.F90:27-75)
rbc3d_status rbc3d_set_cell_grid(rbc3d_ctx* ctx, const double* th, const double* phi, const double* w) {
  if (!ctx || !th || !phi || !w) return RBC3D_ERR_ARG;
  const int nlat = ctx->nlat, nlon = ctx->nlon;
  ctx->h_th.assign(th, th + nlat); ctx->h_phi.assign(phi, phi + nlon); ctx->h_w.assign(w, w + nlat);
  ctx->shtab.L = 0;  // transform tables of the previous grid
  CUDA_TRY(ctx->th.upload(th, nlat, ctx->st)); CUDA_TRY(ctx->phi.upload(phi, nlon, ctx->st));
  CUDA_TRY(ctx->w.upload(w, nlat, ctx->st));
  std::vector<float4> us(nlat * nlon);
  for (int j = 0; j < nlon; ++j)
    for (int i = 0; i < nlat; ++i)
      us[i + nlat * j] = make_float4((float)(std::sin(th[i]) * std::cos(phi[j])), (float)(std::sin(th[i]) * std::sin(phi[j])),
                                     (float)std::cos(th[i]), 0.f);
  CUDA_TRY(ctx->usph.upload(us.data(), us.size(), ctx->st));
  // polar patch
  std::vector<double> mk(MASK_NTAB + 1);
  for (int i = 0; i <= MASK_NTAB; ++i) mk[i] = mask_exact((double)i / MASK_NTAB);
  const std::vector<double>& mk_tab = mk;
  ctx->radius = RBC3D_PI / std::sqrt((double)nlat);
  double h = RBC3D_PI / nlat;
  ctx->nrad = 2 * (int)std::round(ctx->radius / h);
  ctx->nazm = 2 * ctx->nrad;
  const int nrad = ctx->nrad, nazm = ctx->nazm, NQ = nrad * nazm;
  std::vector<double> thL(nrad), pw(nrad), phiL(nazm);
  host_gauleg(0., ctx->radius, nrad, thL.data(), pw.data());
  for (int i = 0; i < nrad; ++i) {
    pw[i] = pw[i] * std::sin(thL[i]) * (RBC3D_TWO_PI / nazm);
    pw[i] = pw[i] * mask_lerp(mk, thL[i] / ctx->radius);
  }
  for (int j = 0; j < nazm; ++j) phiL[j] = j * RBC3D_TWO_PI / nazm;
  // PolarPatch_Build: thG depends on th0 only; phiG = atan2(...) + phi0 with a
  // wrap, so the atan2 part is stored and phi0 added in the kernel.
  std::vector<double> thG((size_t)NQ * nlat), phiA((size_t)NQ * nlat);
  for (int i0 = 0; i0 < nlat; ++i0) {
    double st0 = std::sin(th[i0]), ct0 = std::cos(th[i0]);
    for (int ir = 0; ir < nrad; ++ir) {
      double sth = std::sin(thL[ir]), cth = std::cos(thL[ir]);
      for (int ia = 0; ia < nazm; ++ia) {
        double x0 = sth * std::cos(phiL[ia]), x1 = sth * std::sin(phiL[ia]), x2 = cth;
        double y0 = ct0 * x0 + 0. * x1 + st0 * x2, y1 = 0. * x0 + 1. * x1 + 0. * x2, y2 = -st0 * x0 + 0. * x1 + ct0 * x2;
        y2 = std::fmax(-1.0, std::fmin(1.0, y2));
        size_t q = (size_t)i0 * NQ + ir + nrad * ia;
        thG[q] = std::acos(y2);
        phiA[q] = std::atan2(y1, y0);
      }
    }
  }
  CUDA_TRY(ctx->pw.upload(pw.data(), nrad, ctx->st));
  ctx->phi_uniform = true;
  for (int j = 0; j < nlon; ++j)
    if (std::fabs(phi[j] - j * RBC3D_TWO_PI / nlon) > 1e-12) ctx->phi_uniform = false;
  if (ctx->phi_uniform) {
    // MaskFunc(DistOnSphere / radius) of every pair of grid points of one cell
    // (ModIntOnRbcs.F90:77-80): with phi(j) = j 2 pi / nlon it depends on the two
    // latitudes and the longitude difference d (and d ~ nlon - d) only
    const int nh = nlon / 2 + 1;
    std::vector<double> m64((size_t)nlat * nlat * nh);
    std::vector<float> w32(m64.size());
    for (int i0 = 0; i0 < nlat; ++i0)
      for (int i1 = 0; i1 < nlat; ++i1)
        for (int d = 0; d < nh; ++d) {
          double c = std::cos(th[i0] - th[i1]) - std::sin(th[i0]) * std::sin(th[i1]) * (1. - std::cos(phi[0] - phi[d]));
          c = std::fmin(1., std::fmax(-1., c));
          const double mk = mask_lerp(mk_tab, std::acos(c) / ctx->radius);
          m64[((size_t)i0 * nlat + i1) * nh + d] = mk;
          w32[((size_t)i0 * nlat + i1) * nh + d] = (float)(1.0 - mk);
        }
    CUDA_TRY(ctx->mtab64.upload(m64.data(), m64.size(), ctx->st));
    CUDA_TRY(ctx->mtab32.upload(w32.data(), w32.size(), ctx->st));
  }
  {
    rbc3d_status s = self_mixed_grid(ctx, thG, phiA, pw);
    if (s) return s;
  }
  {
    // FP64 Spline_Interp weights per (latitude, patch point) for k_self: with
    // phi(j) = j 2 pi / nlon, phiG = atan2(...) + phi0 moves the stencil by
    // whole columns, so only the column offset depends on the target's longitude
    const int m = 2 * nlat;
    const double hx = RBC3D_TWO_PI / m, hy = RBC3D_TWO_PI / nlon, ihx = 1. / hx, ihy = 1. / hy;
    std::vector<SelfW64> W((size_t)nlat * NQ);
    for (size_t i = 0; i < W.size(); ++i) {
      const double x = thG[i] * ihx, y = phiA[i] * ihy;
      const int i1 = (int)std::floor(x), j1 = (int)std::floor(y);
      const double s = x - i1, t = y - j1;
      SelfW64 e;
      e.i1 = ((i1 % m) + m) % m;
      e.j1b = j1;
      double cx[4], cy[4];
      cx[0] = 1 + s * s * (-3. + 2. * s); cx[1] = s * s * (3. - 2. * s);
      cx[2] = hx * s * (1. + s * (-2. + s)); cx[3] = hx * s * s * (-1. + s);
      cy[0] = 1 + t * t * (-3. + 2. * t); cy[1] = t * t * (3. - 2. * t);
      cy[2] = hy * t * (1. + t * (-2. + t)); cy[3] = hy * t * t * (-1. + t);
      // node (i1,j1): u u1 u2 u12, then (i1,j2), (i2,j1), (i2,j2), as spline_w16
      const int ax[4] = {0, 0, 1, 1}, ay[4] = {0, 1, 0, 1};
      for (int k = 0; k < 4; ++k) {
        e.w[4 * k + 0] = cx[ax[k]] * cy[ay[k]];
        e.w[4 * k + 1] = cx[ax[k] + 2] * cy[ay[k]];
        e.w[4 * k + 2] = cx[ax[k]] * cy[ay[k] + 2];
        e.w[4 * k + 3] = cx[ax[k] + 2] * cy[ay[k] + 2];
      }
      W[i] = e;
    }
    CUDA_TRY(ctx->self_w64.upload(reinterpret_cast<const char*>(W.data()), W.size() * sizeof(SelfW64), ctx->st));
    rbc3d_status s = self_ff_grid(ctx, W, pw);
    if (s) return s;
  }
  CUDA_TRY(ctx->thG.upload(thG.data(), thG.size(), ctx->st));
  CUDA_TRY(ctx->phiA.upload(phiA.data(), phiA.size(), ctx->st));
  std::vector<double> x0(16), w0(16);
  host_gauleg(0., ctx->radius, 16, x0.data(), w0.data());
  CUDA_TRY(ctx->rd_x0.upload(x0.data(), 16, ctx->st));
  CUDA_TRY(ctx->rd_w0.upload(w0.data(), 16, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status cells_tail(rbc3d_ctx* ctx, bool side_tables = false);

rbc3d_status rbc3d_set_cells(rbc3d_ctx* ctx, int ncell, const int* celltype, const double* x, const double* a3,
                             const double* detJ, const double* area, const double* meshSize, const double* spl_x,
                             const double* spl_a3, const double* spl_detJ) {
  if (!ctx || ncell < 0 || (ncell > 0 && (!celltype || !x || !a3 || !detJ || !area || !meshSize || !spl_x ||
                                         !spl_a3 || !spl_detJ)))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "set_cells: bad arguments");
  if (ctx->h_th.empty()) return ctx_fail(ctx, RBC3D_ERR_STATE, "cell grid not set");
  for (int c = 0; c < ncell; ++c)
    if (celltype[c] < 0 || celltype[c] >= ctx->prm.ncelltypes) return ctx_fail(ctx, RBC3D_ERR_ARG, "bad celltype");
  const int nv = ctx->nlat * ctx->nlon;
  ctx->ncell = ncell;
  ctx->npt = ncell * nv;
  ctx->has_f = ctx->has_g = false;
  ctx->src_density = false;
  if (ncell == 0) return RBC3D_OK;
  size_t N = ctx->npt;
  ctx->h_celltype.assign(celltype, celltype + ncell);
  spl_wait(ctx);
  {
    double mn = meshSize[0];
    for (int c = 1; c < ncell; ++c) mn = std::min(mn, meshSize[c]);
    ctx->near_rthr = 0.5 * mn;
    ctx->rthr_pending = false;
  }
  CUDA_TRY(ctx->celltype.upload(celltype, ncell, ctx->st));
  CUDA_TRY(ctx->x.upload(x, 3 * N, ctx->st)); CUDA_TRY(ctx->a3.upload(a3, 3 * N, ctx->st));
  CUDA_TRY(ctx->detJ.upload(detJ, N, ctx->st));
  CUDA_TRY(ctx->area.upload(area, ncell, ctx->st)); CUDA_TRY(ctx->meshSize.upload(meshSize, ncell, ctx->st));
  CUDA_TRY(ctx->f.alloc(3 * N)); CUDA_TRY(ctx->g.alloc(3 * N)); CUDA_TRY(ctx->sf.alloc(3 * N)); CUDA_TRY(ctx->sg.alloc(3 * N));
  CUDA_TRY(cudaMemsetAsync(ctx->sg.p, 0, sizeof(double) * 3 * N, ctx->st));
  CUDA_TRY(cudaMemsetAsync(ctx->g.p, 0, sizeof(double) * 3 * N, ctx->st));
  CUDA_TRY(ctx->spl.alloc((size_t)ncell * SPL_NSET * ctx->m * ctx->nlon * SPL_NODE));
  CUDA_TRY(ctx->stage.alloc((size_t)ncell * 4 * ctx->m * ctx->nlon * 3));  // before any side-stream work
  rbc3d_status s;
  // the spline tables (the bulk of the upload) go up on the side stream
  // while the main stream builds the source list from the positions
  CUDA_TRY(cudaEventRecord(ctx->ev_fork, ctx->st));
  CUDA_TRY(cudaStreamWaitEvent(ctx->st2, ctx->ev_fork, 0));
  std::swap(ctx->st, ctx->st2);
  s = upload_splines(ctx, spl_x, 3, SPL_X);
  if (!s) s = upload_splines(ctx, spl_a3, 3, SPL_A3);
  if (!s) s = upload_splines(ctx, spl_detJ, 1, SPL_DJ);
  std::swap(ctx->st, ctx->st2);
  CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->st2));
  if (s) return s;
  return cells_tail(ctx);
}

// The position-dependent set-up after the cells' arrays are on the device
// (the spline tables may still be in flight on the side stream, joined by
// ev_join): source list, tlist_rbc, PME spread plan, FP32M records.
// side_tables: set_cells_x, whose side stream builds the tables and the
// target positions derived from them itself (readers wait on ev_spl); the
// main stream then neither joins it nor waits for the device at the end.
rbc3d_status cells_tail(rbc3d_ctx* ctx, bool side_tables) {
  rbc3d_status s;
  const int nv = ctx->nlat * ctx->nlon;
  const size_t N = ctx->npt;
  // set_cells_x: the positions' part now, the normals once the side stream's
  // geometry is done
  if ((s = build_source_list(ctx, !side_tables))) return s;
  // tlist_rbc (TargetList_Update, ModTargetList.F90:95-131): its work units
  // and the PME spread plan depend on the positions only, and are built while
  // the spline tables are still being written on the side stream
  TargetSet& t = ctx->tl[RBC3D_TLIST_RBC];
  t.n = ctx->npt;
  t.sorted = false;
  if ((s = sort_targets(ctx, RBC3D_TLIST_RBC))) return s;
  if ((s = pme_prepare_cells(ctx))) return s;
  if (side_tables) {
    CUDA_TRY(cudaStreamWaitEvent(ctx->st, ctx->ev_geom, 0));
    if ((s = source_normals(ctx))) return s;
  } else {
    CUDA_TRY(cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0));
    if ((s = self_mixed_geom(ctx))) return s;
  }
  DBuf<double>& Ac = ctx->acoef_dev;
  CUDA_TRY(Ac.upload(ctx->Acoef, RBC3D_MAX_CELLTYPES, ctx->st));
  CUDA_TRY(t.x.alloc(3 * N)); CUDA_TRY(t.Acoef.alloc(N)); CUDA_TRY(t.meta.alloc(N));
  CUDA_TRY(cudaMemcpyAsync(t.x.p, ctx->x.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, ctx->st));
  { k_fill_acoef<<<nblk(N, 256), 256, 0, ctx->st>>>(t.n, nv, ctx->celltype.p, Ac.p, t.Acoef.p); ++ctx->launches; }
  { k_fill_meta<<<nblk(N, 256), 256, 0, ctx->st>>>(t.n, nv, ctx->nlat, t.meta.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  int want = 12 * std::max(ctx->npt, 1024);
  if (ctx->items_cap < want) { ctx->items_cap = want; CUDA_TRY(ctx->items.alloc(want)); }
  if (!side_tables) CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status rbc3d_set_cell_density(rbc3d_ctx* ctx, const double* f, const double* g, const double* spl_F,
                                    const double* spl_G) {
  if (!ctx) return RBC3D_ERR_ARG;
  if (ctx->npt == 0) return RBC3D_OK;
  if ((f && !spl_F) || (g && !spl_G)) return ctx_fail(ctx, RBC3D_ERR_ARG, "density without spline table");
  size_t N = ctx->npt;
  rbc3d_status s;
  spl_wait(ctx);  // tables still being built on the side stream are finished first
  if (f) {
    CUDA_TRY(ctx->f.upload(f, 3 * N, ctx->st));
    if ((s = upload_splines(ctx, spl_F, 3, SPL_F))) return s;
    ctx->has_f = true;
  }
  if (g) {
    CUDA_TRY(ctx->g.upload(g, 3 * N, ctx->st));
    if ((s = upload_splines(ctx, spl_G, 3, SPL_G))) return s;
    ctx->has_g = true;
  }
  if ((s = self_mixed_density(ctx, f != nullptr, g != nullptr))) return s;
  if ((s = build_source_density(ctx))) return s;
  CUDA_TRY(cudaStreamSynchronize(ctx->st));  // the caller's host buffers are free again
  return RBC3D_OK;
}

__global__ void k_mesh_size(int ncell, int nlat, const double* __restrict__ area, double* __restrict__ msz) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncell) msz[c] = sqrt(area[c] / ((double)nlat * nlat));  // ModRbc.F90:504
}

// out = 0.5 * min(v[0..n)) (one block)
__global__ void __launch_bounds__(256) k_half_min(int n, const double* __restrict__ v, double* __restrict__ out) {
  __shared__ double red[256];
  double m = HUGE_VAL;
  for (int i = threadIdx.x; i < n; i += 256) m = fmin(m, v[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = 0.5 * red[0];
}

// Cells from their positions alone: RBC_ComputeGeometry (a3, detJ, area,
// meshSize; ModRbc.F90:404-509) and Rbc_BuildSurfaceSource(xFlag) (the x, a3
// and detJ tables, ShFilter to degree < nlat0; ModRbc.F90:716-807) on the
// device, then SourceList_UpdateCoord / TargetList_Update as rbc3d_set_cells.
rbc3d_status rbc3d_set_cells_x(rbc3d_ctx* ctx, int ncell, const int* celltype, int nlat0, const double* x) {
  if (!ctx || ncell < 0 || (ncell > 0 && (!celltype || !x)))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "set_cells_x: bad arguments");
  if (ctx->h_th.empty()) return ctx_fail(ctx, RBC3D_ERR_STATE, "cell grid not set");
  if (nlat0 < 1 || nlat0 > ctx->nlat || 2 * (nlat0 - 1) >= ctx->nlon)
    return ctx_fail(ctx, RBC3D_ERR_ARG, "set_cells_x: need 1 <= nlat0 <= nlat, 2 (nlat0 - 1) < nlon");
  for (int c = 0; c < ncell; ++c)
    if (celltype[c] < 0 || celltype[c] >= ctx->prm.ncelltypes) return ctx_fail(ctx, RBC3D_ERR_ARG, "bad celltype");
  const int nv = ctx->nlat * ctx->nlon;
  ctx->ncell = ncell;
  ctx->npt = ncell * nv;
  ctx->has_f = ctx->has_g = false;
  ctx->src_density = false;
  if (ncell == 0) return RBC3D_OK;
  const size_t N = ctx->npt;
  ctx->h_celltype.assign(celltype, celltype + ncell);
  spl_wait(ctx);  // side-stream readers of the previous cells are done before they are overwritten
  CUDA_TRY(ctx->celltype.upload(celltype, ncell, ctx->st));
  CUDA_TRY(ctx->x.upload(x, 3 * N, ctx->st));
  // the caller's x may be reused once it has been copied
  CUDA_TRY(cudaEventRecord(ctx->ev_up, ctx->st));
  CUDA_TRY(ctx->a3.alloc(3 * N)); CUDA_TRY(ctx->detJ.alloc(N));
  CUDA_TRY(ctx->area.alloc(ncell)); CUDA_TRY(ctx->meshSize.alloc(ncell));
  CUDA_TRY(ctx->f.alloc(3 * N)); CUDA_TRY(ctx->g.alloc(3 * N)); CUDA_TRY(ctx->sf.alloc(3 * N)); CUDA_TRY(ctx->sg.alloc(3 * N));
  CUDA_TRY(cudaMemsetAsync(ctx->sg.p, 0, sizeof(double) * 3 * N, ctx->st));
  CUDA_TRY(cudaMemsetAsync(ctx->g.p, 0, sizeof(double) * 3 * N, ctx->st));
  CUDA_TRY(ctx->spl.alloc((size_t)ncell * SPL_NSET * ctx->m * ctx->nlon * SPL_NODE));
  rbc3d_status s;
  CUDA_TRY(ctx->rthr_dev.alloc(1));
  // The side stream derives the geometry (RBC_ComputeGeometry), then the
  // spline tables and the target positions taken from them, while the main
  // stream builds the source list, the target work units and the PME plan
  // from the positions; it takes the sources' normals once the geometry is
  // done (ev_geom), and the tables' readers wait on ev_spl.  near_rthr =
  // 0.5 min(meshSize) comes back to the host in the background.
  CUDA_TRY(cudaEventRecord(ctx->ev_fork, ctx->st));
  CUDA_TRY(cudaStreamWaitEvent(ctx->st2, ctx->ev_fork, 0));
  std::swap(ctx->st, ctx->st2);
  s = cells_geometry_dev(ctx);
  if (!s) {
    { k_mesh_size<<<nblk(ncell, 128), 128, 0, ctx->st>>>(ncell, ctx->nlat, ctx->area.p, ctx->meshSize.p); ++ctx->launches; }
    { k_half_min<<<1, 256, 0, ctx->st>>>(ncell, ctx->meshSize.p, ctx->rthr_dev.p); ++ctx->launches; }
    if (cudaMemcpyAsync(ctx->h_rthr, ctx->rthr_dev.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess ||
        cudaEventRecord(ctx->ev_rthr, ctx->st) != cudaSuccess || cudaEventRecord(ctx->ev_geom, ctx->st) != cudaSuccess)
      s = RBC3D_ERR_CUDA;
    ctx->rthr_pending = true;
  }
  if (!s) s = surface_sources_dev(ctx, nlat0, true, false, false);
  if (!s) s = self_mixed_geom(ctx);
  std::swap(ctx->st, ctx->st2);
  CUDA_TRY(cudaEventRecord(ctx->ev_spl, ctx->st2));
  CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->st2));
  ctx->spl_pending = true;
  if (s) return s;
  CUDA_TRY(cudaEventSynchronize(ctx->ev_up));
  return cells_tail(ctx, true);
}

// Densities from the raw surface values alone: Rbc_BuildSurfaceSource(fFlag /
// gFlag) (the f detJ and g detJ tables, ShFilter to degree < nlat0) on the
// device, then SourceList_UpdateDensity as rbc3d_set_cell_density.
rbc3d_status rbc3d_set_cell_density_x(rbc3d_ctx* ctx, int nlat0, const double* f, const double* g) {
  if (!ctx) return RBC3D_ERR_ARG;
  if (ctx->npt == 0) return RBC3D_OK;
  const size_t N = ctx->npt;
  rbc3d_status s;
  // the side stream's reads of the previous densities are done
  if (ctx->dens_pending) CUDA_TRY(cudaStreamWaitEvent(ctx->st, ctx->ev_dens, 0));
  if (f) CUDA_TRY(ctx->f.upload(f, 3 * N, ctx->st));
  if (g) CUDA_TRY(ctx->g.upload(g, 3 * N, ctx->st));
  CUDA_TRY(cudaEventRecord(ctx->ev_up, ctx->st));
  // the f detJ / g detJ tables on the side stream (readers wait on ev_spl),
  // the source densities on the main stream
  CUDA_TRY(cudaStreamWaitEvent(ctx->st2, ctx->ev_up, 0));
  std::swap(ctx->st, ctx->st2);
  s = surface_sources_dev(ctx, nlat0, false, f != nullptr, g != nullptr);
  if (!s && f) ctx->has_f = true;
  if (!s && g) ctx->has_g = true;
  if (!s) s = self_mixed_density(ctx, f != nullptr, g != nullptr);
  // a context whose matvecs run in FP32D gets its float-float node records
  // here, on the side stream, ahead of the first matvec's patch
  if (!s && ctx->ff_rec.p && ctx->phi_uniform)
    s = self_ff_records(ctx, 1 | (ctx->has_f ? 2 : 0) | (ctx->has_g ? 4 | 8 : 0));
  std::swap(ctx->st, ctx->st2);
  CUDA_TRY(cudaEventRecord(ctx->ev_spl, ctx->st2));
  CUDA_TRY(cudaEventRecord(ctx->ev_dens, ctx->st2));
  ctx->spl_pending = ctx->dens_pending = true;
  if (s) return s;
  if ((s = build_source_density(ctx))) return s;
  CUDA_TRY(cudaEventSynchronize(ctx->ev_up));  // the caller's host buffers are free again
  return RBC3D_OK;
}

rbc3d_status rbc3d_set_walls(rbc3d_ctx* ctx, int nvert, int nele, const double* x, const int* e2v, const int* glb) {
  if (!ctx || nvert < 0 || nele < 0 || (nvert > 0 && (!x || !e2v || !glb)))
    return ctx_fail(ctx, RBC3D_ERR_ARG, "set_walls: bad arguments");
  WallState& W = ctx->wall;
  W.nvert = nvert; W.nele = nele;
  W.hx.assign(x, x + 3 * (size_t)nvert);
  W.he2v.resize(3 * (size_t)nele);
  for (size_t i = 0; i < W.he2v.size(); ++i) {
    W.he2v[i] = e2v[i] - 1;
    if (W.he2v[i] < 0 || W.he2v[i] >= nvert) return ctx_fail(ctx, RBC3D_ERR_ARG, "e2v out of range");
  }
  W.hglb.resize(nvert);
  W.ndof = 0;
  for (int i = 0; i < nvert; ++i) {
    W.hglb[i] = glb[i] - 1;
    if (W.hglb[i] < 0) return ctx_fail(ctx, RBC3D_ERR_ARG, "indxVertGlb out of range");
    W.ndof = std::max(W.ndof, 3 * glb[i]);
  }
  W.hf.assign(3 * (size_t)nvert, 0.);
  W.prepared = false;
  wall_spec_release(ctx);  // a new mesh invalidates the learned spectral operator
  ctx->pme.wplan.valid = false;
  rbc3d_status s = wall_setup(ctx);
  if (s) return s;
  // tlist_wall (TargetList_Update walls: Acoef = 2, ModTargetList.F90:119-127)
  TargetSet& t = ctx->tl[RBC3D_TLIST_WALL];
  t.n = nvert;
  t.sorted = false;
  CUDA_TRY(t.x.upload(x, 3 * (size_t)nvert, ctx->st));
  CUDA_TRY(t.Acoef.alloc(nvert)); CUDA_TRY(t.meta.alloc(nvert));
  if (nvert) { k_fill_const<<<nblk(nvert, 256), 256, 0, ctx->st>>>(nvert, make_int4(-1000, -1, -1, 0), 2.0, t.meta.p, t.Acoef.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status rbc3d_set_wall_density(rbc3d_ctx* ctx, const double* f) {
  if (!ctx || (!f && ctx->wall.nvert)) return RBC3D_ERR_ARG;
  WallState& W = ctx->wall;
  W.hf.assign(f, f + 3 * (size_t)W.nvert);
  CUDA_TRY(W.f.upload(f, 3 * (size_t)W.nvert, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}
rbc3d_status rbc3d_get_wall_density(rbc3d_ctx* ctx, double* f) {
  if (!ctx || (!f && ctx->wall.nvert)) return RBC3D_ERR_ARG;
  WallState& W = ctx->wall;
  if (W.nvert) {
    CUDA_TRY(cudaMemcpyAsync(f, W.f.p, sizeof(double) * 3 * W.nvert, cudaMemcpyDeviceToHost, ctx->st));
    CUDA_TRY(cudaStreamSynchronize(ctx->st));
  }
  return RBC3D_OK;
}

rbc3d_status rbc3d_set_raw_targets(rbc3d_ctx* ctx, int n, const double* x) {
  if (!ctx || n < 0 || (n > 0 && !x)) return RBC3D_ERR_ARG;
  TargetSet& t = ctx->tl[RBC3D_TLIST_RAW];
  t.n = n;
  t.sorted = false;
  if (n == 0) return RBC3D_OK;
  CUDA_TRY(t.x.upload(x, 3 * (size_t)n, ctx->st));
  CUDA_TRY(t.Acoef.alloc(n)); CUDA_TRY(t.meta.alloc(n));
  { k_fill_const<<<nblk(n, 256), 256, 0, ctx->st>>>(n, make_int4(-1, -1, -1, 0), 2.0, t.meta.p, t.Acoef.p); ++ctx->launches; }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

int rbc3d_num_targets(const rbc3d_ctx* ctx, int which) {
  if (!ctx || which < 0 || which > 2) return -1;
  return ctx->tl[which].n;
}

rbc3d_status rbc3d_add_int_on_rbcs(rbc3d_ctx* ctx, int which, double c1, double c2, int prec, double* v) {
  TargetSet* t = ctx ? tset(ctx, which) : nullptr;
  if (!t || !v || !valid_prec(prec)) return ctx_fail(ctx, RBC3D_ERR_ARG, "add_int_on_rbcs");
  rbc3d_status s;
  if ((s = begin(ctx, *t))) return s;
  if ((s = rbcs_dev(ctx, which, c1, c2, prec, RBC3D_TERM_REAL | RBC3D_TERM_CORR | RBC3D_TERM_LINEAR))) return s;
  return finish_add(ctx, *t, v);
}

rbc3d_status rbc3d_add_int_on_walls(rbc3d_ctx* ctx, int which, double c1, int prec, double* v) {
  TargetSet* t = ctx ? tset(ctx, which) : nullptr;
  if (!t || !v) return ctx_fail(ctx, RBC3D_ERR_ARG, "add_int_on_walls");
  rbc3d_status s;
  if ((s = begin(ctx, *t))) return s;
  if (which == RBC3D_TLIST_WALL) s = run_wall_self(ctx, c1);
  else s = run_wall_quad(ctx, which, c1, prec);
  if (s) return s;
  return finish_add(ctx, *t, v);
}

rbc3d_status rbc3d_prepare_sing_int_on_wall(rbc3d_ctx* ctx) {
  if (!ctx) return RBC3D_ERR_ARG;
  return wall_prepare_self(ctx);
}

rbc3d_status rbc3d_pme_distrib_source(rbc3d_ctx* ctx, double c1, double c2, int cells, int walls, int prec) {
  if (!ctx || !valid_prec(prec)) return RBC3D_ERR_ARG;
  return pme_spread(ctx, c1, c2, cells, walls, prec);
}
rbc3d_status rbc3d_pme_transform(rbc3d_ctx* ctx) {
  if (!ctx) return RBC3D_ERR_ARG;
  return pme_transform(ctx);
}
rbc3d_status rbc3d_pme_add_interp_vel(rbc3d_ctx* ctx, int which, double* v) {
  TargetSet* t = ctx ? tset(ctx, which) : nullptr;
  if (!t || !v) return ctx_fail(ctx, RBC3D_ERR_ARG, "pme_add_interp_vel");
  rbc3d_status s;
  if ((s = begin(ctx, *t))) return s;
  if ((s = pme_gather(ctx, which))) return s;
  return finish_add(ctx, *t, v);
}

rbc3d_status rbc3d_matvec(rbc3d_ctx* ctx, int which, double c1, double c2, unsigned terms, int prec, double* v) {
  TargetSet* t = ctx ? tset(ctx, which) : nullptr;
  if (!t || !valid_prec(prec)) return ctx_fail(ctx, RBC3D_ERR_ARG, "matvec");
  rbc3d_status s = matvec_dev(ctx, which, c1, c2, terms, prec);
  if (s) return s;
  if (!v) return RBC3D_OK;  // result stays on the device
  return finish_add(ctx, *t, v);
}

rbc3d_status rbc3d_set_profiling(rbc3d_ctx* ctx, int on) {
  if (!ctx) return RBC3D_ERR_ARG;
  ctx->prof = on != 0;
  ctx->nrec = 0;
  return RBC3D_OK;
}

rbc3d_status rbc3d_stage_times(rbc3d_ctx* ctx, double ms[RBC3D_NSTAGE], int count[RBC3D_NSTAGE]) {
  if (!ctx || !ms) return RBC3D_ERR_ARG;
  for (int i = 0; i < RBC3D_NSTAGE; ++i) { ms[i] = 0.; if (count) count[i] = 0; }
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  for (size_t r = 0; r < ctx->nrec; ++r) {
    float e = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&e, ctx->evpool[2 * r], ctx->evpool[2 * r + 1]));
    ms[ctx->rec_stage[r]] += e;
    if (count) count[ctx->rec_stage[r]]++;
  }
  ctx->nrec = 0;
  return RBC3D_OK;
}

rbc3d_status rbc3d_timer_start(rbc3d_ctx* ctx) {
  if (!ctx) return RBC3D_ERR_ARG;
  if (!ctx->t0) { CUDA_TRY(cudaEventCreate(&ctx->t0)); CUDA_TRY(cudaEventCreate(&ctx->t1)); }
  CUDA_TRY(cudaEventRecord(ctx->t0, ctx->st));
  return RBC3D_OK;
}
rbc3d_status rbc3d_timer_stop(rbc3d_ctx* ctx, double* ms) {
  if (!ctx || !ms || !ctx->t0) return RBC3D_ERR_ARG;
  CUDA_TRY(cudaEventRecord(ctx->t1, ctx->st));
  CUDA_TRY(cudaEventSynchronize(ctx->t1));
  float e = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&e, ctx->t0, ctx->t1));
  *ms = e;
  return RBC3D_OK;
}

// CalcVelocityField, ModPostProcess.F90:29-63 (overwrites v)
rbc3d_status rbc3d_calc_velocity_field(rbc3d_ctx* ctx, int which, int prec, double* v) {
  TargetSet* t = ctx ? tset(ctx, which) : nullptr;
  if (!t || !v) return ctx_fail(ctx, RBC3D_ERR_ARG, "calc_velocity_field");
  double c = 1.0 / (4. * RBC3D_PI);
  rbc3d_status s = matvec_dev(ctx, which, c, c, RBC3D_TERM_ALL, prec);
  if (s) return s;
  std::fill(v, v + 3 * (size_t)t->n, 0.);
  if ((s = finish_add(ctx, *t, v))) return s;
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < t->n; ++i) v[i + (size_t)k * t->n] += ctx->prm.vBkg[k];
  return RBC3D_OK;
}

rbc3d_status rbc3d_compute_wall_residual_vel(rbc3d_ctx* ctx, int prec, double* v) {
  if (!ctx || !v) return RBC3D_ERR_ARG;
  rbc3d_status s = wall_residual_dev(ctx, prec);
  if (s) return s;
  TargetSet& t = ctx->tl[RBC3D_TLIST_WALL];
  std::fill(v, v + 3 * (size_t)t.n, 0.);
  return finish_add(ctx, t, v);
}

rbc3d_status rbc3d_wall_matmult(rbc3d_ctx* ctx, int prec, const double* u, double* y) {
  if (!ctx || !u || !y) return RBC3D_ERR_ARG;
  int n = ctx->wall.ndof;
  DBuf<double> du, dy, fsave;
  CUDA_TRY(du.upload(u, n, ctx->st));
  CUDA_TRY(dy.alloc(n));
  // MyMatMult overwrites the wall density; keep the caller's density intact
  size_t nf = 3 * (size_t)ctx->wall.nvert;
  CUDA_TRY(fsave.alloc(nf));
  CUDA_TRY(cudaMemcpyAsync(fsave.p, ctx->wall.f.p, sizeof(double) * nf, cudaMemcpyDeviceToDevice, ctx->st));
  rbc3d_status s = wall_matmult_dev(ctx, prec, du.p, dy.p);
  CUDA_TRY(cudaMemcpyAsync(ctx->wall.f.p, fsave.p, sizeof(double) * nf, cudaMemcpyDeviceToDevice, ctx->st));
  if (s) return s;
  CUDA_TRY(cudaMemcpyAsync(y, dy.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st));
  CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return RBC3D_OK;
}

rbc3d_status rbc3d_no_slip_wall(rbc3d_ctx* ctx, const rbc3d_solve_opts* opt, const double* guess,
                                rbc3d_solve_stats* st) {
  if (!ctx || !opt || opt->guess < 0 || opt->guess > 5 || (opt->guess > 0 && opt->guess < 4 && !guess) ||
      opt->rtol < 0 || opt->max_it < 0 || !valid_prec(opt->prec))
    return RBC3D_ERR_ARG;
  if (opt->guess >= 4 && !ctx->wspec.ready) return ctx_fail(ctx, RBC3D_ERR_STATE, "wall spectral model not initialised");
  return wall_solve(ctx, opt, guess, st);
}

rbc3d_status rbc3d_get_counts(const rbc3d_ctx* ctx, rbc3d_counts* out) {
  if (!ctx || !out) return RBC3D_ERR_ARG;
  *out = ctx->counts;
  out->kernel_launches = ctx->launches;
  return RBC3D_OK;
}

rbc3d_status rbc3d_host_alloc(unsigned long long bytes, void** out) {
  if (!out) return RBC3D_ERR_ARG;
  return cudaMallocHost(out, bytes) == cudaSuccess ? RBC3D_OK : RBC3D_ERR_NOMEM;
}
rbc3d_status rbc3d_host_free(void* p) { return cudaFreeHost(p) == cudaSuccess ? RBC3D_OK : RBC3D_ERR_CUDA; }

rbc3d_status rbc3d_fma_peak(int prec, double* tflops) {
  if (!tflops) return RBC3D_ERR_ARG;
  return fma_peak(prec, tflops);
}

rbc3d_status rbc3d_h2d_bandwidth(unsigned long long bytes, double* gbs) {
  if (!gbs || bytes == 0) return RBC3D_ERR_ARG;
  void* h = nullptr;
  void* d = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  rbc3d_status s = RBC3D_OK;
  float best = 0.f;
  if (cudaMallocHost(&h, bytes) != cudaSuccess || cudaMalloc(&d, bytes) != cudaSuccess ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess || cudaMemsetAsync(d, 0, bytes, st) != cudaSuccess) {
    s = RBC3D_ERR_NOMEM;
  } else {
    std::memset(h, 0, bytes);
    for (int it = 0; it < 4 && !s; ++it) {
      float ms = 0.f;
      if (cudaEventRecord(e0, st) != cudaSuccess ||
          cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
          cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        s = RBC3D_ERR_CUDA;
      else if (it > 0 && (best == 0.f || ms < best))
        best = ms;
    }
  }
  if (!s) *gbs = best > 0.f ? (double)bytes / (best * 1e-3) / 1e9 : 0.0;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (d) cudaFree(d);
  if (h) cudaFreeHost(h);
  return s;
}

}  // extern "C"
