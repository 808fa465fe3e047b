// ctx.hpp -- device-resident state of one rbc3d context (one CUDA stream).
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>

#include <string>
#include <vector>

#include "../../include/rbc3d_gpu.h"
#include "common.cuh"

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t upload(const T* h, size_t count, cudaStream_t s) {
    cudaError_t e = alloc(count);
    if (e) return e;
    return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
  }
  ~DBuf() { release(); }
};

// Uniform cell list over the periodic box (HashTable_ComputeNumBlocks,
// ModHashTable.F90:99-126, single rank): Nc = max(floor(L/rc), 3) per axis.
struct HashGrid {
  int Nc[3] = {0, 0, 0};
  double h[3] = {0, 0, 0};
  double L[3] = {0, 0, 0};
  int ncells = 0;
};

// One target list (t_TargetList) on the device, sorted by cell-list cell.
struct TargetSet {
  int n = 0;
  DBuf<double> x;       // 3n, FP64 SoA
  DBuf<double> Acoef;   // n
  DBuf<int4> meta;      // (surf, ilat, ilon, 0); surf 1-based, -1 for raw
  DBuf<int> order;      // sorted position -> target index
  DBuf<int> cstart, cend;
  DBuf<int4> units;     // (hash cell, first sorted position, count, 0): up to TILE targets (FP64 pair sums)
  int nunits = 0;
  DBuf<int4> wunits;    // the same with up to 32 targets, one per warp (FP32 pair sums)
  int nwunits = 0;
  bool sorted = false;
  DBuf<double> v;       // 3n accumulator of the current matvec
  DBuf<double> v2;      // 3n accumulator of the stages on the side stream
};

// exchange the buffers of two DBufs (no copy, no free)
template <class T>
inline void dbuf_swap(DBuf<T>& a, DBuf<T>& b) {
  T* p = a.p; size_t n = a.n;
  a.p = b.p; a.n = b.n;
  b.p = p; b.n = n;
}

// Sources binned by the PME grid tile that holds their B-spline stencil's
// origin: perm lists source indices tile by tile, chunk = (tile, begin, end)
// with at most SPREAD_CHUNK sources per chunk.
struct SpreadPlan {
  DBuf<int> perm;
  DBuf<int4> chunk;
  int n = 0, nchunk = 0;
  bool valid = false;
};

struct PmeState {
  SpreadPlan cplan, wplan;  // cell and wall sources
  DBuf<int2> sched;         // stencil-node schedule of the tiled spread
  int sched_P = 0;
  int N1 = 0, N2 = 0, N3 = 0, NH = 0;
  size_t G = 0, GC = 0;
  DBuf<float> grid32;      // 12*G real grids
  DBuf<double> grid64;
  DBuf<float2> spec32;     // 12*GC spectra
  DBuf<double2> spec64;
  DBuf<float2> vspec32;    // 3*GC
  DBuf<double2> vspec64;
  DBuf<float> vel32;       // 3*G velocity grid
  DBuf<double> vel64;
  DBuf<double> bbx, bby, bbz;
  cufftHandle r2c32_3 = 0, r2c32_12 = 0, c2r32_3 = 0;
  cufftHandle r2c64_3 = 0, r2c64_12 = 0, c2r64_3 = 0;
  bool planned32 = false, planned64 = false;
  bool sl = false, dl = false;
  int prec = RBC3D_FP64;
  bool ready = false;  // velocity grid valid
};

struct WallState {
  int nvert = 0, nele = 0, ndof = 0;
  std::vector<double> hx, hf;       // host copies (x, density)
  std::vector<int> he2v, hglb;
  DBuf<double> x, f, area, eps, cen;  // vertices 3*nvert, density 3*nvert, per element
  DBuf<double> src_x, src_f;          // PME centroid sources (3*nele)
  DBuf<int> e2v;                      // 3*nele (0-based)
  DBuf<int> glb;                      // nvert (0-based unique id)
  DBuf<int> writer;                   // 1 for the last vertex of each unique id (AssembleArray order)
  DBuf<int> order, cstart, cend;      // centroid cell list
  bool prepared = false;
  DBuf<int> rowptr, col;              // self-wall CSR (3nvert x 3nvert)
  DBuf<double> val;
  long long nnz = 0;
};

// Learned spectral operator of the wall solve (wallspec.cu): for a wall that
// is a uniform stack of nring rings of nper vertices along z, per axial
// Fourier mode an orthonormal basis Q of the transformed right-hand sides of
// past solves and the matching transformed solutions Z (A_m Z = Q), so that
// x_m = Z Q^H b_m predicts the solution of a new right-hand side.
struct WallSpec {
  bool ready = false, record = false;
  int nring = 0, dim = 0, nm = 0, kmax = 0;  // dim = 3 nper, nm = nring / 2 + 1
  double tau = 1e-7;                        // basis growth threshold (relative to the mode's norm)
  cufftHandle d2z = 0, z2d = 0;
  DBuf<double2> Q, Z;                       // [mode][kmax][dim]
  DBuf<int> nb;                             // basis size per mode
  DBuf<double2> bh, xh, rh;                 // transformed vectors [mode][dim]
  DBuf<double> tmp, fin;                    // 2 ndof host-call staging; ndof transform input
  DBuf<int> added;                          // per mode, last add
  long long pairs = 0;
};

// Spherical-harmonic transform tables of the cell grid at degree < L
// (cellsolve.cu): Gauss and equiangular pbar rows, the meridian FFT_Diff of
// the equiangular rows, weights, cos / sin(m phi); kept across calls until
// the grid or L changes.
struct ShTabs {
  int L = 0;
  bool equi_lon = false;  // phi equispaced over an even nlon (FFT_Diff's axis)
  DBuf<double> PG, PE, dPE, wf, cs, sn;
};

struct rbc3d_ctx {
  rbc3d_params prm{};
  double iLb[3]{};
  double Acoef[RBC3D_MAX_CELLTYPES]{}, Bcoef[RBC3D_MAX_CELLTYPES]{};
  std::string err;
  cudaStream_t st = nullptr;   // main stream (highest priority)
  cudaStream_t st2 = nullptr;  // matvec side stream: self patch and PME next to the pair sums
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // set_cells_x / set_cell_density_x build the spline tables on the side
  // stream and return; readers on the main stream wait on ev_spl (spl_wait)
  cudaEvent_t ev_spl = nullptr, ev_up = nullptr, ev_geom = nullptr;
  cudaEvent_t ev_dens = nullptr;  // after the side stream's last reads of f and g
  bool spl_pending = false, dens_pending = false;
  int device = 0;

  // Ewald / mask tables
  Tables T{};
  DBuf<double> t_sl1, t_sl2, t_dl, t_mask;
  DBuf<float4> t_sl32;
  DBuf<float2> t_dl32, t_mask32;

  HashGrid hg;

  // cell surface grid and polar patch
  int nlat = 0, nlon = 0, m = 0;  // m = 2*nlat spline rows
  std::vector<double> h_th, h_phi, h_w;
  DBuf<double> th, phi, w;
  DBuf<float4> usph;              // unit-sphere coordinates per grid point (FP32)
  int nrad = 0, nazm = 0;
  double radius = 0;
  DBuf<double> pw, thG, phiA;     // patch weights (nrad); thG/phiA [ilat0][q]
  DBuf<double> rd_s, rd_w;        // GauLeg(-1,1,16) for RBC_NearSingInt_ReAdd
  DBuf<double> rd_x0, rd_w0;      // GauLeg(0,radius,16)

  // cells
  int ncell = 0, npt = 0;
  std::vector<int> h_celltype;
  DBuf<int> celltype;
  DBuf<double> x, a3, detJ, f, g, sf, sg, area, meshSize;
  DBuf<double> spl;               // ncell * SPL_NSET * m*nlon * SPL_NODE
  DBuf<double> tan1, tan2;        // set_cells_x: the tangents dx/dtheta, dx/dphi (point layout)
  bool has_f = false, has_g = false;
  double near_rthr = 0;            // 0.5 * min(meshSize): FP32C cross-surface pairs below it go to FP64
  bool rthr_pending = false;       // set_cells_x: near_rthr still on its way from the device
  double* h_rthr = nullptr;        // its pinned landing slot
  cudaEvent_t ev_rthr = nullptr;   // recorded after the copy into h_rthr
  DBuf<double> rthr_dev;

  // sorted sources (cell surface points)
  DBuf<int> s_order, s_cstart, s_cend;
  DBuf<double> s_x, s_f, s_g, s_a3;  // sorted, SoA 3*npt; s_g carries Bcoef
  DBuf<int4> s_meta;                 // (surf, ilat, ilon, original index)
  // FP32 pair-sum records of the sorted sources: hi/lo coordinates relative
  // to the source's hash-cell centre (+ surf / id bits), unit-sphere point,
  // a3; c1 f and c2 g of the current call; per-cell tile offsets and boxes
  DBuf<float4> s_p0, s_p1, s_u4, s_a4, s_F4, s_G4;
  DBuf<int> s_toff, s_coff;
  DBuf<float4> s_tbox, s_cbox;  // per 128-source tile and per 32-source chunk
  DBuf<float4> s_op0, s_op1;    // own-cell pair records in point order (k_pair_own32)
  DBuf<int> s_inv;              // point -> sorted source position
  int s_ntiles = 0;
  DBuf<unsigned long long> near_queue;  // work counter of the near-singular kernel
  DBuf<double> dBcoef;                  // Bcoef per cell type on the device
  DBuf<char> self_w64;                  // FP64 patch weights per (latitude, patch point)
  DBuf<double> mtab64;                  // same-cell mask per (latitude, latitude, longitude gap)
  DBuf<float> mtab32;                   // 1 - mask, FP32
  DBuf<int> near_l1, near_l2;           // near-singular candidates after the screen / the FP32 replay
  DBuf<float> rep_rec;                  // the FP32 replay's node values: x and a3, 4 slots each (24 floats a node)
  DBuf<double> near_plan, near_part;    // the staged near pass: per-item plans, per-quadrature warp sums
  bool rep_valid = false;               // rep_rec matches the current geometry
  float erfcx_q[16] = {0};   // FP32 erfc fit of the pair kernel
  double erfcx_X = -1.0;
  bool src_sorted = false, src_density = false;

  TargetSet tl[3];

  // near-singular work list
  DBuf<int4> items;               // (target, surf, ilat, ilon)
  int items_cap = 0;
  DBuf<unsigned long long> dcnt;  // device counters: [0] items, [1] pairs, [2] overflow targets, [3] nearsing, [4] wall pairs, [5] duffy, [6] screen misses
  DBuf<double> xvint;             // linear-term reduction (3)

  PmeState pme;
  WallState wall;
  WallSpec wspec;

  // FP32M self patch: FP32 node records, per-(latitude, patch point) weights,
  // target positions relative to the cell centre (hi/lo)
  DBuf<float> mix_rec, mix_pw;
  DBuf<char> mix_w;
  DBuf<float4> mix_thi, mix_tlo;
  int mix_sets = 0;  // current FP32M node-record parts: bit 0 geometry, 1 f, 2 g
  bool phi_uniform = false;

  // FP32D self patch: float-float node records [cell][slot x quad][node tile][hi, lo],
  // the patch weights of k_self as hi/lo planes, pw and the Ewald tables as
  // hi/lo; ff_sets: which record sets (bit 0 x, 1 f, 2 g, 3 a3) are current
  DBuf<int2> ff_widx;
  DBuf<float4> ff_rec, ff_w, ff_tab;
  DBuf<float2> ff_pw;
  DBuf<unsigned> ff_bnd;  // [set][cell][slot]: max |value| (float bits) for the sums' offsets
  int ff_sets = 0;
  DBuf<short> ff_perm;    // [latitude][k]: lane order of the patch points

  // membrane mechanics (membrane.cu): transform tables of the degree < nlat
  // expansion and the reference cells' a_rcp and b, [type][4][nv]
  struct MbState {
    int L = 0;
    DBuf<double> P, DP, wf, cs, sn, sinth;
    int nref = 0;
    DBuf<double> ref_ar, ref_b;
    std::vector<double> ES, ED, EB;
    int excl_nv = 0;
    DBuf<unsigned char> excl;  // repulsion: grid pairs within the patch radius on the reference sphere
  } mb;

  ShTabs shtab;                   // transform tables of the cell solve and the device surface sources
  DBuf<double> scratch;           // GMRES basis / temporaries
  DBuf<double> dotpart;           // GMRES: per-slice partial dot products
  DBuf<double> stage;             // staging of uploaded spline tables (grow-only)
  // grow-only temporaries of the set-up passes (cudaFree would synchronise the device)
  DBuf<int> sort_key, sort_key2, sort_idx;  // sort_points
  DBuf<char> scan_tmp;                      // device list builders: scan storage
  DBuf<int> unit_cnt, unit_off, unit_idx, unit_zero;  // work units: per-cell counts, offsets, sort indices
  DBuf<long long> unit_key;                 // work units: work keys (before and after the sort)
  DBuf<int4> unit_tmp;                      // work units before the sort
  DBuf<char> sort_tmp;
  DBuf<int2> list_tmp;                      // build_source_list: tile / chunk lists
  DBuf<int> plan_key, plan_key2, plan_idx;  // build_spread_plan (may run on the side stream)
  DBuf<char> plan_tmp, plan_scan;
  DBuf<int> plan_ts, plan_te, plan_cnt, plan_off;  // build_spread_plan: tile ranges, chunk counts and offsets
  DBuf<double> vadd;                        // finish_add: the caller's accumulator on the device
  DBuf<double> acoef_dev, mix_xc; // Acoef per cell type; FP32M cell centres
  rbc3d_counts counts{};

  // stage timers: event pairs recorded around each stage, read on demand
  bool prof = false;
  bool verify_screen = false;  // RBC3D_VERIFY_SCREEN=1: check near-singular screens in FP64
  int near_stage_cap = NEAR_STAGE_CAP;  // RBC3D_NEAR_STAGE_CAP: list entries of the staged near pass
  long long launches = 0;  // kernels of this library launched on the context
  std::vector<cudaEvent_t> evpool;
  std::vector<int> rec_stage;
  size_t nrec = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
};

// RAII stage timer (records nothing when profiling is off)
struct StageScope {
  rbc3d_ctx* c;
  int slot;
  StageScope(rbc3d_ctx* ctx, int stage);
  ~StageScope();
};

rbc3d_status ctx_fail(rbc3d_ctx* ctx, int code, const std::string& msg);
rbc3d_status ctx_fail_cuda(rbc3d_ctx* ctx, cudaError_t e, const char* what);

// pair.cu
rbc3d_status build_source_list(rbc3d_ctx* ctx, bool with_normals = true);
rbc3d_status source_normals(rbc3d_ctx* ctx);
// selfff.cu: the float-float node records of the sets in `need` (bit 0 x,
// 1 f, 2 g, 3 a3) that are out of date, on the current stream
rbc3d_status self_ff_records(rbc3d_ctx* ctx, int need);
rbc3d_status sort_points_by_cell(rbc3d_ctx* ctx, int n, const double* x_dev, DBuf<int>& order, DBuf<int>& cs,
                                DBuf<int>& ce);
rbc3d_status matvec_dev(rbc3d_ctx* ctx, int which, double c1, double c2, unsigned terms, int prec);
rbc3d_status build_source_density(rbc3d_ctx* ctx);
rbc3d_status sort_targets(rbc3d_ctx* ctx, int tlist);
rbc3d_status pme_prepare_cells(rbc3d_ctx* ctx);
rbc3d_status run_pair_sum(rbc3d_ctx* ctx, int tlist, double c1, double c2, int prec, bool collect_nbr);
rbc3d_status run_linear(rbc3d_ctx* ctx, int tlist, double c2);
// corr.cu
rbc3d_status run_self_corr(rbc3d_ctx* ctx, int tlist, double c1, double c2);
rbc3d_status run_near_corr(rbc3d_ctx* ctx, int tlist, double c1, double c2, int prec);
// pme.cu
rbc3d_status pme_setup(rbc3d_ctx* ctx);
rbc3d_status pme_release(rbc3d_ctx* ctx);
rbc3d_status pme_spread(rbc3d_ctx* ctx, double c1, double c2, int cells, int walls, int prec);
// FP32 erfc of the pair and self kernels: erfc(x) = exp(-x^2) t Q(t),
// t = 1/(1 + x/2), Q of degree ERFCX_DEG fitted on [0, rc sqrt(pi/alpha)]
constexpr int ERFCX_DEG = 8;
void fit_erfcx(double X, float* q);
void erfcx_coeffs(rbc3d_ctx* ctx);  // fills ctx->erfcx_q for the context's rc, alpha
rbc3d_status pme_transform(rbc3d_ctx* ctx);
rbc3d_status pme_gather(rbc3d_ctx* ctx, int tlist);
// walls.cu
rbc3d_status wall_setup(rbc3d_ctx* ctx);
rbc3d_status wall_prepare_self(rbc3d_ctx* ctx);
rbc3d_status run_wall_quad(rbc3d_ctx* ctx, int tlist, double c1, int prec);
rbc3d_status run_wall_self(rbc3d_ctx* ctx, double c1);
rbc3d_status wall_solve(rbc3d_ctx* ctx, const rbc3d_solve_opts* opt, const double* guess, rbc3d_solve_stats* st);
rbc3d_status wall_matmult_dev(rbc3d_ctx* ctx, int prec, const double* u_dev, double* y_dev);
rbc3d_status wall_residual_dev(rbc3d_ctx* ctx, int prec);
// wallspec.cu
rbc3d_status wall_spec_predict_dev(rbc3d_ctx* ctx, const double* b_dev, double* x0_dev, double* rem_dev);
rbc3d_status wall_spec_add_dev(rbc3d_ctx* ctx, const double* b_dev, const double* x_dev);
rbc3d_status wall_spec_apply_dev(rbc3d_ctx* ctx, const double* v_dev, double* out_dev);
void wall_spec_release(rbc3d_ctx* ctx);

// selfmix.cu
rbc3d_status self_mixed_grid(rbc3d_ctx* ctx, const std::vector<double>& thG, const std::vector<double>& phiA,
                             const std::vector<double>& pw);
rbc3d_status self_mixed_geom(rbc3d_ctx* ctx);
rbc3d_status self_mixed_density(rbc3d_ctx* ctx, bool f, bool g);
rbc3d_status run_self_mixed(rbc3d_ctx* ctx, int tlist, double c1, double c2);
rbc3d_status self_ff_tables(rbc3d_ctx* ctx, const std::vector<double>& c1, const std::vector<double>& c2,
                            const std::vector<double>& dl);
rbc3d_status self_ff_grid(rbc3d_ctx* ctx, const std::vector<SelfW64>& W, const std::vector<double>& pw);
void self_ff_invalidate(rbc3d_ctx* ctx, bool geom, bool f, bool g);
rbc3d_status run_self_ff(rbc3d_ctx* ctx, int tlist, double c1, double c2);
inline bool valid_prec(int p) {
  return p == RBC3D_FP64 || p == RBC3D_FP32C || p == RBC3D_FP32M || p == RBC3D_FP32D;
}
// mixed-precision solves: relative residual reduction asked of each inner
// FP32 GMRES solve (well above the FP32 operators' ~3e-7 relative error)
constexpr double RBC3D_IR_ETA = 1e-5;

// cellsolve.cu: Spherepack pbar(m, n, theta), P[m*L + n] for 0 <= m <= n < L
void pbar_table(int L, double theta, double* P);
// Rbc_BuildSurfaceSource on the device from the context's point fields:
// geom -> the x, a3 and detJ tables, f / g -> the f detJ / g detJ tables
rbc3d_status surface_sources_dev(rbc3d_ctx* ctx, int nlat0, bool geom, bool f, bool g);
// membrane.cu: RBC_ComputeGeometry of the context's cells from ctx->x
// (device): a3, detJ (point layout) and area into the context's arrays,
// queued on the context stream
rbc3d_status cells_geometry_dev(rbc3d_ctx* ctx);
// api.cu: near_rthr once its device value has landed (set_cells_x computes it
// on the device); the current stream waits for spline tables still being
// built on the side stream
double near_rthr_now(rbc3d_ctx* ctx);
void spl_wait(rbc3d_ctx* ctx);

// peak.cu
rbc3d_status fma_peak(int prec, double* tflops);

// shared host helper: GauLeg of ModQuadRule.F90:135-214
void host_gauleg(double x1, double x2, int n, double* x, double* w);
