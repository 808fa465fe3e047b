// noalloc.cu -- allocation-free variant of the linear double-layer term
// (AddLinearInt) for callers that must not allocate device memory.
//
// Who needs it: host programs whose device memory is owned by someone else
// -- a Fortran time integrator that keeps every array in an OpenACC or CUDA
// Fortran data region, or an application whose memory pool forbids foreign
// allocations -- and code that runs in a loop where cudaMalloc / cudaFree
// would synchronise the whole device every call.  Such a caller hands over
// device pointers for all inputs and outputs; the only scratch this entry
// point needs (per-cell moments) lives in a fixed array compiled into the
// library.
//
// Scratch: RBC3D_NOALLOC_MAX_CELLS x 3 doubles (8192 cells, 192 KiB), a
// file-scope __device__ array.  Every GPU that loads the library keeps it
// until the process exits.  Each call overwrites the slots of its ncell
// cells before reading them, so nothing has to be zeroed between calls; two
// calls that run at the same time on the GPU (different streams or host
// threads) share the array and race.
#include <algorithm>
#include <mutex>

#include "ctx.hpp"

#define RBC3D_NOALLOC_MAX_CELLS 8192

static __device__ __align__(256) double g_cell_moment[RBC3D_NOALLOC_MAX_CELLS * 3];

namespace {

struct LinArgs {
  int ncell, nv, nlat, npt;
  const double* x;
  const double* g;
  const double* a3;
  const double* detJ;
  const double* w;
  const int* celltype;
  double B[RBC3D_MAX_CELLTYPES];
  double* moment;  // device address of g_cell_moment
};

// One block per cell: sum over its points of Bcoef * x * (g.a3) * detJ * w,
// the integrand of AddLinearInt (ModIntOnRbcs.F90:173-185).
__global__ void __launch_bounds__(256) k_cell_moment(LinArgs a) {
  const int cell = blockIdx.x;
  double s[3] = {0, 0, 0};
  const size_t base = (size_t)cell * a.nv;
  for (int r = threadIdx.x; r < a.nv; r += blockDim.x) {
    size_t p = base + r;
    int ilat = r % a.nlat;
    double ds = a.w[ilat] * a.detJ[p];
    double vn = a.g[p] * a.a3[p] + a.g[p + a.npt] * a.a3[p + a.npt] + a.g[p + 2 * (size_t)a.npt] * a.a3[p + 2 * (size_t)a.npt];
    for (int k = 0; k < 3; ++k) s[k] += a.x[p + (size_t)k * a.npt] * vn * ds;
  }
  __shared__ double red[3][8];
  for (int k = 0; k < 3; ++k) {
    double t = warp_sum(s[k]);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double B = a.B[a.celltype[cell]];
    for (int k = 0; k < 3; ++k) {
      double t = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[k][i];
      a.moment[3 * cell + k] = B * t;
    }
  }
}

// Every block sums the per-cell moments in cell order (deterministic), then
// adds c2 * xvint / Acoef to its share of the targets (ModIntOnRbcs.F90:187-198).
__global__ void __launch_bounds__(256) k_apply_linear(int ncell, const double* __restrict__ moment, double scale,
                                                      int nt, const double* __restrict__ Acoef, double* __restrict__ v) {
  __shared__ double xv[3];
  if (threadIdx.x < 3) {
    double t = 0;
    for (int c = 0; c < ncell; ++c) t += moment[3 * c + threadIdx.x];
    xv[threadIdx.x] = scale * t;
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
    double iA = 1.0 / Acoef[i];
    for (int k = 0; k < 3; ++k) v[i + (size_t)k * nt] += xv[k] * iA;
  }
}

// Device address of the scratch array, resolved once per device with that
// device current (host code cannot use the symbol itself as a pointer).
std::mutex g_mu;
void* g_addr[64] = {};

rbc3d_status scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RBC3D_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_cell_moment) != cudaSuccess || !p) return RBC3D_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = (double*)g_addr[dev];
  return RBC3D_OK;
}

}  // namespace

extern "C" rbc3d_status rbc3d_add_linear_int_noalloc(int ncell, int nlat, int nlon, const double* x, const double* g,
                                                     const double* a3, const double* detJ, const double* w,
                                                     const int* celltype, int ncelltypes, const double* viscRat,
                                                     const double Lb[3], double c2, int nt, const double* Acoef,
                                                     double* v, void* stream) {
  if (ncell < 0 || ncell > RBC3D_NOALLOC_MAX_CELLS) return RBC3D_ERR_ARG;  // scratch holds 8192 cells
  if (nlat < 1 || nlon < 1 || nt < 0 || ncelltypes < 1 || ncelltypes > RBC3D_MAX_CELLTYPES || !viscRat || !Lb)
    return RBC3D_ERR_ARG;
  if (ncell == 0 || nt == 0 || c2 == 0.0) return RBC3D_OK;
  if (!x || !g || !a3 || !detJ || !w || !celltype || !Acoef || !v) return RBC3D_ERR_ARG;
  double* moment = nullptr;
  rbc3d_status s = scratch_address(&moment);
  if (s) return s;
  LinArgs a;
  a.ncell = ncell; a.nlat = nlat; a.nv = nlat * nlon; a.npt = ncell * nlat * nlon;
  a.x = x; a.g = g; a.a3 = a3; a.detJ = detJ; a.w = w; a.celltype = celltype; a.moment = moment;
  for (int l = 0; l < RBC3D_MAX_CELLTYPES; ++l) a.B[l] = 0.;
  for (int l = 0; l < ncelltypes; ++l) a.B[l] = viscRat[l] > 0 ? 1. - viscRat[l] : -1.;  // initCOEFs
  cudaStream_t st = (cudaStream_t)stream;
  k_cell_moment<<<ncell, 256, 0, st>>>(a);
  double scale = c2 * (-8 * RBC3D_PI) / (Lb[0] * Lb[1] * Lb[2]);
  k_apply_linear<<<std::min(152 * 4, (nt + 255) / 256), 256, 0, st>>>(ncell, moment, scale, nt, Acoef, v);
  return cudaGetLastError() == cudaSuccess ? RBC3D_OK : RBC3D_ERR_CUDA;
}
