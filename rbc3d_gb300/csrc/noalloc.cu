// noalloc.cu -- allocation-free variant of the linear double-layer term
// (AddLinearInt) for callers that must not allocate device memory.
//
// Who needs it: host programs whose device memory is owned by someone else
// -- a Fortran time integrator that keeps every array in an OpenACC or CUDA
// Fortran data region, or an application whose memory pool forbids foreign
// allocations -- and code that runs in a loop where cudaMalloc / cudaFree
// would synchronise the whole device every call.  Such a caller hands over
// device pointers for all inputs and outputs; the only scratch this entry
// point needs (per-cell moments and their total) lives in a fixed array
// compiled into the library.
//
// Scratch: RBC3D_NOALLOC_MAX_CELLS x 3 doubles of per-cell moments (8192
// cells, 192 KiB) followed by one 3-double slot for their sum, a file-scope
// __device__ array.  Every GPU that loads the library keeps it until the
// process exits.  Each call overwrites the slots of its ncell cells and the
// sum slot before reading them, so nothing has to be zeroed between calls;
// two calls that run at the same time on the GPU (different streams or host
// threads) share the array and race.
//
// Cell types come from caller-owned device memory and cannot be checked on
// the host: a cell whose type lies outside [0, ncelltypes) contributes
// nothing (its Bcoef is taken as 0).
#include <algorithm>
#include <climits>

#include "ctx.hpp"

#define RBC3D_NOALLOC_MAX_CELLS 8192
#define RBC3D_NOALLOC_SUM_SLOT (RBC3D_NOALLOC_MAX_CELLS * 3)

static __device__ __align__(256) double g_cell_moment[RBC3D_NOALLOC_MAX_CELLS * 3 + 4];

namespace {

constexpr int kReduceThreads = 256;

struct LinArgs {
  int ncell, nv, nlat, ncelltypes;
  long long npt;
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
  const size_t npt = (size_t)a.npt;
  for (int r = threadIdx.x; r < a.nv; r += blockDim.x) {
    size_t p = base + r;
    int ilat = r % a.nlat;
    double ds = a.w[ilat] * a.detJ[p];
    double vn = a.g[p] * a.a3[p] + a.g[p + npt] * a.a3[p + npt] + a.g[p + 2 * npt] * a.a3[p + 2 * npt];
    for (int k = 0; k < 3; ++k) s[k] += a.x[p + k * npt] * vn * ds;
  }
  __shared__ double red[3][8];
  for (int k = 0; k < 3; ++k) {
    double t = warp_sum(s[k]);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int ct = a.celltype[cell];
    // A type outside the valid range contributes nothing (no read past B).
    double B = 0.0;
    for (int l = 0; l < a.ncelltypes; ++l)
      if (l == ct) B = a.B[l];
    for (int k = 0; k < 3; ++k) {
      double t = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[k][i];
      a.moment[3 * cell + k] = B * t;
    }
  }
}

// One block: the sum of the per-cell moments into the sum slot.  Each thread
// adds a fixed strided subset in cell order, then a fixed-shape tree, so the
// result does not depend on timing.
__global__ void __launch_bounds__(kReduceThreads) k_moment_total(int ncell, double* __restrict__ moment,
                                                                 double scale) {
  __shared__ double red[3][kReduceThreads];
  double s[3] = {0, 0, 0};
  for (int c = threadIdx.x; c < ncell; c += kReduceThreads)
    for (int k = 0; k < 3; ++k) s[k] += moment[3 * c + k];
  for (int k = 0; k < 3; ++k) red[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int h = kReduceThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 3) moment[RBC3D_NOALLOC_SUM_SLOT + threadIdx.x] = scale * red[threadIdx.x][0];
}

// Adds c2 * xvint / Acoef to every target (ModIntOnRbcs.F90:187-198).
__global__ void __launch_bounds__(256) k_apply_linear(const double* __restrict__ moment, int nt,
                                                      const double* __restrict__ Acoef, double* __restrict__ v) {
  const double xv0 = moment[RBC3D_NOALLOC_SUM_SLOT], xv1 = moment[RBC3D_NOALLOC_SUM_SLOT + 1],
               xv2 = moment[RBC3D_NOALLOC_SUM_SLOT + 2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
    double iA = 1.0 / Acoef[i];
    v[i] += xv0 * iA;
    v[i + (size_t)nt] += xv1 * iA;
    v[i + 2 * (size_t)nt] += xv2 * iA;
  }
}

// Device address of the scratch array on the current device.  Host code
// cannot use the symbol itself as a pointer (in host code it names a
// host-side stand-in); the lookup is repeated on every call so that it stays
// valid after the device's context has been torn down and recreated.
rbc3d_status scratch_address(double** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_cell_moment) != cudaSuccess || !p) return RBC3D_ERR_CUDA;
  *out = (double*)p;
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
  const long long nv = (long long)nlat * nlon;
  const long long npt = nv * ncell;
  if (nv > INT_MAX || npt > INT_MAX) return RBC3D_ERR_ARG;  // point indices are 32-bit in the kernels
  if (ncell == 0 || nt == 0 || c2 == 0.0) return RBC3D_OK;
  if (!x || !g || !a3 || !detJ || !w || !celltype || !Acoef || !v) return RBC3D_ERR_ARG;
  double* moment = nullptr;
  rbc3d_status s = scratch_address(&moment);
  if (s) return s;
  LinArgs a;
  a.ncell = ncell; a.nlat = nlat; a.nv = (int)nv; a.npt = npt; a.ncelltypes = ncelltypes;
  a.x = x; a.g = g; a.a3 = a3; a.detJ = detJ; a.w = w; a.celltype = celltype; a.moment = moment;
  for (int l = 0; l < RBC3D_MAX_CELLTYPES; ++l) a.B[l] = 0.;
  for (int l = 0; l < ncelltypes; ++l) a.B[l] = viscRat[l] > 0 ? 1. - viscRat[l] : -1.;  // initCOEFs
  cudaStream_t st = (cudaStream_t)stream;
  k_cell_moment<<<ncell, 256, 0, st>>>(a);
  const double scale = c2 * (-8 * RBC3D_PI) / (Lb[0] * Lb[1] * Lb[2]);
  k_moment_total<<<1, kReduceThreads, 0, st>>>(ncell, moment, scale);
  k_apply_linear<<<std::min(152 * 4, (nt + 255) / 256), 256, 0, st>>>(moment, nt, Acoef, v);
  return cudaGetLastError() == cudaSuccess ? RBC3D_OK : RBC3D_ERR_CUDA;
}
