// peak.cu -- FMA-throughput microbenchmark used as the roofline denominator of
// the CUDA-core-bound kernels (FP32 pair sums, FP64 corrections).
#include <chrono>

#include "ctx.hpp"

namespace {

// 8 independent FMA chains per thread, ITER iterations: 16*ITER flops/thread.
template <typename R, int ITER>
__global__ void __launch_bounds__(256) k_fma(R* out, R a, R b) {
  R x0 = (R)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 16
  for (int i = 0; i < ITER; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  R s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (R)-12345.678) out[0] = s;  // keeps the chains live
}

template <typename R, int ITER>
double run(int nsm) {
  R* out = nullptr;
  if (cudaMalloc(&out, sizeof(R))) return -1;
  int blocks = nsm * 8;
  k_fma<R, ITER><<<blocks, 256>>>(out, (R)0.999999, (R)1e-7);  // warm-up
  cudaDeviceSynchronize();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  cudaEventRecord(e0);
  const int REP = 5;
  for (int r = 0; r < REP; ++r) k_fma<R, ITER><<<blocks, 256>>>(out, (R)0.999999, (R)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  cudaError_t err = cudaGetLastError();
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0) return -1;
  double flops = 16.0 * ITER * 256.0 * blocks * REP;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

rbc3d_status fma_peak(int prec, double* tflops) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  double t = (prec == RBC3D_FP64) ? run<double, 4096>(nsm) : run<float, 65536>(nsm);
  if (t <= 0) return RBC3D_ERR_CUDA;
  *tflops = t;
  return RBC3D_OK;
}
