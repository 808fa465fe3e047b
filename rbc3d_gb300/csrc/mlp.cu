// mlp.cu -- the MLP of the learned wall-density initial guess: forward,
// backward and Adam on the GPU.  No counterpart in the reference.
//
// Layers: nin -> width (SiLU) -> ... -> width (SiLU) -> nout, "depth" hidden
// layers.  GEMM operands are BF16 (inputs, activations, weights, gradients),
// products accumulate in FP32 on the tensor cores through
// mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32; master weights, Adam
// moments and the loss are FP32.  One tiled GEMM kernel (64x64x32 tiles, four
// warps of 32x32, operands staged in shared memory with generic strides so the
// same kernel serves x W^T, dz^T a and dz W) plus small element-wise kernels.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "ctx.hpp"

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

constexpr int BM = 64, BN = 64, BK = 32, PADK = BK + 8;

struct GemmArgs {
  int M, N, K;
  const __nv_bfloat16* A;  // element (m,k) at A[m*sam + k*sak]
  long long sam, sak;
  const __nv_bfloat16* B;  // element (k,n) at B[k*sbk + n*sbn]
  long long sbk, sbn;
  float* C;                // row-major M x N (ldc)
  int ldc;
  const float* bias;       // per column n (EPI 1, 2)
  __nv_bfloat16* Abf;      // EPI 1: SiLU(z) in BF16, row-major ldc
};

__device__ __forceinline__ unsigned pack2(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }

// EPI 0: C = A B;  EPI 1: z = A B + bias -> C, SiLU(z) -> Abf;  EPI 2: C = A B + bias
template <int EPI>
__global__ void __launch_bounds__(128) k_gemm(GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 As[BM][PADK];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][PADK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int gq = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    // stage A (BM x BK) and B^T (BN x BK), k contiguous in shared memory
    for (int e = tid; e < BM * BK; e += 128) {
      int r = e / BK, kk = e % BK;
      int m = m0 + r, k = k0 + kk;
      As[r][kk] = (m < g.M && k < g.K) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : zero;
      int n = n0 + r;
      Bs[r][kk] = (n < g.N && k < g.K) ? g.B[(long long)k * g.sbk + (long long)n * g.sbn] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      unsigned af[2][4], bf[4][2];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        int r = wm * 32 + mt * 16 + gq;
        af[mt][0] = pack2(&As[r][ks + 2 * tq]);
        af[mt][1] = pack2(&As[r + 8][ks + 2 * tq]);
        af[mt][2] = pack2(&As[r][ks + 2 * tq + 8]);
        af[mt][3] = pack2(&As[r + 8][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        int c = wn * 32 + nt * 8 + gq;
        bf[nt][0] = pack2(&Bs[c][ks + 2 * tq]);
        bf[nt][1] = pack2(&Bs[c][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bf[nt]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          int m = m0 + wm * 32 + mt * 16 + gq + 8 * h;
          int n = n0 + wn * 32 + nt * 8 + 2 * tq + q;
          if (m >= g.M || n >= g.N) continue;
          float v = acc[mt][nt][2 * h + q];
          if (EPI != 0) v += g.bias[n];
          g.C[(long long)m * g.ldc + n] = v;
          if (EPI == 1) g.Abf[(long long)m * g.ldc + n] = __float2bfloat16(silu(v));
        }
}

__global__ void k_to_bf16(long long n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// dy = 2 (y - t) / (n*nout); loss = mean (y - t)^2
__global__ void k_mse(long long n, const float* __restrict__ y, const float* __restrict__ t, float scale,
                      float* __restrict__ dy, __nv_bfloat16* __restrict__ dyb, float* loss) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  if (i < n) {
    float d = y[i] - t[i];
    e = d * d;
    dy[i] = 2.f * d * scale;
    dyb[i] = __float2bfloat16(2.f * d * scale);
  }
  e = warp_sumf(e);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, e * scale);
}

// dz = da * SiLU'(z)
__global__ void k_silu_back(long long n, const float* __restrict__ da, const float* __restrict__ z,
                            __nv_bfloat16* __restrict__ dzb) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 1.f / (1.f + expf(-z[i]));
  dzb[i] = __float2bfloat16(da[i] * s * (1.f + z[i] * (1.f - s)));
}

// column sums of a row-major rows x cols matrix (bias gradient)
__global__ void k_colsum(int rows, int cols, const __nv_bfloat16* __restrict__ dz, float* __restrict__ out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += __bfloat162float(dz[(long long)r * cols + c]);
  out[c] = s;
}

__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ wb) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
}

}  // namespace

struct rbc3d_mlp {
  int nin, width, depth, nout, nl;
  std::vector<int> din, dout;
  std::vector<size_t> woff, boff;  // offsets into the packed parameter vector
  size_t nparam = 0;
  DBuf<float> P, G, Mo, Vo;         // master weights, gradients, Adam moments
  DBuf<__nv_bfloat16> Wb;           // BF16 copy of the packed parameters
  int cap = 0;                      // rows the activation buffers hold
  std::vector<DBuf<float>> Z;       // pre-activations (f32), per layer
  std::vector<DBuf<__nv_bfloat16>> A;  // layer inputs (bf16), A[0] = x
  DBuf<float> X, T, Y, DY, DA, loss;
  DBuf<__nv_bfloat16> DZ, DZ2;
  long long step = 0;
  cudaStream_t st = nullptr;
  long long launches = 0;
};

namespace {

rbc3d_status mlp_ensure(rbc3d_mlp* m, int n) {
  if (n <= m->cap) return RBC3D_OK;
  m->cap = n;
  m->Z.resize(m->nl);
  m->A.resize(m->nl);
  for (int l = 0; l < m->nl; ++l) {
    if (m->Z[l].alloc((size_t)n * m->dout[l]) || m->A[l].alloc((size_t)n * m->din[l])) return RBC3D_ERR_NOMEM;
  }
  int wmax = std::max(m->width, std::max(m->nin, m->nout));
  if (m->X.alloc((size_t)n * m->nin) || m->T.alloc((size_t)n * m->nout) || m->Y.alloc((size_t)n * m->nout) ||
      m->DY.alloc((size_t)n * m->nout) || m->DA.alloc((size_t)n * wmax) || m->DZ.alloc((size_t)n * wmax) ||
      m->DZ2.alloc((size_t)n * wmax) || m->loss.alloc(1))
    return RBC3D_ERR_NOMEM;
  return RBC3D_OK;
}

void gemm(rbc3d_mlp* m, int epi, int M, int N, int K, const __nv_bfloat16* A, long long sam, long long sak,
          const __nv_bfloat16* B, long long sbk, long long sbn, float* C, int ldc, const float* bias,
          __nv_bfloat16* Abf) {
  GemmArgs g{M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, Abf};
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  if (epi == 0) k_gemm<0><<<grid, 128, 0, m->st>>>(g);
  else if (epi == 1) k_gemm<1><<<grid, 128, 0, m->st>>>(g);
  else k_gemm<2><<<grid, 128, 0, m->st>>>(g);
  ++m->launches;
}

// forward pass on n rows already in m->X; output in m->Y
rbc3d_status mlp_fwd(rbc3d_mlp* m, int n) {
  { k_to_bf16<<<nblk((long long)n * m->nin, 256), 256, 0, m->st>>>((long long)n * m->nin, m->X.p, m->A[0].p); ++m->launches; }
  for (int l = 0; l < m->nl; ++l) {
    const __nv_bfloat16* W = m->Wb.p + m->woff[l];  // [dout, din] row-major
    const float* b = m->P.p + m->boff[l];
    bool last = l == m->nl - 1;
    // z[n, dout] = a[n, din] W^T : B(k=i, n=o) = W[o][i]
    gemm(m, last ? 2 : 1, n, m->dout[l], m->din[l], m->A[l].p, m->din[l], 1, W, 1, m->din[l],
         last ? m->Y.p : m->Z[l].p, m->dout[l], b, last ? nullptr : m->A[l + 1].p);
  }
  return cudaGetLastError() == cudaSuccess ? RBC3D_OK : RBC3D_ERR_CUDA;
}

// loss + gradients into m->G (packed like P)
rbc3d_status mlp_bwd(rbc3d_mlp* m, int n, float* loss_out) {
  cudaMemsetAsync(m->loss.p, 0, sizeof(float), m->st);
  long long ny = (long long)n * m->nout;
  { k_mse<<<nblk(ny, 256), 256, 0, m->st>>>(ny, m->Y.p, m->T.p, 1.f / (float)ny, m->DY.p, m->DZ.p, m->loss.p); ++m->launches; }
  __nv_bfloat16* dz = m->DZ.p;   // gradient w.r.t. the current layer's pre-activation (bf16)
  __nv_bfloat16* dzn = m->DZ2.p;
  for (int l = m->nl - 1; l >= 0; --l) {
    int di = m->din[l], dd = m->dout[l];
    // dW[dd, di] = dz^T[dd, n] a[n, di]
    gemm(m, 0, dd, di, n, dz, 1, dd, m->A[l].p, di, 1, m->G.p + m->woff[l], di, nullptr, nullptr);
    { k_colsum<<<nblk(dd, 128), 128, 0, m->st>>>(n, dd, dz, m->G.p + m->boff[l]); ++m->launches; }
    if (l == 0) break;
    // da[n, di] = dz[n, dd] W[dd, di]
    const __nv_bfloat16* W = m->Wb.p + m->woff[l];
    gemm(m, 0, n, di, dd, dz, dd, 1, W, di, 1, m->DA.p, di, nullptr, nullptr);
    long long na = (long long)n * di;
    { k_silu_back<<<nblk(na, 256), 256, 0, m->st>>>(na, m->DA.p, m->Z[l - 1].p, dzn); ++m->launches; }
    std::swap(dz, dzn);
  }
  if (loss_out) {
    if (cudaMemcpyAsync(loss_out, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost, m->st)) return RBC3D_ERR_CUDA;
  }
  if (cudaStreamSynchronize(m->st)) return RBC3D_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? RBC3D_OK : RBC3D_ERR_CUDA;
}

}  // namespace

extern "C" {

rbc3d_status rbc3d_mlp_create(int nin, int width, int depth, int nout, unsigned long long seed, rbc3d_mlp** out) {
  if (!out || nin < 1 || width < 1 || depth < 1 || nout < 1 || depth > 64) return RBC3D_ERR_ARG;
  rbc3d_mlp* m = new rbc3d_mlp();
  m->nin = nin; m->width = width; m->depth = depth; m->nout = nout; m->nl = depth + 1;
  for (int l = 0; l < m->nl; ++l) {
    m->din.push_back(l == 0 ? nin : width);
    m->dout.push_back(l == m->nl - 1 ? nout : width);
  }
  size_t off = 0;
  for (int l = 0; l < m->nl; ++l) {
    m->woff.push_back(off); off += (size_t)m->din[l] * m->dout[l];
    m->boff.push_back(off); off += m->dout[l];
  }
  m->nparam = off;
  // He-uniform initialisation (seeded), zero biases
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < m->nl; ++l) {
    float lim = std::sqrt(6.f / m->din[l]) * (l == m->nl - 1 ? 0.1f : 1.f);
    std::uniform_real_distribution<float> U(-lim, lim);
    for (size_t i = 0; i < (size_t)m->din[l] * m->dout[l]; ++i) h[m->woff[l] + i] = U(rng);
  }
  if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) || m->P.upload(h.data(), off, m->st) ||
      m->G.alloc(off) || m->Mo.alloc(off) || m->Vo.alloc(off) || m->Wb.alloc(off)) {
    delete m;
    return RBC3D_ERR_CUDA;
  }
  cudaMemsetAsync(m->Mo.p, 0, off * sizeof(float), m->st);
  cudaMemsetAsync(m->Vo.p, 0, off * sizeof(float), m->st);
  { k_to_bf16<<<nblk(off, 256), 256, 0, m->st>>>(off, m->P.p, m->Wb.p); ++m->launches; }
  if (cudaStreamSynchronize(m->st)) { delete m; return RBC3D_ERR_CUDA; }
  *out = m;
  return RBC3D_OK;
}

rbc3d_status rbc3d_mlp_destroy(rbc3d_mlp* m) {
  if (!m) return RBC3D_OK;
  cudaStream_t st = m->st;
  if (st) cudaStreamSynchronize(st);
  delete m;
  if (st) cudaStreamDestroy(st);
  return RBC3D_OK;
}

long long rbc3d_mlp_num_params(const rbc3d_mlp* m) { return m ? (long long)m->nparam : -1; }

// Packed FP32 parameters [W_0 (dout x din, row-major), b_0, W_1, b_1, ...]: get or set.
rbc3d_status rbc3d_mlp_params(rbc3d_mlp* m, float* host, int get) {
  if (!m || !host) return RBC3D_ERR_ARG;
  if (get) {
    if (cudaMemcpyAsync(host, m->P.p, m->nparam * sizeof(float), cudaMemcpyDeviceToHost, m->st)) return RBC3D_ERR_CUDA;
  } else {
    if (cudaMemcpyAsync(m->P.p, host, m->nparam * sizeof(float), cudaMemcpyHostToDevice, m->st)) return RBC3D_ERR_CUDA;
    { k_to_bf16<<<nblk(m->nparam, 256), 256, 0, m->st>>>(m->nparam, m->P.p, m->Wb.p); ++m->launches; }
  }
  return cudaStreamSynchronize(m->st) ? RBC3D_ERR_CUDA : RBC3D_OK;
}

// y (n x nout, row-major FP32) = MLP(x (n x nin, row-major FP32))
rbc3d_status rbc3d_mlp_forward(rbc3d_mlp* m, int n, const float* x, float* y) {
  if (!m || n < 0 || (n && (!x || !y))) return RBC3D_ERR_ARG;
  if (n == 0) return RBC3D_OK;
  if (mlp_ensure(m, n)) return RBC3D_ERR_NOMEM;
  if (cudaMemcpyAsync(m->X.p, x, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->st)) return RBC3D_ERR_CUDA;
  rbc3d_status s = mlp_fwd(m, n);
  if (s) return s;
  if (cudaMemcpyAsync(y, m->Y.p, sizeof(float) * n * m->nout, cudaMemcpyDeviceToHost, m->st)) return RBC3D_ERR_CUDA;
  return cudaStreamSynchronize(m->st) ? RBC3D_ERR_CUDA : RBC3D_OK;
}

// Loss (mean squared error) and packed FP32 gradients (for checks).
rbc3d_status rbc3d_mlp_gradients(rbc3d_mlp* m, int n, const float* x, const float* t, float* grads, float* loss) {
  if (!m || n <= 0 || !x || !t) return RBC3D_ERR_ARG;
  if (mlp_ensure(m, n)) return RBC3D_ERR_NOMEM;
  if (cudaMemcpyAsync(m->X.p, x, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->st) ||
      cudaMemcpyAsync(m->T.p, t, sizeof(float) * n * m->nout, cudaMemcpyHostToDevice, m->st))
    return RBC3D_ERR_CUDA;
  rbc3d_status s = mlp_fwd(m, n);
  if (s) return s;
  if ((s = mlp_bwd(m, n, loss))) return s;
  if (grads && cudaMemcpy(grads, m->G.p, m->nparam * sizeof(float), cudaMemcpyDeviceToHost)) return RBC3D_ERR_CUDA;
  return RBC3D_OK;
}

// One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the batch; returns the loss before the step.
rbc3d_status rbc3d_mlp_train_step(rbc3d_mlp* m, int n, const float* x, const float* t, float lr, float* loss) {
  rbc3d_status s = rbc3d_mlp_gradients(m, n, x, t, nullptr, loss);
  if (s) return s;
  m->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f / (1.f - std::pow(b1, (float)m->step)), c2 = 1.f / (1.f - std::pow(b2, (float)m->step));
  { k_adam<<<nblk(m->nparam, 256), 256, 0, m->st>>>(m->nparam, m->P.p, m->G.p, m->Mo.p, m->Vo.p, lr, b1, b2, 1e-8f,
                                                    c1, c2, m->Wb.p); ++m->launches; }
  return cudaStreamSynchronize(m->st) ? RBC3D_ERR_CUDA : RBC3D_OK;
}

}  // extern "C"
