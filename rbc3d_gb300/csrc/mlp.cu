// mlp.cu -- the MLP of the learned wall-density initial guess: forward,
// backward and Adam on the GPU.  No counterpart in the reference.
//
// Layers: nin -> width (SiLU) -> ... -> width (SiLU) -> nout, "depth" hidden
// layers.  GEMM operands are BF16 (inputs, activations, weights, gradients),
// products accumulate in FP32 in tensor memory through tcgen05.mma (k_umma);
// master weights, Adam moments and the loss are FP32.  One GEMM kernel
// (operands gathered with generic strides, so it serves x W^T, dz^T a and
// dz W) plus small element-wise kernels.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "ctx.hpp"

namespace {

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }


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
  int ksplit;              // EPI 0: K split over gridDim.z; partial tiles to ws[z][M][N]
  float* ws;
};

__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }

// ---------------------------------------------------------------------------
// tcgen05 GEMM: 128 x 128 output tile per CTA, K staged 64 at a time into a
// UNST-deep shared-memory ring (cp.async 16-byte copies, UNST - 1 stages in
// flight while the tensor core works on the oldest) in the canonical no-swizzle
// K-major layout (8-row x 16-byte core matrices: element (r, k) at byte
// ((r/8)*8 + k/8)*128 + (r%8)*16 + (k%8)*2, so core matrices adjacent in K are
// 128 B apart and 8-row groups 1024 B apart), one elected thread issuing
// tcgen05.mma.cta_group::1.kind::f16 (M 128, N 128, K 16, BF16 in, FP32
// accumulate in 128 TMEM columns) and committing each stage to an mbarrier;
// the four warps read their 32 accumulator rows back with tcgen05.ld and run
// the epilogue.  Operands are gathered with generic strides (asynchronous
// 16-byte copies when k is contiguous, else synchronous gathers), so one kernel
// serves x W^T, dz^T a and dz W.  GEMMs with few output tiles and a long K (the
// weight gradients, K = batch rows) split K over gridDim.z; the partial tiles
// are summed in a fixed order by k_splitk_sum.
constexpr int UBM = 128, UBN = 128, UBK = 64, UNST = 4;
constexpr int USTAGE = UBM * UBK * 2;  // bytes per operand per stage (16 KB)
constexpr unsigned UMMA_IDESC = (1u << 4)              // D: FP32
                                | (1u << 7)            // A: BF16
                                | (1u << 10)           // B: BF16
                                | ((UBN >> 3) << 17)   // N / 8
                                | ((UBM >> 4) << 24);  // M / 16  (A, B K-major)
constexpr long long UMMA_WAIT_LIMIT = 1ll << 26;       // bounded mbarrier waits

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4, LBO >> 4 (K-adjacent core
// matrices), SBO >> 4 (8-row groups), version 1, no swizzle
__device__ __forceinline__ unsigned long long umma_desc(unsigned addr) {
  return (unsigned long long)((addr >> 4) & 0x3FFF) | ((unsigned long long)(128 >> 4) << 16) |
         ((unsigned long long)(1024 >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (long long it = 0; it < UMMA_WAIT_LIMIT; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ bool umma_async_ok(const __nv_bfloat16* X, long long sr, long long sk, int K) {
  return sk == 1 && (sr % 8) == 0 && (K % 8) == 0 && ((reinterpret_cast<size_t>(X) & 15) == 0);
}

// asynchronous form of the k-contiguous stage (umma_async_ok): one 16-byte
// cp.async per core-matrix row, zero-filled outside rows x K
__device__ __forceinline__ void umma_stage_async(unsigned dst, const __nv_bfloat16* X, long long sr, int rows, int K,
                                                 int r0, int k0) {
  for (int e = threadIdx.x; e < UBM * (UBK / 8); e += blockDim.x) {
    const int r = e / (UBK / 8), k8 = e % (UBK / 8);
    const int gr = r0 + r, gk = k0 + 8 * k8;
    const bool in = gr < rows && gk < K;  // K % 8 == 0: a vector is wholly in or out
    const __nv_bfloat16* src = in ? X + (long long)gr * sr + gk : X;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst + ((r >> 3) * 8 + k8) * 128 + (r & 7) * 16),
                 "l"(src), "r"(in ? 16 : 0)
                 : "memory");
  }
}

// stage rows [r0, r0+128) x k [k0, k0+64) of X (element (r, k) at X[r*sr + k*sk],
// zero outside rows x K) into the core-matrix layout at dst
__device__ __forceinline__ void umma_stage(unsigned char* dst, const __nv_bfloat16* X, long long sr, long long sk,
                                           int rows, int K, int r0, int k0) {
  const int tid = threadIdx.x;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  if (sk == 1 && (sr % 8) == 0 && ((reinterpret_cast<size_t>(X) & 15) == 0)) {
    // k contiguous: one 16-byte vector = one core-matrix row
    for (int e = tid; e < UBM * (UBK / 8); e += blockDim.x) {
      const int r = e / (UBK / 8), k8 = e % (UBK / 8);
      const int gr = r0 + r, gk = k0 + 8 * k8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (gr < rows && gk + 8 <= K) v = *reinterpret_cast<const uint4*>(X + (long long)gr * sr + gk);
      else if (gr < rows)
        for (int q = 0; q < 8; ++q)
          reinterpret_cast<__nv_bfloat16*>(&v)[q] = gk + q < K ? X[(long long)gr * sr + gk + q] : zero;
      *reinterpret_cast<uint4*>(dst + ((r >> 3) * 8 + k8) * 128 + (r & 7) * 16) = v;
    }
  } else if (sr == 1 && (sk % 8) == 0 && ((reinterpret_cast<size_t>(X) & 15) == 0)) {
    // rows contiguous: 8 consecutive rows of one k per vector, transposed into place
    for (int e = tid; e < (UBM / 8) * UBK; e += blockDim.x) {
      const int r8 = e % (UBM / 8), k = e / (UBM / 8);
      const int gr = r0 + 8 * r8, gk = k0 + k;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (gk < K && gr + 8 <= rows) v = *reinterpret_cast<const uint4*>(X + gr + (long long)gk * sk);
      else if (gk < K)
        for (int q = 0; q < 8; ++q)
          reinterpret_cast<__nv_bfloat16*>(&v)[q] = gr + q < rows ? X[gr + q + (long long)gk * sk] : zero;
      const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&v);
      unsigned char* base = dst + (r8 * 8 + (k >> 3)) * 128 + (k & 7) * 2;
#pragma unroll
      for (int q = 0; q < 8; ++q) *reinterpret_cast<__nv_bfloat16*>(base + q * 16) = h[q];
    }
  } else {
    for (int e = tid; e < UBM * UBK; e += blockDim.x) {
      const int r = e / UBK, k = e % UBK;
      const int gr = r0 + r, gk = k0 + k;
      const __nv_bfloat16 v = (gr < rows && gk < K) ? X[(long long)gr * sr + (long long)gk * sk] : zero;
      *reinterpret_cast<__nv_bfloat16*>(dst + ((r >> 3) * 8 + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2) = v;
    }
  }
}

// EPI 0: C = A B;  EPI 1: z = A B + bias -> C, SiLU(z) -> Abf;  EPI 2: C = A B + bias
template <int EPI>
__global__ void __launch_bounds__(128) k_umma(GemmArgs g, int* err) {
  extern __shared__ __align__(1024) unsigned char usm[];
  unsigned char* As = usm;                    // UNST stages
  unsigned char* Bs = usm + UNST * USTAGE;    // UNST stages
  __shared__ __align__(8) unsigned long long mbar[UNST];
  __shared__ unsigned tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.y * UBM, n0 = blockIdx.x * UBN;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                 "r"(UBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int b = 0; b < UNST; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[b])));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const unsigned taddr = tmem_slot;
  // this CTA's K chunks [kb, ke)
  const int nkall = (g.K + UBK - 1) / UBK;
  const int kb = (int)((long long)nkall * blockIdx.z / gridDim.z), ke = (int)((long long)nkall * (blockIdx.z + 1) / gridDim.z);
  const int nk = ke - kb;
  const bool asyncA = umma_async_ok(g.A, g.sam, g.sak, g.K), asyncB = umma_async_ok(g.B, g.sbn, g.sbk, g.K);
  // A: rows m (sam), k (sak);  B as [n][k]: rows n (sbn), k (sbk)
  auto issue = [&](int c) {
    const int buf = c % UNST, k0 = (kb + c) * UBK;
    if (asyncA) umma_stage_async(smem_u32(As + buf * USTAGE), g.A, g.sam, g.M, g.K, m0, k0);
    else umma_stage(As + buf * USTAGE, g.A, g.sam, g.sak, g.M, g.K, m0, k0);
    if (asyncB) umma_stage_async(smem_u32(Bs + buf * USTAGE), g.B, g.sbn, g.N, g.K, n0, k0);
    else umma_stage(Bs + buf * USTAGE, g.B, g.sbn, g.sbk, g.N, g.K, n0, k0);
  };
  bool ok = true;
  for (int c = 0; c < UNST - 1; ++c) {
    if (c < nk) issue(c);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  for (int c = 0; c < nk; ++c) {
    const int buf = c % UNST;
    asm volatile("cp.async.wait_group %0;\n" ::"n"(UNST - 2) : "memory");  // chunk c has landed
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n");
      const unsigned a0 = smem_u32(As + buf * USTAGE), b0 = smem_u32(Bs + buf * USTAGE);
#pragma unroll
      for (int j = 0; j < UBK / 16; ++j) {
        const unsigned long long da = umma_desc(a0 + j * 256), db = umma_desc(b0 + j * 256);
        const unsigned acc = (c > 0 || j > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
            "l"(da), "l"(db), "r"(UMMA_IDESC), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_u32(&mbar[buf])));
    }
    // refill the buffer of chunk c - 1 with chunk c + UNST - 1 once chunk c - 1's MMAs are done
    const int nx = c + UNST - 1;
    if (nx < nk) {
      if (c >= 1 && !mbar_wait(smem_u32(&mbar[(c - 1) % UNST]), ((c - 1) / UNST) & 1)) ok = false;
      issue(nx);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  // all MMAs done: the last commit tracks every earlier MMA of the thread
  if (nk > 0 && !mbar_wait(smem_u32(&mbar[(nk - 1) % UNST]), ((nk - 1) / UNST) & 1)) ok = false;
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    const int row = m0 + warp * 32 + (tid & 31);
#pragma unroll 1
    for (int c0 = 0; c0 < UBN; c0 += 32) {
      unsigned r[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr + ((unsigned)(warp * 32) << 16) + (unsigned)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < g.M) {
        float v[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]) + ((EPI != 0 && n0 + c0 + q < g.N) ? g.bias[n0 + c0 + q] : 0.f);
        const bool part = EPI == 0 && g.ksplit > 1;
        const int ldc = part ? g.N : g.ldc;
        float* crow = (part ? g.ws + (long long)blockIdx.z * g.M * g.N : g.C) + (long long)row * ldc + n0 + c0;
        const bool vec = n0 + c0 + 32 <= g.N && (ldc % 8) == 0 && ((reinterpret_cast<size_t>(crow) & 15) == 0) &&
                         (EPI != 1 || ((reinterpret_cast<size_t>(g.Abf + (long long)row * g.ldc + n0 + c0) & 15) == 0));
        if (vec) {
          // a row segment of 32: 8 float4 (and 4 x 8 bf16) stores
#pragma unroll
          for (int q = 0; q < 8; ++q)
            reinterpret_cast<float4*>(crow)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          if (EPI == 1) {
            __nv_bfloat16* arow = g.Abf + (long long)row * g.ldc + n0 + c0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              __nv_bfloat16 h[8];
#pragma unroll
              for (int e = 0; e < 8; ++e) h[e] = __float2bfloat16(silu(v[8 * q + e]));
              reinterpret_cast<uint4*>(arow)[q] = *reinterpret_cast<const uint4*>(h);
            }
          }
        } else {
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const int n = n0 + c0 + q;
            if (n >= g.N) break;
            crow[q] = v[q];
            if (EPI == 1) g.Abf[(long long)row * g.ldc + n] = __float2bfloat16(silu(v[q]));
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(UBN));
}

// C[m][n] = sum over z of ws[z][m][n] (the split-K partial tiles, fixed order)
__global__ void k_splitk_sum(int M, int N, int S, const float* __restrict__ ws, float* __restrict__ C, int ldc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x, MN = (long long)M * N;
  if (i >= MN) return;
  float s = 0.f;
  for (int z = 0; z < S; ++z) s += ws[z * MN + i];
  C[(i / N) * ldc + i % N] = s;
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

// column sums of a row-major rows x cols matrix (bias gradient): 32 columns
// per block, its 8 warps over the rows, a shared-memory reduction
__global__ void k_colsum(int rows, int cols, const __nv_bfloat16* __restrict__ dz, float* __restrict__ out) {
  __shared__ float part[8][32];
  const int c = blockIdx.x * 32 + (threadIdx.x & 31), w = threadIdx.x >> 5;
  float s = 0.f;
  if (c < cols)
    for (int r = w; r < rows; r += 8) s += __bfloat162float(dz[(long long)r * cols + c]);
  part[w][threadIdx.x & 31] = s;
  __syncthreads();
  if (w == 0 && c < cols) {
    float t = 0.f;
    for (int k = 0; k < 8; ++k) t += part[k][threadIdx.x & 31];
    out[c] = t;
  }
}

// out[c][r] = in[r][c] for a row-major rows x cols BF16 matrix (32 x 32 tiles)
__global__ void k_transpose(int rows, int cols, const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[i][threadIdx.x] = in[(long long)r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(long long)c * rows + r] = t[threadIdx.x][i];
  }
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
  DBuf<__nv_bfloat16> TA, TB;       // transposed GEMM operands of the backward pass
  long long step = 0;
  cudaStream_t st = nullptr;
  long long launches = 0;
  DBuf<int> err;  // set by a GEMM whose mbarrier wait ran out
  DBuf<float> WS;  // split-K partial tiles
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
      m->DZ2.alloc((size_t)n * wmax) || m->loss.alloc(1) || m->TA.alloc((size_t)n * wmax) ||
      m->TB.alloc((size_t)std::max((size_t)n * wmax, (size_t)wmax * wmax)))
    return RBC3D_ERR_NOMEM;
  return RBC3D_OK;
}

void gemm(rbc3d_mlp* m, int epi, int M, int N, int K, const __nv_bfloat16* A, long long sam, long long sak,
          const __nv_bfloat16* B, long long sbk, long long sbn, float* C, int ldc, const float* bias,
          __nv_bfloat16* Abf) {
  GemmArgs g{M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, Abf, 1, nullptr};
  dim3 grid((N + UBN - 1) / UBN, (M + UBM - 1) / UBM);
  // weight gradients (few tiles, K = batch rows): split K to fill the SMs
  const int tiles = grid.x * grid.y, nk = (K + UBK - 1) / UBK;
  if (epi == 0 && tiles < 76 && nk >= 4) {
    int sm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    const int S = std::min(nk, std::max(1, sm / tiles));
    if (S > 1 && !m->WS.alloc((size_t)S * M * N)) {
      g.ksplit = S;
      g.ws = m->WS.p;
      grid.z = S;
    }
  }
  const int smem = 2 * UNST * USTAGE;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_umma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_umma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_umma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  if (epi == 0) k_umma<0><<<grid, 128, smem, m->st>>>(g, m->err.p);
  else if (epi == 1) k_umma<1><<<grid, 128, smem, m->st>>>(g, m->err.p);
  else k_umma<2><<<grid, 128, smem, m->st>>>(g, m->err.p);
  ++m->launches;
  if (g.ksplit > 1) {
    k_splitk_sum<<<nblk((long long)M * N, 256), 256, 0, m->st>>>(M, N, g.ksplit, g.ws, C, ldc);
    ++m->launches;
  }
}

void transpose(rbc3d_mlp* m, int rows, int cols, const __nv_bfloat16* in, __nv_bfloat16* out) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose<<<grid, block, 0, m->st>>>(rows, cols, in, out);
  ++m->launches;
}

// a GEMM whose mbarrier wait ran out left err set (read after a synchronisation)
rbc3d_status gemm_status(rbc3d_mlp* m) {
  int e = 0;
  if (cudaMemcpyAsync(&e, m->err.p, sizeof(int), cudaMemcpyDeviceToHost, m->st) || cudaStreamSynchronize(m->st))
    return RBC3D_ERR_CUDA;
  return e ? RBC3D_ERR_TIMEOUT : RBC3D_OK;
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
    // dW[dd, di] = dz^T[dd, n] a[n, di], from K-major copies dz^T [dd][n] and a^T [di][n]
    transpose(m, n, dd, dz, m->TA.p);
    transpose(m, n, di, m->A[l].p, m->TB.p);
    gemm(m, 0, dd, di, n, m->TA.p, n, 1, m->TB.p, 1, n, m->G.p + m->woff[l], di, nullptr, nullptr);
    { k_colsum<<<nblk(dd, 32), 256, 0, m->st>>>(n, dd, dz, m->G.p + m->boff[l]); ++m->launches; }
    if (l == 0) break;
    // da[n, di] = dz[n, dd] W[dd, di], from W^T [di][dd]
    const __nv_bfloat16* W = m->Wb.p + m->woff[l];
    transpose(m, dd, di, W, m->TB.p);
    gemm(m, 0, n, di, dd, dz, dd, 1, m->TB.p, 1, dd, m->DA.p, di, nullptr, nullptr);
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
      m->G.alloc(off) || m->Mo.alloc(off) || m->Vo.alloc(off) || m->Wb.alloc(off) || m->err.alloc(1)) {
    delete m;
    return RBC3D_ERR_CUDA;
  }
  cudaMemsetAsync(m->err.p, 0, sizeof(int), m->st);
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
  return gemm_status(m);
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
  if ((s = gemm_status(m))) return s;
  if (grads && (cudaMemcpyAsync(grads, m->G.p, m->nparam * sizeof(float), cudaMemcpyDeviceToHost, m->st) ||
                cudaStreamSynchronize(m->st)))
    return RBC3D_ERR_CUDA;
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
