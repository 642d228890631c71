// Neural operator for the learned warm start: a small MLP mapping the six
// physical parameters of an instance (bias, generation amplitude, absorption
// coefficient, doping, lifetime, interface rate) to the coefficients of a
// fixed low-rank (POD) basis of the steady-state fields.  No counterpart in
// the reference: it is the warm-start component the benchmark adds.
//
// Arithmetic: GEMM operands are BF16 (weights stored in BF16, activations
// rounded to BF16 when staged), accumulation FP32 on the tensor cores
// (tcgen05.mma into TMEM); FP32 master weights and Adam moments.  Layers: z = x W^T + b, y = tanh(z) for hidden layers, linear
// output; loss = mean squared error.  The decoder (mean + V c) is an FP32 GEMM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "common.hpp"

namespace pecs {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16, kGemmThreads = 256;

template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ float round_bf16(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// C[M,N] = alpha * op(A)[M,K] op(B)[K,N] + beta * C + bias[n], then act.
// op(A)(m,k) = TA ? A[k*lda+m] : A[m*lda+k]; op(B)(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n].
// kBf16In rounds both operands to BF16 before the product (FP32 accumulate).
template <typename TAe, typename TBe, bool TA, bool TB, bool kBf16In>
__global__ void __launch_bounds__(kGemmThreads)
    k_gemm(int M, int N, int K, const TAe* __restrict__ A, int lda, const TBe* __restrict__ B, int ldb,
           float* __restrict__ C, int ldc, float alpha, float beta, const float* __restrict__ bias,
           int act) {
  __shared__ float As[kBK][kBM + 1];
  __shared__ float Bs[kBK][kBN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += kBK) {
    for (int t = threadIdx.x; t < kBK * kBM; t += kGemmThreads) {
      const int kk = t % kBK, mm = t / kBK;
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < M && k < K) v = to_f(TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]);
      As[kk][mm] = kBf16In ? round_bf16(v) : v;
    }
    for (int t = threadIdx.x; t < kBK * kBN; t += kGemmThreads) {
      const int nn = t % kBN, kk = t / kBN;
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.f;
      if (n < N && k < K) v = to_f(TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]);
      Bs[kk][nn] = kBf16In ? round_bf16(v) : v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = alpha * acc[i][j];
      if (beta != 0.f) v += beta * C[(size_t)m * ldc + n];
      if (bias) v += bias[n];
      if (act == 1) v = tanhf(v);
      C[(size_t)m * ldc + n] = v;
    }
  }
}

template <typename TAe, typename TBe, bool TA, bool TB, bool kBf16In>
void gemm(int M, int N, int K, const TAe* A, int lda, const TBe* B, int ldb, float* C, int ldc,
          float alpha, float beta, const float* bias, int act, cudaStream_t st) {
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM);
  k_gemm<TAe, TBe, TA, TB, kBf16In><<<grid, kGemmThreads, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc,
                                                                    alpha, beta, bias, act);
  PECS_CUDA(cudaGetLastError());
}

// ---- tensor-core GEMM: tcgen05.mma, BF16 operands, FP32 accumulator in TMEM ----
// The layers' GEMMs C = act(alpha op(A) op(B) + beta C + bias) with BF16-rounded
// operands run on the 5th-generation tensor cores: each CTA owns a 128 x 128
// tile of C, whose FP32 accumulator lives in 128 TMEM columns.  Per K chunk of
// 64, the CTA's threads stage op(A) (128 x 64) and op(B)^T (128 x 64) as BF16
// in shared memory in the canonical K-major layout without swizzle (8-row x
// 16-byte core matrices; K-adjacent core matrices 128 B apart, 8-row groups
// 1024 B apart), one thread issues four tcgen05.mma (K = 16 each) and commits
// them to an mbarrier, and every thread waits on it -- with a bounded number of
// polls: a wait that runs out sets the error flag, the tile is skipped and the
// TMEM is still freed -- before the buffers are refilled.  The epilogue reads
// the accumulator with tcgen05.ld (warp w: TMEM lanes 32w..32w+31 = rows).
constexpr int kTcM = 128, kTcN = 128, kTcK = 64, kTcThreads = 128;
constexpr uint32_t kTcCols = 128;
constexpr long long kTcPollLimit = 1LL << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, k) of a 128 x 64 K-major tile
__device__ __forceinline__ uint32_t tc_off(int row, int k) {
  return (uint32_t)((row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading-dimension byte
// offset (K direction, 128 B), stride byte offset (8-row groups, 1024 B),
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)(1024u >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (long long i = 0; i < kTcPollLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <typename TAe, typename TBe, bool TA, bool TB>
__global__ void __launch_bounds__(kTcThreads)
    k_gemm_tc(int M, int N, int K, const TAe* __restrict__ A, int lda, const TBe* __restrict__ B, int ldb,
              float* __restrict__ C, int ldc, float alpha, float beta, const float* __restrict__ bias,
              int act, int* __restrict__ err) {
  __shared__ __align__(1024) unsigned char As[kTcM * kTcK * 2];
  __shared__ __align__(1024) unsigned char Bs[kTcN * kTcK * 2];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
  const uint32_t mbar_a = smem_u32(&mbar);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar_a) : "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  // instruction descriptor (kind::f16): FP32 accumulator, BF16 A and B, both
  // K-major, N = 128, M = 128
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                         ((uint32_t)(kTcM >> 4) << 24);
  uint32_t parity = 0;
  bool failed = false;
  const int nk = (K + kTcK - 1) / kTcK;
  for (int kc = 0; kc < nk && !failed; ++kc) {
    const int k0 = kc * kTcK;
    for (int t = tid; t < kTcM * kTcK; t += kTcThreads) {
      int r, k;
      if (TA) { r = t % kTcM; k = t / kTcM; } else { k = t % kTcK; r = t / kTcK; }
      const int m = m0 + r, kk = k0 + k;
      float v = 0.f;
      if (m < M && kk < K) v = to_f(TA ? A[(size_t)kk * lda + m] : A[(size_t)m * lda + kk]);
      *reinterpret_cast<__nv_bfloat16*>(As + tc_off(r, k)) = __float2bfloat16_rn(v);
    }
    for (int t = tid; t < kTcN * kTcK; t += kTcThreads) {
      int r, k;
      if (TB) { k = t % kTcK; r = t / kTcK; } else { r = t % kTcN; k = t / kTcN; }
      const int n = n0 + r, kk = k0 + k;
      float v = 0.f;
      if (n < N && kk < K) v = to_f(TB ? B[(size_t)n * ldb + kk] : B[(size_t)kk * ldb + n]);
      *reinterpret_cast<__nv_bfloat16*>(Bs + tc_off(r, k)) = __float2bfloat16_rn(v);
    }
    // the staged tiles are read by the tensor cores (async proxy)
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (tid == 0) {
#pragma unroll
      for (int s = 0; s < kTcK / 16; ++s) {
        const uint64_t ad = tc_desc(smem_u32(As) + s * 256);
        const uint64_t bd = tc_desc(smem_u32(Bs) + s * 256);
        const uint32_t accumulate = (kc > 0 || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar_a)
                   : "memory");
    }
    const bool ok = tc_wait(mbar_a, parity);
    parity ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    failed = __syncthreads_or(!ok) != 0;
  }
  if (failed) {
    if (tid == 0) atomicExch(err, 1);
    // let MMAs still in flight finish (bounded) before the TMEM is freed
    tc_wait(mbar_a, parity ^ 1u);
  } else {
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < kTcN; c0 += 32) {
      if (n0 + c0 >= N) break;
      uint32_t v[32];
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                   : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                   : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0)
                   : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c0 + j;
          if (n >= N) break;
          float x = alpha * __uint_as_float(v[j]);
          if (beta != 0.f) x += beta * C[(size_t)row * ldc + n];
          if (bias) x += bias[n];
          if (act == 1) x = tanhf(x);
          C[(size_t)row * ldc + n] = x;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcCols) : "memory");
}

// BF16-operand GEMMs of the network: on the tensor cores
template <typename TAe, typename TBe, bool TA, bool TB>
void gemm_tc(int M, int N, int K, const TAe* A, int lda, const TBe* B, int ldb, float* C, int ldc,
             float alpha, float beta, const float* bias, int act, int* err, cudaStream_t st) {
  dim3 grid((N + kTcN - 1) / kTcN, (M + kTcM - 1) / kTcM);
  k_gemm_tc<TAe, TBe, TA, TB><<<grid, kTcThreads, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta,
                                                           bias, act, err);
  PECS_CUDA(cudaGetLastError());
}

// dz = dy * (1 - y^2)   (tanh backward), in place on dy
__global__ void k_tanh_bwd(float* __restrict__ dy, const float* __restrict__ y, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) dy[i] *= (1.f - y[i] * y[i]);
}

// db[n] = sum_b dz[b, n]
__global__ void k_colsum(const float* __restrict__ dz, float* __restrict__ db, int B, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += dz[(size_t)b * N + n];
  db[n] = s;
}

// dy = 2 (y - t) / (B N); per-block partial loss sums
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy,
                      size_t n, float* __restrict__ loss_partial) {
  __shared__ float s[256];
  float acc = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = 2.f * d / (float)n;
    acc += d * d;
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = s[0];
}

// Adam on FP32 masters, refreshes the BF16 copy
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ wb, size_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

__global__ void k_add_rowvec(float* __restrict__ y, const float* __restrict__ mean, int B, int N) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < (size_t)B * N) y[i] += mean[i % N];
}

}  // namespace

struct Mlp {
  std::vector<int> w;          // widths, layers = w.size()-1
  size_t n_params = 0;
  std::vector<size_t> woff, boff;  // offsets of W_l (out x in) and b_l in the packed vector
  DBuf<float> P, G, Mo, Vo;    // masters, grads, Adam moments
  DBuf<__nv_bfloat16> Pb;      // BF16 copy
  int max_batch = 0;
  std::vector<DBuf<float>> act;  // act[l]: batch x w[l] (act[0] = input copy)
  std::vector<DBuf<float>> dact;
  DBuf<float> loss_part;
  DBuf<int> err;  // set by a tensor-core GEMM whose MMA-completion wait ran out
  int adam_t = 0;
  cudaStream_t st = nullptr;
  ~Mlp() {
    if (st) cudaStreamDestroy(st);
  }

  void ensure_batch(int B) {
    if (B <= max_batch) return;
    act.clear();
    dact.clear();
    act.resize(w.size());
    dact.resize(w.size());
    for (size_t l = 0; l < w.size(); ++l) {
      act[l].alloc((size_t)B * w[l]);
      dact[l].alloc((size_t)B * w[l]);
    }
    max_batch = B;
  }

  const __nv_bfloat16* Wb(int l) const { return Pb.p + woff[l]; }
  const float* bias(int l) const { return P.p + boff[l]; }

  void forward(int B, const float* x, cudaStream_t s) {
    ensure_batch(B);
    const int L = (int)w.size() - 1;
    PECS_CUDA(cudaMemcpyAsync(act[0].p, x, (size_t)B * w[0] * 4, cudaMemcpyDeviceToDevice, s));
    for (int l = 0; l < L; ++l) {
      // act[l+1] = act(act[l] W_l^T + b_l); W_l stored out x in (row-major)
      gemm_tc<float, __nv_bfloat16, false, true>(B, w[l + 1], w[l], act[l].p, w[l], Wb(l), w[l],
                                                 act[l + 1].p, w[l + 1], 1.f, 0.f, bias(l),
                                                 l < L - 1 ? 1 : 0, err.p, s);
    }
  }

  // gradients of mean((y - t)^2) into G; returns via loss_part (device)
  void backward(int B, const float* target, cudaStream_t s) {
    const int L = (int)w.size() - 1;
    const size_t nout = (size_t)B * w[L];
    const int nblk = 64;
    if (loss_part.n < (size_t)nblk) loss_part.alloc(nblk);
    k_mse<<<nblk, 256, 0, s>>>(act[L].p, target, dact[L].p, nout, loss_part.p);
    PECS_CUDA(cudaGetLastError());
    for (int l = L - 1; l >= 0; --l) {
      float* dz = dact[l + 1].p;
      if (l < L - 1) {
        const size_t n = (size_t)B * w[l + 1];
        k_tanh_bwd<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dz, act[l + 1].p, n);
        PECS_CUDA(cudaGetLastError());
      }
      // dW_l (out x in) = dz^T (out x B) * act[l] (B x in)
      gemm_tc<float, float, true, false>(w[l + 1], w[l], B, dz, w[l + 1], act[l].p, w[l],
                                         G.p + woff[l], w[l], 1.f, 0.f, nullptr, 0, err.p, s);
      k_colsum<<<(w[l + 1] + 127) / 128, 128, 0, s>>>(dz, G.p + boff[l], B, w[l + 1]);
      PECS_CUDA(cudaGetLastError());
      if (l > 0) {
        // d act[l] (B x in) = dz (B x out) * W_l (out x in)
        gemm_tc<float, __nv_bfloat16, false, false>(B, w[l], w[l + 1], dz, w[l + 1], Wb(l), w[l],
                                                    dact[l].p, w[l], 1.f, 0.f, nullptr, 0, err.p, s);
      }
    }
  }

  // after the stream has synchronised: report (and clear) a GEMM that gave up
  void check_err() {
    int h = 0;
    PECS_CUDA(cudaMemcpy(&h, err.p, 4, cudaMemcpyDeviceToHost));
    if (h) {
      err.zero();
      throw PecsError(PECS_E_CUDA, "a tensor-core GEMM gave up waiting for its MMAs; outputs are invalid");
    }
  }

  float read_loss(cudaStream_t s, int B) {
    std::vector<float> h(64);
    PECS_CUDA(cudaMemcpyAsync(h.data(), loss_part.p, 64 * 4, cudaMemcpyDeviceToHost, s));
    PECS_CUDA(cudaStreamSynchronize(s));
    double t = 0;
    for (float v : h) t += v;
    return (float)(t / ((double)B * w.back()));
  }

  void adam(float lr, cudaStream_t s) {
    ++adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
    k_adam<<<(unsigned)((n_params + 255) / 256), 256, 0, s>>>(P.p, Mo.p, Vo.p, G.p, Pb.p, n_params, lr,
                                                              b1, b2, 1e-8f, c1, c2);
    PECS_CUDA(cudaGetLastError());
  }

  void sync_bf16(cudaStream_t s) {
    k_to_bf16<<<(unsigned)((n_params + 255) / 256), 256, 0, s>>>(P.p, Pb.p, n_params);
    PECS_CUDA(cudaGetLastError());
  }
};

}  // namespace pecs

using namespace pecs;

struct pecs_mlp {
  Mlp m;
};

namespace pecs {
void set_error_external(const std::string& m);
}

#define NN_TRY(...)                                     \
  try {                                                 \
    __VA_ARGS__;                                        \
    return PECS_OK;                                     \
  } catch (const PecsError& ex) {                       \
    pecs::set_error_external(ex.what());                \
    return ex.code;                                     \
  } catch (const std::exception& ex) {                  \
    pecs::set_error_external(ex.what());                \
    return PECS_E_ARG;                                  \
  }

extern "C" {

int pecs_mlp_create(int n_layers, const int* widths, unsigned long long seed, pecs_mlp** out) {
  NN_TRY({
    if (!out || !widths || n_layers < 1 || n_layers > 16) throw PecsError(PECS_E_ARG, "bad layers");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
      throw PecsError(PECS_E_NODEVICE, "no CUDA device available");
    std::unique_ptr<pecs_mlp> h(new pecs_mlp());
    Mlp& m = h->m;
    m.w.assign(widths, widths + n_layers + 1);
    for (int x : m.w)
      if (x < 1 || x > 65536) throw PecsError(PECS_E_ARG, "bad width");
    size_t off = 0;
    for (int l = 0; l < n_layers; ++l) {
      m.woff.push_back(off);
      off += (size_t)m.w[l] * m.w[l + 1];
      m.boff.push_back(off);
      off += m.w[l + 1];
    }
    m.n_params = off;
    std::vector<float> init(off, 0.f);
    std::mt19937_64 g(seed);
    for (int l = 0; l < n_layers; ++l) {
      const float sc = std::sqrt(1.0f / m.w[l]);  // LeCun-uniform-like for tanh
      std::uniform_real_distribution<float> U(-sc * std::sqrt(3.f), sc * std::sqrt(3.f));
      for (size_t t = 0; t < (size_t)m.w[l] * m.w[l + 1]; ++t) init[m.woff[l] + t] = U(g);
    }
    PECS_CUDA(cudaStreamCreateWithFlags(&m.st, cudaStreamNonBlocking));
    m.P.upload(init);
    m.G.alloc(off);
    m.G.zero();
    m.err.alloc(1);
    m.err.zero();
    m.Mo.alloc(off);
    m.Mo.zero();
    m.Vo.alloc(off);
    m.Vo.zero();
    m.Pb.alloc(off);
    m.sync_bf16(m.st);
    PECS_CUDA(cudaStreamSynchronize(m.st));
    *out = h.release();
  })
}

void pecs_mlp_destroy(pecs_mlp* m) { delete m; }

int pecs_mlp_n_params(pecs_mlp* h, long long* n) {
  NN_TRY({
    if (!h || !n) throw PecsError(PECS_E_ARG, "NULL argument");
    *n = (long long)h->m.n_params;
  })
}

int pecs_mlp_get_params(pecs_mlp* h, float* host) {
  NN_TRY({
    if (!h || !host) throw PecsError(PECS_E_ARG, "NULL argument");
    PECS_CUDA(cudaMemcpy(host, h->m.P.p, h->m.n_params * 4, cudaMemcpyDeviceToHost));
  })
}

int pecs_mlp_set_params(pecs_mlp* h, const float* host) {
  NN_TRY({
    if (!h || !host) throw PecsError(PECS_E_ARG, "NULL argument");
    Mlp& m = h->m;
    PECS_CUDA(cudaMemcpy(m.P.p, host, m.n_params * 4, cudaMemcpyHostToDevice));
    m.sync_bf16(m.st);
    m.Mo.zero();
    m.Vo.zero();
    m.adam_t = 0;
    PECS_CUDA(cudaStreamSynchronize(m.st));
  })
}

// y (batch x out) = network(x (batch x in)); device pointers
int pecs_mlp_forward(pecs_mlp* h, int batch, const float* x_dev, float* y_dev, void* stream) {
  NN_TRY({
    if (!h || batch < 1 || !x_dev || !y_dev) throw PecsError(PECS_E_ARG, "invalid arguments");
    Mlp& m = h->m;
    cudaStream_t s = stream ? (cudaStream_t)stream : m.st;
    m.forward(batch, x_dev, s);
    PECS_CUDA(cudaMemcpyAsync(y_dev, m.act.back().p, (size_t)batch * m.w.back() * 4,
                              cudaMemcpyDeviceToDevice, s));
    PECS_CUDA(cudaStreamSynchronize(s));
    m.check_err();
  })
}

// gradients of the MSE loss (no update); grad_host receives n_params floats
int pecs_mlp_gradients(pecs_mlp* h, int batch, const float* x_dev, const float* t_dev, float* grad_host,
                       float* loss) {
  NN_TRY({
    if (!h || batch < 1 || !x_dev || !t_dev) throw PecsError(PECS_E_ARG, "invalid arguments");
    Mlp& m = h->m;
    m.forward(batch, x_dev, m.st);
    m.backward(batch, t_dev, m.st);
    if (loss) *loss = m.read_loss(m.st, batch);
    if (grad_host) PECS_CUDA(cudaMemcpy(grad_host, m.G.p, m.n_params * 4, cudaMemcpyDeviceToHost));
    PECS_CUDA(cudaStreamSynchronize(m.st));
    m.check_err();
  })
}

// one Adam step on the MSE loss of (x, t); loss (may be NULL) returns the pre-update loss
int pecs_mlp_train_step(pecs_mlp* h, int batch, const float* x_dev, const float* t_dev, float lr,
                        float* loss) {
  NN_TRY({
    if (!h || batch < 1 || !x_dev || !t_dev || !(lr > 0)) throw PecsError(PECS_E_ARG, "invalid arguments");
    Mlp& m = h->m;
    m.forward(batch, x_dev, m.st);
    m.backward(batch, t_dev, m.st);
    m.adam(lr, m.st);
    if (loss)
      *loss = m.read_loss(m.st, batch);
    else
      PECS_CUDA(cudaStreamSynchronize(m.st));
    m.check_err();
  })
}

// Warm-start carrier vectors straight from the network's coefficients: for
// each row b, y_i = mean_i + sum_j V_ij c_bj (FP32) over the 2 n_u density
// outputs, and the full carrier vectors (nd doubles, currents zero) get
// exp(y) in their density block at u_off: electrons from y_0..y_{n_u-1},
// holes from y_{n_u}..y_{2 n_u - 1}.
__global__ void k_warm_start(int batch, int r, int n_u, const float* __restrict__ c, const float* __restrict__ V,
                             const float* __restrict__ mean, int nd, int u_off, double* __restrict__ vn,
                             double* __restrict__ vp) {
  const int b = blockIdx.y;
  extern __shared__ float cs[];
  for (int j = threadIdx.x; j < r; j += blockDim.x) cs[j] = c[(size_t)b * r + j];
  __syncthreads();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * nd; t += gridDim.x * blockDim.x) {
    const int which = t / nd, d = t - which * nd;
    double* out = (which ? vp : vn) + (size_t)b * nd;
    const int i = d - u_off;
    if (i < 0 || i >= n_u) {
      out[d] = 0.0;
      continue;
    }
    const int o = which * n_u + i;
    const float* v = V + (size_t)o * r;
    float y = mean[o];
    for (int j = 0; j < r; ++j) y = fmaf(v[j], cs[j], y);
    out[d] = (double)expf(y);
  }
}

// FP32 decoder: y (batch x n) = mean (n) + c (batch x r) V^T, V stored n x r (row-major)
int pecs_decode(int batch, int r, int n, const float* c_dev, const float* V_dev, const float* mean_dev,
                float* y_dev, void* stream) {
  NN_TRY({
    if (batch < 1 || r < 1 || n < 1 || !c_dev || !V_dev || !mean_dev || !y_dev)
      throw PecsError(PECS_E_ARG, "invalid arguments");
    cudaStream_t s = (cudaStream_t)stream;
    gemm<float, float, false, true, false>(batch, n, r, c_dev, r, V_dev, r, y_dev, n, 1.f, 0.f, nullptr,
                                           0, s);
    const size_t tot = (size_t)batch * n;
    k_add_rowvec<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(y_dev, mean_dev, batch, n);
    PECS_CUDA(cudaGetLastError());
    PECS_CUDA(cudaStreamSynchronize(s));
  })
}

int pecs_warm_start_vectors(int batch, int r, int n_u, const float* c_dev, const float* V_dev,
                            const float* mean_dev, int nd, int u_off, double* vn_dev, double* vp_dev,
                            void* stream) {
  NN_TRY({
    if (batch < 1 || r < 1 || n_u < 1 || nd < 1 || u_off < 0 || u_off + n_u > nd || !c_dev || !V_dev ||
        !mean_dev || !vn_dev || !vp_dev)
      throw PecsError(PECS_E_ARG, "invalid arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 grid((unsigned)std::min<long long>(((long long)2 * nd + 255) / 256, 1024), batch);
    k_warm_start<<<grid, 256, (size_t)r * sizeof(float), s>>>(batch, r, n_u, c_dev, V_dev, mean_dev, nd, u_off,
                                                               vn_dev, vp_dev);
    PECS_CUDA(cudaGetLastError());
    PECS_CUDA(cudaStreamSynchronize(s));
  })
}

}  // extern "C"
