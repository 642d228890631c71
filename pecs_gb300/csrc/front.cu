// FP64 factorisation of the largest multifrontal fronts on the GPU.
//
// mf_factorize (mf.cpp) assembles each front F = [F11 F12; F21 F22] (s
// fully-summed rows and columns, m update rows and columns) on the host.  For
// fronts of at least FrontOffload::min_front rows it hands the dense work to
// this file: the LU with partial pivoting among the s fully-summed rows, the
// Schur complement S = F22 - L21 U12, and the blocks the solve sweeps apply,
//   Gf = [L11^-1 P ; L21 L11^-1 P]   ((s+m) x s),
//   Hb = [U11^-1 | -U11^-1 U12]      (s x (s+m)).
// These are the numerics of the host path (dense.cpp, mf.cpp) -- the
// factorisation UMFPACK performs in Carrier::set_solver /
// PoissonData::set_solver (source/Carrier.cpp:26-32, source/Poisson.cpp:90-96
// of the reference) -- in FP64 on the device:
//   * block columns of 64: the panel (rows k0..f-1, 64 columns) is factored by
//     one CTA, column by column (pivot search over the fully-summed rows, the
//     whole row swapped, column scaled, rank-1 update of the rest of the
//     panel); the block row to its right is solved with the panel's unit
//     lower triangle (a thread per column); the trailing matrix gets the
//     rank-64 update as a DGEMM;
//   * L11^-1 and U11^-1 are built block column by block column from 64 x 64
//     diagonal-block inverses (a thread per column) and DGEMMs;
//   * Gf's lower part and Hb's right part are DGEMMs.
// The GEMMs are cuBLAS DGEMM (plain library GEMMs on row-major data, called
// as their column-major transposes); everything else is the kernels below.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "common.hpp"
#include "mf.hpp"

namespace pecs {
namespace {

constexpr int kFB = 64;            // block-column width
constexpr int kPanelThreads = 1024;

#define PECS_CUBLAS(x)                                                                     \
  do {                                                                                     \
    cublasStatus_t s_ = (x);                                                               \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                       \
      throw PecsError(PECS_E_CUDA, std::string(#x) + ": cuBLAS status " + std::to_string((int)s_)); \
  } while (0)

// C (M x N, row-major, ldc) = alpha A (M x K, lda) B (K x N, ldb) + beta C
void gemm_rm(cublasHandle_t h, int M, int N, int K, double alpha, const double* A, int lda,
             const double* B, int ldb, double beta, double* C, int ldc) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  PECS_CUBLAS(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &alpha, B, ldb, A, lda, &beta, C, ldc));
}

// One CTA: LU with partial pivoting of columns k0..k0+kb-1 of the front
// (rows k0..f-1), pivots among rows < s, whole rows swapped.  perm[t] = the
// original row now at row t.  status: -1, or the first bad column (pivot not
// above tiny or not finite; *bad receives its magnitude).
__global__ void __launch_bounds__(kPanelThreads)
    k_front_panel(int f, int s, double* __restrict__ A, int lda, int k0, int kb, int* __restrict__ perm,
                  double tiny, int* __restrict__ status, double* __restrict__ bad) {
  __shared__ double sv[32];
  __shared__ int si[32];
  __shared__ int piv_s;
  __shared__ double pv_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  if (*status >= 0) return;
  for (int j = k0; j < k0 + kb; ++j) {
    // pivot: the largest |A[r][j]| over r in [j, s), the first one on ties
    double best = -1.0;
    int bi = j;
    for (int r = j + tid; r < s; r += blockDim.x) {
      const double v = fabs(A[(size_t)r * lda + j]);
      if (v > best || (v == best && r < bi)) {
        best = v;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      sv[warp] = best;
      si[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      best = lane < nw ? sv[lane] : -1.0;
      bi = lane < nw ? si[lane] : 0x7fffffff;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) {
        piv_s = bi;
        pv_s = best;
      }
    }
    __syncthreads();
    const int piv = piv_s;
    const double pmag = pv_s;
    if (!(pmag > tiny) || !isfinite(pmag)) {
      if (tid == 0) {
        *status = j;
        *bad = pmag;
      }
      return;
    }
    if (piv != j) {
      for (int c = tid; c < f; c += blockDim.x) {
        const double a = A[(size_t)j * lda + c];
        A[(size_t)j * lda + c] = A[(size_t)piv * lda + c];
        A[(size_t)piv * lda + c] = a;
      }
      if (tid == 0) {
        const int t = perm[j];
        perm[j] = perm[piv];
        perm[piv] = t;
      }
    }
    __syncthreads();
    const double inv = 1.0 / A[(size_t)j * lda + j];
    const int ncol = k0 + kb - (j + 1);  // panel columns right of j
    // scale column j and update the panel's remaining columns, row by row
    for (int r = j + 1 + tid / 32; r < f; r += nw) {
      double* row = A + (size_t)r * lda;
      double l = 0.0;
      if (lane == 0) {
        l = row[j] * inv;
        row[j] = l;
      }
      l = __shfl_sync(0xffffffffu, l, 0);
      for (int c = lane; c < ncol; c += 32) row[j + 1 + c] -= l * A[(size_t)j * lda + j + 1 + c];
    }
    __syncthreads();
  }
}

// Rows k0..k0+kb-1, columns c0..f-1 <- L^-1 (those rows), L the unit lower
// triangle of the diagonal block at (k0, k0); a thread per column.
__global__ void k_front_trsm_rows(int f, double* __restrict__ A, int lda, int k0, int kb, int c0,
                                  const int* __restrict__ status) {
  __shared__ double L[kFB][kFB + 1];
  if (*status >= 0) return;
  for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
    const int r = t / kb, c = t - r * kb;
    L[r][c] = A[(size_t)(k0 + r) * lda + k0 + c];
  }
  __syncthreads();
  const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= f) return;
  double x[kFB];
#pragma unroll
  for (int r = 0; r < kFB; ++r)
    if (r < kb) x[r] = A[(size_t)(k0 + r) * lda + c];
#pragma unroll
  for (int r = 1; r < kFB; ++r) {
    if (r >= kb) break;
    double acc = x[r];
#pragma unroll
    for (int t = 0; t < kFB; ++t)
      if (t < r) acc -= L[r][t] * x[t];
    x[r] = acc;
  }
#pragma unroll
  for (int r = 1; r < kFB; ++r)
    if (r < kb) A[(size_t)(k0 + r) * lda + c] = x[r];
}

// Inverses of the diagonal blocks (b x b, b <= 64) of an n x n triangle:
// lower unit (lower = 1) or upper with its diagonal (lower = 0); block J's
// inverse goes to X at (J*64, J*64); a thread per column of a block.
__global__ void k_front_tri_inv_blocks(int n, const double* __restrict__ T, int ldt, double* __restrict__ X,
                                       int ldx, int lower) {
  __shared__ double Ts[kFB][kFB + 1];
  const int o = blockIdx.x * kFB, b = min(kFB, n - o);
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
    const int r = t / b, c = t - r * b;
    Ts[r][c] = T[(size_t)(o + r) * ldt + o + c];
  }
  __syncthreads();
  const int j = threadIdx.x;
  if (j >= b) return;
  double x[kFB];
  if (lower) {
    // L x = e_j, unit diagonal: x_r = delta_rj - sum_{t<r} L_rt x_t
#pragma unroll
    for (int r = 0; r < kFB; ++r) {
      if (r >= b) break;
      double acc = (r == j) ? 1.0 : 0.0;
#pragma unroll
      for (int t = 0; t < kFB; ++t)
        if (t < r) acc -= Ts[r][t] * x[t];
      x[r] = acc;
    }
  } else {
    // U x = e_j: x_r = (delta_rj - sum_{t>r} U_rt x_t) / U_rr, r from the bottom
#pragma unroll
    for (int rr = 0; rr < kFB; ++rr) {
      const int r = b - 1 - rr;
      if (r < 0) break;
      double acc = (r == j) ? 1.0 : 0.0;
#pragma unroll
      for (int t = 0; t < kFB; ++t)
        if (t > r && t < b) acc -= Ts[r][t] * x[t];
      x[r] = acc / Ts[r][r];
    }
  }
#pragma unroll
  for (int r = 0; r < kFB; ++r)
    if (r < b) X[(size_t)(o + r) * ldx + o + j] = x[r];
}

// X (n x n) = T^-1 for the unit lower (lower = 1) or upper (lower = 0)
// triangle of T, block column by block column: for lower, from the last
// block to the first, X[J+, J] = -X[J+, J+] (L[J+, J] X[J, J]); for upper,
// from the first to the last, X[:J, J] = -(X[:J, :J] U[:J, J]) X[J, J].  X's
// other triangle is zero.  tmp: n x 64.
void tri_inverse(cublasHandle_t h, cudaStream_t st, int n, const double* T, int ldt, double* X, int ldx,
                 double* tmp, bool lower) {
  PECS_CUDA(cudaMemset2DAsync(X, (size_t)ldx * sizeof(double), 0, (size_t)n * sizeof(double), n, st));
  const int nb = (n + kFB - 1) / kFB;
  k_front_tri_inv_blocks<<<nb, kFB, 0, st>>>(n, T, ldt, X, ldx, lower ? 1 : 0);
  PECS_CUDA(cudaGetLastError());
  if (lower) {
    for (int J = nb - 2; J >= 0; --J) {
      const int o = J * kFB, b = kFB, r0 = o + b, nr = n - r0;
      // tmp (nr x b) = L[r0:, o:o+b] X[o:o+b, o:o+b]
      gemm_rm(h, nr, b, b, 1.0, T + (size_t)r0 * ldt + o, ldt, X + (size_t)o * ldx + o, ldx, 0.0, tmp, kFB);
      // X[r0:, o:o+b] = -X[r0:, r0:] tmp  (X[r0:, r0:] lower triangular, zeros above)
      gemm_rm(h, nr, b, nr, -1.0, X + (size_t)r0 * ldx + r0, ldx, tmp, kFB, 0.0, X + (size_t)r0 * ldx + o, ldx);
    }
  } else {
    for (int J = 1; J < nb; ++J) {
      const int o = J * kFB, b = std::min(kFB, n - o);
      // tmp (o x b) = X[:o, :o] U[:o, o:o+b]
      gemm_rm(h, o, b, o, 1.0, X, ldx, T + o, ldt, 0.0, tmp, kFB);
      // X[:o, o:o+b] = -tmp X[o:o+b, o:o+b]
      gemm_rm(h, o, b, b, -1.0, tmp, kFB, X + (size_t)o * ldx + o, ldx, 0.0, X + o, ldx);
    }
  }
}

// G[r][perm[t]] = X[r][t] (the column permutation of Gf)
__global__ void k_front_permute_cols(int rows, int s, const double* __restrict__ X, const int* __restrict__ perm,
                                     double* __restrict__ G) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * s) return;
  const int r = (int)(i / s), t = (int)(i - (size_t)r * s);
  G[(size_t)r * s + perm[t]] = X[i];
}

struct GpuFront {
  std::mutex mu;
  int device = 0;
  cudaStream_t st = nullptr;
  cublasHandle_t h = nullptr;
  ~GpuFront() {
    if (h) cublasDestroy(h);
    if (st) cudaStreamDestroy(st);
  }
};

int gpu_factor_front(void* ctx, int f, int s, const double* Fm, double tiny, int* perm, double* bad,
                     std::vector<double>& G, std::vector<double>& H, std::vector<double>& S) {
  GpuFront& g = *static_cast<GpuFront*>(ctx);
  std::lock_guard<std::mutex> lock(g.mu);
  PECS_CUDA(cudaSetDevice(g.device));
  if (!g.st) {
    PECS_CUDA(cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking));
    PECS_CUBLAS(cublasCreate(&g.h));
    PECS_CUBLAS(cublasSetStream(g.h, g.st));
    PECS_CUBLAS(cublasSetMathMode(g.h, CUBLAS_DEFAULT_MATH));
  }
  cudaStream_t st = g.st;
  const int m = f - s;
  DBuf<double> A, X, T, Gd, Hd;
  DBuf<int> permd, status;
  DBuf<double> badd;
  A.alloc((size_t)f * f);
  PECS_CUDA(cudaMemcpyAsync(A.p, Fm, (size_t)f * f * sizeof(double), cudaMemcpyHostToDevice, st));
  std::vector<int> p0(s);
  for (int t = 0; t < s; ++t) p0[t] = t;
  permd.alloc(s);
  PECS_CUDA(cudaMemcpyAsync(permd.p, p0.data(), (size_t)s * sizeof(int), cudaMemcpyHostToDevice, st));
  status.alloc(1);
  const int minus1 = -1;
  PECS_CUDA(cudaMemcpyAsync(status.p, &minus1, sizeof(int), cudaMemcpyHostToDevice, st));
  badd.alloc(1);
  // LU of the first s columns, block column by block column
  for (int k0 = 0; k0 < s; k0 += kFB) {
    const int kb = std::min(kFB, s - k0), k1 = k0 + kb;
    k_front_panel<<<1, kPanelThreads, 0, st>>>(f, s, A.p, f, k0, kb, permd.p, tiny, status.p, badd.p);
    PECS_CUDA(cudaGetLastError());
    if (k1 < f) {
      k_front_trsm_rows<<<(f - k1 + 127) / 128, 128, 0, st>>>(f, A.p, f, k0, kb, k1, status.p);
      PECS_CUDA(cudaGetLastError());
      gemm_rm(g.h, f - k1, f - k1, kb, -1.0, A.p + (size_t)k1 * f + k0, f, A.p + (size_t)k0 * f + k1, f, 1.0,
              A.p + (size_t)k1 * f + k1, f);
    }
  }
  int stat = -1;
  PECS_CUDA(cudaMemcpyAsync(&stat, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  PECS_CUDA(cudaStreamSynchronize(st));
  if (stat >= 0) {
    PECS_CUDA(cudaMemcpy(bad, badd.p, sizeof(double), cudaMemcpyDeviceToHost));
    return stat;
  }
  // S = A[s:, s:]
  S.assign((size_t)m * m, 0.0);
  if (m > 0)
    PECS_CUDA(cudaMemcpy2DAsync(S.data(), (size_t)m * sizeof(double), A.p + (size_t)s * f + s,
                                (size_t)f * sizeof(double), (size_t)m * sizeof(double), m,
                                cudaMemcpyDeviceToHost, st));
  X.alloc((size_t)s * s);
  T.alloc((size_t)std::max(s, 1) * kFB);
  // Gf: X = L11^-1, then [X ; L21 X] with the columns permuted
  tri_inverse(g.h, st, s, A.p, f, X.p, s, T.p, true);
  Gd.alloc((size_t)f * s);
  {
    DBuf<double> Gx;
    Gx.alloc((size_t)f * s);
    PECS_CUDA(cudaMemcpyAsync(Gx.p, X.p, (size_t)s * s * sizeof(double), cudaMemcpyDeviceToDevice, st));
    gemm_rm(g.h, m, s, s, 1.0, A.p + (size_t)s * f, f, X.p, s, 0.0, Gx.p + (size_t)s * s, s);
    const size_t tot = (size_t)f * s;
    k_front_permute_cols<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(f, s, Gx.p, permd.p, Gd.p);
    PECS_CUDA(cudaGetLastError());
    PECS_CUDA(cudaStreamSynchronize(st));
  }
  // Hb: [U11^-1 | -U11^-1 U12]
  Hd.alloc((size_t)s * f);
  tri_inverse(g.h, st, s, A.p, f, X.p, s, T.p, false);
  PECS_CUDA(cudaMemcpy2DAsync(Hd.p, (size_t)f * sizeof(double), X.p, (size_t)s * sizeof(double),
                              (size_t)s * sizeof(double), s, cudaMemcpyDeviceToDevice, st));
  gemm_rm(g.h, s, m, s, -1.0, X.p, s, A.p + s, f, 0.0, Hd.p + s, f);
  G.resize((size_t)f * s);
  H.resize((size_t)s * f);
  PECS_CUDA(cudaMemcpyAsync(G.data(), Gd.p, (size_t)f * s * sizeof(double), cudaMemcpyDeviceToHost, st));
  PECS_CUDA(cudaMemcpyAsync(H.data(), Hd.p, (size_t)s * f * sizeof(double), cudaMemcpyDeviceToHost, st));
  PECS_CUDA(cudaMemcpyAsync(perm, permd.p, (size_t)s * sizeof(int), cudaMemcpyDeviceToHost, st));
  PECS_CUDA(cudaStreamSynchronize(st));
  return -1;
}

}  // namespace

std::shared_ptr<FrontOffload> make_gpu_front_offload(int device, int min_front) {
  auto g = std::make_shared<GpuFront>();
  g->device = device;
  auto off = std::shared_ptr<FrontOffload>(new FrontOffload(), [g](FrontOffload* p) { delete p; });
  off->min_front = min_front;
  off->ctx = g.get();
  off->factor = &gpu_factor_front;
  return off;
}

}  // namespace pecs
