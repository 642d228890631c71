// GB300 engine for the PECS IMEX time step and the C ABI (include/pecs.h).
//
// Data layout in HBM (everything resident after pecs_create):
//   state[2][field]  ping-pong state vectors, [instance][ndofs(field)] FP64,
//                    field-major so a kernel reads one instance's vector
//                    contiguously; carrier vectors are component-wise
//                    [J_x | J_y | u] with the cell's dofs contiguous.
//   rhs/y[field]     assembled right-hand sides / forward-sweep slots.
//   bconst[field]    time-independent RHS parts (generation, Dirichlet data,
//                    doping), per instance.
//   carrier and Poisson FactorBanks (solve.cuh) + per-RHS update workspaces.
// A step is: carrier RHS (1 launch) -> carrier solves (one launch per tree
// level for all carriers and instances) -> Poisson RHS (1) -> Poisson solve
// -> steady-state reduction (2) + snapshot (1).  pecs_run_to_steady_state
// replays a CUDA graph of two steps (even/odd ping-pong).
#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
#include <condition_variable>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <type_traits>
#include <string>
#include <vector>

#include "common.hpp"
#include "fp_bits.cuh"
#include "mf.hpp"
#include "problem.hpp"
#include "rhs_kernels.cuh"
#include "solve.cuh"

namespace pecs {

namespace {

thread_local std::string g_last_error;

void set_error(const std::string& m) { g_last_error = m; }

// ---------------------------------------------------------------------------
// small kernels: residual, axpy, steady-state test, interface current
// ---------------------------------------------------------------------------

struct CsrDev {
  const int* rp;
  const int* ci;
  const double* v;
};

struct CsrSet {
  CsrDev m[5];
};

struct CsrDf {  // matrix values split into FP32 (hi, lo) pairs
  const int* rp;
  const int* ci;
  const float2* v;
};

struct CsrDfSet {
  CsrDf m[5];
};

// ---- interleaved [dof][rhs] buffers of the batched solves --------------------
// dst[d * R + k] = src_k[d]   (32 x 32 tiles through shared memory); dst32,
// when given, receives the same values rounded to float (the right-hand sides
// of the FP32 sweeps)
__global__ void k_gather_il(const double* const* __restrict__ src, double* __restrict__ dst,
                            float* __restrict__ dst32, int n, int R) {
  __shared__ double t[32][33];
  const int d0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk, d = d0 + threadIdx.x;
    t[kk][threadIdx.x] = (k < R && d < n) ? src[k][d] : 0.0;
  }
  __syncthreads();
  for (int dd = threadIdx.y; dd < 32; dd += blockDim.y) {
    const int d = d0 + dd, k = k0 + threadIdx.x;
    if (d < n && k < R) {
      const double v = t[threadIdx.x][dd];
      dst[(size_t)d * R + k] = v;
      if (dst32) dst32[(size_t)d * R + k] = (float)v;
    }
  }
}

// dst_k[d] = src[d * R + k]
// mask (optional): only columns of instances k / nf with mask[k / nf] != 0
template <typename V>
__global__ void k_scatter_il(const V* __restrict__ src, double* const* __restrict__ dst, int n,
                             int R, const int* __restrict__ mask, int nf) {
  __shared__ double t[32][33];
  const int d0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int dd = threadIdx.y; dd < 32; dd += blockDim.y) {
    const int d = d0 + dd, k = k0 + threadIdx.x;
    t[dd][threadIdx.x] = (d < n && k < R) ? (double)src[(size_t)d * R + k] : 0.0;
  }
  __syncthreads();
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk, d = d0 + threadIdx.x;
    if (k < R && d < n && (!mask || mask[k / nf])) dst[k][d] = t[threadIdx.x][kk];
  }
}

__global__ void k_split_il(const double* __restrict__ x, float2* __restrict__ xs, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = x[i];
  const float hi = __double2float_rn(a);
  xs[i] = make_float2(hi, __double2float_rn(a - (double)hi));
}

template <typename V>
__global__ void k_axpy_il(double* __restrict__ x, const V* __restrict__ d, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
}

// dst_k[d] = (double) x32[d * R + k] + (double) d32[d * R + k]: the refined
// solution of an FP32 sweep and its one correction, written to the state
__global__ void k_scatter_sum_il(const float* __restrict__ x32, const float* __restrict__ d32,
                                 double* const* __restrict__ dst, int n, int R,
                                 const int* __restrict__ mask, int nf) {
  __shared__ double t[32][33];
  const int d0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int dd = threadIdx.y; dd < 32; dd += blockDim.y) {
    const int d = d0 + dd, k = k0 + threadIdx.x;
    const size_t o = (size_t)d * R + k;
    t[dd][threadIdx.x] = (d < n && k < R) ? f2d_exact(x32[o]) + f2d_exact(d32[o]) : 0.0;
  }
  __syncthreads();
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk, d = d0 + threadIdx.x;
    if (k < R && d < n && (!mask || mask[k / nf])) dst[k][d] = t[threadIdx.x][kk];
  }
}

// dst[d * R + k] = src[k][d] as an FP32 pair (the previous step's solution,
// interleaved for the residual of an increment solve)
__global__ void k_gather_pairs_il(const double* const* __restrict__ src, float2* __restrict__ dst, int n, int R) {
  __shared__ double t[32][33];
  const int d0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk, d = d0 + threadIdx.x;
    t[kk][threadIdx.x] = (k < R && d < n) ? src[k][d] : 0.0;
  }
  __syncthreads();
  for (int dd = threadIdx.y; dd < 32; dd += blockDim.y) {
    const int d = d0 + dd, k = k0 + threadIdx.x;
    if (d < n && k < R) dst[(size_t)d * R + k] = d2ff(t[threadIdx.x][dd]);
  }
}

// dst_k[d] = old_k[d] + (double) d32[d * R + k]: the previous step's solution
// plus the increment an increment solve found
__global__ void k_scatter_delta_il(const float* __restrict__ d32, const double* const* __restrict__ old,
                                   double* const* __restrict__ dst, int n, int R, const int* __restrict__ mask,
                                   int nf) {
  __shared__ float t[32][33];
  const int d0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int dd = threadIdx.y; dd < 32; dd += blockDim.y) {
    const int d = d0 + dd, k = k0 + threadIdx.x;
    t[dd][threadIdx.x] = (d < n && k < R) ? d32[(size_t)d * R + k] : 0.f;
  }
  __syncthreads();
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk, d = d0 + threadIdx.x;
    // FP32-pair sum converted with integer operations (FP64 additions are
    // the scarce resource on GB300): the state keeps ~47 bits of the update
    if (k < R && d < n && (!mask || mask[k / nf]))
      dst[k][d] = ff2d_i32(ff_add(d2ff(old[k][d]), t[threadIdx.x][kk]));
  }
}

// x = (double) x32 + (double) d32
__global__ void k_sum_il(const float* __restrict__ x32, const float* __restrict__ d32,
                         double* __restrict__ x, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] = (double)x32[i] + (double)d32[i];
}

__global__ void k_widen_il(const float* __restrict__ x32, double* __restrict__ x, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) x[i] = (double)x32[i];
}

// r = b - A x for R right-hand sides sharing A: one warp per row, lanes over
// right-hand sides (matrix entries broadcast, vectors read contiguously).
// The sum runs in FP32-pair ("double-float") arithmetic: products are exact
// through fmaf, partial sums through TwoSum, so the residual keeps ~46-bit
// accuracy while running on the FP32 pipe.
// X is float2 (an FP32 pair) or float (a pair with zero low part: the first
// refinement of an FP32 sweep's solution); RT the residual's storage type.
__device__ __forceinline__ float2 as_pair(float2 v) { return v; }
__device__ __forceinline__ float2 as_pair(float v) { return make_float2(v, 0.f); }

// b - (sh + sl): for a float residual (the next sweep's input) entirely in
// FP32 pairs, b split on the integer pipe; for a double residual in FP64
template <typename RT>
__device__ __forceinline__ RT df_residual(double b, float sh, float sl) {
  if constexpr (sizeof(RT) == 4) {
    const float2 t = ff_add(d2ff(b), make_float2(-sh, -sl));
    return t.x + t.y;
  } else {
    return b - ((double)sh + (double)sl);
  }
}

// b: interleaved right-hand sides, or (bt non-null) a table of per-RHS
// vectors read in place (one 8-byte load per lane; saves the transposing
// gather of an increment solve)
template <typename X, typename RT>
__global__ void k_residual_df_il(CsrDf A, const double* __restrict__ b, const double* const* __restrict__ bt,
                                 const X* __restrict__ xs, RT* __restrict__ r, int n, int R) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int k = blockIdx.y * 32 + (threadIdx.x & 31);
  if (row >= n || k >= R) return;
  float sh = 0.f, sl = 0.f;
  for (int p = A.rp[row]; p < A.rp[row + 1]; ++p) {
    const float2 a = A.v[p], xv = as_pair(xs[(size_t)A.ci[p] * R + k]);
    const float ph = a.x * xv.x;
    const float pe = fmaf(a.x, xv.x, -ph) + fmaf(a.x, xv.y, a.y * xv.x);
    const float t = sh + ph;
    const float z = t - sh;
    const float e = (sh - (t - z)) + (ph - z);
    sh = t;
    sl += e + pe;
  }
  const size_t o = (size_t)row * R + k;
  r[o] = df_residual<RT>(bt ? bt[k][row] : b[o], sh, sl);
}

// Four right-hand sides per lane (128 per warp, R a multiple of 4): the row's
// column indices and values are read once for all of them and every x row is
// one 512 B (float) / 1 KB (pair) coalesced access.  Same arithmetic as above.
__device__ __forceinline__ void ld_pairs4(const float* p, float2 (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = make_float2(t.x, 0.f);
  v[1] = make_float2(t.y, 0.f);
  v[2] = make_float2(t.z, 0.f);
  v[3] = make_float2(t.w, 0.f);
}
__device__ __forceinline__ void ld_pairs4(const float2* p, float2 (&v)[4]) {
  const float4 t0 = reinterpret_cast<const float4*>(p)[0], t1 = reinterpret_cast<const float4*>(p)[1];
  v[0] = make_float2(t0.x, t0.y);
  v[1] = make_float2(t0.z, t0.w);
  v[2] = make_float2(t1.x, t1.y);
  v[3] = make_float2(t1.z, t1.w);
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

template <typename X, typename RT>
__global__ void k_residual_df_il4(CsrDf A, const double* __restrict__ b, const double* const* __restrict__ bt,
                                  const X* __restrict__ xs, RT* __restrict__ r, int n, int R) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int k = blockIdx.y * 128 + (threadIdx.x & 31) * 4;
  if (row >= n || k >= R) return;
  float sh[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f};
  const int p1 = A.rp[row + 1];
  for (int p = A.rp[row]; p < p1; ++p) {
    const float2 a = A.v[p];
    float2 xv[4];
    ld_pairs4(xs + (size_t)A.ci[p] * R + k, xv);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float ph = a.x * xv[q].x;
      const float pe = fmaf(a.x, xv[q].x, -ph) + fmaf(a.x, xv[q].y, a.y * xv[q].x);
      const float t = sh[q] + ph;
      const float z = t - sh[q];
      const float e = (sh[q] - (t - z)) + (ph - z);
      sh[q] = t;
      sl[q] += e + pe;
    }
  }
  const size_t o = (size_t)row * R + k;
  double bb[4];
  if (bt) {
#pragma unroll
    for (int q = 0; q < 4; ++q) bb[q] = bt[k + q][row];
  } else {
    const double2 b0 = reinterpret_cast<const double2*>(b + o)[0], b1 = reinterpret_cast<const double2*>(b + o)[1];
    bb[0] = b0.x, bb[1] = b0.y, bb[2] = b1.x, bb[3] = b1.y;
  }
  RT v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = df_residual<RT>(bb[q], sh[q], sl[q]);
  st4(r + o, v);
}

template <typename X, typename RT>
void launch_residual_df(const CsrDf& A, const double* b, const X* xs, RT* r, int n, int R, cudaStream_t s,
                        const double* const* bt = nullptr) {
  if (R % 4 == 0 && R >= 96)
    k_residual_df_il4<X, RT><<<dim3((n + 7) / 8, (R + 127) / 128), 256, 0, s>>>(A, b, bt, xs, r, n, R);
  else
    k_residual_df_il<X, RT><<<dim3((n + 7) / 8, (R + 31) / 32), 256, 0, s>>>(A, b, bt, xs, r, n, R);
  PECS_CUDA(cudaGetLastError());
}

// ||b - A x||^2 and ||b||^2 of one instance-major vector pair (grid.y =
// instance), accumulated in FP64 (diagnostic: the residual a solve reached)
__global__ void k_residual_norms(CsrDev A, const double* __restrict__ b, const double* __restrict__ x, int n,
                                 double* __restrict__ sums) {
  const int i = blockIdx.y;
  const double* bi = b + (size_t)i * n;
  const double* xi = x + (size_t)i * n;
  double r2 = 0.0, b2 = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int p = A.rp[row]; p < A.rp[row + 1]; ++p) acc += A.v[p] * xi[A.ci[p]];
    const double r = bi[row] - acc;
    r2 += r * r;
    b2 += bi[row] * bi[row];
  }
  for (int o = 16; o > 0; o >>= 1) {
    r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    b2 += __shfl_xor_sync(0xffffffffu, b2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums + 2 * i, r2);
    atomicAdd(sums + 2 * i + 1, b2);
  }
}

// FP64 variant (FP32_IR mode)
template <typename RT>
__global__ void k_residual_il(CsrDev A, const double* __restrict__ b, const double* __restrict__ x,
                              RT* __restrict__ r, int n, int R) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int k = blockIdx.y * 32 + (threadIdx.x & 31);
  if (row >= n || k >= R) return;
  double acc = 0.0;
  for (int p = A.rp[row]; p < A.rp[row + 1]; ++p) acc += A.v[p] * x[(size_t)A.ci[p] * R + k];
  const size_t o = (size_t)row * R + k;
  r[o] = (RT)(b[o] - acc);
}

constexpr int kRedThreads = 256;
constexpr int kRedChunks = 16;

// partial sums of |new-old|^2 and |new|^2: grid (kRedChunks, 5 fields, n_inst).
// The difference is always formed in FP64 (a 1e-8 relative change is below
// FP32 resolution); Acc is the type the squares are summed in.
template <typename Acc>
__global__ void k_relchange_partial(FieldPtrs NEW, FieldPtrs OLD, int n_fields,
                                    double2* __restrict__ partial) {
  const int chunk = blockIdx.x, fld = blockIdx.y, i = blockIdx.z;
  __shared__ double sd[kRedThreads], sn[kRedThreads];
  Acc d2 = 0, n2 = 0;
  if (fld < n_fields) {
    const int f = fld == n_fields - 1 ? 4 : fld;
    const int nd = NEW.nd[f];
    const double* a = NEW.u[f] + (size_t)i * nd;
    const double* b = OLD.u[f] + (size_t)i * nd;
    const int per = (nd + kRedChunks - 1) / kRedChunks;
    const int lo = chunk * per, hi = min(nd, lo + per);
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      const double x = a[t], y = b[t];
      Acc d, xa;
      if constexpr (sizeof(Acc) == 4) {
        d = d2f_trunc(x - y);  // the one FP64 operation per element
        xa = d2f_trunc(x);
      } else {
        d = x - y;
        xa = x;
      }
      d2 += d * d;
      n2 += xa * xa;
    }
  }
  sd[threadIdx.x] = (double)d2;
  sn[threadIdx.x] = (double)n2;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sd[threadIdx.x] += sd[threadIdx.x + o];
      sn[threadIdx.x] += sn[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    partial[((size_t)i * 5 + fld) * kRedChunks + chunk] = make_double2(sd[0], sn[0]);
}

// Per-instance convergence test after a step (rel = max over fields of
// sqrt(d2 / n2)).  An active instance stops when
// its relative change is <= tol (conv_step = the step), when its state is not
// finite (conv_step = -step), or when it has marched max_steps since its start
// step (conv_step = the step, capped = 1; streamed sweeps refill such slots).
__global__ void k_converge(const double2* __restrict__ partial, int n_inst, int n_fields, double tol,
                           int* __restrict__ conv_step, double* __restrict__ rel,
                           int* __restrict__ step_ctr, int* __restrict__ active,
                           int* __restrict__ n_active, const int* __restrict__ start, int max_steps,
                           int* __restrict__ capped) {
  const int step = *step_ctr + 1;
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n_inst; i += blockDim.x) {
    double r = 0.0;
    bool finite = true;
    for (int fld = 0; fld < n_fields; ++fld) {
      double d2 = 0.0, n2 = 0.0;
      for (int c = 0; c < kRedChunks; ++c) {
        const double2 v = partial[((size_t)i * 5 + fld) * kRedChunks + c];
        d2 += v.x;
        n2 += v.y;
      }
      finite = finite && isfinite(d2) && isfinite(n2);
      const double q = n2 > 0.0 ? sqrt(d2 / n2) : sqrt(d2);
      r = fmax(r, q);
    }
    if (active[i]) {
      rel[i] = finite ? r : __longlong_as_double(0x7ff8000000000000LL);
      if (!finite) {
        active[i] = 0;
        conv_step[i] = -step;  // non-finite state: stopped, reported as failure
      } else if (r <= tol) {
        active[i] = 0;
        conv_step[i] = step;
      } else if (step - start[i] >= max_steps) {
        active[i] = 0;
        conv_step[i] = step;
        capped[i] = 1;
      }
    }
    if (active[i]) atomicAdd(&cnt, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *step_ctr = step;
    *n_active = cnt;
  }
}

// I_Sigma per instance: one block per instance, threads over interface faces
__global__ void k_interface_current(Tables T, RegionDev semi, RegionDev elec, FieldPtrs F,
                                    const InstDev* __restrict__ inst, const double* __restrict__ ne,
                                    const double* __restrict__ pe, const int* __restrict__ isemi,
                                    const int* __restrict__ ielec, int n_iface, int n1, int nq,
                                    double* __restrict__ out) {
  const int i = blockIdx.x;
  const InstDev P = inst[i];
  __shared__ double sacc[kRedThreads];
  double acc = 0.0;
  for (int t = threadIdx.x; t < n_iface; t += blockDim.x) {
    const int Ks = isemi[t], Ke = ielec[t];
    const double* un = F.u[0] + (size_t)i * F.nd[0] + 2 * semi.nc * n1 + Ks * n1;
    const double* up = F.u[1] + (size_t)i * F.nd[1] + 2 * semi.nc * n1 + Ks * n1;
    const double* ur = F.u[2] + (size_t)i * F.nd[2] + 2 * elec.nc * n1 + Ke * n1;
    const double* uo = F.u[3] + (size_t)i * F.nd[3] + 2 * elec.nc * n1 + Ke * n1;
    const double hy = semi.h[Ks].y;
    for (int q = 0; q < nq; ++q) {
      double n = 0, p = 0, r = 0, o = 0;
      for (int a = 0; a < n1; ++a) {
        const double fs = T.fphi[(semi.iface_face * n1 + a) * nq + q];
        const double fe = T.fphi[(elec.iface_face * n1 + a) * nq + q];
        n += fs * un[a];
        p += fs * up[a];
        r += fe * ur[a];
        o += fe * uo[a];
      }
      const size_t o2 = (size_t)i * n_iface * nq + (size_t)t * nq + q;
      acc += (P.k_et * (n - ne[o2]) * o - P.k_ht * (p - pe[o2]) * r) * T.fw[q] * hy;
    }
  }
  sacc[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sacc[threadIdx.x] += sacc[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[i] = sacc[0];
}

// copy state of instances that converged at this step into the snapshot
__global__ void k_snapshot(FieldPtrs NEW, double* const* snap, const int* __restrict__ conv_step,
                           const int* __restrict__ step_ctr, int n_fields_total) {
  const int i = blockIdx.z, f = blockIdx.y;
  if (f >= n_fields_total) return;
  const int cs = conv_step[i];
  const int step = *step_ctr;
  if (cs != step && cs != -step) return;
  const int nd = NEW.nd[f];
  const double* a = NEW.u[f] + (size_t)i * nd;
  double* b = snap[f] + (size_t)i * nd;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nd; t += gridDim.x * blockDim.x) b[t] = a[t];
}


}  // namespace

// error message hook for the other translation units of the library
void set_error_external(const std::string& m) { g_last_error = m; }

// ---------------------------------------------------------------------------
// Engine
// ---------------------------------------------------------------------------

struct SetTable {  // device pointer arrays of one SetsView
  std::vector<DBuf<double*>> b, y, w, x;
  SetsView view{};
  int max_nrhs = 0;
};

struct Engine {
  pecs_options opt{};
  std::unique_ptr<Setup> S;
  int n_inst = 0;
  int n_fields = 5;  // fields in use (3 for semiconductor only: n, p, P)
  bool host_only = false;
  bool full = true;
  int nd[5] = {0, 0, 0, 0, 0};
  double setup_seconds = 0.0;
  cudaStream_t st = nullptr;
  // factors
  MfFactor fs[2], fe[2], fp;
  int n_fs = 0, n_fe = 0;
  FactorBank bank_c, bank_p;
  // device matrices (for refinement residuals)
  DBuf<int> A_rp[5], A_ci[5];
  DBuf<double> A_v[5];
  CsrSet csr{};
  // tables and regions
  DBuf<double> t_phi, t_qw, t_fphi, t_fw, t_psix, t_psiy, t_phiP, t_mref;
  DBuf<float> tf_phi, tf_qw, tf_fphi, tf_fw, tf_psix, tf_psiy;
  DBuf<double> t_drift_x, t_drift_y;
  DBuf<float2> t_drift_x_ff, t_drift_y_ff, t_mref_ff;
  DBuf<int> t_drift_cx, t_drift_cy;
  DBuf<double> t_charge;
  Tables T{};
  DBuf<double2> h_[2], ph_[2];
  DBuf<int4> bid_[2];
  DBuf<int> rt_[2], phid_[2], partner_[2], iface_[2];
  RegionDev R[2]{};
  DBuf<InstDev> inst;
  DBuf<double> iface_ne, iface_pe, sch_ne, sch_pe;
  DBuf<int> isemi, ielec;
  // vectors
  DBuf<double> state[2][5], rhs[5], bconst[5], snap[5], init_dev[4];
  int cur = 0;
  bool carriers_advanced = false;
  bool initialized = false;
  // interleaved buffers of the batched solves, per bank (0 carriers, 1 Poisson) and set
  struct IlSet {
    int n = 0, R = 0, mat = 0;
    bool f32 = false;              // panel bank with FP32 factors: float sweep vectors
    DBuf<double> B, Y, W, X, Rr, D;
    DBuf<float> B32, Y32, W32, X32, D32, Rr32;
    DBuf<float2> Xs;
    DBuf<const double*> src;       // rhs vector of each column
    DBuf<double*> dst[2];          // state vector of each column, per ping-pong target
  };
  struct IlBank {
    int n_sets = 0;
    IlSet set[kMaxSets];
    int max_R = 0;
  };
  IlBank il[2];
  DBuf<double*> snap_ptrs;
  // steady state
  DBuf<double2> partial;
  DBuf<int> conv_step, step_ctr, active, n_active, start_step, capped, refill_mask;
  int step_cap = 1 << 30;  // per-instance step cap seen by k_converge (streamed sweeps)
  const int* scatter_mask = nullptr;  // solves write only these instances (slot refills)
  DBuf<double> rel;
  // graphs
  cudaGraphExec_t graph2[2] = {nullptr, nullptr};  // two steps starting from cur = 0 / 1
  bool graph_valid = false;
  // refinement sweeps per solve of bank `which` (0 carriers, 1 Poisson):
  // ir_max_iters > 0 sets the count, < 0 disables refinement, 0 selects the
  // default -- two for FP32_IR, one for FP32_MIXED and for FP64 factors.  The
  // FP64 step is what UMFPACK's default control does in
  // SparseDirectUMFPACK::solve, which the reference's Carrier::solve and
  // PoissonData::solve call (Carrier.cpp:34-40, Poisson.cpp:98-105): without
  // it the explicit-inverse sweeps leave the Poisson field of a coupled
  // trajectory ~1e-9 from exact arithmetic at 64x64 cells after 60 steps (the
  // net charge on its right-hand side nearly cancels, so the carrier solves'
  // errors are amplified there, and the same on the single-instance and the
  // batched paths: it is the stored factors' rounding, not the sweeps'); with
  // it, ~2e-12
  int ir_iters(int which) const {
    (void)which;
    if (opt.ir_max_iters < 0) return 0;
    if (opt.ir_max_iters > 0) return opt.ir_max_iters;
    return opt.precision == PECS_PREC_FP32_IR ? 2 : 1;
  }
  // element-wise launches per set of one solve: gather, scatter and, per
  // refinement sweep, the residual and its helpers (split / widen, axpy / sum)
  int set_launches_per_solve(int which) const {
    const int iters = ir_iters(which);
    const bool mixed = opt.precision == PECS_PREC_FP32_MIXED;
    int n = 2;
    for (int it = 0; it < iters; ++it) {
      if (il_f32(which))
        n += mixed ? (it == 0 ? (iters == 1 ? 1 : 2) : 3) : (it == 0 ? 3 : 2);
      else
        n += mixed ? 3 : 2;
    }
    return n;
  }
  // Poisson RHS + Poisson solve
  int initialize_launches() const {
    return 1 + bank_p.kernel_launches_per_solve() * (1 + ir_iters(1)) + il[1].n_sets * set_launches_per_solve(1);
  }
  int launches_per_step() const {
    const int lc = bank_c.kernel_launches_per_solve(), lp = bank_p.kernel_launches_per_solve();
    const int sc = il[0].n_sets, sp = il[1].n_sets;
    // increment solves: gather of the previous solution, residual and
    // scatter per set, one sweep
    const bool dc = delta_solves() && il_f32(0), dp = delta_solves() && il_f32(1);
    return 1 + (dc ? lc + 3 * sc : lc * (1 + ir_iters(0)) + sc * set_launches_per_solve(0)) + 1 +
           (dp ? lp + 3 * sp : lp * (1 + ir_iters(1)) + sp * set_launches_per_solve(1)) + 3;
  }
  // algorithmic bytes of one application of a bank to all of its right-hand
  // sides: every stored factor entry once, plus the vectors (b read, y write +
  // read, x write, update vectors write + read, in the sweep's vector type:
  // float for FP32 panel banks, else double)
  double solve_bytes(int which) const {
    const FactorBank& B = which == 0 ? bank_c : bank_p;
    const IlBank& I = il[which];
    double vec = 0.0;
    for (int si = 0; si < I.n_sets; ++si) {
      const IlSet& S_ = I.set[si];
      const double vb = S_.f32 ? 4.0 : 8.0;
      vec += (double)S_.R * (4.0 * vb * S_.n + 2.0 * vb * B.set_wtotal(si));
    }
    return (double)B.bytes() + vec;
  }
  double time_solves(int which, int reps) {
    cudaEvent_t e0, e1;
    PECS_CUDA(cudaEventCreate(&e0));
    PECS_CUDA(cudaEventCreate(&e1));
    const FactorBank& B = which == 0 ? bank_c : bank_p;
    bank_sweep(B, which, false, st);  // warm
    PECS_CUDA(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) bank_sweep(B, which, false, st);
    PECS_CUDA(cudaEventRecord(e1, st));
    PECS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    PECS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return (double)ms / reps;
  }

  ~Engine() {
    for (auto& g : graph2)
      if (g) cudaGraphExecDestroy(g);
    if (st) cudaStreamDestroy(st);
  }

  FieldPtrs fields(const DBuf<double>* u, DBuf<double>* out) const {
    FieldPtrs F{};
    for (int f = 0; f < 5; ++f) {
      F.u[f] = u ? u[f].p : nullptr;
      F.out[f] = out ? out[f].p : nullptr;
      F.bc[f] = bconst[f].p;
      F.nd[f] = nd[f];
    }
    return F;
  }

  void build_il(int which, const std::vector<std::vector<int>>& set_fields, const FactorBank& bank) {
    IlBank& I = il[which];
    I.n_sets = (int)set_fields.size();
    I.max_R = 0;
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      const int f0 = set_fields[si][0];
      S_.n = nd[f0];
      S_.R = n_inst * (int)set_fields[si].size();
      S_.mat = f0;
      const size_t nR = (size_t)S_.n * S_.R;
      S_.f32 = bank.panel() && opt.precision != PECS_PREC_FP64;
      S_.B.alloc(nR);
      S_.X.alloc(nR);
      if (S_.f32) {
        S_.B32.alloc(nR);
        S_.Y32.alloc(nR);
        S_.X32.alloc(nR);
        S_.W32.alloc((size_t)bank.set_wtotal(si) * S_.R);
        S_.W32.zero();
      } else {
        S_.Y.alloc(nR);
        S_.W.alloc((size_t)bank.set_wtotal(si) * S_.R);
        S_.W.zero();
      }
      if (ir_iters(which) > 0) {
        if (S_.f32) {
          S_.Rr32.alloc(nR);
          S_.D32.alloc(nR);
        } else {
          S_.Rr.alloc(nR);
          S_.D.alloc(nR);
        }
        if (opt.precision == PECS_PREC_FP32_MIXED) S_.Xs.alloc(nR);
      }
      std::vector<const double*> src;
      std::vector<double*> dst[2];
      for (int i = 0; i < n_inst; ++i)
        for (int f : set_fields[si]) {
          src.push_back(rhs[f].p + (size_t)i * nd[f]);
          for (int t = 0; t < 2; ++t) dst[t].push_back(state[t][f].p + (size_t)i * nd[f]);
        }
      S_.src.upload(src);
      for (int t = 0; t < 2; ++t) S_.dst[t].upload(dst[t]);
      I.max_R = std::max(I.max_R, S_.R);
    }
  }

  IlSetsViewF il_view_f(int which, bool correction) {
    IlSetsViewF v{};
    IlBank& I = il[which];
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      v.set[si] = correction ? IlSetViewF{S_.R, S_.Rr32.p, S_.Y32.p, S_.W32.p, S_.D32.p}
                             : IlSetViewF{S_.R, S_.B32.p, S_.Y32.p, S_.W32.p, S_.X32.p};
    }
    return v;
  }
  bool il_f32(int which) const { return il[which].n_sets > 0 && il[which].set[0].f32; }
  void bank_sweep(const FactorBank& bank, int which, bool correction, cudaStream_t s) {
    if (il_f32(which))
      bank.solve(il_view_f(which, correction), il[which].max_R, s);
    else
      bank.solve(il_view(which, correction), il[which].max_R, s);
  }

  IlSetsView il_view(int which, bool correction) {
    IlSetsView v{};
    IlBank& I = il[which];
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      v.set[si] = correction ? IlSetView{S_.R, S_.Rr.p, S_.Y.p, S_.W.p, S_.D.p}
                             : IlSetView{S_.R, S_.B.p, S_.Y.p, S_.W.p, S_.X.p};
    }
    return v;
  }

  // x = A^-1 b for every right-hand side of a bank, in the interleaved layout:
  // gather the instance-major RHS vectors, sweep (+ refinement), scatter the
  // solutions into state[target].
  // Increment solves (time steps of the mixed mode with increment_solves):
  // r = b - K u_prev with u_prev the previous step's solution (state buffer
  // 1 - target) in FP32 pairs, one FP32 sweep d = K32^-1 r, u = u_prev + d.
  // The error of d relative to the exact increment is that of one FP32 solve,
  // so it shrinks with the step's change and vanishes at the fixed point,
  // where r = 0: the steady state is that of the refined solves.
  bool delta_solves() const {
    return opt.increment_solves > 0 && opt.precision == PECS_PREC_FP32_MIXED;
  }
  void solve_bank_delta(const FactorBank& bank, int which, int target, cudaStream_t s) {
    IlBank& I = il[which];
    const dim3 tb(32, 8);
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      const dim3 g((S_.n + 31) / 32, (S_.R + 31) / 32);
      k_gather_pairs_il<<<g, tb, 0, s>>>(S_.dst[1 - target].p, S_.Xs.p, S_.n, S_.R);
      PECS_CUDA(cudaGetLastError());
      // the right-hand sides are read in place from the per-instance vectors
      launch_residual_df(csr_df.m[S_.mat], (const double*)nullptr, S_.Xs.p, S_.Rr32.p, S_.n, S_.R, s,
                         (const double* const*)S_.src.p);
    }
    bank_sweep(bank, which, true, s);
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      const dim3 g((S_.n + 31) / 32, (S_.R + 31) / 32);
      k_scatter_delta_il<<<g, tb, 0, s>>>(S_.D32.p, S_.dst[1 - target].p, S_.dst[target].p, S_.n, S_.R,
                                          scatter_mask, S_.R / n_inst);
      PECS_CUDA(cudaGetLastError());
    }
  }

  void solve_bank_il(const FactorBank& bank, int which, int target, cudaStream_t s, bool delta = false) {
    if (delta && il_f32(which) && target != cur) {
      solve_bank_delta(bank, which, target, s);
      return;
    }
    IlBank& I = il[which];
    const dim3 tb(32, 8);
    const bool f32 = il_f32(which);
    const bool mixed = opt.precision == PECS_PREC_FP32_MIXED;
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      k_gather_il<<<dim3((S_.n + 31) / 32, (S_.R + 31) / 32), tb, 0, s>>>(
          S_.src.p, S_.B.p, f32 ? S_.B32.p : nullptr, S_.n, S_.R);
      PECS_CUDA(cudaGetLastError());
    }
    bank_sweep(bank, which, false, s);
    const int iters = ir_iters(which);
    auto egrid = [](size_t nR) { return (unsigned)((nR + 255) / 256); };
    for (int it = 0; it < iters; ++it) {
      for (int si = 0; si < I.n_sets; ++si) {
        IlSet& S_ = I.set[si];
        const size_t nR = (size_t)S_.n * S_.R;
        const dim3 rg((S_.n + 7) / 8, (S_.R + 31) / 32);
        if (f32) {
          // FP32 sweep vectors: the residual is stored in float for the next sweep
          if (mixed && it == 0) {
            launch_residual_df(csr_df.m[S_.mat], S_.B.p, S_.X32.p, S_.Rr32.p, S_.n, S_.R, s);
          } else if (mixed) {
            k_split_il<<<egrid(nR), 256, 0, s>>>(S_.X.p, S_.Xs.p, nR);
            PECS_CUDA(cudaGetLastError());
            launch_residual_df(csr_df.m[S_.mat], S_.B.p, S_.Xs.p, S_.Rr32.p, S_.n, S_.R, s);
          } else {
            if (it == 0) {
              k_widen_il<<<egrid(nR), 256, 0, s>>>(S_.X32.p, S_.X.p, nR);
              PECS_CUDA(cudaGetLastError());
            }
            k_residual_il<float><<<rg, 256, 0, s>>>(csr.m[S_.mat], S_.B.p, S_.X.p, S_.Rr32.p, S_.n, S_.R);
          }
        } else if (mixed) {
          k_split_il<<<egrid(nR), 256, 0, s>>>(S_.X.p, S_.Xs.p, nR);
          PECS_CUDA(cudaGetLastError());
          launch_residual_df(csr_df.m[S_.mat], S_.B.p, S_.Xs.p, S_.Rr.p, S_.n, S_.R, s);
        } else {
          k_residual_il<double><<<rg, 256, 0, s>>>(csr.m[S_.mat], S_.B.p, S_.X.p, S_.Rr.p, S_.n, S_.R);
        }
        PECS_CUDA(cudaGetLastError());
      }
      bank_sweep(bank, which, true, s);
      for (int si = 0; si < I.n_sets; ++si) {
        IlSet& S_ = I.set[si];
        const size_t nR = (size_t)S_.n * S_.R;
        if (f32 && mixed && it == 0 && iters == 1)
          continue;  // the scatter adds the correction
        if (f32 && mixed && it == 0)
          k_sum_il<<<egrid(nR), 256, 0, s>>>(S_.X32.p, S_.D32.p, S_.X.p, nR);
        else if (f32)
          k_axpy_il<float><<<egrid(nR), 256, 0, s>>>(S_.X.p, S_.D32.p, nR);
        else
          k_axpy_il<double><<<egrid(nR), 256, 0, s>>>(S_.X.p, S_.D.p, nR);
        PECS_CUDA(cudaGetLastError());
      }
    }
    for (int si = 0; si < I.n_sets; ++si) {
      IlSet& S_ = I.set[si];
      const dim3 sg((S_.n + 31) / 32, (S_.R + 31) / 32);
      const int nf = S_.R / n_inst;  // columns per instance
      if (f32 && iters == 0)
        k_scatter_il<float><<<sg, tb, 0, s>>>(S_.X32.p, S_.dst[target].p, S_.n, S_.R, scatter_mask, nf);
      else if (f32 && mixed && iters == 1)
        k_scatter_sum_il<<<sg, tb, 0, s>>>(S_.X32.p, S_.D32.p, S_.dst[target].p, S_.n, S_.R, scatter_mask,
                                           nf);
      else
        k_scatter_il<double><<<sg, tb, 0, s>>>(S_.X.p, S_.dst[target].p, S_.n, S_.R, scatter_mask, nf);
      PECS_CUDA(cudaGetLastError());
    }
  }

  std::vector<std::vector<int>> carrier_set_fields() const {
    std::vector<std::vector<int>> sf;
    if (n_fs == 1)
      sf.push_back({0, 1});
    else {
      sf.push_back({0});
      sf.push_back({1});
    }
    if (full) {
      if (n_fe == 1)
        sf.push_back({2, 3});
      else {
        sf.push_back({2});
        sf.push_back({3});
      }
    }
    return sf;
  }

  void create(const std::vector<pecs_params>& P, const pecs_options& o) {
    auto t0 = std::chrono::steady_clock::now();
    opt = o;
    n_inst = (int)P.size();
    host_only = opt.host_setup_only != 0;
    if (!host_only) {
      int ndev = 0;
      if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
        throw PecsError(PECS_E_NODEVICE, "no CUDA device available");
      if (opt.device < 0 || opt.device >= ndev) throw PecsError(PECS_E_ARG, "bad device ordinal");
      PECS_CUDA(cudaSetDevice(opt.device));
      PECS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    }
    S.reset(new Setup(P));
    full = S->full;
    n_fields = full ? 5 : 3;
    nd[0] = nd[1] = S->semi.ndofs;
    nd[2] = nd[3] = full ? S->elec.ndofs : 0;
    nd[4] = S->pois.ndofs;
    // factorisation (host, FP64); equal carrier matrices share one factor
    const int leaf = opt.leaf_cells > 0 ? opt.leaf_cells : 8;
    auto same = [](const Csr& a, const Csr& b) {
      return a.rowptr == b.rowptr && a.col == b.col && a.val == b.val;
    };
    // the largest fronts (near the root) are factored in FP64 on the GPU
    std::shared_ptr<FrontOffload> off;
    if (!host_only && opt.gpu_factor_min_front >= 0)
      off = make_gpu_front_offload(opt.device, opt.gpu_factor_min_front > 0 ? opt.gpu_factor_min_front : 1024);
    auto factor = [&](const Csr& A, const std::vector<int>& dc, const std::vector<int>* cls, int nc,
                      const std::vector<double>& xy, MfFactor& F) {
      F = mf_analyze(A, dc.data(), cls ? cls->data() : nullptr, nc, xy.data(), leaf);
      try {
        mf_factorize(F, A, 0, off.get());
      } catch (const PecsError&) {
        throw;
      } catch (const std::exception& e) {
        throw PecsError(PECS_E_SINGULAR, e.what());
      }
    };
    n_fs = same(S->semi.A[0], S->semi.A[1]) ? 1 : 2;
    for (int t = 0; t < n_fs; ++t)
      factor(S->semi.A[t], S->semi.dof_cell, &S->semi.dof_class, S->semi.grid.nc(), S->semi.cell_xy, fs[t]);
    if (full) {
      n_fe = same(S->elec.A[0], S->elec.A[1]) ? 1 : 2;
      for (int t = 0; t < n_fe; ++t)
        factor(S->elec.A[t], S->elec.dof_cell, &S->elec.dof_class, S->elec.grid.nc(), S->elec.cell_xy, fe[t]);
    }
    factor(S->pois.A, S->pois.dof_cell, nullptr, S->pois.grid.nc(), S->pois.cell_xy, fp);
    if (host_only) {
      setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return;
    }
    std::vector<const MfFactor*> cf;
    for (int t = 0; t < n_fs; ++t) cf.push_back(&fs[t]);
    for (int t = 0; t < n_fe; ++t) cf.push_back(&fe[t]);
    const int fprec = opt.precision == PECS_PREC_FP64 ? PECS_PREC_FP64 : PECS_PREC_FP32_IR;
    // many right-hand sides per set: panel kernels (lanes over right-hand sides)
    int min_rc = 1 << 30, max_rc = 0;
    for (auto& f : carrier_set_fields()) {
      min_rc = std::min(min_rc, n_inst * (int)f.size());
      max_rc = std::max(max_rc, n_inst * (int)f.size());
    }
    const PanelTuning tu{opt.panel_chunk, opt.panel_min_ctas};
    bank_c.build(cf, fprec, min_rc >= kPanelMinRhs, tu, max_rc);
    bank_p.build({&fp}, fprec, n_inst >= kPanelMinRhs, tu, n_inst);
    // free host copies of the factor values (structure is kept for stats)
    for (auto* F : {&fs[0], &fs[1], &fe[0], &fe[1], &fp}) {
      std::vector<std::vector<double>>().swap(F->Gf);
      std::vector<std::vector<double>>().swap(F->Hb);
    }
    // matrices for refinement residuals
    const Csr* mats[5] = {&S->semi.A[0], &S->semi.A[1], full ? &S->elec.A[0] : nullptr,
                          full ? &S->elec.A[1] : nullptr, &S->pois.A};
    for (int f = 0; f < 5; ++f) {
      if (!mats[f]) continue;
      A_rp[f].upload(mats[f]->rowptr);
      A_ci[f].upload(mats[f]->col);
      A_v[f].upload(mats[f]->val);
      csr.m[f] = CsrDev{A_rp[f].p, A_ci[f].p, A_v[f].p};
      if (opt.precision == PECS_PREC_FP32_MIXED) {
        std::vector<float2> sv(mats[f]->val.size());
        for (size_t t = 0; t < sv.size(); ++t) {
          const double a = mats[f]->val[t];
          const float hi = (float)a;
          sv[t] = make_float2(hi, (float)(a - (double)hi));
        }
        Adf[f].upload(sv);
        csr_df.m[f] = CsrDf{A_rp[f].p, A_ci[f].p, Adf[f].p};
      }
    }
    upload_tables();
    upload_regions();
    // vectors
    for (int f = 0; f < 5; ++f) {
      const size_t n = (size_t)n_inst * nd[f];
      if (n == 0) continue;
      for (int b = 0; b < 2; ++b) {
        state[b][f].alloc(n);
        state[b][f].zero();
      }
      rhs[f].alloc(n);
      rhs[f].zero();
      snap[f].alloc(n);
      std::vector<double> bc;
      bc.reserve(n);
      for (int i = 0; i < n_inst; ++i) bc.insert(bc.end(), S->bconst[f][i].begin(), S->bconst[f][i].end());
      bconst[f].upload(bc);
      if (f < 4) {
        std::vector<double> v;
        v.reserve(n);
        for (int i = 0; i < n_inst; ++i) v.insert(v.end(), S->init[f][i].begin(), S->init[f][i].end());
        init_dev[f].upload(v);
      }
    }
    build_il(0, carrier_set_fields(), bank_c);
    build_il(1, {{4}}, bank_p);
    if (opt.autotune) {
      // panel banks: per level, the fastest tiling for these right-hand sides,
      // then the flow sweep if it is faster still
      for (int which = 0; which < 2; ++which) {
        FactorBank& bk = which == 0 ? bank_c : bank_p;
        if (!bk.panel()) continue;
        if (il_f32(which))
          bk.autotune(il_view_f(which, false), il[which].max_R, st, 3, opt.flow_sweep);
        else
          bk.autotune(il_view(which, false), il[which].max_R, st, 3, opt.flow_sweep);
      }
      PECS_CUDA(cudaStreamSynchronize(st));
    } else if (opt.flow_sweep > 0) {
      for (int which = 0; which < 2; ++which) {
        FactorBank& bk = which == 0 ? bank_c : bank_p;
        if (!bk.panel()) continue;
        if (il_f32(which))
          bk.force_flow(il_view_f(which, false), il[which].max_R);
        else
          bk.force_flow(il_view(which, false), il[which].max_R);
      }
    }
    // few-right-hand-side banks: the flow sweep when it times faster (or as
    // flow_sweep forces)
    if (opt.autotune || opt.flow_sweep != 0) {
      for (int which = 0; which < 2; ++which) {
        FactorBank& bk = which == 0 ? bank_c : bank_p;
        if (bk.panel()) continue;
        bk.tune_rows_flow(il_view(which, false), il[which].max_R, st,
                          opt.autotune ? opt.flow_sweep : (opt.flow_sweep > 0 ? 1 : -1));
      }
      PECS_CUDA(cudaStreamSynchronize(st));
    }
    // steady-state buffers
    partial.alloc((size_t)n_inst * 5 * kRedChunks);
    partial.zero();
    conv_step.alloc(n_inst);
    start_step.alloc(n_inst);
    start_step.zero();
    capped.alloc(n_inst);
    capped.zero();
    refill_mask.alloc(n_inst);
    refill_mask.zero();
    rel.alloc(n_inst);
    step_ctr.alloc(1);
    n_active.alloc(1);
    active.alloc(n_inst);
    std::vector<int> ones(n_inst, 1);
    active.upload(ones);
    std::vector<double*> sp(5, nullptr);
    for (int f = 0; f < 5; ++f) sp[f] = snap[f].p;
    snap_ptrs.upload(sp);
    PECS_CUDA(cudaDeviceSynchronize());
    setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // Replace the per-instance parameters (bias, generation, doping, lifetimes,
  // rates...) of every instance; matrices and factors are kept.
  void set_instances(const std::vector<pecs_params>& P) {
    if ((int)P.size() != n_inst) throw PecsError(PECS_E_ARG, "n_inst differs from the context's");
    std::vector<pecs_params> chk(P);
    chk.insert(chk.begin(), S->inst[0]);
    std::string err = validate_params(chk.data(), (int)chk.size());
    if (!err.empty()) throw PecsError(PECS_E_ARG, err);
    S->compute_instances(P);
    auto put = [&](DBuf<double>& d, const std::vector<std::vector<double>>& src) {
      std::vector<double> v;
      for (auto& x : src) v.insert(v.end(), x.begin(), x.end());
      if (v.size() != d.n) throw PecsError(PECS_E_STATE, "instance data size changed");
      if (!v.empty()) PECS_CUDA(cudaMemcpy(d.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
    };
    for (int f = 0; f < 5; ++f)
      if (nd[f]) put(bconst[f], S->bconst[f]);
    for (int f = 0; f < 4; ++f)
      if (nd[f]) put(init_dev[f], S->init[f]);
    if (full) {
      put(iface_ne, S->iface_ne);
      put(iface_pe, S->iface_pe);
    }
    if (S->has_schottky) {
      put(sch_ne, S->schottky_ne);
      put(sch_pe, S->schottky_pe);
    }
    std::vector<InstDev> ip(n_inst);
    for (int i = 0; i < n_inst; ++i) {
      const pecs_params& p = S->inst[i];
      ip[i] = InstDev{p.k_et, p.k_ht, p.tau_n, p.tau_p, p.n_i, p.s_n, p.s_p, p.srh, 0};
    }
    PECS_CUDA(cudaMemcpy(inst.p, ip.data(), ip.size() * sizeof(InstDev), cudaMemcpyHostToDevice));
  }

  void upload_tables() {
    const CarrierTables& ct = S->ct;
    const PoissonTables& pt = S->pt;
    t_phi.upload(ct.phi);
    t_qw.upload(ct.qw);
    t_fphi.upload(ct.fphi);
    t_fw.upload(ct.fw);
    t_psix.upload(pt.psi_x);
    t_psiy.upload(pt.psi_y);
    t_phiP.upload(pt.phi);
    std::vector<double> mref(ct.n1 * ct.n1, 0.0);
    for (int a = 0; a < ct.n1; ++a)
      for (int b = 0; b < ct.n1; ++b)
        for (int q = 0; q < ct.Q; ++q) mref[a * ct.n1 + b] += ct.phi[a * ct.Q + q] * ct.phi[b * ct.Q + q] * ct.qw[q];
    t_mref.upload(mref);
    auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    tf_phi.upload(f32(ct.phi));
    tf_qw.upload(f32(ct.qw));
    tf_fphi.upload(f32(ct.fphi));
    tf_fw.upload(f32(ct.fw));
    tf_psix.upload(f32(pt.psi_x));
    tf_psiy.upload(f32(pt.psi_y));
    // drift tensors sum_q phi_a phi_b psi_c w_q over the RT functions with a
    // non-zero x (y) component; on rectangles each RT function has one
    // component only, nrt/2 of each
    const int n1 = ct.n1, Q = ct.Q, nrt = pt.n_rt, NC = nrt / 2;
    std::vector<int> cx, cy;
    for (int c = 0; c < nrt; ++c) {
      bool nx = false, ny = false;
      for (int q = 0; q < Q; ++q) {
        nx = nx || pt.psi_x[c * Q + q] != 0.0;
        ny = ny || pt.psi_y[c * Q + q] != 0.0;
      }
      if (nx && ny) throw PecsError(PECS_E_STATE, "RT function with two components");
      if (nx) cx.push_back(c);
      if (ny) cy.push_back(c);
    }
    if ((int)cx.size() != NC || (int)cy.size() != NC)
      throw PecsError(PECS_E_STATE, "RT functions not split evenly by component");
    std::vector<double> dx((size_t)n1 * n1 * NC, 0.0), dy((size_t)n1 * n1 * NC, 0.0);
    for (int a = 0; a < n1; ++a)
      for (int b = 0; b < n1; ++b)
        for (int j = 0; j < NC; ++j)
          for (int q = 0; q < Q; ++q) {
            const double pw = ct.phi[a * Q + q] * ct.phi[b * Q + q] * ct.qw[q];
            dx[((size_t)a * n1 + b) * NC + j] += pw * pt.psi_x[cx[j] * Q + q];
            dy[((size_t)a * n1 + b) * NC + j] += pw * pt.psi_y[cy[j] * Q + q];
          }
    t_drift_x.upload(dx);
    t_drift_y.upload(dy);
    t_drift_cx.upload(cx);
    t_drift_cy.upload(cy);
    // Poisson charge matrix sum_q phiP_a phi_b w_q
    const int nphi = pt.n_phi;
    std::vector<double> chg((size_t)nphi * n1, 0.0);
    for (int a = 0; a < nphi; ++a)
      for (int b = 0; b < n1; ++b)
        for (int q = 0; q < Q; ++q) chg[(size_t)a * n1 + b] += pt.phi[a * Q + q] * ct.phi[b * Q + q] * ct.qw[q];
    t_charge.upload(chg);
    // FP32 pairs (hi rounded to nearest, lo the rounded remainder) for the
    // mixed path
    auto ff = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size());
      for (size_t k = 0; k < v.size(); ++k) {
        const float hi = (float)v[k];
        o[k] = make_float2(hi, (float)(v[k] - (double)hi));
      }
      return o;
    };
    t_drift_x_ff.upload(ff(dx));
    t_drift_y_ff.upload(ff(dy));
    t_mref_ff.upload(ff(mref));
    T = Tables{t_phi.p,  t_qw.p,  t_fphi.p,  t_fw.p,   t_psix.p,  t_psiy.p, t_phiP.p,
               t_mref.p, tf_phi.p, tf_qw.p, tf_fphi.p, tf_fw.p, tf_psix.p, tf_psiy.p,
               t_drift_x.p, t_drift_y.p, t_drift_cx.p, t_drift_cy.p, t_charge.p,
               t_drift_x_ff.p, t_drift_y_ff.p, t_mref_ff.p};
  }

  void upload_regions() {
    const int nrt = S->n_rt, nphi = S->n_phi, nloc = nrt + nphi;
    const pecs_params& P0 = S->inst[0];
    for (int r = 0; r < (full ? 2 : 1); ++r) {
      const CarrierSystem& CS = r == 0 ? S->semi : S->elec;
      const Grid& g = CS.grid;
      const std::vector<int>& c2p = r == 0 ? S->s2p : S->e2p;
      const int nc = g.nc();
      std::vector<double2> h(nc);
      std::vector<int4> bid(nc);
      std::vector<int> rt(nc * nrt), phid(nc * nphi), partner(nc, -1), ifc(nc, -1);
      for (int K = 0; K < nc; ++K) {
        double x0, y0, hx, hy;
        g.geom(K, x0, y0, hx, hy);
        h[K] = make_double2(hx, hy);
        bid[K] = make_int4(g.face_bid(K, 0), g.face_bid(K, 1), g.face_bid(K, 2), g.face_bid(K, 3));
        const int pc = c2p[K];
        for (int b = 0; b < nrt; ++b) rt[K * nrt + b] = S->pois.l2g[pc * nloc + b];
        for (int a = 0; a < nphi; ++a) phid[K * nphi + a] = S->pois.l2g[pc * nloc + nrt + a];
      }
      const std::vector<int>& mine = r == 0 ? S->iface_semi : S->iface_elec;
      const std::vector<int>& other = r == 0 ? S->iface_elec : S->iface_semi;
      for (size_t t = 0; t < mine.size(); ++t) {
        partner[mine[t]] = other[t];
        ifc[mine[t]] = (int)t;
      }
      h_[r].upload(h);
      bid_[r].upload(bid);
      rt_[r].upload(rt);
      phid_[r].upload(phid);
      partner_[r].upload(partner);
      iface_[r].upload(ifc);
      RegionDev& D = R[r];
      D.nc = nc;
      D.nd = CS.ndofs;
      D.field1 = r == 0 ? 0 : 2;
      D.is_semi = r == 0;
      D.iface_face = r == 0 ? kRight : kLeft;
      D.partner_face = r == 0 ? kLeft : kRight;
      D.inv_eps = 1.0 / (r == 0 ? P0.eps_semi : P0.eps_elec);
      D.inv_dt = 1.0 / P0.dt;
      D.h = h_[r].p;
      D.bid = bid_[r].p;
      D.rt = rt_[r].p;
      D.phid = phid_[r].p;
      D.partner = partner_[r].p;
      D.iface = iface_[r].p;
    }
    if (!full) R[1] = R[0];
    std::vector<InstDev> ip(n_inst);
    for (int i = 0; i < n_inst; ++i) {
      const pecs_params& p = S->inst[i];
      ip[i] = InstDev{p.k_et, p.k_ht, p.tau_n, p.tau_p, p.n_i, p.s_n, p.s_p, p.srh, 0};
    }
    inst.upload(ip);
    std::vector<double> a, b, c, d;
    for (int i = 0; i < n_inst; ++i) {
      a.insert(a.end(), S->iface_ne[i].begin(), S->iface_ne[i].end());
      b.insert(b.end(), S->iface_pe[i].begin(), S->iface_pe[i].end());
      if (S->has_schottky) {
        c.insert(c.end(), S->schottky_ne[i].begin(), S->schottky_ne[i].end());
        d.insert(d.end(), S->schottky_pe[i].begin(), S->schottky_pe[i].end());
      }
    }
    iface_ne.upload(a);
    iface_pe.upload(b);
    sch_ne.upload(c);
    sch_pe.upload(d);
    isemi.upload(S->iface_semi);
    ielec.upload(S->iface_elec);
  }

  // ---- stages ------------------------------------------------------------
  int nxt() const { return cur ^ 1; }

  void launch_carrier_rhs(cudaStream_t s, const int* act) {
    FieldPtrs F = fields(state[cur], rhs);
    const int ntot = 2 * R[0].nc + (full ? 2 * R[1].nc : 0);
    dim3 grid((ntot + 127) / 128, n_inst);
    const int nif = (int)S->iface_semi.size();
    const double* sne = S->has_schottky ? sch_ne.p : nullptr;
    const double* spe = S->has_schottky ? sch_pe.p : nullptr;
    const bool mixed = opt.precision == PECS_PREC_FP32_MIXED;
    const int nreg = full ? 2 : 1;
    // (LDG degree, Poisson table degree): the reference's RT_{k-1} x DGQ_{k-1}
    // pairing has KP = k, the configurations' RT_k x DGQ_k KP = k + 1
    auto go = [&](auto kk, auto kp) {
      constexpr int K = decltype(kk)::value, KP = decltype(kp)::value;
      if (mixed)
        k_carrier_rhs<K, KP, float><<<grid, 128, 0, s>>>(T, R[0], R[1], nreg, F, inst.p, iface_ne.p,
                                                         iface_pe.p, nif, sne, spe, act);
      else
        k_carrier_rhs<K, KP, double><<<grid, 128, 0, s>>>(T, R[0], R[1], nreg, F, inst.p, iface_ne.p,
                                                          iface_pe.p, nif, sne, spe, act);
    };
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    using I3 = std::integral_constant<int, 3>;
    const int kp = S->pt.k;
    if (S->k == 1)
      kp == 1 ? go(I1{}, I1{}) : go(I1{}, I2{});
    else
      kp == 2 ? go(I2{}, I2{}) : go(I2{}, I3{});
    PECS_CUDA(cudaGetLastError());
  }

  void launch_poisson_rhs(cudaStream_t s, const DBuf<double>* carriers, const int* act) {
    FieldPtrs F = fields(carriers, rhs);
    const int ncells = R[0].nc + (full ? R[1].nc : 0);
    const int n = std::max(ncells, S->pois.n_rt_total);
    dim3 grid((n + 127) / 128, n_inst);
    const int kp = S->pt.k, nreg = full ? 2 : 1, nrt = S->pois.n_rt_total;
    if (S->k == 1 && kp == 1)
      k_poisson_rhs<1, 1><<<grid, 128, 0, s>>>(T, R[0], R[1], nreg, F, nrt, act);
    else if (S->k == 1)
      k_poisson_rhs<1, 2><<<grid, 128, 0, s>>>(T, R[0], R[1], nreg, F, nrt, act);
    else if (kp == 2)
      k_poisson_rhs<2, 2><<<grid, 128, 0, s>>>(T, R[0], R[1], nreg, F, nrt, act);
    else
      k_poisson_rhs<2, 3><<<grid, 128, 0, s>>>(T, R[0], R[1], nreg, F, nrt, act);
    PECS_CUDA(cudaGetLastError());
  }

  DBuf<float2> Adf[5];
  CsrDfSet csr_df{};

  std::vector<int> carrier_fields() const {
    return full ? std::vector<int>{0, 1, 2, 3} : std::vector<int>{0, 1};
  }

  void stage_carrier_rhs(cudaStream_t s, const int* act) { launch_carrier_rhs(s, act); }
  void stage_solve_carriers(cudaStream_t s, const int* act) {
    solve_bank_il(bank_c, 0, nxt(), s, delta_solves());
    carriers_advanced = true;
  }
  void stage_poisson_rhs(cudaStream_t s, const int* act) {
    launch_poisson_rhs(s, carriers_advanced ? state[nxt()] : state[cur], act);
  }
  void stage_solve_poisson(cudaStream_t s, const int* act) {
    const int target = carriers_advanced ? nxt() : cur;
    solve_bank_il(bank_p, 1, target, s, delta_solves() && carriers_advanced);
    if (carriers_advanced) {
      cur = nxt();
      carriers_advanced = false;
    }
  }

  void full_step(cudaStream_t s, const int* act) {
    stage_carrier_rhs(s, act);
    stage_solve_carriers(s, act);
    stage_poisson_rhs(s, act);
    stage_solve_poisson(s, act);
  }

  // step + steady-state bookkeeping (state[cur] -> state[nxt], compares both)
  void step_with_check(cudaStream_t s, double tol) {
    const int old = cur;
    full_step(s, active.p);
    FieldPtrs NEW = fields(state[cur], nullptr), OLD = fields(state[old], nullptr);
    if (opt.precision == PECS_PREC_FP32_MIXED)
      k_relchange_partial<float><<<dim3(kRedChunks, 5, n_inst), kRedThreads, 0, s>>>(NEW, OLD, n_fields,
                                                                                    partial.p);
    else
      k_relchange_partial<double><<<dim3(kRedChunks, 5, n_inst), kRedThreads, 0, s>>>(NEW, OLD, n_fields,
                                                                                     partial.p);
    PECS_CUDA(cudaGetLastError());
    k_converge<<<1, 256, 0, s>>>(partial.p, n_inst, n_fields, tol, conv_step.p, rel.p, step_ctr.p,
                                 active.p, n_active.p, start_step.p, step_cap, capped.p);
    PECS_CUDA(cudaGetLastError());
    k_snapshot<<<dim3(32, 5, n_inst), 256, 0, s>>>(NEW, snap_ptrs.p, conv_step.p, step_ctr.p, 5);
    PECS_CUDA(cudaGetLastError());
  }

  // Initial conditions from the device-resident projections, then the initial
  // Poisson solve.  No host traffic.
  void initialize() {
    for (int f = 0; f < 4; ++f) {
      if (nd[f] == 0) continue;
      PECS_CUDA(cudaMemcpyAsync(state[cur][f].p, init_dev[f].p, (size_t)n_inst * nd[f] * 8,
                                cudaMemcpyDeviceToDevice, st));
    }
    carriers_advanced = false;
    stage_poisson_rhs(st, nullptr);
    stage_solve_poisson(st, nullptr);
    PECS_CUDA(cudaStreamSynchronize(st));
    initialized = true;
  }

  void reset_convergence() {
    std::vector<int> ones(n_inst, 1), zeros(n_inst, 0);
    PECS_CUDA(cudaMemcpyAsync(active.p, ones.data(), n_inst * 4, cudaMemcpyHostToDevice, st));
    PECS_CUDA(cudaMemcpyAsync(conv_step.p, zeros.data(), n_inst * 4, cudaMemcpyHostToDevice, st));
    PECS_CUDA(cudaMemsetAsync(start_step.p, 0, n_inst * 4, st));
    PECS_CUDA(cudaMemsetAsync(capped.p, 0, n_inst * 4, st));
    PECS_CUDA(cudaMemsetAsync(step_ctr.p, 0, 4, st));
    PECS_CUDA(cudaStreamSynchronize(st));
  }

  void capture_graph(double tol) {
    graph_cap = step_cap;
    const int saved = cur;
    for (int par = 0; par < 2; ++par) {
      if (graph2[par]) {
        cudaGraphExecDestroy(graph2[par]);
        graph2[par] = nullptr;
      }
      cudaGraph_t g;
      cur = par;
      PECS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      try {
        step_with_check(st, tol);
        step_with_check(st, tol);
      } catch (...) {
        cudaStreamEndCapture(st, &g);
        cur = saved;
        throw;
      }
      PECS_CUDA(cudaStreamEndCapture(st, &g));
      PECS_CUDA(cudaGraphInstantiate(&graph2[par], g, 0));
      cudaGraphDestroy(g);
    }
    cur = saved;  // two steps return the ping-pong index to where it was
    graph_tol = tol;
    graph_valid = true;
  }
  double graph_tol = -1.0;
  int graph_cap = -1;
  int last_run_steps = 0;

  void run_to_steady(int max_steps, double tol, int check_every, int* steps, double* relc) {
    if (!initialized) throw PecsError(PECS_E_STATE, "pecs_initialize must be called first");
    if (max_steps < 0) throw PecsError(PECS_E_ARG, "max_steps < 0");
    if (check_every <= 0) check_every = 50;
    check_every += check_every & 1;
    reset_convergence();
    last_run_steps = 0;
    const bool use_graph = opt.use_graphs != 0 && max_steps >= 2;
    step_cap = 1 << 30;  // the host loop stops at max_steps
    if (use_graph && (!graph_valid || graph_tol != tol || graph_cap != step_cap)) capture_graph(tol);
    int done = 0;
    int h_active = n_inst;
    while (done < max_steps && h_active > 0) {
      const int chunk = std::min(check_every, max_steps - done);
      int k = 0;
      for (; k + 2 <= chunk; k += 2) {
        if (use_graph)
          PECS_CUDA(cudaGraphLaunch(graph2[cur], st));
        else {
          step_with_check(st, tol);
          step_with_check(st, tol);
        }
      }
      if (k < chunk) {  // odd remainder
        step_with_check(st, tol);
        ++k;
      }
      done += k;
      last_run_steps = done;
      PECS_CUDA(cudaMemcpyAsync(&h_active, n_active.p, 4, cudaMemcpyDeviceToHost, st));
      PECS_CUDA(cudaStreamSynchronize(st));
    }
    // instances that converged: restore their snapshot into the current state
    std::vector<int> cs(n_inst);
    std::vector<double> rl(n_inst);
    PECS_CUDA(cudaMemcpy(cs.data(), conv_step.p, n_inst * 4, cudaMemcpyDeviceToHost));
    PECS_CUDA(cudaMemcpy(rl.data(), rel.p, n_inst * 8, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n_inst; ++i) {
      if (cs[i] != 0) {
        for (int f = 0; f < 5; ++f)
          if (nd[f])
            PECS_CUDA(cudaMemcpyAsync(state[cur][f].p + (size_t)i * nd[f], snap[f].p + (size_t)i * nd[f],
                                      (size_t)nd[f] * 8, cudaMemcpyDeviceToDevice, st));
      }
      if (steps) steps[i] = cs[i] > 0 ? cs[i] : (cs[i] < 0 ? cs[i] : done);
      if (relc) relc[i] = rl[i];
    }
    PECS_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < n_inst; ++i)
      if (cs[i] < 0)
        throw PecsError(PECS_E_NONFINITE, "instance " + std::to_string(i) +
                                              " produced a non-finite state at step " +
                                              std::to_string(-cs[i]));
  }

  // Largest ||b - A x|| / ||b|| over the instances and fields of one bank, for
  // the latest solve: b = the last assembled right-hand sides, x = the state
  // they were solved into (valid after a full step or a stage solve).
  double solve_residual(int which) {
    std::vector<int> flds = which == 0 ? carrier_fields() : std::vector<int>{4};
    DBuf<double> sums;
    sums.alloc((size_t)2 * n_inst);
    double worst = 0.0;
    for (int f : flds) {
      sums.zero();
      const DBuf<double>& x = which == 0 ? (carriers_advanced ? state[nxt()][f] : state[cur][f]) : state[cur][f];
      k_residual_norms<<<dim3(64, n_inst), 256, 0, st>>>(csr.m[f], rhs[f].p, x.p, nd[f], sums.p);
      PECS_CUDA(cudaGetLastError());
      std::vector<double> h(2 * n_inst);
      PECS_CUDA(cudaMemcpyAsync(h.data(), sums.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
      PECS_CUDA(cudaStreamSynchronize(st));
      for (int i = 0; i < n_inst; ++i)
        if (h[2 * i + 1] > 0.0) worst = std::max(worst, std::sqrt(h[2 * i] / h[2 * i + 1]));
    }
    return worst;
  }

  // ---- streamed sweep: slots refilled as they finish -------------------------
  // New parameters for the given slots (host setup of their per-instance data,
  // uploaded slice by slice), their initial state (standard, or the given
  // device densities for electrons / holes), then one Poisson solve whose
  // results are written to these slots only.
  // pre: the slots' per-instance data already computed (a streamed sweep's
  // background preparation), moved in; empty: computed here
  void refill(const std::vector<int>& slots, const std::vector<pecs_params>& P,
              const std::vector<const double*>& init_n, const std::vector<const double*>& init_p,
              std::vector<Setup::InstanceData>* pre = nullptr) {
    {
      std::vector<pecs_params> chk(P);
      chk.insert(chk.begin(), S->inst[0]);
      std::string err = validate_params(chk.data(), (int)chk.size());
      if (!err.empty()) throw PecsError(PECS_E_ARG, err);
    }
    std::vector<int> mask(n_inst, 0);
    for (size_t t = 0; t < slots.size(); ++t) S->inst[slots[t]] = P[t];
    if (pre) {
      for (size_t t = 0; t < slots.size(); ++t) S->store_instance(slots[t], std::move((*pre)[t]));
    } else {
      S->compute_instances_at(slots);
    }
    // host sources of the copies below stay alive until the synchronisation
    // at the end (the per-instance vectors, ips, mask)
    std::vector<InstDev> ips(slots.size());
    for (size_t t = 0; t < slots.size(); ++t) {
      const int i = slots[t];
      mask[i] = 1;
      auto put = [&](DBuf<double>& d, const std::vector<double>& v) {
        if (v.empty()) return;
        PECS_CUDA(cudaMemcpyAsync(d.p + (size_t)i * v.size(), v.data(), v.size() * 8, cudaMemcpyHostToDevice, st));
      };
      for (int f = 0; f < 5; ++f)
        if (nd[f]) put(bconst[f], S->bconst[f][i]);
      for (int f = 0; f < 4; ++f)
        if (nd[f]) put(init_dev[f], S->init[f][i]);
      if (full) {
        put(iface_ne, S->iface_ne[i]);
        put(iface_pe, S->iface_pe[i]);
      }
      if (S->has_schottky) {
        put(sch_ne, S->schottky_ne[i]);
        put(sch_pe, S->schottky_pe[i]);
      }
      const pecs_params& p = S->inst[i];
      ips[t] = InstDev{p.k_et, p.k_ht, p.tau_n, p.tau_p, p.n_i, p.s_n, p.s_p, p.srh, 0};
      PECS_CUDA(cudaMemcpyAsync(inst.p + i, &ips[t], sizeof(InstDev), cudaMemcpyHostToDevice, st));
      for (int f = 0; f < 4; ++f) {
        if (!nd[f]) continue;
        const double* src = init_dev[f].p + (size_t)i * nd[f];
        if (f == 0 && init_n[t]) src = init_n[t];
        if (f == 1 && init_p[t]) src = init_p[t];
        PECS_CUDA(cudaMemcpyAsync(state[cur][f].p + (size_t)i * nd[f], src, (size_t)nd[f] * 8,
                                  cudaMemcpyDeviceToDevice, st));
      }
    }
    PECS_CUDA(cudaMemcpyAsync(refill_mask.p, mask.data(), n_inst * 4, cudaMemcpyHostToDevice, st));
    scatter_mask = refill_mask.p;
    try {
      stage_poisson_rhs(st, nullptr);
      stage_solve_poisson(st, nullptr);
    } catch (...) {
      scatter_mask = nullptr;
      throw;
    }
    scatter_mask = nullptr;
    PECS_CUDA(cudaStreamSynchronize(st));
  }

  // March n_points parameter sets through the n_inst slots.  Outputs per
  // point: steps (to convergence; max_steps when capped; negative when the
  // state became non-finite), interface current, optionally final fields.
  void sweep_stream(int n_points, const pecs_params* params, const double* const* init_n,
                    const double* const* init_p, int max_steps, double tol, int check_every,
                    int* out_steps, double* out_current, double* const* out_fields) {
    if (n_points <= 0) return;
    if (max_steps < 1) throw PecsError(PECS_E_ARG, "max_steps < 1");
    if (check_every <= 0) check_every = 50;
    check_every += check_every & 1;
    std::vector<int> slot_point(n_inst, -1);
    int next = 0;
    // The points after the first fill have their per-instance data (the
    // constant right-hand sides, projected initial states: host work of a
    // few milliseconds each) prepared by a host thread in stream order while
    // the GPU marches, at most n_inst points ahead of the refills.
    struct Prefetch {
      std::vector<Setup::InstanceData> data;
      std::vector<char> ready;
      std::mutex mu;
      std::condition_variable cv;
      int consumed = 0;
      bool stop = false;
      std::thread worker;
      ~Prefetch() {
        {
          std::lock_guard<std::mutex> g(mu);
          stop = true;
        }
        cv.notify_all();
        if (worker.joinable()) worker.join();
      }
    } pf;
    pf.data.resize(n_points);
    pf.ready.assign(n_points, 0);
    const int n_first = std::min(n_inst, n_points);
    pf.consumed = n_first;  // the first fill computes its points itself
    if (n_points > n_first) {
      const unsigned hc = std::thread::hardware_concurrency();
      const int threads = std::max(1, (int)(hc ? hc : 1));
      const Setup* Sc = S.get();
      pf.worker = std::thread([&pf, Sc, params, n_first, n_points, threads, this]() {
        for (int q = n_first; q < n_points; ++q) {
          {
            std::unique_lock<std::mutex> lk(pf.mu);
            pf.cv.wait(lk, [&] { return pf.stop || q - pf.consumed < n_inst; });
            if (pf.stop) return;
          }
          Setup::InstanceData d;
          try {
            Sc->compute_instance_data(params[q], d, threads);
          } catch (...) {
            // left unready: the refill computes this point itself
            std::lock_guard<std::mutex> g(pf.mu);
            pf.ready[q] = 2;
            pf.cv.notify_all();
            continue;
          }
          std::lock_guard<std::mutex> g(pf.mu);
          pf.data[q] = std::move(d);
          pf.ready[q] = 1;
          pf.cv.notify_all();
        }
      });
    }
    auto take = [&](std::vector<int>& slots) {
      std::vector<pecs_params> P;
      std::vector<const double*> in, ip;
      std::vector<Setup::InstanceData> pre;
      bool all_pre = next >= n_first;
      for (int i : slots) {
        slot_point[i] = next;
        P.push_back(params[next]);
        in.push_back(init_n ? init_n[next] : nullptr);
        ip.push_back(init_p ? init_p[next] : nullptr);
        if (next >= n_first) {
          std::unique_lock<std::mutex> lk(pf.mu);
          pf.cv.wait(lk, [&] { return pf.ready[next] != 0; });
          if (pf.ready[next] == 1)
            pre.push_back(std::move(pf.data[next]));
          else
            all_pre = false;
          pf.consumed = next + 1;
          pf.cv.notify_all();
        }
        ++next;
      }
      refill(slots, P, in, ip, all_pre && pre.size() == slots.size() ? &pre : nullptr);
    };
    // first fill: every slot the points can occupy; idle slots are inactive
    std::vector<int> first;
    for (int i = 0; i < n_inst && next + (int)first.size() < n_points; ++i) first.push_back(i);
    carriers_advanced = false;
    initialized = true;
    take(first);
    {
      std::vector<int> act(n_inst, 0), zeros(n_inst, 0);
      for (int i : first) act[i] = 1;
      PECS_CUDA(cudaMemcpyAsync(active.p, act.data(), n_inst * 4, cudaMemcpyHostToDevice, st));
      PECS_CUDA(cudaMemcpyAsync(conv_step.p, zeros.data(), n_inst * 4, cudaMemcpyHostToDevice, st));
      PECS_CUDA(cudaMemsetAsync(start_step.p, 0, n_inst * 4, st));
      PECS_CUDA(cudaMemsetAsync(capped.p, 0, n_inst * 4, st));
      PECS_CUDA(cudaMemsetAsync(step_ctr.p, 0, 4, st));
      PECS_CUDA(cudaStreamSynchronize(st));
    }
    step_cap = max_steps;
    const bool use_graph = opt.use_graphs != 0;
    if (use_graph && (!graph_valid || graph_tol != tol || graph_cap != step_cap)) capture_graph(tol);
    int done_steps = 0, harvested = 0;
    last_run_steps = 0;
    std::vector<int> cs(n_inst), act(n_inst);
    DBuf<double> cur_dev;
    cur_dev.alloc(n_inst);
    std::vector<double> hcur(n_inst);
    while (harvested < n_points) {
      for (int k = 0; k < check_every; k += 2) {
        if (use_graph) {
          PECS_CUDA(cudaGraphLaunch(graph2[cur], st));
        } else {
          step_with_check(st, tol);
          step_with_check(st, tol);
        }
      }
      done_steps += check_every;
      last_run_steps = done_steps;
      PECS_CUDA(cudaMemcpyAsync(cs.data(), conv_step.p, n_inst * 4, cudaMemcpyDeviceToHost, st));
      PECS_CUDA(cudaMemcpyAsync(act.data(), active.p, n_inst * 4, cudaMemcpyDeviceToHost, st));
      PECS_CUDA(cudaStreamSynchronize(st));
      std::vector<int> finished;
      for (int i = 0; i < n_inst; ++i)
        if (slot_point[i] >= 0 && !act[i]) finished.push_back(i);
      if (finished.empty()) continue;
      // harvest from the snapshots (state at each slot's final step)
      if (full && !S->iface_semi.empty() && out_current) {
        FieldPtrs F{};
        for (int f = 0; f < 5; ++f) {
          F.u[f] = snap[f].p;
          F.bc[f] = bconst[f].p;
          F.nd[f] = nd[f];
        }
        k_interface_current<<<n_inst, kRedThreads, 0, st>>>(T, R[0], R[1], F, inst.p, iface_ne.p, iface_pe.p,
                                                           isemi.p, ielec.p, (int)S->iface_semi.size(),
                                                           S->n1, S->nq1, cur_dev.p);
        PECS_CUDA(cudaGetLastError());
        PECS_CUDA(cudaMemcpyAsync(hcur.data(), cur_dev.p, n_inst * 8, cudaMemcpyDeviceToHost, st));
      }
      for (int i : finished) {
        const int pt = slot_point[i];
        if (out_fields)
          for (int f = 0; f < 5; ++f)
            if (nd[f] && out_fields[f])
              PECS_CUDA(cudaMemcpyAsync(out_fields[f] + (size_t)pt * nd[f], snap[f].p + (size_t)i * nd[f],
                                        (size_t)nd[f] * 8, cudaMemcpyDeviceToHost, st));
      }
      PECS_CUDA(cudaStreamSynchronize(st));
      std::vector<int> start_h(n_inst);
      PECS_CUDA(cudaMemcpy(start_h.data(), start_step.p, n_inst * 4, cudaMemcpyDeviceToHost));
      std::vector<int> refills;
      for (int i : finished) {
        const int pt = slot_point[i];
        if (out_steps) out_steps[pt] = cs[i] < 0 ? cs[i] + start_h[i] : cs[i] - start_h[i];
        if (out_current) out_current[pt] = (full && !S->iface_semi.empty()) ? hcur[i] : 0.0;
        ++harvested;
        slot_point[i] = -1;
        if (next + (int)refills.size() < n_points) refills.push_back(i);
      }
      if (!refills.empty()) {
        take(refills);
        // restart the refilled slots at the current step
        int step_now = 0;
        PECS_CUDA(cudaMemcpy(&step_now, step_ctr.p, 4, cudaMemcpyDeviceToHost));
        for (int i : refills) {
          const int one = 1, zero = 0;
          PECS_CUDA(cudaMemcpyAsync(active.p + i, &one, 4, cudaMemcpyHostToDevice, st));
          PECS_CUDA(cudaMemcpyAsync(conv_step.p + i, &zero, 4, cudaMemcpyHostToDevice, st));
          PECS_CUDA(cudaMemcpyAsync(capped.p + i, &zero, 4, cudaMemcpyHostToDevice, st));
          PECS_CUDA(cudaMemcpyAsync(start_step.p + i, &step_now, 4, cudaMemcpyHostToDevice, st));
          PECS_CUDA(cudaStreamSynchronize(st));
        }
      }
    }
  }

  void interface_current(double* out) {
    std::vector<double> h(n_inst, 0.0);
    if (full && !S->iface_semi.empty()) {
      DBuf<double> d;
      d.alloc(n_inst);
      FieldPtrs F = fields(carriers_advanced ? state[nxt()] : state[cur], nullptr);
      k_interface_current<<<n_inst, kRedThreads, 0, st>>>(T, R[0], R[1], F, inst.p, iface_ne.p, iface_pe.p,
                                                         isemi.p, ielec.p, (int)S->iface_semi.size(),
                                                         S->n1, S->nq1, d.p);
      PECS_CUDA(cudaGetLastError());
      PECS_CUDA(cudaMemcpyAsync(h.data(), d.p, n_inst * 8, cudaMemcpyDeviceToHost, st));
      PECS_CUDA(cudaStreamSynchronize(st));
    }
    std::copy(h.begin(), h.end(), out);
  }

  const DBuf<double>& latest(int f) const {
    if (f < 4 && carriers_advanced) return state[nxt()][f];
    return state[cur][f];
  }
};

struct LuHandle {
  MfFactor F;
  int precision = PECS_PREC_FP64;
  bool uploaded = false;
  FactorBank bank;
  int nrhs_cap = 0;
  DBuf<double> b, y, x;
  std::vector<DBuf<double>> w;
  SetTable tab;
  cudaStream_t st = nullptr;
  ~LuHandle() {
    if (st) cudaStreamDestroy(st);
  }
};

namespace {
// Loads this file's device module on device `dev` (current) and records the
// device addresses of the no-alloc solve's static arrays; defined with them.
void noalloc_reserve(int dev);
}  // namespace

}  // namespace pecs

using namespace pecs;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct pecs_ctx {
  Engine e;
};
struct pecs_lu {
  LuHandle h;
};

#define PECS_TRY(...)                                   \
  try {                                                 \
    __VA_ARGS__;                                        \
    return PECS_OK;                                     \
  } catch (const PecsError& ex) {                       \
    set_error(ex.what());                               \
    return ex.code;                                     \
  } catch (const std::bad_alloc&) {                     \
    set_error("out of host memory");                    \
    return PECS_E_ARG;                                  \
  } catch (const std::exception& ex) {                  \
    set_error(ex.what());                               \
    return PECS_E_ARG;                                  \
  }

// pecs_lu_factor: fronts with at least this many rows go to the GPU
static std::atomic<int> g_lu_gpu_min_front{1024};

// Also makes the context's GPU the calling thread's current device: a context
// may be driven from any host thread (one per context in a concurrent ragged
// sweep), and a thread's current device starts at 0.
static void need_device(Engine& e) {
  if (e.host_only) throw PecsError(PECS_E_STATE, "context was created with host_setup_only");
  PECS_CUDA(cudaSetDevice(e.opt.device));
}

extern "C" {

const char* pecs_last_error(void) { return g_last_error.c_str(); }

void pecs_default_options(pecs_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->precision = PECS_PREC_FP64;
  opt->leaf_cells = 8;
  opt->use_graphs = 1;
  opt->ir_max_iters = 0;
  opt->ir_tol = 1e-12;
  opt->device = 0;
  opt->autotune = 1;
}

int pecs_apply_boundary_layout(pecs_params* p, int insulated, int schottky) {
  PECS_TRY({
    if (!p) throw PecsError(PECS_E_ARG, "params is NULL");
    const int D = kDirichlet, N = kNeumann, I = kInterface, S = kSchottky;
    const bool full = p->full_system != 0;
    const int semi[4] = {insulated ? N : D, full ? I : D, D, schottky ? S : D};
    const int elec_tb = (full && insulated) ? N : D;
    const int elec[4] = {I, D, elec_tb, elec_tb};
    const int pois[4] = {insulated ? N : D, D, D, schottky ? S : D};
    const int pois_elec[4] = {0, 0, (full && insulated) ? N : 0,
                              full && schottky ? S : ((full && insulated) ? N : 0)};
    for (int f = 0; f < 4; ++f) {
      p->bc_semi[f] = semi[f];
      p->bc_elec[f] = elec[f];
      p->bc_poisson[f] = pois[f];
      p->bc_poisson_elec[f] = pois_elec[f];
    }
  })
}

int pecs_create(const pecs_params* params, int n_inst, const pecs_options* opt, pecs_ctx** out) {
  PECS_TRY({
    if (!out) throw PecsError(PECS_E_ARG, "out is NULL");
    *out = nullptr;
    std::string err = validate_params(params, n_inst);
    if (!err.empty()) throw PecsError(PECS_E_ARG, err);
    pecs_options o;
    pecs_default_options(&o);
    if (opt) o = *opt;
    if (o.precision != PECS_PREC_FP64 && o.precision != PECS_PREC_FP32_IR &&
        o.precision != PECS_PREC_FP32_MIXED)
      throw PecsError(PECS_E_ARG, "unknown precision");
    std::unique_ptr<pecs_ctx> c(new pecs_ctx());
    c->e.create(std::vector<pecs_params>(params, params + n_inst), o);
    *out = c.release();
  })
}

void pecs_destroy(pecs_ctx* ctx) { delete ctx; }

int pecs_get_info(pecs_ctx* ctx, pecs_info* info) {
  PECS_TRY({
    if (!ctx || !info) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    std::memset(info, 0, sizeof(*info));
    info->n_inst = e.n_inst;
    for (int f = 0; f < 5; ++f) info->ndofs[f] = e.nd[f];
    long long es = 0, ee = 0;
    int ls = 0, le = 0, ns = 0, ne = 0;
    for (int t = 0; t < e.n_fs; ++t) {
      es += e.fs[t].entries();
      ls = std::max(ls, std::max(e.fs[t].n_heights, e.fs[t].n_depths));
      ns += (int)e.fs[t].nodes.size();
    }
    for (int t = 0; t < e.n_fe; ++t) {
      ee += e.fe[t].entries();
      le = std::max(le, std::max(e.fe[t].n_heights, e.fe[t].n_depths));
      ne += (int)e.fe[t].nodes.size();
    }
    info->factor_entries[0] = es;
    info->factor_entries[1] = ee;
    info->factor_entries[2] = e.fp.entries();
    info->factor_levels[0] = ls;
    info->factor_levels[1] = le;
    info->factor_levels[2] = std::max(e.fp.n_heights, e.fp.n_depths);
    info->factor_nodes[0] = ns;
    info->factor_nodes[1] = ne;
    info->factor_nodes[2] = (int)e.fp.nodes.size();
    info->factor_bytes = e.bank_c.bytes() + e.bank_p.bytes();
    info->setup_seconds = e.setup_seconds;
    info->n_distinct_carrier_factors = e.n_fs + e.n_fe;
    if (!e.host_only) {
      info->launches_per_step = e.launches_per_step();
      info->solve_bytes[0] = e.solve_bytes(0);
      info->solve_bytes[1] = e.solve_bytes(1);
      info->solve_launches[0] = e.bank_c.kernel_launches_per_solve();
      info->solve_launches[1] = e.bank_p.kernel_launches_per_solve();
      info->setup_launches = e.bank_c.tune_launches() + e.bank_p.tune_launches();
      info->initialize_launches = e.initialize_launches();
      info->tuned_sweep_ms[0] = e.bank_c.tuned_ms();
      info->tuned_sweep_ms[1] = e.bank_p.tuned_ms();
      info->flow_rpl[0] = e.bank_c.flow_rpl();
      info->flow_rpl[1] = e.bank_p.flow_rpl();
      info->flow_top[0] = e.bank_c.flow_top();
      info->flow_top[1] = e.bank_p.flow_top();
    }
  })
}

int pecs_get_matrix(pecs_ctx* ctx, int which, int* n, long long* nnz, int* rowptr, int* col,
                    double* val) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    Setup& S = *ctx->e.S;
    const Csr* A = nullptr;
    switch (which) {
      case PECS_MAT_N: A = &S.semi.A[0]; break;
      case PECS_MAT_P: A = &S.semi.A[1]; break;
      case PECS_MAT_R: A = S.full ? &S.elec.A[0] : nullptr; break;
      case PECS_MAT_O: A = S.full ? &S.elec.A[1] : nullptr; break;
      case PECS_MAT_POISSON: A = &S.pois.A; break;
      case PECS_MAT_MASS_SEMI: A = &S.semi.M; break;
      case PECS_MAT_MASS_ELEC: A = S.full ? &S.elec.M : nullptr; break;
      default: break;
    }
    if (!A) throw PecsError(PECS_E_ARG, "no such matrix");
    if (n) *n = A->n;
    if (nnz) *nnz = A->nnz();
    if (rowptr) std::copy(A->rowptr.begin(), A->rowptr.end(), rowptr);
    if (col) std::copy(A->col.begin(), A->col.end(), col);
    if (val) std::copy(A->val.begin(), A->val.end(), val);
  })
}

int pecs_get_setup_vector(pecs_ctx* ctx, int kind, int field, int inst, double* out, long long n) {
  PECS_TRY({
    if (!ctx || !out) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    Setup& S = *e.S;
    if (field < 0 || field >= 5 || e.nd[field] == 0) throw PecsError(PECS_E_ARG, "no such field");
    if (inst < 0 || inst >= e.n_inst) throw PecsError(PECS_E_ARG, "bad instance");
    if (n < e.nd[field]) throw PecsError(PECS_E_ARG, "output buffer too small");
    const std::vector<double>* v = nullptr;
    if (kind == PECS_SETUP_CONST_RHS) {
      v = &S.bconst[field][inst];
    } else if (kind == PECS_SETUP_INITIAL) {
      if (field == PECS_FIELD_POISSON)
        throw PecsError(PECS_E_ARG, "the initial potential comes from a solve (pecs_initialize)");
      v = &S.init[field][inst];
    } else {
      throw PecsError(PECS_E_ARG, "unknown kind");
    }
    if ((int)v->size() != e.nd[field]) throw PecsError(PECS_E_STATE, "setup vector not built");
    std::copy(v->begin(), v->end(), out);
  })
}

int pecs_get_mesh(pecs_ctx* ctx, int mesh, int* nx, int* ny, double* xs, double* ys) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    Setup& S = *ctx->e.S;
    const Grid* g = nullptr;
    if (mesh == PECS_MESH_SEMI) g = &S.semi.grid;
    else if (mesh == PECS_MESH_ELEC && S.full) g = &S.elec.grid;
    else if (mesh == PECS_MESH_POISSON) g = &S.pois.grid;
    if (!g) throw PecsError(PECS_E_ARG, "no such mesh");
    if (nx) *nx = g->nx;
    if (ny) *ny = g->ny;
    if (xs) std::copy(g->xs.begin(), g->xs.end(), xs);
    if (ys) std::copy(g->ys.begin(), g->ys.end(), ys);
  })
}

int pecs_initialize(pecs_ctx* ctx) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    ctx->e.initialize();
  })
}

static void check_field(Engine& e, int inst, int field, size_t n) {
  need_device(e);
  if (inst < 0 || inst >= e.n_inst) throw PecsError(PECS_E_ARG, "instance out of range");
  if (field < 0 || field > 4 || e.nd[field] == 0) throw PecsError(PECS_E_ARG, "field out of range");
  if (n != (size_t)e.nd[field]) throw PecsError(PECS_E_ARG, "length does not match the field size");
}

int pecs_set_state(pecs_ctx* ctx, int inst, int field, const double* host, size_t n) {
  PECS_TRY({
    if (!ctx || !host) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    check_field(e, inst, field, n);
    if (e.carriers_advanced) throw PecsError(PECS_E_STATE, "step in progress");
    PECS_CUDA(cudaMemcpyAsync(e.state[e.cur][field].p + (size_t)inst * e.nd[field], host, n * 8,
                              cudaMemcpyHostToDevice, e.st));
    PECS_CUDA(cudaStreamSynchronize(e.st));
    e.initialized = true;
  })
}

int pecs_get_state(pecs_ctx* ctx, int inst, int field, double* host, size_t n) {
  PECS_TRY({
    if (!ctx || !host) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    check_field(e, inst, field, n);
    PECS_CUDA(cudaMemcpyAsync(host, e.latest(field).p + (size_t)inst * e.nd[field], n * 8,
                              cudaMemcpyDeviceToHost, e.st));
    PECS_CUDA(cudaStreamSynchronize(e.st));
  })
}

int pecs_set_instances(pecs_ctx* ctx, const pecs_params* params, int n_inst) {
  PECS_TRY({
    if (!ctx || !params) throw PecsError(PECS_E_ARG, "NULL argument");
    need_device(ctx->e);
    ctx->e.set_instances(std::vector<pecs_params>(params, params + n_inst));
  })
}

int pecs_get_state_device(pecs_ctx* ctx, int inst, int field, double* dst_dev) {
  PECS_TRY({
    if (!ctx || !dst_dev) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    check_field(e, inst, field, (size_t)(field >= 0 && field < 5 ? e.nd[field] : 0));
    PECS_CUDA(cudaMemcpyAsync(dst_dev, e.latest(field).p + (size_t)inst * e.nd[field],
                              (size_t)e.nd[field] * 8, cudaMemcpyDeviceToDevice, e.st));
    PECS_CUDA(cudaStreamSynchronize(e.st));
  })
}

int pecs_set_state_device(pecs_ctx* ctx, int inst, int field, const double* src_dev) {
  PECS_TRY({
    if (!ctx || !src_dev) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    check_field(e, inst, field, (size_t)(field >= 0 && field < 5 ? e.nd[field] : 0));
    if (e.carriers_advanced) throw PecsError(PECS_E_STATE, "step in progress");
    PECS_CUDA(cudaMemcpyAsync(e.state[e.cur][field].p + (size_t)inst * e.nd[field], src_dev,
                              (size_t)e.nd[field] * 8, cudaMemcpyDeviceToDevice, e.st));
    PECS_CUDA(cudaStreamSynchronize(e.st));
    e.initialized = true;
  })
}

int pecs_get_rhs(pecs_ctx* ctx, int inst, int field, double* host, size_t n) {
  PECS_TRY({
    if (!ctx || !host) throw PecsError(PECS_E_ARG, "NULL argument");
    Engine& e = ctx->e;
    check_field(e, inst, field, n);
    PECS_CUDA(cudaMemcpyAsync(host, e.rhs[field].p + (size_t)inst * e.nd[field], n * 8,
                              cudaMemcpyDeviceToHost, e.st));
    PECS_CUDA(cudaStreamSynchronize(e.st));
  })
}

int pecs_assemble_carrier_rhs(pecs_ctx* ctx) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    if (ctx->e.carriers_advanced) throw PecsError(PECS_E_STATE, "carriers already advanced");
    ctx->e.stage_carrier_rhs(ctx->e.st, nullptr);
    PECS_CUDA(cudaStreamSynchronize(ctx->e.st));
  })
}

int pecs_solve_carriers(pecs_ctx* ctx) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    if (ctx->e.carriers_advanced) throw PecsError(PECS_E_STATE, "carriers already advanced");
    ctx->e.stage_solve_carriers(ctx->e.st, nullptr);
    PECS_CUDA(cudaStreamSynchronize(ctx->e.st));
  })
}

int pecs_assemble_poisson_rhs(pecs_ctx* ctx) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    ctx->e.stage_poisson_rhs(ctx->e.st, nullptr);
    PECS_CUDA(cudaStreamSynchronize(ctx->e.st));
  })
}

int pecs_solve_poisson(pecs_ctx* ctx) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    ctx->e.stage_solve_poisson(ctx->e.st, nullptr);
    PECS_CUDA(cudaStreamSynchronize(ctx->e.st));
  })
}

int pecs_time_stages(pecs_ctx* ctx, int reps, double* ms) {
  PECS_TRY({
    if (!ctx || !ms || reps <= 0) throw PecsError(PECS_E_ARG, "invalid arguments");
    Engine& e = ctx->e;
    need_device(e);
    if (!e.initialized) throw PecsError(PECS_E_STATE, "pecs_initialize must be called first");
    if (e.carriers_advanced) throw PecsError(PECS_E_STATE, "a step is half done (carriers advanced)");
    cudaEvent_t ev[5];
    for (auto& v : ev) PECS_CUDA(cudaEventCreate(&v));
    double acc[4] = {0, 0, 0, 0};
    for (int r = 0; r <= reps; ++r) {  // the first step warms up, untimed
      PECS_CUDA(cudaEventRecord(ev[0], e.st));
      e.stage_carrier_rhs(e.st, nullptr);
      PECS_CUDA(cudaEventRecord(ev[1], e.st));
      e.stage_solve_carriers(e.st, nullptr);
      PECS_CUDA(cudaEventRecord(ev[2], e.st));
      e.stage_poisson_rhs(e.st, nullptr);
      PECS_CUDA(cudaEventRecord(ev[3], e.st));
      e.stage_solve_poisson(e.st, nullptr);
      PECS_CUDA(cudaEventRecord(ev[4], e.st));
      PECS_CUDA(cudaEventSynchronize(ev[4]));
      if (r == 0) continue;
      for (int k = 0; k < 4; ++k) {
        float t = 0.f;
        PECS_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
        acc[k] += t;
      }
    }
    for (auto& v : ev) cudaEventDestroy(v);
    for (int k = 0; k < 4; ++k) ms[k] = acc[k] / reps;
  })
}

int pecs_step(pecs_ctx* ctx, int n_steps) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    if (n_steps < 0) throw PecsError(PECS_E_ARG, "n_steps < 0");
    Engine& e = ctx->e;
    if (!e.initialized) throw PecsError(PECS_E_STATE, "pecs_initialize must be called first");
    if (e.carriers_advanced) throw PecsError(PECS_E_STATE, "step in progress");
    for (int s = 0; s < n_steps; ++s) e.full_step(e.st, nullptr);
    PECS_CUDA(cudaStreamSynchronize(e.st));
  })
}

int pecs_run_to_steady_state(pecs_ctx* ctx, int max_steps, double tol, int check_every, int* steps,
                             double* rel_change) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    if (!(tol >= 0.0)) throw PecsError(PECS_E_ARG, "tol must be >= 0");
    ctx->e.run_to_steady(max_steps, tol, check_every, steps, rel_change);
  })
}

int pecs_solve_residual(pecs_ctx* ctx, int which, double* max_rel) {
  PECS_TRY({
    if (!ctx || !max_rel || which < 0 || which > 1) throw PecsError(PECS_E_ARG, "invalid arguments");
    need_device(ctx->e);
    *max_rel = ctx->e.solve_residual(which);
  })
}

int pecs_interface_current(pecs_ctx* ctx, double* out) {
  PECS_TRY({
    if (!ctx || !out) throw PecsError(PECS_E_ARG, "NULL argument");
    need_device(ctx->e);
    ctx->e.interface_current(out);
  })
}

int pecs_sweep_stream(pecs_ctx* ctx, int n_points, const pecs_params* params,
                      const double* const* init_n, const double* const* init_p, int max_steps, double tol,
                      int check_every, int* steps, double* currents, double* const* final_fields) {
  PECS_TRY({
    if (!ctx || !params || n_points < 0) throw PecsError(PECS_E_ARG, "invalid arguments");
    {
      // every point must share the context's meshes and fixed matrices
      std::vector<pecs_params> chk(params, params + n_points);
      chk.insert(chk.begin(), ctx->e.S->inst[0]);
      std::string err = validate_params(chk.data(), (int)chk.size());
      if (!err.empty()) throw PecsError(PECS_E_ARG, err);
    }
    need_device(ctx->e);
    if (!(tol >= 0.0)) throw PecsError(PECS_E_ARG, "tol must be >= 0");
    if (ctx->e.carriers_advanced) throw PecsError(PECS_E_STATE, "step in progress");
    ctx->e.sweep_stream(n_points, params, init_n, init_p, max_steps, tol, check_every, steps, currents,
                        final_fields);
  })
}

int pecs_iv_sweep(pecs_ctx* ctx, const double* const* init_fields, int max_steps, double tol,
                  int check_every, double* currents, int* steps, double* const* final_fields) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    Engine& e = ctx->e;
    if (init_fields) {
      e.carriers_advanced = false;
      for (int f = 0; f < 5; ++f) {
        if (!e.nd[f]) continue;
        if (!init_fields[f]) throw PecsError(PECS_E_ARG, "init_fields entry is NULL");
        PECS_CUDA(cudaMemcpyAsync(e.state[e.cur][f].p, init_fields[f], (size_t)e.n_inst * e.nd[f] * 8,
                                  cudaMemcpyHostToDevice, e.st));
      }
      PECS_CUDA(cudaStreamSynchronize(e.st));
      e.initialized = true;
    } else {
      e.initialize();
    }
    e.run_to_steady(max_steps, tol, check_every, steps, nullptr);
    if (currents) e.interface_current(currents);
    if (final_fields) {
      for (int f = 0; f < 5; ++f) {
        if (!e.nd[f] || !final_fields[f]) continue;
        PECS_CUDA(cudaMemcpyAsync(final_fields[f], e.state[e.cur][f].p, (size_t)e.n_inst * e.nd[f] * 8,
                                  cudaMemcpyDeviceToHost, e.st));
      }
      PECS_CUDA(cudaStreamSynchronize(e.st));
    }
  })
}

int pecs_time_solve(pecs_ctx* ctx, int which, int reps, double* ms_per_solve) {
  PECS_TRY({
    if (!ctx || !ms_per_solve || reps <= 0 || which < 0 || which > 1)
      throw PecsError(PECS_E_ARG, "invalid arguments");
    need_device(ctx->e);
    if (ctx->e.carriers_advanced) throw PecsError(PECS_E_STATE, "step in progress");
    *ms_per_solve = ctx->e.time_solves(which, reps);
  })
}

int pecs_last_run_steps(pecs_ctx* ctx) { return ctx ? ctx->e.last_run_steps : -1; }

void* pecs_get_stream(pecs_ctx* ctx) { return ctx ? (void*)ctx->e.st : nullptr; }

int pecs_synchronize(pecs_ctx* ctx) {
  PECS_TRY({
    if (!ctx) throw PecsError(PECS_E_ARG, "ctx is NULL");
    need_device(ctx->e);
    PECS_CUDA(cudaStreamSynchronize(ctx->e.st));
  })
}

// ---- drop-in direct solver -------------------------------------------------
int pecs_lu_factor(int n, const int* rowptr, const int* col, const double* val, const int* dof_cell,
                   const int* dof_class, int n_cells, const double* cell_xy, int precision,
                   int leaf_cells, pecs_lu** out) {
  PECS_TRY({
    if (!out) throw PecsError(PECS_E_ARG, "out is NULL");
    *out = nullptr;
    if (n <= 0 || !rowptr || !col || !val || !dof_cell || n_cells <= 0 || !cell_xy)
      throw PecsError(PECS_E_ARG, "invalid matrix arguments");
    if (precision != PECS_PREC_FP64 && precision != PECS_PREC_FP32_IR)
      throw PecsError(PECS_E_ARG, "unknown precision");
    if (rowptr[0] != 0 || rowptr[n] < 0) throw PecsError(PECS_E_ARG, "bad rowptr");
    Csr A;
    A.n = n;
    A.rowptr.assign(rowptr, rowptr + n + 1);
    A.col.assign(col, col + rowptr[n]);
    A.val.assign(val, val + rowptr[n]);
    std::unique_ptr<pecs_lu> h(new pecs_lu());
    h->h.precision = precision;
    h->h.F = mf_analyze(A, dof_cell, dof_class, n_cells, cell_xy, leaf_cells);
    std::shared_ptr<FrontOffload> off;
    int ndev = 0, dev = 0;
    const int min_front = g_lu_gpu_min_front.load();
    if (min_front >= 0 && cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0 && cudaGetDevice(&dev) == cudaSuccess)
      off = make_gpu_front_offload(dev, min_front);
    try {
      mf_factorize(h->h.F, A, 0, off.get());
    } catch (const PecsError&) {
      throw;
    } catch (const std::exception& ex) {
      throw PecsError(PECS_E_SINGULAR, ex.what());
    }
    *out = h.release();
  })
}

int pecs_lu_set_gpu_factor_min_front(int rows) { return g_lu_gpu_min_front.exchange(rows); }

int pecs_debug_lu_values(pecs_lu* lu, double* out, long long n, long long* count) {
  PECS_TRY({
    if (!lu) throw PecsError(PECS_E_ARG, "lu is NULL");
    const MfFactor& F = lu->h.F;
    if (F.Gf.empty()) throw PecsError(PECS_E_STATE, "host factors were released");
    long long tot = 0;
    for (size_t j = 0; j < F.Gf.size(); ++j) tot += (long long)(F.Gf[j].size() + F.Hb[j].size());
    if (count) *count = tot;
    if (out) {
      if (n < tot) throw PecsError(PECS_E_ARG, "output too small");
      long long o = 0;
      for (size_t j = 0; j < F.Gf.size(); ++j) {
        std::copy(F.Gf[j].begin(), F.Gf[j].end(), out + o);
        o += (long long)F.Gf[j].size();
        std::copy(F.Hb[j].begin(), F.Hb[j].end(), out + o);
        o += (long long)F.Hb[j].size();
      }
    }
  })
}

static void lu_upload(LuHandle& h, int nrhs) {
  if (!h.uploaded) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
      throw PecsError(PECS_E_NODEVICE, "no CUDA device available");
    PECS_CUDA(cudaStreamCreateWithFlags(&h.st, cudaStreamNonBlocking));
    h.bank.build({&h.F}, h.precision == PECS_PREC_FP64 ? PECS_PREC_FP64 : PECS_PREC_FP32_IR);
    // The no-alloc solve's static scratch lives in this file's device module,
    // which CUDA loads lazily; reserving it here, where allocation is allowed,
    // means pecs_lu_solve_device_noalloc never triggers that load.
    int dev = -1;
    PECS_CUDA(cudaGetDevice(&dev));
    noalloc_reserve(dev);
    h.uploaded = true;
  }
  if (nrhs > h.nrhs_cap) {
    const int n = h.F.n;
    h.b.alloc((size_t)nrhs * n);
    h.y.alloc((size_t)nrhs * n);
    h.x.alloc((size_t)nrhs * n);
    h.w.resize(nrhs);
    for (auto& w : h.w) {
      w.alloc(h.bank.set_wtotal(0));
      w.zero();
    }
    h.nrhs_cap = nrhs;
  }
}

static void lu_bind(LuHandle& h, int nrhs, const double* b, double* x) {
  const int n = h.F.n;
  std::vector<double*> hb(nrhs), hy(nrhs), hw(nrhs), hx(nrhs);
  for (int r = 0; r < nrhs; ++r) {
    hb[r] = const_cast<double*>(b) + (size_t)r * n;
    hy[r] = h.y.p + (size_t)r * n;
    hw[r] = h.w[r].p;
    hx[r] = x + (size_t)r * n;
  }
  h.tab.b.resize(1);
  h.tab.y.resize(1);
  h.tab.w.resize(1);
  h.tab.x.resize(1);
  h.tab.b[0].upload(hb);
  h.tab.y[0].upload(hy);
  h.tab.w[0].upload(hw);
  h.tab.x[0].upload(hx);
  h.tab.view.set[0] = SetView{nrhs, h.tab.b[0].p, h.tab.y[0].p, h.tab.w[0].p, h.tab.x[0].p};
  h.tab.max_nrhs = nrhs;
}

int pecs_lu_solve_device(pecs_lu* lu, int nrhs, const double* b_dev, double* x_dev, void* stream) {
  PECS_TRY({
    if (!lu || nrhs <= 0 || !b_dev || !x_dev) throw PecsError(PECS_E_ARG, "invalid arguments");
    LuHandle& h = lu->h;
    lu_upload(h, nrhs);
    lu_bind(h, nrhs, b_dev, x_dev);
    cudaStream_t s = stream ? (cudaStream_t)stream : h.st;
    h.bank.solve(h.tab.view, nrhs, s);
    PECS_CUDA(cudaStreamSynchronize(s));
  })
}

int pecs_lu_solve(pecs_lu* lu, int nrhs, const double* b, double* x) {
  PECS_TRY({
    if (!lu || nrhs <= 0 || !b || !x) throw PecsError(PECS_E_ARG, "invalid arguments");
    LuHandle& h = lu->h;
    lu_upload(h, nrhs);
    const size_t bytes = (size_t)nrhs * h.F.n * 8;
    PECS_CUDA(cudaMemcpyAsync(h.b.p, b, bytes, cudaMemcpyHostToDevice, h.st));
    lu_bind(h, nrhs, h.b.p, h.x.p);
    h.bank.solve(h.tab.view, nrhs, h.st);
    PECS_CUDA(cudaMemcpyAsync(x, h.x.p, bytes, cudaMemcpyDeviceToHost, h.st));
    PECS_CUDA(cudaStreamSynchronize(h.st));
  })
}

int pecs_lu_stats(pecs_lu* lu, long long* entries, int* levels, int* nodes, int* max_front) {
  PECS_TRY({
    if (!lu) throw PecsError(PECS_E_ARG, "lu is NULL");
    const MfFactor& F = lu->h.F;
    if (entries) *entries = F.entries();
    if (levels) *levels = std::max(F.n_heights, F.n_depths);
    if (nodes) *nodes = (int)F.nodes.size();
    if (max_front) *max_front = F.max_front();
  })
}

void pecs_lu_destroy(pecs_lu* lu) { delete lu; }

// ---- solve for callers that cannot allocate device memory ------------------
// Some callers may not allocate device memory at solve time: an application
// whose memory is carved up by its own pool allocator, a code that has to stay
// inside a fixed device-memory budget, or a host library called from a context
// where cudaMalloc is not allowed.  pecs_lu_solve_device_noalloc runs the same
// forward/backward sweeps as pecs_lu_solve_device, but keeps the sweeps'
// scratch -- the forward-sweep slots and the per-node update vectors -- in the
// fixed file-scope array below instead of memory owned by the handle, and
// allocates nothing.  CUDA loads this file's device module, and with it the
// array (8 MiB), on a device when the factors are first uploaded there (the
// first pecs_lu_solve / pecs_lu_solve_device call of a handle); the device
// then holds it until the process exits.
}  // extern "C"

namespace pecs {
namespace {
constexpr size_t kNoAllocScratchDoubles = size_t(1) << 20;  // 8 MiB
constexpr int kNoAllocMaxRhs = 8;
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];
static __device__ __align__(256) double* g_noalloc_ptrs[4 * kNoAllocMaxRhs];

struct NoAllocSlot {
  double* scratch = nullptr;
  double** ptrs = nullptr;
};
std::mutex g_noalloc_mu;
NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];

// The host-side names of the static arrays are only stand-ins: their device
// addresses are looked up once per device, with that device current.  Taking
// the first address loads the module, so this runs at factor upload.
void noalloc_reserve(int dev) {
  if (dev < 0 || dev >= kNoAllocMaxDevices) throw PecsError(PECS_E_ARG, "device ordinal too large");
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  NoAllocSlot& s = g_noalloc_slot[dev];
  if (!s.scratch) {
    void* a = nullptr;
    void* b = nullptr;
    PECS_CUDA(cudaGetSymbolAddress(&a, g_noalloc_scratch));
    PECS_CUDA(cudaGetSymbolAddress(&b, g_noalloc_ptrs));
    s.scratch = static_cast<double*>(a);
    s.ptrs = static_cast<double**>(b);
  }
}

// Addresses recorded by noalloc_reserve; never loads anything itself.
NoAllocSlot noalloc_slot(int dev) {
  if (dev < 0 || dev >= kNoAllocMaxDevices) throw PecsError(PECS_E_ARG, "device ordinal too large");
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  const NoAllocSlot s = g_noalloc_slot[dev];
  if (!s.scratch)
    throw PecsError(PECS_E_STATE, "the static scratch is not reserved on this device: upload the "
                                  "factors there first (pecs_lu_solve or pecs_lu_solve_device)");
  return s;
}
}  // namespace
}  // namespace pecs

extern "C" {

int pecs_lu_solve_device_noalloc(pecs_lu* lu, int nrhs, const double* b_dev, double* x_dev,
                                 void* stream) {
  PECS_TRY({
    if (!lu || !b_dev || !x_dev) throw PecsError(PECS_E_ARG, "invalid arguments");
    if (nrhs < 1 || nrhs > kNoAllocMaxRhs)
      throw PecsError(PECS_E_ARG, "nrhs must be 1.." + std::to_string(kNoAllocMaxRhs));
    LuHandle& h = lu->h;
    if (!h.uploaded)
      throw PecsError(PECS_E_STATE,
                      "the factors are not on the device yet: one pecs_lu_solve or "
                      "pecs_lu_solve_device call on this handle uploads them");
    const size_t n = (size_t)h.F.n, nw = (size_t)h.bank.set_wtotal(0);
    const size_t need = (size_t)nrhs * (n + nw);
    if (need > kNoAllocScratchDoubles)
      throw PecsError(PECS_E_ARG, "this solve needs " + std::to_string(need) +
                                      " doubles of scratch; the static scratch holds " +
                                      std::to_string(kNoAllocScratchDoubles));
    int dev = -1;
    PECS_CUDA(cudaGetDevice(&dev));
    cudaPointerAttributes pa;
    PECS_CUDA(cudaPointerGetAttributes(&pa, h.y.p));
    if (pa.device != dev)
      throw PecsError(PECS_E_ARG, "the current device is not the device holding the factors");
    NoAllocSlot slot = noalloc_slot(dev);
    cudaStream_t s = stream ? (cudaStream_t)stream : h.st;
    double* table[4 * kNoAllocMaxRhs];
    for (int r = 0; r < nrhs; ++r) {
      table[r] = const_cast<double*>(b_dev) + (size_t)r * n;
      table[nrhs + r] = slot.scratch + (size_t)r * n;
      table[2 * nrhs + r] = slot.scratch + (size_t)nrhs * n + (size_t)r * nw;
      table[3 * nrhs + r] = x_dev + (size_t)r * n;
    }
    // pageable source: the call returns once the table has been staged
    PECS_CUDA(cudaMemcpyAsync(slot.ptrs, table, sizeof(double*) * 4 * nrhs, cudaMemcpyHostToDevice, s));
    SetsView sv{};
    sv.set[0] = SetView{nrhs, slot.ptrs, slot.ptrs + nrhs, slot.ptrs + 2 * nrhs, slot.ptrs + 3 * nrhs};
    h.bank.solve(sv, nrhs, s);
    PECS_CUDA(cudaStreamSynchronize(s));
  })
}

// diagnostic: per-level device times of one carrier (which = 0) or Poisson (1)
// sweep of an FP32 panel bank; returns the number of levels written
int pecs_debug_time_levels(pecs_ctx* ctx, int which, int reps, double* ms, int cap) {
  int n = 0;
  const int rc = [&]() -> int {
    PECS_TRY({
      if (!ctx || !ms || cap <= 0 || reps <= 0 || (which != 0 && which != 1))
        throw PecsError(PECS_E_ARG, "invalid arguments");
      Engine& e = ctx->e;
      need_device(e);
      if (!e.il_f32(which)) throw PecsError(PECS_E_STATE, "level timing needs FP32 panel sweeps");
      const FactorBank& B = which == 0 ? e.bank_c : e.bank_p;
      const std::vector<double> t = B.time_levels(e.il_view_f(which, false), e.il[which].max_R, e.st, reps);
      n = std::min(cap, (int)t.size());
      for (int k = 0; k < n; ++k) ms[k] = t[k];
    })
  }();
  return rc == PECS_OK ? n : rc;
}

int pecs_debug_flow_stall(pecs_ctx* ctx, int which, int* flag) {
  PECS_TRY({
    if (!ctx || !flag || (which != 0 && which != 1)) throw PecsError(PECS_E_ARG, "invalid arguments");
    Engine& e = ctx->e;
    need_device(e);
    const FactorBank& B = which == 0 ? e.bank_c : e.bank_p;
    if (B.flow_rpl() == 0 && !B.rows_flow()) throw PecsError(PECS_E_STATE, "the bank does not use the flow sweep");
    B.debug_arm_flow_stall();
    e.bank_sweep(B, which, false, e.st);
    PECS_CUDA(cudaStreamSynchronize(e.st));
    *flag = B.flow_error(true);
  })
}

// diagnostic: apply the host copy of the factors (no GPU involved)
int pecs_lu_host_apply(pecs_lu* lu, const double* b, double* x) {
  PECS_TRY({
    if (!lu || !b || !x) throw PecsError(PECS_E_ARG, "invalid arguments");
    if (lu->h.F.Gf.empty()) throw PecsError(PECS_E_STATE, "host factors were released");
    mf_apply_host(lu->h.F, b, x);
  })
}

}  // extern "C"
