// Multifrontal solve kernels and their host-side plans (solve.cuh): one
// launch per tree level (few-right-hand-side and panel kernels), or one
// persistent dataflow launch per direction (flow sweeps) over the same items.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "solve.cuh"

namespace pecs {

namespace {

// Programmatic dependent launch: a sweep level is launched while the previous
// level still runs; it stages what does not depend on that level (item
// records, index metadata, its block tile) and then waits for the previous
// grid's completion and memory (griddepcontrol.wait) before reading vectors.
// A level lets the next one start once its CTAs are past their main loop.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// Polls of one wait before it gives up (with 64 ns sleeps and a global load
// each: tens to hundreds of milliseconds, against a whole sweep of well under
// a millisecond).
constexpr unsigned kFlowPollLimit = 1u << 18;

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_gpu(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Bounded wait for *ctr >= target; false (and the error flag set) when the
// poll limit runs out.
__device__ __noinline__ bool flow_wait(const int* ctr, int target, int* err) {
  if (ld_acquire_gpu(ctr) >= target) return true;
  for (unsigned n = 0; n < kFlowPollLimit; ++n) {
    __nanosleep(64);
    if (ld_acquire_gpu(ctr) >= target) return true;
  }
  atomicExch(err, 1);
  return false;
}


// Loads RB consecutive staged values (16-byte aligned) with vector loads.
template <typename T, int RB>
__device__ __forceinline__ void load_rhs(const T* p, T (&v)[RB]) {
  if constexpr (sizeof(T) == 4 && RB % 4 == 0) {
#pragma unroll
    for (int q = 0; q < RB / 4; ++q) {
      const float4 t = reinterpret_cast<const float4*>(p)[q];
      v[4 * q] = t.x;
      v[4 * q + 1] = t.y;
      v[4 * q + 2] = t.z;
      v[4 * q + 3] = t.w;
    }
  } else if constexpr (sizeof(T) == 8 && RB % 2 == 0) {
#pragma unroll
    for (int q = 0; q < RB / 2; ++q) {
      const double2 t = reinterpret_cast<const double2*>(p)[q];
      v[2 * q] = t.x;
      v[2 * q + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int r = 0; r < RB; ++r) v[r] = p[r];
  }
}

template <typename T>
__device__ __forceinline__ T group_sum(T v, int g) {
  // xor-butterfly inside aligned groups of g lanes (g a power of two <= 32)
  for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Vector access for the two RHS layouts: an array of per-RHS vectors
// (SetView) or one interleaved [dof][rhs] buffer per set (IlSetView).
__device__ __forceinline__ double getb(const SetView& s, int r, int d) { return s.b[r][d]; }
__device__ __forceinline__ double gety(const SetView& s, int r, int d) { return s.y[r][d]; }
__device__ __forceinline__ double getx(const SetView& s, int r, int d) { return s.x[r][d]; }
__device__ __forceinline__ double getw(const SetView& s, int r, int d) { return s.w[r][d]; }
// L2-coherent reads (ld.global.cg) of vectors written inside the same launch
// (flow sweeps: other CTAs' update and solution rows, which share cache lines
// with rows this SM may have read earlier)
__device__ __forceinline__ double getw_cg(const SetView& s, int r, int d) { return __ldcg(s.w[r] + d); }
__device__ __forceinline__ double getx_cg(const SetView& s, int r, int d) { return __ldcg(s.x[r] + d); }
__device__ __forceinline__ void puty(const SetView& s, int r, int d, double v) { s.y[r][d] = v; }
__device__ __forceinline__ void putx(const SetView& s, int r, int d, double v) { s.x[r][d] = v; }
__device__ __forceinline__ void putw(const SetView& s, int r, int d, double v) { s.w[r][d] = v; }
__device__ __forceinline__ double getb(const IlSetView& s, int r, int d) {
  return s.b[(size_t)d * s.nrhs + r];
}
__device__ __forceinline__ double gety(const IlSetView& s, int r, int d) {
  return s.y[(size_t)d * s.nrhs + r];
}
__device__ __forceinline__ double getx(const IlSetView& s, int r, int d) {
  return s.x[(size_t)d * s.nrhs + r];
}
__device__ __forceinline__ double getw(const IlSetView& s, int r, int d) {
  return s.w[(size_t)d * s.nrhs + r];
}
__device__ __forceinline__ double getw_cg(const IlSetView& s, int r, int d) {
  return __ldcg(s.w + (size_t)d * s.nrhs + r);
}
__device__ __forceinline__ double getx_cg(const IlSetView& s, int r, int d) {
  return __ldcg(s.x + (size_t)d * s.nrhs + r);
}
__device__ __forceinline__ void puty(const IlSetView& s, int r, int d, double v) {
  s.y[(size_t)d * s.nrhs + r] = v;
}
__device__ __forceinline__ void putx(const IlSetView& s, int r, int d, double v) {
  s.x[(size_t)d * s.nrhs + r] = v;
}
__device__ __forceinline__ void putw(const IlSetView& s, int r, int d, double v) {
  s.w[(size_t)d * s.nrhs + r] = v;
}

// Sum of the children's update entries that land on front position p.
template <bool CG, typename SVi>
__device__ __forceinline__ double gather_updates(const BankView& B, const SVi& st, int r, int c0,
                                                 int c1) {
  double v = 0.0;
  for (int c = c0; c < c1; ++c) v += CG ? getw_cg(st, r, B.cmap_idx[c]) : getw(st, r, B.cmap_idx[c]);
  return v;
}

// Forward sweep, large node: CTA computes rows [r0, r1) of Gf * d.
template <typename T, int RB, typename SV, bool CG = false>
__device__ void fwd_large(const BankView& B, const SV& S, int4 it, T* sm, int chunk) {
  const int j = it.x, r0 = it.y, r1 = it.z;
  const int s = B.s[j];
  const auto& st = S.set[B.node_set[j]];
  const int* own = B.own_idx + B.own_off[j];
  const int* cptr = B.cmap_ptr + B.cm_off[j];
  const T* G = static_cast<const T*>(B.G) + B.goff[j];
  const int wo = B.w_off[j];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  {
    // one chunk of RB right-hand sides (blockIdx.y in the level kernels)
    const int rb = chunk * RB;
    if (rb >= st.nrhs) return;
    const int nr = min(RB, st.nrhs - rb);
    for (int p = threadIdx.x; p < s; p += blockDim.x) {
      const int gd = own[p];
      const int c0 = cptr[p], c1 = cptr[p + 1];
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        double v = 0.0;
        if (r < nr) v = getb(st, rb + r, gd) - gather_updates<CG>(B, st, rb + r, c0, c1);
        sm[r * s + p] = (T)v;  // RHS-major: lanes of a warp read consecutive columns
      }
    }
    __syncthreads();
    // warps per row: 1 (8 rows per item) .. 8 (1 row per item, columns split)
    const int nrows = r1 - r0;
    const int wpr = nrows <= 1 ? 8 : (nrows <= 2 ? 4 : (nrows <= 4 ? 2 : 1));
    T* red = sm + (size_t)s * RB;  // nw x RB partial sums
    for (int rbase = r0; rbase < r1; rbase += nw / wpr) {
      const int row = rbase + warp / wpr, part = warp % wpr;
      T acc[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = T(0);
      if (row < r1) {
        const T* g = G + (long long)row * s;
        for (int c = part * 32 + lane; c < s; c += 32 * wpr) {
          const T gv = __ldg(g + c);
#pragma unroll
          for (int r = 0; r < RB; ++r) acc[r] += gv * sm[r * s + c];
        }
      }
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = group_sum(acc[r], 32);
      if (wpr > 1) {
        if (lane == 0)
#pragma unroll
          for (int r = 0; r < RB; ++r) red[warp * RB + r] = acc[r];
        __syncthreads();
        if (part == 0)
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            T t = T(0);
            for (int q = 0; q < wpr; ++q) t += red[(warp + q) * RB + r];
            acc[r] = t;
          }
      }
      if (part == 0 && row < r1) {
#pragma unroll
        for (int r = 0; r < RB; ++r) {
          if (lane == r && r < nr) {
            if (row < s) {
              puty(st, rb + r, own[row], (double)acc[r]);
            } else {
              const int t = row - s;
              const double cu = gather_updates<CG>(B, st, rb + r, cptr[row], cptr[row + 1]);
              putw(st, rb + r, wo + t, cu + (double)acc[r]);
            }
          }
        }
      }
      if (wpr > 1) __syncthreads();
    }
    __syncthreads();
  }
}

// Forward sweep, thin node (s <= kThinCols): the node's Gf is stored
// column-major, so lane `row` reads Gf[c][row] for c = 0..s-1: consecutive
// lanes read consecutive addresses and every lane has s independent loads in
// flight; no cross-lane reduction.  A warp item covers rows [r0, r1).
template <typename T, int RB, typename SV, bool CG = false>
__device__ void fwd_thin(const BankView& B, const SV& S, int4 it, T* sm, int chunk) {
  const int j = it.x, r0 = it.y, r1 = it.z;
  const int s = B.s[j], m = B.m[j], f = s + m;
  const auto& st = S.set[B.node_set[j]];
  const int* own = B.own_idx + B.own_off[j];
  const int* cptr = B.cmap_ptr + B.cm_off[j];
  const T* G = static_cast<const T*>(B.G) + B.goff[j];
  const int wo = B.w_off[j];
  const int lane = threadIdx.x & 31;
  {
    // one chunk of RB right-hand sides (blockIdx.y in the level kernels)
    const int rb = chunk * RB;
    if (rb >= st.nrhs) return;
    const int nr = min(RB, st.nrhs - rb);
    for (int p = lane; p < s; p += 32) {
      const int gd = own[p];
      const int c0 = cptr[p], c1 = cptr[p + 1];
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        double v = 0.0;
        if (r < nr) v = getb(st, rb + r, gd) - gather_updates<CG>(B, st, rb + r, c0, c1);
        sm[p * RB + r] = (T)v;
      }
    }
    __syncwarp();
    for (int row = r0 + lane; row < r1; row += 32) {
      T acc[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = T(0);
      const T* g = G + row;
#pragma unroll 4
      for (int c = 0; c < s; ++c) {
        const T gv = __ldg(g + (long long)c * f);
        T dv[RB];
        load_rhs<T, RB>(sm + c * RB, dv);
#pragma unroll
        for (int r = 0; r < RB; ++r) acc[r] += gv * dv[r];
      }
      if (row < s) {
#pragma unroll
        for (int r = 0; r < RB; ++r)
          if (r < nr) puty(st, rb + r, own[row], (double)acc[r]);
      } else {
        const int c0 = cptr[row], c1 = cptr[row + 1];
#pragma unroll
        for (int r = 0; r < RB; ++r)
          if (r < nr) putw(st, rb + r, wo + row - s, gather_updates<CG>(B, st, rb + r, c0, c1) + (double)acc[r]);
      }
    }
    __syncwarp();
  }
}

// Backward sweep, large node: rows [r0, r1) of Hb * [y_own ; x_upd].
template <typename T, int RB, typename SV, bool CG = false>
__device__ void bwd_large(const BankView& B, const SV& S, int4 it, T* sm, int chunk) {
  const int j = it.x, r0 = it.y, r1 = it.z;
  const int s = B.s[j], m = B.m[j], f = s + m;
  const auto& st = S.set[B.node_set[j]];
  const int* own = B.own_idx + B.own_off[j];
  const int* upd = B.upd_idx + B.upd_off[j];
  const T* H = static_cast<const T*>(B.H) + B.hoff[j];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  {
    // one chunk of RB right-hand sides (blockIdx.y in the level kernels)
    const int rb = chunk * RB;
    if (rb >= st.nrhs) return;
    const int nr = min(RB, st.nrhs - rb);
    for (int p = threadIdx.x; p < f; p += blockDim.x) {
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        double v = 0.0;
        if (r < nr) v = (p < s) ? gety(st, rb + r, own[p]) : (CG ? getx_cg(st, rb + r, upd[p - s]) : getx(st, rb + r, upd[p - s]));
        sm[r * f + p] = (T)v;
      }
    }
    __syncthreads();
    const int nrows = r1 - r0;
    const int wpr = nrows <= 1 ? 8 : (nrows <= 2 ? 4 : (nrows <= 4 ? 2 : 1));
    T* red = sm + (size_t)f * RB;
    for (int rbase = r0; rbase < r1; rbase += nw / wpr) {
      const int row = rbase + warp / wpr, part = warp % wpr;
      T acc[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = T(0);
      if (row < r1) {
        const T* h = H + (long long)row * f;
        for (int c = part * 32 + lane; c < f; c += 32 * wpr) {
          const T hv = __ldg(h + c);
#pragma unroll
          for (int r = 0; r < RB; ++r) acc[r] += hv * sm[r * f + c];
        }
      }
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = group_sum(acc[r], 32);
      if (wpr > 1) {
        if (lane == 0)
#pragma unroll
          for (int r = 0; r < RB; ++r) red[warp * RB + r] = acc[r];
        __syncthreads();
        if (part == 0)
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            T t = T(0);
            for (int q = 0; q < wpr; ++q) t += red[(warp + q) * RB + r];
            acc[r] = t;
          }
      }
      if (part == 0 && row < r1) {
#pragma unroll
        for (int r = 0; r < RB; ++r)
          if (lane == r && r < nr) putx(st, rb + r, own[row], (double)acc[r]);
      }
      if (wpr > 1) __syncthreads();
    }
    __syncthreads();
  }
}

// Backward sweep, thin node (s + m <= kThinCols): Hb stored column-major.
template <typename T, int RB, typename SV, bool CG = false>
__device__ void bwd_thin(const BankView& B, const SV& S, int4 it, T* sm, int chunk) {
  const int j = it.x, r0 = it.y, r1 = it.z;
  const int s = B.s[j], m = B.m[j], f = s + m;
  const auto& st = S.set[B.node_set[j]];
  const int* own = B.own_idx + B.own_off[j];
  const int* upd = B.upd_idx + B.upd_off[j];
  const T* H = static_cast<const T*>(B.H) + B.hoff[j];
  const int lane = threadIdx.x & 31;
  {
    // one chunk of RB right-hand sides (blockIdx.y in the level kernels)
    const int rb = chunk * RB;
    if (rb >= st.nrhs) return;
    const int nr = min(RB, st.nrhs - rb);
    for (int p = lane; p < f; p += 32) {
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        double v = 0.0;
        if (r < nr) v = (p < s) ? gety(st, rb + r, own[p]) : (CG ? getx_cg(st, rb + r, upd[p - s]) : getx(st, rb + r, upd[p - s]));
        sm[p * RB + r] = (T)v;
      }
    }
    __syncwarp();
    for (int row = r0 + lane; row < r1; row += 32) {
      T acc[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = T(0);
      const T* h = H + row;
#pragma unroll 4
      for (int c = 0; c < f; ++c) {
        const T hv = __ldg(h + (long long)c * s);
        T dv[RB];
        load_rhs<T, RB>(sm + c * RB, dv);
#pragma unroll
        for (int r = 0; r < RB; ++r) acc[r] += hv * dv[r];
      }
#pragma unroll
      for (int r = 0; r < RB; ++r)
        if (r < nr) putx(st, rb + r, own[row], (double)acc[r]);
    }
    __syncwarp();
  }
}

template <typename T, int RB, typename SV>
__global__ void __launch_bounds__(kSolveThreads)
    k_forward(BankView B, SV S, const int4* __restrict__ items, int n_large,
              const int4* __restrict__ thin, int n_thin) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  pdl_trigger();  // the next level may start launching once every CTA here has started
  pdl_wait();     // every access below may read the previous level's results
  if ((int)blockIdx.x < n_large) {
    fwd_large<T, RB, SV>(B, S, items[blockIdx.x], sm, (int)blockIdx.y);
  } else {
    const int wib = threadIdx.x >> 5;
    const int idx = ((int)blockIdx.x - n_large) * (kSolveThreads / 32) + wib;
    if (idx < n_thin) fwd_thin<T, RB, SV>(B, S, thin[idx], sm + wib * kThinCols * RB, (int)blockIdx.y);
  }
}

template <typename T, int RB, typename SV>
__global__ void __launch_bounds__(kSolveThreads)
    k_backward(BankView B, SV S, const int4* __restrict__ items, int n_large,
               const int4* __restrict__ thin, int n_thin) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  pdl_trigger();
  pdl_wait();
  if ((int)blockIdx.x < n_large) {
    bwd_large<T, RB, SV>(B, S, items[blockIdx.x], sm, (int)blockIdx.y);
  } else {
    const int wib = threadIdx.x >> 5;
    const int idx = ((int)blockIdx.x - n_large) * (kSolveThreads / 32) + wib;
    if (idx < n_thin) bwd_thin<T, RB, SV>(B, S, thin[idx], sm + wib * kThinCols * RB, (int)blockIdx.y);
  }
}

template <typename T, int RB, typename SV>
void launch_level(bool forward, const BankView& B, const SV& S, const LevelPlan& L,
                  int max_nrhs, cudaStream_t st) {
  const int warps = kSolveThreads / 32;
  const int nblk = L.n_large + (L.n_thin + warps - 1) / warps;
  if (nblk == 0) return;
  size_t sm_large = ((size_t)L.max_cols + kSolveThreads / 32) * RB * sizeof(T);
  size_t sm_thin = L.n_thin ? (size_t)warps * kThinCols * RB * sizeof(T) : 0;
  size_t smem = std::max(sm_large, sm_thin);
  const dim3 grid(nblk, (max_nrhs + RB - 1) / RB);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kSolveThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (forward)
    PECS_CUDA(cudaLaunchKernelEx(&cfg, k_forward<T, RB, SV>, B, S, (const int4*)L.items.p, L.n_large,
                                 (const int4*)L.thin.p, L.n_thin));
  else
    PECS_CUDA(cudaLaunchKernelEx(&cfg, k_backward<T, RB, SV>, B, S, (const int4*)L.items.p, L.n_large,
                                 (const int4*)L.thin.p, L.n_thin));
}

// The output rows of one item (RHS chunk `chunk`) set to NaN by threads
// t0 = 0 .. nt-1: a flow item whose wait ran out, so that the solve's results
// are flagged non-finite.
template <int RB, bool FWD, typename SV>
__device__ void poison_rows(const BankView& B, const SV& S, int4 it, int chunk, int t0, int nt) {
  const int j = it.x, r0 = it.y, r1 = it.z;
  const int s = B.s[j];
  const auto& st = S.set[B.node_set[j]];
  const int* own = B.own_idx + B.own_off[j];
  const int rb = chunk * RB;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  for (int e = t0; e < (r1 - r0) * RB; e += nt) {
    const int row = r0 + e / RB, r = rb + e % RB;
    if (r >= st.nrhs) continue;
    if (!FWD)
      putx(st, r, own[row], nan);
    else if (row < s)
      puty(st, r, own[row], nan);
    else
      putw(st, r, B.w_off[j] + row - s, nan);
  }
}

// Flow sweep of the few-right-hand-side path: one persistent launch per
// direction over the level plans' items -- wide-node row chunks (kind 0, a
// CTA) and groups of up to eight thin-node row chunks (kind 1, a warp each)
// -- in topological order, with the panel flow sweep's tickets, per-node
// counters, bounded waits, deferred release signals and reset of the other
// direction's counters (see k_panel_flow).  Vectors written inside the
// launch are read with ld.global.cg: their rows (8 or 16 bytes per dof)
// share cache lines.
struct RowsFlowView {
  const int4* entries;  // (kind, first item, item count, RHS chunk)
  const int4* items;    // (node, row0, row1, 0)
  const int4* sync;     // (wait counter or -1, target, signal counter or -1, 0)
  int* ctr;
  int* other_ctr;
  int n_ctr;
  int* queue;
  int* other_queue;
  int* err;
  int n_entries;
};

template <typename T, int RB, bool FWD, typename SV>
__global__ void __launch_bounds__(kSolveThreads)
    k_rows_flow(BankView B, SV S, RowsFlowView F) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  __shared__ int s_ticket, s_ok;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = blockIdx.x * kSolveThreads + tid; i < F.n_ctr; i += gridDim.x * kSolveThreads) F.other_ctr[i] = 0;
  if (blockIdx.x == 0 && tid == 0) *F.other_queue = 0;
  int pending = -1;
  if (tid == 0) s_ticket = atomicAdd(F.queue, 1);
  for (;;) {
    __syncthreads();
    const int t = s_ticket;
    if (lane == 0 && pending >= 0) red_release_gpu(F.ctr + pending, 1);
    pending = -1;
    __syncthreads();
    if (t >= F.n_entries) break;
    if (tid == 0) s_ticket = atomicAdd(F.queue, 1);
    const int4 e = F.entries[t];
    if (e.x == 0) {
      const int4 sy = F.sync[e.y];
      if (tid == 0) s_ok = sy.x < 0 || flow_wait(F.ctr + sy.x, sy.y, F.err);
      __syncthreads();
      if (s_ok) {
        if (FWD)
          fwd_large<T, RB, SV, true>(B, S, F.items[e.y], sm, e.w);
        else
          bwd_large<T, RB, SV, true>(B, S, F.items[e.y], sm, e.w);
      } else {
        poison_rows<RB, FWD, SV>(B, S, F.items[e.y], e.w, tid, kSolveThreads);
      }
      if (tid == 0) pending = sy.z;
    } else if (warp < e.z) {
      const int4 sy = F.sync[e.y + warp];
      int ok = 1;
      if (lane == 0) ok = sy.x < 0 || flow_wait(F.ctr + sy.x, sy.y, F.err);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (ok) {
        T* wsm = sm + warp * kThinCols * RB;
        if (FWD)
          fwd_thin<T, RB, SV, true>(B, S, F.items[e.y + warp], wsm, e.w);
        else
          bwd_thin<T, RB, SV, true>(B, S, F.items[e.y + warp], wsm, e.w);
      } else {
        poison_rows<RB, FWD, SV>(B, S, F.items[e.y + warp], e.w, lane, 32);
      }
      __syncwarp();
      if (lane == 0) pending = sy.z;
    }
  }
}

template <typename T, int RB>
void set_smem_limit(size_t bytes) {
  PECS_CUDA(cudaFuncSetAttribute(k_forward<T, RB, SetsView>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  PECS_CUDA(cudaFuncSetAttribute(k_backward<T, RB, SetsView>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  PECS_CUDA(cudaFuncSetAttribute(k_forward<T, RB, IlSetsView>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  PECS_CUDA(cudaFuncSetAttribute(k_backward<T, RB, IlSetsView>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

template <typename T, typename SV>
void launch_rb(int rb, bool forward, const BankView& B, const SV& S, const LevelPlan& L,
               int max_nrhs, cudaStream_t st) {
  switch (rb) {
    case 1: launch_level<T, 1, SV>(forward, B, S, L, max_nrhs, st); break;
    case 2: launch_level<T, 2, SV>(forward, B, S, L, max_nrhs, st); break;
    case 4: launch_level<T, 4, SV>(forward, B, S, L, max_nrhs, st); break;
    case 8: launch_level<T, 8, SV>(forward, B, S, L, max_nrhs, st); break;
    default: launch_level<T, 16, SV>(forward, B, S, L, max_nrhs, st); break;
  }
}


// ---- panel path --------------------------------------------------------------
constexpr int kPanelKcF32 = 128;  // staged columns per chunk, FP32 blocks
constexpr int kPanelKcF64 = 64;   // staged columns per chunk, FP64 blocks
// chunk sizes the launch may fall back to (per-level child-row counts are
// precomputed for each)
constexpr int kPanelKcSteps = 8;
constexpr int kPanelKc[kPanelKcSteps] = {128, 64, 32, 16, 8, 4, 2, 1};
constexpr size_t kPanelSmem = 160 * 1024;
constexpr int kPanelCmMax = 4096;  // staged child-update rows per node (more: read from global)
constexpr int kSplitMaxParts = 8;  // split-K: at most this many column parts per tile
constexpr int kSplitPart = 128;    // split-K: columns per part (a multiple of every chunk size)
constexpr int kSplitMinK = 192;    // split-K: only nodes with at least this many columns
constexpr size_t kWarpSmem = 48 * 1024;  // leaf levels: shared memory per CTA

// RPL consecutive values of one interleaved row (offset a multiple of RPL),
// double or float storage, registers of type VR (the storage type converts
// only where the two differ -- on GB300 every FP64 operation, conversions
// included, runs on the narrow FP64 unit, so the FP32 path keeps none).
template <int RPL, typename VR>
__device__ __forceinline__ void ld_rhs(const double* p, VR (&v)[RPL]) {
  if constexpr (RPL == 1) {
    v[0] = (VR)p[0];
  } else {
#pragma unroll
    for (int q = 0; q < RPL / 2; ++q) {
      const double2 t = reinterpret_cast<const double2*>(p)[q];
      v[2 * q] = (VR)t.x;
      v[2 * q + 1] = (VR)t.y;
    }
  }
}

template <int RPL, typename VR>
__device__ __forceinline__ void ld_rhs(const float* p, VR (&v)[RPL]) {
  if constexpr (RPL == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = (VR)t.x, v[1] = (VR)t.y, v[2] = (VR)t.z, v[3] = (VR)t.w;
  } else if constexpr (RPL == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = (VR)t.x, v[1] = (VR)t.y;
  } else {
    v[0] = (VR)p[0];
  }
}

template <int RPL, typename VR>
__device__ __forceinline__ void st_rhs(double* p, const VR (&v)[RPL]) {
  if constexpr (RPL == 1) {
    p[0] = (double)v[0];
  } else {
#pragma unroll
    for (int q = 0; q < RPL / 2; ++q)
      reinterpret_cast<double2*>(p)[q] = make_double2((double)v[2 * q], (double)v[2 * q + 1]);
  }
}

template <int RPL, typename VR>
__device__ __forceinline__ void st_rhs(float* p, const VR (&v)[RPL]) {
  if constexpr (RPL == 4) {
    *reinterpret_cast<float4*>(p) = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
  } else if constexpr (RPL == 2) {
    *reinterpret_cast<float2*>(p) = make_float2((float)v[0], (float)v[1]);
  } else {
    p[0] = (float)v[0];
  }
}

// n consecutive shared-memory values (16-byte aligned when n * sizeof(T) >= 16).
template <typename T, int N>
__device__ __forceinline__ void lds(const T* p, T (&v)[N]) {
  if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
    for (int q = 0; q < N / 4; ++q) {
      const float4 t = reinterpret_cast<const float4*>(p)[q];
      v[4 * q] = t.x;
      v[4 * q + 1] = t.y;
      v[4 * q + 2] = t.z;
      v[4 * q + 3] = t.w;
    }
  } else if constexpr (sizeof(T) == 8 && N % 2 == 0) {
#pragma unroll
    for (int q = 0; q < N / 2; ++q) {
      const double2 t = reinterpret_cast<const double2*>(p)[q];
      v[2 * q] = t.x;
      v[2 * q + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int q = 0; q < N; ++q) v[q] = p[q];
  }
}

template <typename T, int N, typename VR>
__device__ __forceinline__ void sts(T* p, const VR (&v)[N]) {
  if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
    for (int q = 0; q < N / 4; ++q)
      reinterpret_cast<float4*>(p)[q] =
          make_float4((float)v[4 * q], (float)v[4 * q + 1], (float)v[4 * q + 2], (float)v[4 * q + 3]);
  } else if constexpr (sizeof(T) == 8 && N % 2 == 0) {
#pragma unroll
    for (int q = 0; q < N / 2; ++q)
      reinterpret_cast<double2*>(p)[q] = make_double2((double)v[2 * q], (double)v[2 * q + 1]);
  } else {
#pragma unroll
    for (int q = 0; q < N; ++q) p[q] = (T)v[q];
  }
}

// One item = rows [r0, r1) of one node's block (Gf for the forward sweep, Hb
// for the backward sweep; both column-major with leading dimension = row
// count), applied to the right-hand-side chunk blockIdx.y (32 * RPL RHS).
// Rows are tiled ri at a time (ri in {4, 8, 16, 32}): warp (g, part) owns rows
// 4g..4g+3 of the tile and the chunk columns k = part (mod 32 / ri); partial
// sums of the column parts are added through shared memory.
//
// The kernel is bound by memory latency, so each column chunk is staged with
// asynchronous copies (cp.async: global -> shared without registers): the
// block tile, the chunk's right-hand-side rows (lanes over right-hand sides,
// coalesced) and, in the forward sweep, the children's update rows that land
// on the chunk's columns are all in flight at once, followed by one wait.
// The item record carries everything about its node (sizes, offsets, the
// node's child-map range), and the node's index metadata is staged once, so
// the chain of dependent loads per item is: record -> metadata -> copies.
// nbuf = 2: the staging buffers are doubled and chunk c + 1 is copied while
// chunk c is multiplied (items with more than one chunk).
template <typename T>
__host__ __device__ constexpr size_t panel_smem_bytes(int ds_rows, int rc, int kc, int ri_max,
                                                      int sc_rows, int meta_ints, int nbuf = 1) {
  return (size_t)nbuf * ((size_t)ds_rows * rc + (size_t)kc * ri_max + (size_t)sc_rows * rc) * sizeof(T) +
         (size_t)meta_ints * sizeof(int);
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(BYTES)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}



// RPL consecutive T of one interleaved row -> shared memory (16-byte pieces
// where the row segment allows; zero fill for lanes past the last RHS)
template <typename T, int RPL>
__device__ __forceinline__ void stage_row(T* dst, const T* src, bool ok) {
  constexpr int BYTES = RPL * (int)sizeof(T);
  if (!ok) {
#pragma unroll
    for (int q = 0; q < RPL; ++q) dst[q] = T(0);
    return;
  }
  if constexpr (BYTES <= 16) {
    cp_async<BYTES>(dst, src);
  } else {
#pragma unroll
    for (int o = 0; o < BYTES / 16; ++o) cp_async<16>(reinterpret_cast<char*>(dst) + 16 * o,
                                                      reinterpret_cast<const char*>(src) + 16 * o);
  }
}

template <typename T>
__device__ __forceinline__ T quiet_nan() {
  if constexpr (sizeof(T) == 4)
    return __int_as_float(0x7fc00000);
  else
    return __longlong_as_double(0x7ff8000000000000ll);
}

// Staging shape of a panel launch (its shared-memory layout): staged block
// columns per chunk, staged right-hand-side rows, the tallest row tile, staged
// child-update rows per chunk, and the index metadata sizes.
struct PanelShape {
  int kc_cap, ds_rows, ri_max, sc_rows, max_s, max_f, cm_cap;
  int nbuf;  // staging buffers (2: the next chunk is copied during this one's products)
};

// One panel item (rows [r0, r1) of one node) applied to the right-hand-side
// chunk starting at rc0 (chunk index `chunk`).  wait_inputs() is called by
// every thread once the block tile's copies are in flight and before any
// vector is read; it returns false when the inputs could not be waited for,
// and the item then writes NaN (the solve's results are flagged non-finite).
// main_done() is called once the item no longer reads its inputs.
template <typename T, int RPL, bool FWD, typename SVT, typename Wait, typename Done>
__device__ __forceinline__ void panel_tile(const BankView& B, const SVT& S, const PanelItem& I, int rc0,
                                           int chunk, const PanelShape& P, T* __restrict__ partials,
                                           int* __restrict__ counters, int parts_ld, int ychunks,
                                           unsigned char* smem_raw, Wait wait_inputs, Done main_done) {
  constexpr int RC = 32 * RPL;
  constexpr int NW = kSolveThreads / 32;
  const int r0 = I.a.y, r1 = I.a.z, ri = I.a.w;
  const int s = I.b.x, m = I.b.y, f = s + m, w_off = I.b.w;
  const auto st = S.set[I.b.z];
  // the sweep vectors have the block's type (FP64 banks: double, FP32: float)
  static_assert(std::is_same<typename std::remove_cv<typename std::remove_pointer<decltype(st.y)>::type>::type,
                             T>::value, "sweep vectors must have the block's type");
  const int R = st.nrhs;
  if (rc0 >= R) return;
  const int max_s = P.max_s, max_f = P.max_f, cm_cap = P.cm_cap, ri_max = P.ri_max;
  const int ds_rows = P.ds_rows, sc_rows = P.sc_rows;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rl = rc0 + lane * RPL;  // first right-hand side of this lane
  const bool lane_ok = rl < R;      // R is a multiple of RPL
  const int K = FWD ? s : f;
  const int ld = FWD ? f : s;
  const T* M = static_cast<const T*>(FWD ? B.G : B.H) + (((long long)I.c.y << 32) | (unsigned)I.c.x);
  const int nrows = r1 - r0;
  const int wpr = 32 / ri;  // warps sharing a row group (column parts)
  const int g = warp / wpr, part = warp % wpr;
  // split-K: this CTA covers columns [k_lo, k_hi) of a tile split in n_parts;
  // an unsplit item may carry its own (smaller) chunk width in e.x
  const bool split = I.e.z >= 0;
  const int k_lo = split ? I.e.x : 0, k_hi = split ? I.e.y : K;
  const int kc_cap = (!split && I.e.x > 0) ? min(I.e.x, P.kc_cap) : P.kc_cap;
  bool bad = false;
  const int nbuf = P.nbuf;
  // staging buffers, nbuf of each: Ds [ds_rows][RC] (nbuf * ds_rows >= 32 when
  // ri < 32: the column-part reduction reuses them), Gs [kc_cap][ri], Sc
  // [sc_rows][RC] child-update rows of a chunk
  T* Ds0 = reinterpret_cast<T*>(smem_raw);
  T* Gs0 = Ds0 + (size_t)nbuf * ds_rows * RC;
  T* Sc0 = Gs0 + (size_t)nbuf * P.kc_cap * ri_max;
  // index metadata of the whole node:
  //   forward:  src_s[s] = own rows; cp_s[f + 1] = child-update ranges per front
  //             position (relative to the node's first entry); cm_s = child rows
  //   backward: src_s[f] = own rows (y) / ~update rows (x)
  int* src_s = reinterpret_cast<int*>(Sc0 + (size_t)nbuf * sc_rows * RC);
  int* cp_s = src_s + (FWD ? max_s : max_f);
  int* cm_s = cp_s + max_f + 1;
  const int cbase = I.d.y, ncm = I.d.z;
  {
    const int* own = B.own_idx + I.c.z;
    if (FWD) {
      const int* cptr = B.cmap_ptr + I.d.x;
      for (int p = tid; p < s; p += kSolveThreads) src_s[p] = own[p];
      for (int p = tid; p <= f; p += kSolveThreads) cp_s[p] = cptr[p] - cbase;
      const int n = min(ncm, cm_cap);
      for (int c = tid; c < n; c += kSolveThreads) cm_s[c] = B.cmap_idx[cbase + c];
    } else {
      const int* upd = B.upd_idx + I.c.w;
      for (int p = tid; p < f; p += kSolveThreads) src_s[p] = p < s ? own[p] : ~upd[p - s];
    }
  }
  __syncthreads();
  T acc[4][RPL];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < RPL; ++q) acc[i][q] = T(0);
  // (A) asynchronous copies of one chunk into buffer b: block tile (read-only,
  // may start before the inputs are waited for), then right-hand-side rows and
  // child-update rows
  const int ri_log = 31 - __clz(ri);  // ri is a power of two
  auto stage_block = [&](int k0, int b) {
    const int kc = min(kc_cap, k_hi - k0);
    T* Gs = Gs0 + (size_t)b * P.kc_cap * ri_max;
    const T* Mk = M + (size_t)k0 * ld + r0;
    for (int idx = tid; idx < kc * ri; idx += kSolveThreads) {
      const int k = idx >> ri_log, i = idx & (ri - 1);
      if (i < nrows)
        cp_async<sizeof(T)>(Gs + idx, Mk + (size_t)k * ld + i);
      else
        Gs[idx] = T(0);
    }
  };
  auto stage_rows = [&](int k0, int b) {
    const int kc = min(kc_cap, k_hi - k0);
    T* Ds = Ds0 + (size_t)b * ds_rows * RC;
    for (int k = warp; k < kc; k += NW) {
      const int sr = src_s[k0 + k];
      const T* src = FWD ? st.b + (size_t)sr * R
                         : (sr >= 0 ? st.y + (size_t)sr * R : st.x + (size_t)(~sr) * R);
      stage_row<T, RPL>(Ds + (size_t)k * RC + lane * RPL, src + rl, lane_ok);
    }
    if (FWD) {
      T* Sc = Sc0 + (size_t)b * sc_rows * RC;
      const int cb = cp_s[k0];
      const int ne = cp_s[k0 + kc] - cb;  // <= sc_rows (plan)
      for (int e = warp; e < ne; e += NW) {
        const int c = cb + e;
        const int wi = c < cm_cap ? cm_s[c] : B.cmap_idx[cbase + c];
        stage_row<T, RPL>(Sc + (size_t)e * RC + lane * RPL, st.w + (size_t)wi * R + rl, lane_ok);
      }
    }
    cp_async_commit();
  };
  if (k_lo < k_hi) stage_block(k_lo, 0);
  bad = !wait_inputs();  // vectors below are written by earlier work
  if (k_lo < k_hi) stage_rows(k_lo, 0);
  int chunk_i = 0;
  for (int k0 = k_lo; k0 < k_hi; k0 += kc_cap, ++chunk_i) {
    const int kc = min(kc_cap, k_hi - k0);
    const int b = nbuf == 2 ? (chunk_i & 1) : 0;
    const bool more = k0 + kc_cap < k_hi;
    if (more && nbuf == 2) {
      stage_block(k0 + kc_cap, b ^ 1);
      stage_rows(k0 + kc_cap, b ^ 1);
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_group<0>();
    }
    __syncthreads();
    T* Ds = Ds0 + (size_t)b * ds_rows * RC;
    const T* Gs = Gs0 + (size_t)b * P.kc_cap * ri_max;
    if (FWD) {
      // (B) subtract the children's updates from the staged right-hand sides
      const T* Sc = Sc0 + (size_t)b * sc_rows * RC;
      const int cb = cp_s[k0];
      for (int k = warp; k < kc; k += NW) {
        const int p = k0 + k;
        const int e0 = cp_s[p] - cb, e1 = cp_s[p + 1] - cb;
        if (e1 > e0) {
          T v[RPL], u[RPL];
          lds<T, RPL>(Ds + (size_t)k * RC + lane * RPL, v);
          for (int e = e0; e < e1; ++e) {
            lds<T, RPL>(Sc + (size_t)e * RC + lane * RPL, u);
#pragma unroll
            for (int q = 0; q < RPL; ++q) v[q] -= u[q];
          }
          sts<T, RPL>(Ds + (size_t)k * RC + lane * RPL, v);
        }
      }
      __syncthreads();
    }
    // (C) register tiles
    const T* Gp = Gs + 4 * g;
    const T* Dp = Ds + lane * RPL;
#pragma unroll 4
    for (int k = part; k < kc; k += wpr) {
      T gv[4], dv[RPL];
      lds<T, 4>(Gp + k * ri, gv);
      lds<T, RPL>(Dp + (size_t)k * RC, dv);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < RPL; ++q) acc[i][q] += gv[i] * dv[q];
    }
    __syncthreads();  // buffer b is restaged two chunks later (one, single-buffered)
    if (more && nbuf == 1) {
      stage_block(k0 + kc_cap, 0);
      stage_rows(k0 + kc_cap, 0);
    }
  }
  main_done();
  // row i of the item -> its destination
  auto emit = [&](int i, T (&v)[RPL]) {
    const int row = r0 + i;
    if (bad) {
#pragma unroll
      for (int q = 0; q < RPL; ++q) v[q] = quiet_nan<T>();
    }
    if (FWD) {
      if (row < s) {
        st_rhs<RPL>(st.y + (size_t)src_s[row] * R + rl, v);
      } else {
        for (int c = cp_s[row]; c < cp_s[row + 1]; ++c) {
          const int wi = c < cm_cap ? cm_s[c] : B.cmap_idx[cbase + c];
          T u[RPL];
          ld_rhs<RPL>(st.w + (size_t)wi * R + rl, u);
#pragma unroll
          for (int q = 0; q < RPL; ++q) v[q] += u[q];
        }
        st_rhs<RPL>(st.w + (size_t)(w_off + row - s) * R + rl, v);
      }
    } else {
      st_rhs<RPL>(st.x + (size_t)src_s[row] * R + rl, v);
    }
  };
  // row totals -> destination, or (split-K) this part's slab of partials
  auto finish = [&](int i, T (&v)[RPL]) {
    if (!split) {
      emit(i, v);
    } else {
      T* dst = partials + ((size_t)(I.e.z * kSplitMaxParts + I.d.w) * 32 + i) * parts_ld + rl;
#pragma unroll
      for (int q = 0; q < RPL; ++q) dst[q] = v[q];
    }
  };
  if (wpr == 1) {
    if (lane_ok) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (4 * g + i < nrows) finish(4 * g + i, acc[i]);
    }
  } else {
    T* red = Ds0;  // [wpr][ri][RC] = 32 * RC values
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int q = 0; q < RPL; ++q)
        red[((size_t)part * ri + 4 * g + i) * RC + lane * RPL + q] = acc[i][q];
    __syncthreads();
    if (lane_ok) {
      for (int i = warp; i < nrows; i += NW) {
        T v[RPL];
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
          T t = T(0);
          for (int p = 0; p < wpr; ++p) t += red[((size_t)p * ri + i) * RC + lane * RPL + q];
          v[q] = t;
        }
        finish(i, v);
      }
    }
  }
  if (!split) return;
  // split-K: the last CTA of the tile to arrive adds the parts in part order
  // (the result does not depend on which CTA is last) and writes the rows
  __shared__ int ticket;
  __threadfence();
  __syncthreads();
  int* ctr = counters + (size_t)I.e.z * ychunks + chunk;
  if (tid == 0) ticket = atomicAdd(ctr, 1);
  __syncthreads();
  if (ticket != I.e.w - 1) return;
  __threadfence();
  if (lane_ok) {
    for (int i = warp; i < nrows; i += NW) {
      T v[RPL];
#pragma unroll
      for (int q = 0; q < RPL; ++q) v[q] = T(0);
      for (int p = 0; p < I.e.w; ++p) {
        const T* src = partials + ((size_t)(I.e.z * kSplitMaxParts + p) * 32 + i) * parts_ld + rl;
#pragma unroll
        for (int q = 0; q < RPL; ++q) v[q] += __ldcg(src + q);
      }
      emit(i, v);
    }
  }
  if (tid == 0) *ctr = 0;
}

template <typename T, int RPL, bool FWD, typename SVT>
__global__ void __launch_bounds__(kSolveThreads)
    k_panel(BankView B, SVT S, const PanelItem* __restrict__ items, PanelShape P, T* __restrict__ partials,
            int* __restrict__ counters, int parts_ld, int ychunks) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PanelItem I = items[blockIdx.x];
  panel_tile<T, RPL, FWD, SVT>(
      B, S, I, (int)blockIdx.y * 32 * RPL, (int)blockIdx.y, P, partials, counters, parts_ld, ychunks, smem_raw,
      [] {
        pdl_wait();
        return true;
      },
      [] { pdl_trigger(); });
}

// Leaf levels: a warp per node (all of its rows) and right-hand-side chunk,
// eight independent nodes per CTA and no CTA barrier.  A level qualifies when
// its nodes are small (at most kWarpMaxK columns and kWarpMaxRows rows) and,
// in the forward sweep, have no children (so the staged right-hand sides need
// no update subtraction and the outputs no pass-through sums).  The warp
// stages its node's whole block and right-hand-side rows with cp.async.
constexpr int kWarpMaxK = 64;
constexpr int kWarpMaxRows = 64;
constexpr int kWarpNodesPerCta = kSolveThreads / 32;

template <typename T>
__host__ __device__ constexpr size_t panel_warp_bytes(int max_k, int rows_pad, int rc) {
  // rounded to 16 bytes: every warp's slice starts 16-byte aligned
  return ((((size_t)max_k * rc + (size_t)max_k * rows_pad) * sizeof(T) + (size_t)max_k * sizeof(int)) +
          15) & ~(size_t)15;
}

// One leaf-level node applied by one warp to the right-hand-side chunk at rc0;
// `base` is the warp's shared-memory slice.  wait_inputs() (every lane) is
// called once the block's copies are in flight and before any vector is read;
// false: the inputs could not be waited for and the node writes NaN.
template <typename T, int RPL, bool FWD, typename SVT, typename Wait, typename Done>
__device__ __forceinline__ void panel_warp_node(const BankView& B, const SVT& S, const PanelItem& I, int rc0,
                                                int max_k, int rows_pad, unsigned char* base, Wait wait_inputs,
                                                Done main_done) {
  constexpr int RC = 32 * RPL;
  const int lane = threadIdx.x & 31;
  const int s = I.b.x, m = I.b.y, f = s + m, w_off = I.b.w;
  const auto st = S.set[I.b.z];
  const int R = st.nrhs;
  if (rc0 >= R) return;
  const int rl = rc0 + lane * RPL;
  const bool lane_ok = rl < R;
  const int K = FWD ? s : f;
  const int rows = FWD ? f : s;  // = the leading dimension of the block
  const T* M = static_cast<const T*>(FWD ? B.G : B.H) + (((long long)I.c.y << 32) | (unsigned)I.c.x);
  T* Ds = reinterpret_cast<T*>(base);        // [max_k][RC]
  T* Gs = Ds + (size_t)max_k * RC;           // [max_k][rows_pad]
  int* src_s = reinterpret_cast<int*>(Gs + (size_t)max_k * rows_pad);  // [max_k]
  {
    const int* own = B.own_idx + I.c.z;
    const int* upd = B.upd_idx + I.c.w;
    for (int p = lane; p < K; p += 32) src_s[p] = FWD ? own[p] : (p < s ? own[p] : ~upd[p - s]);
  }
  for (int e = lane; e < K * rows_pad; e += 32) {
    const int k = e / rows_pad, r = e - k * rows_pad;
    if (r < rows)
      cp_async<sizeof(T)>(Gs + e, M + (size_t)k * rows + r);
    else
      Gs[e] = T(0);
  }
  __syncwarp();
  const bool bad = !wait_inputs();  // vectors below are written by earlier work
  for (int k = 0; k < K; ++k) {
    const int sr = src_s[k];
    const T* src = FWD ? st.b + (size_t)sr * R
                       : (sr >= 0 ? st.y + (size_t)sr * R : st.x + (size_t)(~sr) * R);
    stage_row<T, RPL>(Ds + (size_t)k * RC + lane * RPL, src + rl, lane_ok);
  }
  cp_async_wait_all();
  __syncwarp();
  main_done();
  if (!lane_ok) return;
  for (int r4 = 0; r4 < rows; r4 += 4) {
    T acc[4][RPL];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int q = 0; q < RPL; ++q) acc[i][q] = T(0);
    for (int k = 0; k < K; ++k) {
      T gv[4], dv[RPL];
      lds<T, 4>(Gs + (size_t)k * rows_pad + r4, gv);
      lds<T, RPL>(Ds + (size_t)k * RC + lane * RPL, dv);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < RPL; ++q) acc[i][q] += gv[i] * dv[q];
    }
    if (bad) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < RPL; ++q) acc[i][q] = quiet_nan<T>();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = r4 + i;
      if (row >= rows) break;
      if (FWD) {
        if (row < s)
          st_rhs<RPL>(st.y + (size_t)src_s[row] * R + rl, acc[i]);
        else
          st_rhs<RPL>(st.w + (size_t)(w_off + row - s) * R + rl, acc[i]);
      } else {
        st_rhs<RPL>(st.x + (size_t)src_s[row] * R + rl, acc[i]);
      }
    }
  }
}

template <typename T, int RPL, bool FWD, typename SVT>
__global__ void __launch_bounds__(kSolveThreads)
    k_panel_warp(BankView B, SVT S, const PanelItem* __restrict__ items, int n_items, int max_k,
                 int rows_pad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  const int idx = blockIdx.x * kWarpNodesPerCta + warp;
  if (idx >= n_items) return;
  const PanelItem I = items[idx];
  panel_warp_node<T, RPL, FWD, SVT>(
      B, S, I, (int)blockIdx.y * 32 * RPL, max_k, rows_pad,
      smem_raw + (size_t)warp * panel_warp_bytes<T>(max_k, rows_pad, 32 * RPL),
      [] {
        pdl_wait();
        return true;
      },
      [] { pdl_trigger(); });
}

// ---- flow sweeps -------------------------------------------------------------
// One persistent launch per sweep direction instead of one launch per tree
// level.  The direction's work entries are listed in topological order
// (forward: by height, backward: by depth); every CTA repeatedly takes the
// next entry from a ticket counter and, before reading any vector, waits until
// the entry's node has its inputs: forward, every item of its children has
// finished (their update rows are written); backward, every item of its
// parent has finished (the parent finished only after its own parent, so all
// ancestors' solution rows are written).  An entry only ever waits on entries
// with smaller tickets, which CTAs already running hold, so the sweep always
// progresses whatever the number of resident CTAs.  Finished items add one to
// a per-node counter with release semantics; waits read it with acquire
// semantics.  Each direction's launch zeroes the other direction's counters
// and ticket, so consecutive sweeps start from zero without extra launches.
// Vectors produced inside a launch are whole 128-byte lines per row (checked
// on the host), so no line read from L1 can be stale.
struct FlowView {
  const int4* entries;  // (0: one CTA item / 1: up to 8 warp items, first item, item count, RHS chunk)
  const PanelItem* items;
  const int4* sync;     // per item: (wait counter or -1, wait target, signal counter or -1, 0)
  int* ctr;             // this direction's per-node counters
  int* other_ctr;       // the other direction's (zeroed here)
  int n_ctr;
  int* queue;           // this direction's ticket counter
  int* other_queue;
  int* err;             // set to 1 when a wait runs out
  int n_entries;
};

template <typename T, int RPL, bool FWD, typename SVT>
__global__ void __launch_bounds__(kSolveThreads, 3)
    k_panel_flow(BankView B, SVT S, FlowView F, PanelShape P, int warp_max_k, int warp_rows_pad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_ticket, s_ok;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = blockIdx.x * kSolveThreads + tid; i < F.n_ctr; i += gridDim.x * kSolveThreads) F.other_ctr[i] = 0;
  if (blockIdx.x == 0 && tid == 0) *F.other_queue = 0;
  // The next ticket is taken while the current entry runs, and an entry's
  // completion is signalled (by lane 0 of the warp that owns it) after the
  // barrier that starts the next one, so neither round trip sits between
  // two entries.
  int pending = -1;  // lane 0: the counter this warp still has to signal
  if (tid == 0) s_ticket = atomicAdd(F.queue, 1);
  for (;;) {
    __syncthreads();
    const int t = s_ticket;
    if (lane == 0 && pending >= 0) red_release_gpu(F.ctr + pending, 1);
    pending = -1;
    __syncthreads();  // every thread has read s_ticket
    if (t >= F.n_entries) break;
    if (tid == 0) s_ticket = atomicAdd(F.queue, 1);
    const int4 e = F.entries[t];
    const int rc0 = e.w * 32 * RPL;
    if (e.x == 0) {
      const int4 sy = F.sync[e.y];
      panel_tile<T, RPL, FWD, SVT>(
          B, S, F.items[e.y], rc0, e.w, P, nullptr, nullptr, 0, 0, smem_raw,
          [&] {
            if (tid == 0) s_ok = sy.x < 0 || flow_wait(F.ctr + sy.x, sy.y, F.err);
            __syncthreads();
            return s_ok != 0;
          },
          [] {});
      if (tid == 0) pending = sy.z;
    } else if (warp < e.z) {
      const int ii = e.y + warp;
      const int4 sy = F.sync[ii];
      panel_warp_node<T, RPL, FWD, SVT>(
          B, S, F.items[ii], rc0, warp_max_k, warp_rows_pad,
          smem_raw + (size_t)warp * panel_warp_bytes<T>(warp_max_k, warp_rows_pad, 32 * RPL),
          [&] {
            int ok = 1;
            if (lane == 0) ok = sy.x < 0 || flow_wait(F.ctr + sy.x, sy.y, F.err);
            return __shfl_sync(0xffffffffu, ok, 0) != 0;
          },
          [] {});
      __syncwarp();
      if (lane == 0) pending = sy.z;
    }
  }
}

constexpr size_t kFlowSmem = 96 * 1024;    // flow launches: leaf-warp slices within this
constexpr size_t kFlowScBytes = 32 * 1024;  // flow launches: staged child-update rows per chunk
constexpr int kFlowCmMax = 1024;            // flow launches: staged child-map entries per node

template <typename T, typename SVT>
const void* flow_kernel(int rpl, bool forward) {
  if (forward)
    return rpl == 1 ? (const void*)k_panel_flow<T, 1, true, SVT>
                    : (rpl == 2 ? (const void*)k_panel_flow<T, 2, true, SVT> : (const void*)k_panel_flow<T, 4, true, SVT>);
  return rpl == 1 ? (const void*)k_panel_flow<T, 1, false, SVT>
                  : (rpl == 2 ? (const void*)k_panel_flow<T, 2, false, SVT> : (const void*)k_panel_flow<T, 4, false, SVT>);
}

template <typename T, int RPL, typename SVT>
void launch_flow(bool forward, const BankView& B, const SVT& S, const FlowPlan& FP, const FlowView& F,
                 cudaStream_t st) {
  const PanelShape shape{FP.kc_cap, FP.ds_rows, FP.ri_max, FP.sc_rows, FP.max_s, FP.max_f, FP.cm_cap, FP.nbuf};
  if (forward)
    k_panel_flow<T, RPL, true, SVT><<<FP.grid, kSolveThreads, FP.smem, st>>>(B, S, F, shape, FP.warp_max_k,
                                                                            FP.warp_rows_pad);
  else
    k_panel_flow<T, RPL, false, SVT><<<FP.grid, kSolveThreads, FP.smem, st>>>(B, S, F, shape, FP.warp_max_k,
                                                                             FP.warp_rows_pad);
  PECS_CUDA(cudaGetLastError());
}

// Tile shape of one level for nrhs right-hand sides: the longest row tiles and
// the most right-hand sides per lane that still give the GPU two CTAs per SM.
// Fewer right-hand sides per CTA is tried first (it keeps the staged columns
// per output value higher than shorter row tiles do).
struct PanelChoice {
  int cap_idx, rpl;
};

PanelChoice choose_panel(const PanelPlan& L, int max_nrhs, int rpl_max, int min_ctas) {
  static const int order[6][2] = {{0, 4}, {0, 2}, {0, 1}, {1, 1}, {2, 1}, {3, 1}};
  PanelChoice best{0, 1};
  long long best_ctas = -1;
  for (auto& o : order) {
    if (o[1] > rpl_max) continue;
    const long long ctas = (long long)L.tiles[o[0]].n_items * ((max_nrhs + 32 * o[1] - 1) / (32 * o[1]));
    if (ctas >= min_ctas) return PanelChoice{o[0], o[1]};
    if (ctas > best_ctas) {
      best_ctas = ctas;
      best = PanelChoice{o[0], o[1]};
    }
  }
  return best;
}

template <typename T, int RPL, typename SVT>
void launch_panel(bool forward, const BankView& B, const SVT& S, const PanelPlan& L,
                  const PanelTiles& P, int max_nrhs, int kcap, int parts_ld, cudaStream_t st) {
  const int ychunks = (parts_ld + 31) / 32;
  if (P.n_items == 0) return;
  constexpr int RC = 32 * RPL;
  const int meta = forward ? L.max_s + L.max_f + 1 + L.cm_cap : L.max_f;
  // columns per chunk: the tuned cap, halved until the chunk's staging fits
  int ci = 0;
  while (ci + 1 < kPanelKcSteps && (kPanelKc[ci] > kcap || kPanelKc[ci + 1] >= std::max(1, L.max_k))) ++ci;
  size_t smem = 0;
  int kc = 1, ds_rows = 32, sc_rows = 0, nbuf = 1;
  for (;; ++ci) {
    kc = std::min(kPanelKc[ci], std::max(1, L.max_k));
    nbuf = 1;  // level launches: single-buffered (measured faster: more CTAs per SM)
    ds_rows = P.min_ri < 32 ? std::max(kc, 32 / nbuf) : kc;
    sc_rows = forward ? L.sc_rows[ci] : 0;
    smem = panel_smem_bytes<T>(ds_rows, RC, kc, P.max_ri, sc_rows, meta, nbuf);
    if (smem <= kPanelSmem || ci + 1 == kPanelKcSteps) break;
  }
  if (smem > kPanelSmem) throw PecsError(PECS_E_ARG, "panel staging exceeds shared memory");
  const dim3 grid(P.n_items, (max_nrhs + RC - 1) / RC);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kSolveThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  T* parts = reinterpret_cast<T*>(L.partials.p);
  const PanelShape shape{kc, ds_rows, P.max_ri, sc_rows, L.max_s, L.max_f, L.cm_cap, nbuf};
  if (forward)
    PECS_CUDA(cudaLaunchKernelEx(&cfg, k_panel<T, RPL, true, SVT>, B, S, (const PanelItem*)P.items.p, shape,
                                 parts, L.counters.p, parts_ld, ychunks));
  else
    PECS_CUDA(cudaLaunchKernelEx(&cfg, k_panel<T, RPL, false, SVT>, B, S, (const PanelItem*)P.items.p, shape,
                                 parts, L.counters.p, parts_ld, ychunks));
}

template <typename T, typename SVT>
void set_panel_smem_limit() {
  const int lim = (int)kPanelSmem;
  auto set = [&](const void* fn) {
    PECS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
  };
  set((const void*)k_panel<T, 1, true, SVT>);
  set((const void*)k_panel<T, 2, true, SVT>);
  set((const void*)k_panel<T, 4, true, SVT>);
  set((const void*)k_panel<T, 1, false, SVT>);
  set((const void*)k_panel<T, 2, false, SVT>);
  set((const void*)k_panel<T, 4, false, SVT>);
  set((const void*)k_panel_warp<T, 1, true, SVT>);
  set((const void*)k_panel_warp<T, 2, true, SVT>);
  set((const void*)k_panel_warp<T, 4, true, SVT>);
  set((const void*)k_panel_warp<T, 1, false, SVT>);
  set((const void*)k_panel_warp<T, 2, false, SVT>);
  set((const void*)k_panel_warp<T, 4, false, SVT>);
}

template <typename T, int RPL, typename SVT>
void launch_panel_warp(bool forward, const BankView& B, const SVT& S, const PanelPlan& L,
                       int max_nrhs, cudaStream_t st) {
  constexpr int RC = 32 * RPL;
  const int rows_pad = (L.warp_rows + 3) & ~3;
  const size_t smem = kWarpNodesPerCta * panel_warp_bytes<T>(L.max_k, rows_pad, RC);
  const dim3 grid((L.warp.n_items + kWarpNodesPerCta - 1) / kWarpNodesPerCta, (max_nrhs + RC - 1) / RC);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kSolveThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (forward)
    PECS_CUDA(cudaLaunchKernelEx(&cfg, k_panel_warp<T, RPL, true, SVT>, B, S, (const PanelItem*)L.warp.items.p,
                                 L.warp.n_items, L.max_k, rows_pad));
  else
    PECS_CUDA(cudaLaunchKernelEx(&cfg, k_panel_warp<T, RPL, false, SVT>, B, S, (const PanelItem*)L.warp.items.p,
                                 L.warp.n_items, L.max_k, rows_pad));
}

// One tiling option of a level: kind 0 = whole-row items (row-tile cap
// 32 >> cap_idx), 1 = split-K items, 2 = leaf warps; rpl = RHS per lane.
template <typename T, typename SVT>
void launch_panel_option(const PanelOption& o, bool forward, const BankView& B, const SVT& S,
                         const PanelPlan& L, int max_nrhs, const PanelTuning& tu, int parts_ld,
                         cudaStream_t st) {
  if (o.kind == 2) {
    switch (o.rpl) {
      case 1: launch_panel_warp<T, 1, SVT>(forward, B, S, L, max_nrhs, st); break;
      case 2: launch_panel_warp<T, 2, SVT>(forward, B, S, L, max_nrhs, st); break;
      default: launch_panel_warp<T, 4, SVT>(forward, B, S, L, max_nrhs, st); break;
    }
    return;
  }
  const PanelTiles& P = o.kind == 1 ? L.split : L.tiles[o.cap_idx];
  switch (o.rpl) {
    case 1: launch_panel<T, 1, SVT>(forward, B, S, L, P, max_nrhs, tu.chunk, parts_ld, st); break;
    case 2: launch_panel<T, 2, SVT>(forward, B, S, L, P, max_nrhs, tu.chunk, parts_ld, st); break;
    default: launch_panel<T, 4, SVT>(forward, B, S, L, P, max_nrhs, tu.chunk, parts_ld, st); break;
  }
}

// The valid options of a level for rpl_max RHS per lane.
template <typename T>
std::vector<PanelOption> panel_options(const PanelPlan& L, int max_nrhs, int rpl_max, int parts_ld) {
  std::vector<PanelOption> v;
  for (int rpl = rpl_max; rpl >= 1; rpl /= 2) {
    if (L.warp.n_items > 0) {
      const int rows_pad = (L.warp_rows + 3) & ~3;
      if (kWarpNodesPerCta * panel_warp_bytes<T>(L.max_k, rows_pad, 32 * rpl) <= kWarpSmem)
        v.push_back(PanelOption{2, 0, rpl});
    }
    for (int ci = 0; ci < 4; ++ci) v.push_back(PanelOption{0, ci, rpl});
    if (L.split.n_items > 0 && max_nrhs <= parts_ld) v.push_back(PanelOption{1, 0, rpl});
  }
  return v;
}

// Heuristic option (untuned banks): leaf warps where the level has them; else
// split-K when full-height tiles give too few CTAs; else the row-tile height
// and RHS per lane of choose_panel.
template <typename T>
PanelOption panel_default_option(const PanelPlan& L, int max_nrhs, int rpl_max, const PanelTuning& tu,
                                 int parts_ld) {
  if (L.warp.n_items > 0) {
    int rpl = rpl_max;
    const int rows_pad = (L.warp_rows + 3) & ~3;
    while (rpl > 1 && kWarpNodesPerCta * panel_warp_bytes<T>(L.max_k, rows_pad, 32 * rpl) > kWarpSmem) rpl /= 2;
    return PanelOption{2, 0, rpl};
  }
  const long long full_tiles = (long long)L.tiles[0].n_items * ((max_nrhs + 31) / 32);
  if (L.split.n_items > 0 && full_tiles < tu.min_ctas && max_nrhs <= parts_ld) {
    int rpl = rpl_max;
    while (rpl > 1 && (long long)L.split.n_items * ((max_nrhs + 32 * rpl - 1) / (32 * rpl)) < tu.min_ctas)
      rpl /= 2;
    return PanelOption{1, 0, rpl};
  }
  const PanelChoice c = choose_panel(L, max_nrhs, rpl_max, tu.min_ctas);
  return PanelOption{0, c.cap_idx, c.rpl};
}

template <typename T, typename SVT>
void launch_panel_level(bool forward, const BankView& B, const SVT& S, const PanelPlan& L,
                        int max_nrhs, int rpl_max, const PanelTuning& tu, int parts_ld,
                        cudaStream_t st) {
  PanelOption o = L.tuned;
  if (o.kind < 0 || o.rpl > rpl_max) o = panel_default_option<T>(L, max_nrhs, rpl_max, tu, parts_ld);
  launch_panel_option<T, SVT>(o, forward, B, S, L, max_nrhs, tu, parts_ld, st);
}
}  // namespace

FlowPlanHost plan_flow(const FlowNodes& nd, bool forward, int top, int rpl, int max_nrhs, int kc_max, int esz,
                       int n_sm) {
  FlowPlanHost H;
  const int n_nodes = (int)nd.s.size();
  const std::vector<std::vector<int>>& lv_all = forward ? nd.by_height : nd.by_depth;
  // the covered levels in ticket order (forward: the highest heights, from
  // the lowest of them up; backward: depths 0 .. top-1)
  const int L = (int)lv_all.size();
  top = std::min(std::max(top, 1), L);
  const std::vector<std::vector<int>> lv(forward ? lv_all.begin() + (L - top) : lv_all.begin(),
                                         forward ? lv_all.end() : lv_all.begin() + top);
  const int RC = 32 * rpl;
  H.n_chunks = (std::max(1, max_nrhs) + RC - 1) / RC;
  kc_max = std::max(1, kc_max);
  const int sc_cap = std::max(8, (int)(kFlowScBytes / ((size_t)RC * esz)));
  auto warp_bytes = [&](int k, int r) {
    return esz == 8 ? panel_warp_bytes<double>(k, r, RC) : panel_warp_bytes<float>(k, r, RC);
  };
  auto rows_of = [&](int g) { return forward ? nd.s[g] + nd.m[g] : nd.s[g]; };
  // per level: leaf warps (small nodes, forward without children, the warp
  // slices within budget) or CTA row tiles (32 rows, fewer where a level has
  // too few tiles to fill the GPU)
  std::vector<int> warp_level(lv.size(), 0), cap_level(lv.size(), 32);
  int wk = 0, wr = 0;
  for (size_t l = 0; l < lv.size(); ++l) {
    bool leaf = true;
    int mk = 0, mr = 0;
    for (int g : lv[l]) {
      const int f = nd.s[g] + nd.m[g];
      const int rows = rows_of(g), k = forward ? nd.s[g] : f;
      const bool kids = nd.cmap_ptr[nd.cm_off[g] + f] > nd.cmap_ptr[nd.cm_off[g]];
      if (k > kWarpMaxK || rows > kWarpMaxRows || (forward && kids)) leaf = false;
      mk = std::max(mk, k);
      mr = std::max(mr, rows);
    }
    const int nk = std::max(wk, mk), nr = std::max(wr, (mr + 3) & ~3);
    if (leaf && kWarpNodesPerCta * warp_bytes(nk, nr) <= kFlowSmem) {
      warp_level[l] = 1;
      wk = nk;
      wr = nr;
      continue;
    }
    int cap = 32;
    while (cap > 4) {
      long long t = 0;
      for (int g : lv[l]) t += (rows_of(g) + cap - 1) / cap;
      if (t * H.n_chunks >= n_sm) break;
      cap /= 2;
    }
    cap_level[l] = cap;
  }
  H.warp_max_k = wk;
  H.warp_rows_pad = wr;
  // items per node (signals per chunk), then the items with their waits
  std::vector<int> nsig(n_nodes, 0), per_node(n_nodes, 1);
  for (size_t l = 0; l < lv.size(); ++l)
    for (int g : lv[l]) {
      const int rows = rows_of(g);
      if (warp_level[l]) {
        nsig[g] = 1;
        per_node[g] = rows;
      } else {
        const int cap = cap_level[l];
        const int nit = (rows + cap - 1) / cap;
        per_node[g] = (rows + nit - 1) / nit;
        nsig[g] = (rows + per_node[g] - 1) / per_node[g];
      }
    }
  std::vector<int> kid_sig(n_nodes, 0);
  for (int g = 0; g < n_nodes; ++g)
    if (nd.parent[g] >= 0) kid_sig[nd.parent[g]] += nsig[g];
  int min_ri = 32, max_k_tiles = 0;
  for (size_t l = 0; l < lv.size(); ++l) {
    const size_t first = H.items.size();
    for (int g : lv[l]) {
      const int s = nd.s[g], m = nd.m[g], f = s + m;
      const int rows = rows_of(g);
      const long long off = forward ? nd.goff[g] : nd.hoff[g];
      const int cb = nd.cmap_ptr[nd.cm_off[g]];
      const int ncm = nd.cmap_ptr[nd.cm_off[g] + f] - cb;
      const int p = nd.parent[g];
      const int4 sy = forward ? make_int4(kid_sig[g] > 0 ? g : -1, kid_sig[g] * H.n_chunks, p, 0)
                              : make_int4(p, p >= 0 ? nsig[p] * H.n_chunks : 0, g, 0);
      PanelItem it;
      it.b = make_int4(s, m, nd.node_set[g], nd.w_off[g]);
      it.c = make_int4((int)(off & 0xffffffffll), (int)(off >> 32), nd.own_off[g], nd.upd_off[g]);
      if (warp_level[l]) {
        it.a = make_int4(g, 0, rows, 32);
        it.d = make_int4(nd.cm_off[g], cb, 0, 0);
        it.e = make_int4(0, 0, -1, 1);
        H.items.push_back(it);
        H.sync.push_back(sy);
        continue;
      }
      // the widest chunk (<= kc_max columns) whose child-update rows fit
      int kc = kc_max, rows_sc = 0;
      for (;; kc /= 2) {
        rows_sc = 0;
        if (forward) {
          const int* cp = nd.cmap_ptr.data() + nd.cm_off[g];
          for (int k0 = 0; k0 < s; k0 += kc) rows_sc = std::max(rows_sc, cp[std::min(k0 + kc, s)] - cp[k0]);
        }
        if (rows_sc <= sc_cap || kc == 1) break;
      }
      H.kc_cap = std::max(H.kc_cap, kc);
      max_k_tiles = std::max(max_k_tiles, forward ? s : f);
      H.sc_rows = std::max(H.sc_rows, rows_sc);
      H.max_s = std::max(H.max_s, s);
      H.max_f = std::max(H.max_f, f);
      H.cm_cap = std::max(H.cm_cap, std::min(ncm, kFlowCmMax));
      const int per = per_node[g];
      int ri = 4;
      while (ri < per) ri *= 2;
      H.ri_max = std::max(H.ri_max, ri);
      min_ri = std::min(min_ri, ri);
      it.d = make_int4(nd.cm_off[g], cb, ncm, 0);
      it.e = make_int4(kc, 0, -1, 1);  // no split; this node's chunk width
      for (int r0 = 0; r0 < rows; r0 += per) {
        it.a = make_int4(g, r0, std::min(rows, r0 + per), ri);
        H.items.push_back(it);
        H.sync.push_back(sy);
      }
    }
    // entries: the level's items, each for every chunk (consecutive, so the
    // chunks of one tile share its block in L2); leaf warps in groups
    for (size_t i = first; i < H.items.size();) {
      const int n = warp_level[l] ? (int)std::min<size_t>(kWarpNodesPerCta, H.items.size() - i) : 1;
      for (int c = 0; c < H.n_chunks; ++c) H.entries.push_back(make_int4(warp_level[l], (int)i, n, c));
      i += n;
    }
  }
  H.nbuf = max_k_tiles > H.kc_cap ? 2 : 1;  // items of several chunks: double-buffered staging
  H.ds_rows = min_ri < 32 ? std::max(H.kc_cap, 32 / H.nbuf) : H.kc_cap;
  const int meta = forward ? H.max_s + H.max_f + 1 + H.cm_cap : H.max_f;
  const size_t tile_smem =
      esz == 8 ? panel_smem_bytes<double>(H.ds_rows, RC, H.kc_cap, H.ri_max, H.sc_rows, meta, H.nbuf)
               : panel_smem_bytes<float>(H.ds_rows, RC, H.kc_cap, H.ri_max, H.sc_rows, meta, H.nbuf);
  const size_t warp_smem = wk == 0 ? 0 : kWarpNodesPerCta * warp_bytes(wk, wr);
  H.smem = std::max(tile_smem, warp_smem);
  H.ok = H.smem <= kPanelSmem;
  return H;
}

BankView FactorBank::view() const {
  BankView v;
  v.s = s_.p;
  v.m = m_.p;
  v.goff = goff_.p;
  v.hoff = hoff_.p;
  v.own_off = own_off_.p;
  v.upd_off = upd_off_.p;
  v.w_off = w_off_.p;
  v.cm_off = cm_off_.p;
  v.own_idx = own_idx_.p;
  v.upd_idx = upd_idx_.p;
  v.cmap_ptr = cmap_ptr_.p;
  v.cmap_idx = cmap_idx_.p;
  v.node_set = node_set_.p;
  v.G = prec_ == PECS_PREC_FP64 ? (const void*)G64_.p : (const void*)G32_.p;
  v.H = prec_ == PECS_PREC_FP64 ? (const void*)H64_.p : (const void*)H32_.p;
  return v;
}

int FactorBank::kernel_launches_per_solve() const {
  if (rows_flow_on_) return 2;
  if (flow_sel_ >= 0) {
    const int top = flow_cfg_[flow_sel_].top;
    int n = 2;
    for (size_t l = 0; l + top < pfwd_.size(); ++l) n += pfwd_[l].tiles[0].n_items > 0;
    for (size_t l = top; l < pbwd_.size(); ++l) n += pbwd_[l].tiles[0].n_items > 0;
    return n;
  }
  int n = 0;
  for (auto& l : pfwd_) n += l.tiles[0].n_items > 0;
  for (auto& l : pbwd_) n += l.tiles[0].n_items > 0;
  for (auto& l : fwd_) n += (l.n_large + l.n_thin) > 0;
  for (auto& l : bwd_) n += (l.n_large + l.n_thin) > 0;
  return n;
}

void FactorBank::build(const std::vector<const MfFactor*>& factors, int precision, bool panel,
                       PanelTuning tuning, int max_nrhs) {
  if (factors.empty() || (int)factors.size() > kMaxSets)
    throw PecsError(PECS_E_ARG, "factor bank needs 1..4 factors");
  prec_ = precision;
  panel_ = panel;
  tune_ = tuning;
  parts_ld_ = std::max(32, max_nrhs);
  if (tune_.chunk < 0 || tune_.chunk > 128 || tune_.min_ctas < 0)
    throw PecsError(PECS_E_ARG, "panel tuning out of range");
  if (tune_.chunk == 0) tune_.chunk = precision == PECS_PREC_FP64 ? kPanelKcF64 : kPanelKcF32;
  if (prec_ == PECS_PREC_FP64) tune_.chunk = std::min(tune_.chunk, kPanelKcF64);
  if (tune_.min_ctas == 0) tune_.min_ctas = kTargetCtas;
  n_sets_ = (int)factors.size();
  std::vector<int> hs, hm, own_off, upd_off, w_off, cm_off, own_idx, upd_idx, cmap_ptr, cmap_idx,
      node_set;
  std::vector<long long> goff, hoff;
  std::vector<double> G, H;
  long long go = 0, ho = 0;
  int wtot = 0;
  struct LevelNodes {
    std::vector<int> nodes;
  };
  std::vector<LevelNodes> fl, bl;
  int base = 0;
  for (int fi = 0; fi < n_sets_; ++fi) {
    const MfFactor& F = *factors[fi];
    const int N = (int)F.nodes.size();
    if ((int)F.Gf.size() != N) throw PecsError(PECS_E_STATE, "factor not factorised");
    // update-vector offsets are local to the factor: each RHS owns a buffer of
    // set_wtotal(set) doubles
    std::vector<int> wbase(N);
    wtot = 0;
    for (int j = 0; j < N; ++j) {
      wbase[j] = wtot;
      wtot += F.nodes[j].m;
    }
    set_wtotal_[fi] = std::max(1, wtot);
    std::vector<int> fpos(F.n, -1);
    for (int j = 0; j < N; ++j) {
      const MfNode& nd = F.nodes[j];
      hs.push_back(nd.s);
      hm.push_back(nd.m);
      own_off.push_back((int)own_idx.size());
      upd_off.push_back((int)upd_idx.size());
      own_idx.insert(own_idx.end(), nd.own.begin(), nd.own.end());
      upd_idx.insert(upd_idx.end(), nd.upd.begin(), nd.upd.end());
      w_off.push_back(wbase[j]);
      node_set.push_back(fi);
      goff.push_back(go);
      hoff.push_back(ho);
      {
        // thin blocks (few columns) are stored column-major for thread-per-row
        // application; wide blocks row-major for warp-per-row application
        const int s_ = nd.s, f_ = nd.s + nd.m;
        const std::vector<double>& g = F.Gf[j];  // f_ x s_ row-major
        if (panel || s_ <= kThinCols) {
          for (int c = 0; c < s_; ++c)
            for (int r = 0; r < f_; ++r) G.push_back(g[(size_t)r * s_ + c]);
        } else {
          G.insert(G.end(), g.begin(), g.end());
        }
        const std::vector<double>& h = F.Hb[j];  // s_ x f_ row-major
        if (panel || f_ <= kThinCols) {
          for (int c = 0; c < f_; ++c)
            for (int r = 0; r < s_; ++r) H.push_back(h[(size_t)r * f_ + c]);
        } else {
          H.insert(H.end(), h.begin(), h.end());
        }
      }
      go += (long long)F.Gf[j].size();
      ho += (long long)F.Hb[j].size();
      // extend-add gather lists per front position
      const int f = nd.s + nd.m;
      for (int t = 0; t < nd.s; ++t) fpos[nd.own[t]] = t;
      for (int t = 0; t < nd.m; ++t) fpos[nd.upd[t]] = nd.s + t;
      std::vector<std::vector<int>> lists(f);
      for (int c : nd.children) {
        const MfNode& ch = F.nodes[c];
        for (int a = 0; a < ch.m; ++a) {
          int p = fpos[ch.upd[a]];
          if (p < 0) throw PecsError(PECS_E_STATE, "extend-add map mismatch");
          lists[p].push_back(wbase[c] + a);
        }
      }
      for (int t = 0; t < nd.s; ++t) fpos[nd.own[t]] = -1;
      for (int t = 0; t < nd.m; ++t) fpos[nd.upd[t]] = -1;
      cm_off.push_back((int)cmap_ptr.size());
      for (int p = 0; p < f; ++p) {
        cmap_ptr.push_back((int)cmap_idx.size());
        cmap_idx.insert(cmap_idx.end(), lists[p].begin(), lists[p].end());
      }
      cmap_ptr.push_back((int)cmap_idx.size());
      if ((int)fl.size() <= nd.height) fl.resize(nd.height + 1);
      if ((int)bl.size() <= nd.depth) bl.resize(nd.depth + 1);
      fl[nd.height].nodes.push_back(base + j);
      bl[nd.depth].nodes.push_back(base + j);
    }
    base += N;
  }
  entries_ = go + ho;
  s_.upload(hs);
  m_.upload(hm);
  own_off_.upload(own_off);
  upd_off_.upload(upd_off);
  w_off_.upload(w_off);
  cm_off_.upload(cm_off);
  own_idx_.upload(own_idx);
  upd_idx_.upload(upd_idx);
  cmap_ptr_.upload(cmap_ptr);
  cmap_idx_.upload(cmap_idx);
  node_set_.upload(node_set);
  goff_.upload(goff);
  hoff_.upload(hoff);
  if (prec_ == PECS_PREC_FP64) {
    G64_.upload(G);
    H64_.upload(H);
    bytes_ = (long long)(G.size() + H.size()) * 8;
  } else {
    std::vector<float> g32(G.begin(), G.end()), h32(H.begin(), H.end());
    G32_.upload(g32);
    H32_.upload(h32);
    bytes_ = (long long)(G.size() + H.size()) * 4;
  }
  // level plans: uniform work units so a level's time is not set by one long
  // item.  Thin nodes (cols <= kThinCols): warp items of <= kThinRows rows.
  // Wide nodes: CTA items of <= kWideRows rows (kWideRows/8 rows per warp).
  std::vector<std::vector<int4>> keep_items[2], keep_thin[2];  // host copies for the flow plans
  auto make = [&](const std::vector<LevelNodes>& lv, bool forward, std::vector<LevelPlan>& out) {
    out.clear();
    out.resize(lv.size());
    keep_items[forward ? 0 : 1].assign(lv.size(), {});
    keep_thin[forward ? 0 : 1].assign(lv.size(), {});
    for (size_t l = 0; l < lv.size(); ++l) {
      std::vector<int4> items, thin;
      int max_cols = 0;
      for (int g : lv[l].nodes) {
        const int s = hs[g], m = hm[g], f = s + m;
        const int cols = forward ? s : f;
        const int rows = forward ? f : s;
        if (cols <= kThinCols) {
          for (int r0 = 0; r0 < rows; r0 += kThinRows)
            thin.push_back(make_int4(g, r0, std::min(rows, r0 + kThinRows), 0));
        } else {
          max_cols = std::max(max_cols, cols);
        }
      }
      // wide nodes: 8 rows per CTA item (one per warp), fewer when the level
      // would not give the GPU enough CTAs -- down to one row whose columns are
      // split over the CTA's eight warps
      long long wide_rows = 0;
      for (int g : lv[l].nodes) {
        const int s = hs[g], m = hm[g];
        const int cols = forward ? s : s + m;
        if (cols > kThinCols) wide_rows += forward ? s + m : s;
      }
      int per = kWideRows;
      while (per > 1 && wide_rows / per < 2 * kTargetCtas) per /= 2;
      for (int g : lv[l].nodes) {
        const int s = hs[g], m = hm[g], f = s + m;
        const int cols = forward ? s : f;
        const int rows = forward ? f : s;
        if (cols <= kThinCols) continue;
        for (int r0 = 0; r0 < rows; r0 += per)
          items.push_back(make_int4(g, r0, std::min(rows, r0 + per), 0));
      }
      out[l].n_large = (int)items.size();
      out[l].n_thin = (int)thin.size();
      out[l].max_cols = max_cols;
      out[l].items.upload(items);
      out[l].thin.upload(thin);
      keep_items[forward ? 0 : 1][l] = items;
      keep_thin[forward ? 0 : 1][l] = thin;
    }
  };
  if (panel) {
    // panel items: a node's rows in tiles of ri <= cap rows, for caps 32, 16,
    // 8 and 4 (levels that would not fill the GPU use shorter tiles: more
    // CTAs, column parts per warp)
    auto make_panel = [&](const std::vector<LevelNodes>& lv, bool forward, std::vector<PanelPlan>& out) {
      out.clear();
      out.resize(lv.size());
      for (size_t l = 0; l < lv.size(); ++l) {
        int max_k = 0, max_s = 1, max_f = 1, max_cm = 0;
        for (int g : lv[l].nodes) {
          const int f = hs[g] + hm[g];
          max_k = std::max(max_k, forward ? hs[g] : f);
          max_s = std::max(max_s, hs[g]);
          max_f = std::max(max_f, f);
          max_cm = std::max(max_cm, cmap_ptr[cm_off[g] + f] - cmap_ptr[cm_off[g]]);
        }
        out[l].max_k = max_k;
        out[l].max_s = max_s;
        out[l].max_f = max_f;
        out[l].cm_cap = std::min(max_cm, kPanelCmMax);
        // forward: most child-update rows landing on one chunk of columns
        for (int ci = 0; ci < kPanelKcSteps; ++ci) {
          int mx = 0;
          if (forward) {
            const int kc = kPanelKc[ci];
            for (int g : lv[l].nodes) {
              const int* cp = cmap_ptr.data() + cm_off[g];
              for (int k0 = 0; k0 < hs[g]; k0 += kc) mx = std::max(mx, cp[std::min(k0 + kc, hs[g])] - cp[k0]);
            }
          }
          out[l].sc_rows[ci] = mx;
        }
        // split-K items: nodes with long rows in 32-row tiles x column parts
        // of kSplitPart (at most kSplitMaxParts); shorter nodes of the level
        // as whole-row items
        if (max_k >= kSplitMinK) {
          std::vector<PanelItem> items;
          int max_ri = 4, min_ri = 32, tiles = 0;
          for (int g : lv[l].nodes) {
            const int rows = forward ? hs[g] + hm[g] : hs[g];
            const int K = forward ? hs[g] : hs[g] + hm[g];
            const int nit = (rows + 31) / 32;
            const int per = (rows + nit - 1) / nit;
            int ri = 4;
            while (ri < per) ri *= 2;
            max_ri = std::max(max_ri, ri);
            min_ri = std::min(min_ri, ri);
            const long long off = forward ? goff[g] : hoff[g];
            const int cb = cmap_ptr[cm_off[g]];
            const int ncm = cmap_ptr[cm_off[g] + hs[g] + hm[g]] - cb;
            int parts = 1, part_len = K;
            if (K >= kSplitMinK) {
              parts = std::min(kSplitMaxParts, (K + kSplitPart - 1) / kSplitPart);
              part_len = ((K + parts - 1) / parts + kSplitPart - 1) / kSplitPart * kSplitPart;
              parts = (K + part_len - 1) / part_len;
            }
            for (int r0 = 0; r0 < rows; r0 += per) {
              const int tile = parts > 1 ? tiles++ : -1;
              for (int p = 0; p < parts; ++p) {
                PanelItem it;
                it.a = make_int4(g, r0, std::min(rows, r0 + per), ri);
                it.b = make_int4(hs[g], hm[g], node_set[g], w_off[g]);
                it.c = make_int4((int)(off & 0xffffffffll), (int)(off >> 32), own_off[g], upd_off[g]);
                it.d = make_int4(cm_off[g], cb, ncm, p);
                it.e = make_int4(p * part_len, std::min(K, (p + 1) * part_len), tile, parts);
                items.push_back(it);
              }
            }
          }
          if (tiles > 0) {
            PanelTiles& P = out[l].split;
            P.n_items = (int)items.size();
            P.max_ri = max_ri;
            P.min_ri = min_ri;
            for (const PanelItem& it : items) P.max_span = std::max(P.max_span, it.e.y - it.e.x);
            P.items.upload(items);
            out[l].split_tiles = tiles;
            const int ych = (parts_ld_ + 31) / 32;
            out[l].counters.alloc((size_t)tiles * ych);
            out[l].counters.zero();
            const size_t esz = prec_ == PECS_PREC_FP64 ? 8 : 4;
            out[l].partials.alloc((size_t)tiles * kSplitMaxParts * 32 * parts_ld_ * esz);
          }
        }
        // leaf level: every node small and, forward, without children
        bool leaf = true;
        int max_rows = 0;
        for (int g : lv[l].nodes) {
          const int f = hs[g] + hm[g];
          const int rows = forward ? f : hs[g];
          const int k = forward ? hs[g] : f;
          const bool kids = cmap_ptr[cm_off[g] + f] > cmap_ptr[cm_off[g]];
          if (k > kWarpMaxK || rows > kWarpMaxRows || (forward && kids)) leaf = false;
          max_rows = std::max(max_rows, rows);
        }
        {
          const size_t esz = prec_ == PECS_PREC_FP64 ? 8 : 4;
          const size_t rows_pad = (size_t)((max_rows + 3) & ~3);
          const size_t wb = (((size_t)max_k * 32 + (size_t)max_k * rows_pad) * esz + (size_t)max_k * 4 + 15) & ~(size_t)15;
          if (kWarpNodesPerCta * wb > kWarpSmem) leaf = false;
        }
        if (leaf) {
          std::vector<PanelItem> items;
          for (int g : lv[l].nodes) {
            const int rows = forward ? hs[g] + hm[g] : hs[g];
            const long long off = forward ? goff[g] : hoff[g];
            PanelItem it;
            it.a = make_int4(g, 0, rows, 32);
            it.b = make_int4(hs[g], hm[g], node_set[g], w_off[g]);
            it.c = make_int4((int)(off & 0xffffffffll), (int)(off >> 32), own_off[g], upd_off[g]);
            it.d = make_int4(cm_off[g], cmap_ptr[cm_off[g]], 0, 0);
            it.e = make_int4(0, 0, -1, 1);
            items.push_back(it);
          }
          out[l].warp.n_items = (int)items.size();
          out[l].warp.items.upload(items);
          out[l].warp_rows = max_rows;
        }
        for (int ci = 0; ci < 4; ++ci) {
          const int cap = 32 >> ci;
          std::vector<PanelItem> items;
          int max_ri = 4, min_ri = 32;
          for (int g : lv[l].nodes) {
            const int rows = forward ? hs[g] + hm[g] : hs[g];
            const int nit = (rows + cap - 1) / cap;
            const int per = (rows + nit - 1) / nit;
            int ri = 4;
            while (ri < per) ri *= 2;
            max_ri = std::max(max_ri, ri);
            min_ri = std::min(min_ri, ri);
            const long long off = forward ? goff[g] : hoff[g];
            const int cb = cmap_ptr[cm_off[g]];
            const int ncm = cmap_ptr[cm_off[g] + hs[g] + hm[g]] - cb;
            for (int r0 = 0; r0 < rows; r0 += per) {
              PanelItem it;
              it.a = make_int4(g, r0, std::min(rows, r0 + per), ri);
              it.b = make_int4(hs[g], hm[g], node_set[g], w_off[g]);
              it.c = make_int4((int)(off & 0xffffffffll), (int)(off >> 32), own_off[g], upd_off[g]);
              it.d = make_int4(cm_off[g], cb, ncm, 0);
              it.e = make_int4(0, 0, -1, 1);  // no split
              items.push_back(it);
            }
          }
          PanelTiles& P = out[l].tiles[ci];
          P.n_items = (int)items.size();
          P.max_ri = max_ri;
          P.min_ri = min_ri;
          P.max_span = max_k;
          P.items.upload(items);
        }
      }
    };
    make_panel(fl, true, pfwd_);
    make_panel(bl, false, pbwd_);
    fwd_.clear();
    bwd_.clear();
    if (prec_ == PECS_PREC_FP64)
      set_panel_smem_limit<double, IlSetsView>();
    else
      set_panel_smem_limit<float, IlSetsViewF>();
    // flow plans: both directions, 1, 2 and 4 right-hand sides per lane
    n_nodes_ = (int)hs.size();
    std::vector<int> parent(n_nodes_, -1);
    {
      int b0 = 0;
      for (int fi = 0; fi < n_sets_; ++fi) {
        const MfFactor& F = *factors[fi];
        for (int j = 0; j < (int)F.nodes.size(); ++j)
          for (int c : F.nodes[j].children) parent[b0 + c] = b0 + j;
        b0 += (int)F.nodes.size();
      }
    }
    flow_state_.alloc(2 * (size_t)n_nodes_ + 3);
    flow_state_.zero();
    stall_node_ = -1;
    for (int g = 0; g < (int)factors[0]->nodes.size() && stall_node_ < 0; ++g)
      if (parent[g] < 0 && !factors[0]->nodes[g].children.empty()) stall_node_ = g;
    int n_sm = 0, dev = 0;
    PECS_CUDA(cudaGetDevice(&dev));
    PECS_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    FlowNodes nodes{hs, hm, node_set, w_off, own_off, upd_off, cm_off, cmap_ptr, goff, hoff, parent, {}, {}};
    for (auto& l : fl) nodes.by_height.push_back(l.nodes);
    for (auto& l : bl) nodes.by_depth.push_back(l.nodes);
    const int esz = prec_ == PECS_PREC_FP64 ? 8 : 4;
    flow_cfg_.clear();
    flow_sel_ = -1;
    const int n_levels = (int)std::max(fl.size(), bl.size());
    std::vector<int> tops{n_levels};
    for (int t : {7, 5, 3})
      if (t < n_levels) tops.push_back(t);
    for (int top : tops) {
      for (int kc : {64, 32}) {
        for (int rpl : {1, 2, 4}) {
          FlowConfig cfg;
          cfg.top = top;
          cfg.kc = std::min(kc, tune_.chunk);
          cfg.rpl = rpl;
          bool ok = true;
          for (int d = 0; d < 2 && ok; ++d) {
            FlowPlan& FP = cfg.plan[d];
            FlowPlanHost H = plan_flow(nodes, d == 0, top, rpl, max_nrhs, cfg.kc, esz, n_sm);
            if (!H.ok) {
              ok = false;
              break;
            }
            FP.top = top;
            FP.rpl = rpl;
            FP.n_chunks = H.n_chunks;
            FP.kc_cap = H.kc_cap;
            FP.nbuf = H.nbuf;
            FP.ds_rows = H.ds_rows;
            FP.ri_max = H.ri_max;
            FP.sc_rows = H.sc_rows;
            FP.max_s = H.max_s;
            FP.max_f = H.max_f;
            FP.cm_cap = H.cm_cap;
            FP.warp_max_k = H.warp_max_k;
            FP.warp_rows_pad = H.warp_rows_pad;
            FP.smem = H.smem;
            FP.n_entries = (int)H.entries.size();
            FP.items.upload(H.items);
            FP.sync.upload(H.sync);
            FP.entries.upload(H.entries);
            const void* fn = esz == 8 ? flow_kernel<double, IlSetsView>(rpl, d == 0)
                                      : flow_kernel<float, IlSetsViewF>(rpl, d == 0);
            PECS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmem));
            int per_sm = 0;
            PECS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSolveThreads, FP.smem));
            FP.grid = std::max(1, std::min(FP.n_entries, std::max(1, per_sm) * n_sm));
          }
          if (ok) flow_cfg_.push_back(std::move(cfg));
        }
      }
    }
    return;
  }
  make(fl, true, fwd_);
  make(bl, false, bwd_);
  // flow plans over the same items: per node the number of its items (its
  // signals), waits on the children's (forward) or the parent's (backward)
  {
    const int n_nodes = (int)hs.size();
    n_nodes_ = n_nodes;
    std::vector<int> parent(n_nodes, -1);
    int b0 = 0;
    for (int fi = 0; fi < n_sets_; ++fi) {
      const MfFactor& F = *factors[fi];
      for (int j = 0; j < (int)F.nodes.size(); ++j)
        for (int c : F.nodes[j].children) parent[b0 + c] = b0 + j;
      b0 += (int)F.nodes.size();
    }
    flow_state_.alloc(2 * (size_t)n_nodes + 3);
    flow_state_.zero();
    rows_flow_on_ = false;
    stall_node_ = -1;
    for (int g = 0; g < (int)factors[0]->nodes.size() && stall_node_ < 0; ++g)
      if (parent[g] < 0 && !factors[0]->nodes[g].children.empty()) stall_node_ = g;
    for (int d = 0; d < 2; ++d) {
      std::vector<int> nsig(n_nodes, 0), kid_sig(n_nodes, 0);
      for (size_t l = 0; l < keep_items[d].size(); ++l) {
        for (const int4& it : keep_items[d][l]) ++nsig[it.x];
        for (const int4& it : keep_thin[d][l]) ++nsig[it.x];
      }
      for (int g = 0; g < n_nodes; ++g)
        if (parent[g] >= 0) kid_sig[parent[g]] += nsig[g];
      std::vector<int4> items, sync, entries;
      auto push = [&](const int4& it) {
        const int g = it.x, pa = parent[g];
        items.push_back(it);
        sync.push_back(d == 0 ? make_int4(kid_sig[g] > 0 ? g : -1, kid_sig[g], pa, 0)
                              : make_int4(pa, pa >= 0 ? nsig[pa] : 0, g, 0));
      };
      for (size_t l = 0; l < keep_items[d].size(); ++l) {
        for (const int4& it : keep_items[d][l]) {
          entries.push_back(make_int4(0, (int)items.size(), 1, 0));
          push(it);
        }
        const std::vector<int4>& th = keep_thin[d][l];
        for (size_t i = 0; i < th.size(); i += kSolveThreads / 32) {
          const int n = (int)std::min<size_t>(kSolveThreads / 32, th.size() - i);
          entries.push_back(make_int4(1, (int)items.size(), n, 0));
          for (int k = 0; k < n; ++k) push(th[i + k]);
        }
      }
      RowsFlowPlan& P = rows_flow_plan_[d];
      P.n_entries = (int)entries.size();
      P.entries.upload(entries);
      P.items.upload(items);
      P.sync.upload(sync);
    }
  }
  max_cols_ = 0;
  for (auto& l : fwd_) max_cols_ = std::max(max_cols_, l.max_cols);
  for (auto& l : bwd_) max_cols_ = std::max(max_cols_, l.max_cols);
  const size_t esz = prec_ == PECS_PREC_FP64 ? 8 : 4;
  const size_t small_need = (size_t)(kSolveThreads / 32) * kThinCols * esz;
  max_rb_ = 16;
  while (max_rb_ > 1 &&
         std::max((size_t)max_cols_ + kSolveThreads / 32, small_need / esz) * max_rb_ * esz > kSmemCap)
    max_rb_ /= 2;
  if ((size_t)max_cols_ * esz > kSmemCap) throw PecsError(PECS_E_ARG, "front too large for shared memory");
  const size_t lim = kSmemCap;
  if (prec_ == PECS_PREC_FP64) {
    set_smem_limit<double, 1>(lim);
    set_smem_limit<double, 2>(lim);
    set_smem_limit<double, 4>(lim);
    set_smem_limit<double, 8>(lim);
    set_smem_limit<double, 16>(lim);
  } else {
    set_smem_limit<float, 1>(lim);
    set_smem_limit<float, 2>(lim);
    set_smem_limit<float, 4>(lim);
    set_smem_limit<float, 8>(lim);
    set_smem_limit<float, 16>(lim);
  }
}

int FactorBank::solve_rb(int max_nrhs) const {
  int rb = max_nrhs <= 1 ? 1 : (max_nrhs <= 2 ? 2 : (max_nrhs <= 4 ? 4 : (max_nrhs <= 8 ? 8 : 16)));
  if (prec_ == PECS_PREC_FP64) rb = std::min(rb, 8);  // FP64: register budget
  return std::min(rb, max_rb_);
}

template <typename T, int RB, typename SV>
void launch_rows_flow(const BankView& B, const SV& S, const RowsFlowView& Ff, const RowsFlowView& Fb,
                      size_t smem, cudaStream_t st) {
  const void* fns[2] = {(const void*)k_rows_flow<T, RB, true, SV>, (const void*)k_rows_flow<T, RB, false, SV>};
  int dev = 0, n_sm = 0;
  PECS_CUDA(cudaGetDevice(&dev));
  PECS_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  for (int d = 0; d < 2; ++d) {
    PECS_CUDA(cudaFuncSetAttribute(fns[d], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap));
    int per_sm = 0;
    PECS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fns[d], kSolveThreads, smem));
    const RowsFlowView& F = d == 0 ? Ff : Fb;
    const int grid = std::max(1, std::min(F.n_entries, std::max(1, per_sm) * n_sm));
    if (d == 0)
      k_rows_flow<T, RB, true, SV><<<grid, kSolveThreads, smem, st>>>(B, S, F);
    else
      k_rows_flow<T, RB, false, SV><<<grid, kSolveThreads, smem, st>>>(B, S, F);
    PECS_CUDA(cudaGetLastError());
  }
}

template <typename SV>
void FactorBank::solve_rows_flow(const SV& sets, int max_nrhs, cudaStream_t st) const {
  const BankView B = view();
  const int rb = solve_rb(max_nrhs);
  const size_t esz = prec_ == PECS_PREC_FP64 ? 8 : 4;
  const size_t smem = std::max(((size_t)max_cols_ + kSolveThreads / 32) * rb * esz,
                               (size_t)(kSolveThreads / 32) * kThinCols * rb * esz);
  int* base = flow_state_.p;
  int* ctr[2] = {base, base + n_nodes_};
  int* queue[2] = {base + 2 * (size_t)n_nodes_, base + 2 * (size_t)n_nodes_ + 1};
  int* err = base + 2 * (size_t)n_nodes_ + 2;
  RowsFlowView F[2];
  for (int d = 0; d < 2; ++d) {
    const RowsFlowPlan& P = rows_flow_plan_[d];
    F[d] = RowsFlowView{P.entries.p, P.items.p, P.sync.p, ctr[d], ctr[1 - d], n_nodes_,
                        queue[d],    queue[1 - d], err,   P.n_entries};
  }
  auto go = [&](auto tag) {
    using T = decltype(tag);
    switch (rb) {
      case 1: launch_rows_flow<T, 1, SV>(B, sets, F[0], F[1], smem, st); break;
      case 2: launch_rows_flow<T, 2, SV>(B, sets, F[0], F[1], smem, st); break;
      case 4: launch_rows_flow<T, 4, SV>(B, sets, F[0], F[1], smem, st); break;
      case 8: launch_rows_flow<T, 8, SV>(B, sets, F[0], F[1], smem, st); break;
      default: launch_rows_flow<T, 16, SV>(B, sets, F[0], F[1], smem, st); break;
    }
  };
  if (prec_ == PECS_PREC_FP64)
    go(double{});
  else
    go(float{});
}

void FactorBank::tune_rows_flow(const IlSetsView& sets, int max_nrhs, cudaStream_t st, int flow_mode, int reps) {
  rows_flow_on_ = false;
  if (panel_ || flow_mode < 0 || max_nrhs > solve_rb(max_nrhs) || rows_flow_plan_[0].n_entries == 0) return;
  if (flow_mode > 0) {
    rows_flow_on_ = true;
    return;
  }
  cudaEvent_t e0, e1;
  PECS_CUDA(cudaEventCreate(&e0));
  PECS_CUDA(cudaEventCreate(&e1));
  auto time = [&](bool flow) {
    rows_flow_on_ = flow;
    solve(sets, max_nrhs, st);  // warm-up
    float best = 1e30f;
    for (int r = 0; r < reps; ++r) {
      PECS_CUDA(cudaEventRecord(e0, st));
      solve(sets, max_nrhs, st);
      PECS_CUDA(cudaEventRecord(e1, st));
      PECS_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      PECS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, ms);
    }
    return best;
  };
  const float lev = time(false), flo = time(true);
  if (flow_error() != 0) throw PecsError(PECS_E_CUDA, "flow sweep: a wait for a node's inputs ran out");
  if (std::getenv("PECS_TUNE_LOG"))
    std::fprintf(stderr, "rows flow: %.4f ms (levels %.4f ms)\n", flo, lev);
  rows_flow_on_ = flo < lev;
  tuned_ms_ = std::min(flo, lev);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

template <typename SV>
void FactorBank::solve_impl(const SV& sets, int max_nrhs, cudaStream_t st) const {
  if (rows_flow_on_ && max_nrhs <= solve_rb(max_nrhs)) {
    solve_rows_flow(sets, max_nrhs, st);
    return;
  }
  const BankView B = view();
  const int rb = solve_rb(max_nrhs);
  for (const LevelPlan& L : fwd_) {
    if (prec_ == PECS_PREC_FP64)
      launch_rb<double, SV>(rb, true, B, sets, L, max_nrhs, st);
    else
      launch_rb<float, SV>(rb, true, B, sets, L, max_nrhs, st);
  }
  for (const LevelPlan& L : bwd_) {
    if (prec_ == PECS_PREC_FP64)
      launch_rb<double, SV>(rb, false, B, sets, L, max_nrhs, st);
    else
      launch_rb<float, SV>(rb, false, B, sets, L, max_nrhs, st);
  }
}

void FactorBank::solve(const SetsView& sets, int max_nrhs, cudaStream_t st) const {
  if (panel_) throw PecsError(PECS_E_STATE, "panel factor bank needs the interleaved layout");
  solve_impl(sets, max_nrhs, st);
}

void FactorBank::solve(const IlSetsView& sets, int max_nrhs, cudaStream_t st) const {
  if (panel_ && prec_ != PECS_PREC_FP64)
    throw PecsError(PECS_E_STATE, "FP32 panel banks take float sweep vectors");
  if (panel_)
    solve_panel(sets, max_nrhs, st);
  else
    solve_impl(sets, max_nrhs, st);
}

template <typename SVT>
int FactorBank::panel_rpl(const SVT& sets, int max_nrhs) const {
  // right-hand sides per lane: at most as many as fill the lanes, dividing every set's count
  int rpl = max_nrhs >= 96 ? 4 : (max_nrhs >= 48 ? 2 : 1);
  for (int si = 0; si < n_sets_; ++si)
    while (rpl > 1 && sets.set[si].nrhs % rpl != 0) rpl /= 2;
  return rpl;
}

int FactorBank::flow_error(bool clear) const {
  if (flow_state_.n == 0) return 0;
  int e = 0;
  int* p = flow_state_.p + 2 * (size_t)n_nodes_ + 2;
  PECS_CUDA(cudaMemcpy(&e, p, sizeof(int), cudaMemcpyDeviceToHost));
  if (clear) PECS_CUDA(cudaMemset(p, 0, sizeof(int)));
  return e;
}

void FactorBank::debug_arm_flow_stall() const {
  if (flow_state_.n == 0 || stall_node_ < 0) throw PecsError(PECS_E_STATE, "no flow sweep to stall");
  PECS_CUDA(cudaDeviceSynchronize());
  const int v = -(1 << 30);
  PECS_CUDA(cudaMemcpy(flow_state_.p + stall_node_, &v, sizeof(int), cudaMemcpyHostToDevice));
}

// A flow configuration applies when its plans cover these right-hand sides
// and every sweep vector row is a whole number of 128-byte lines at a 128-byte
// aligned address (rows written inside the launch never share a line with
// another).
template <typename SVT>
bool FactorBank::flow_ok(const SVT& sets, int max_nrhs, int cfg) const {
  using T = typename std::conditional<std::is_same<SVT, IlSetsViewF>::value, float, double>::type;
  if (!panel_ || cfg < 0 || cfg >= (int)flow_cfg_.size()) return false;
  if ((prec_ == PECS_PREC_FP64) != (sizeof(T) == 8)) return false;
  const FlowConfig& C = flow_cfg_[cfg];
  const int rpl = C.rpl;
  if (C.plan[0].n_entries == 0 || C.plan[1].n_entries == 0) return false;
  if ((max_nrhs + 32 * rpl - 1) / (32 * rpl) != C.plan[0].n_chunks) return false;
  if (panel_rpl(sets, max_nrhs) < rpl) return false;
  auto al = [](const void* p) { return ((uintptr_t)p & 127u) == 0; };
  for (int si = 0; si < n_sets_; ++si) {
    const auto& v = sets.set[si];
    if (v.nrhs > max_nrhs || v.nrhs % rpl != 0 || ((size_t)v.nrhs * sizeof(T)) % 128 != 0) return false;
    if (!al(v.b) || !al(v.y) || !al(v.w) || !al(v.x)) return false;
  }
  return true;
}

// Hybrid sweep: level launches for the levels below the configuration's top
// levels, then one flow launch per direction over those, then level launches
// again (backward) for the rest.
template <typename SVT>
void FactorBank::solve_flow(const SVT& sets, int max_nrhs, int cfg, cudaStream_t st) const {
  using T = typename std::conditional<std::is_same<SVT, IlSetsViewF>::value, float, double>::type;
  const BankView B = view();
  const FlowConfig& C = flow_cfg_[cfg];
  const int lrpl = panel_rpl(sets, max_nrhs);
  int* base = flow_state_.p;
  int* ctr[2] = {base, base + n_nodes_};
  int* queue[2] = {base + 2 * (size_t)n_nodes_, base + 2 * (size_t)n_nodes_ + 1};
  int* err = base + 2 * (size_t)n_nodes_ + 2;
  for (size_t l = 0; l + C.top < pfwd_.size(); ++l)
    launch_panel_level<T, SVT>(true, B, sets, pfwd_[l], max_nrhs, lrpl, tune_, parts_ld_, st);
  for (int d = 0; d < 2; ++d) {
    const FlowPlan& FP = C.plan[d];
    const FlowView F{FP.entries.p, FP.items.p, FP.sync.p, ctr[d], ctr[1 - d], n_nodes_,
                     queue[d],     queue[1 - d], err,     FP.n_entries};
    switch (C.rpl) {
      case 1: launch_flow<T, 1, SVT>(d == 0, B, sets, FP, F, st); break;
      case 2: launch_flow<T, 2, SVT>(d == 0, B, sets, FP, F, st); break;
      default: launch_flow<T, 4, SVT>(d == 0, B, sets, FP, F, st); break;
    }
  }
  for (size_t l = C.top; l < pbwd_.size(); ++l)
    launch_panel_level<T, SVT>(false, B, sets, pbwd_[l], max_nrhs, lrpl, tune_, parts_ld_, st);
}

template <typename SVT>
void FactorBank::solve_panel(const SVT& sets, int max_nrhs, cudaStream_t st) const {
  if (flow_sel_ >= 0 && flow_ok(sets, max_nrhs, flow_sel_)) {
    solve_flow(sets, max_nrhs, flow_sel_, st);
    return;
  }
  const int rpl = panel_rpl(sets, max_nrhs);
  const BankView B = view();
  for (int pass = 0; pass < 2; ++pass) {
    const bool fwd = pass == 0;
    for (const PanelPlan& L : fwd ? pfwd_ : pbwd_) {
      if constexpr (std::is_same<SVT, IlSetsViewF>::value)
        launch_panel_level<float, SVT>(fwd, B, sets, L, max_nrhs, rpl, tune_, parts_ld_, st);
      else
        launch_panel_level<double, SVT>(fwd, B, sets, L, max_nrhs, rpl, tune_, parts_ld_, st);
    }
  }
}

// Per level, choose the tiling option that gives the fastest whole sweep:
// starting from the heuristic choice everywhere, each level in turn tries all
// of its valid options with the other levels fixed, timing complete sweeps
// (minimum of `reps` after one warm-up), so every level is measured with the
// cache state the real sweep gives it.  The sweep's values are meaningless
// while tuning; callers solve again before using any result.
template <typename SVT>
void FactorBank::force_flow_impl(const SVT& sets, int max_nrhs) {
  // every level in the flow launch, the widest chunks and the most
  // right-hand sides per lane that apply
  int best = -1;
  for (int c = 0; c < (int)flow_cfg_.size(); ++c) {
    const FlowConfig& C = flow_cfg_[c];
    if (!flow_ok(sets, max_nrhs, c) || C.top != flow_cfg_[0].top) continue;
    if (best < 0 || C.kc > flow_cfg_[best].kc || (C.kc == flow_cfg_[best].kc && C.rpl > flow_cfg_[best].rpl))
      best = c;
  }
  flow_sel_ = best;
}

void FactorBank::force_flow(const IlSetsViewF& sets, int max_nrhs) {
  force_flow_impl(sets, max_nrhs);
  release_unused_flow();
}
void FactorBank::force_flow(const IlSetsView& sets, int max_nrhs) {
  force_flow_impl(sets, max_nrhs);
  release_unused_flow();
}

void FactorBank::release_unused_flow() {
  for (int c = 0; c < (int)flow_cfg_.size(); ++c) {
    if (c == flow_sel_) continue;
    for (FlowPlan& P : flow_cfg_[c].plan) {
      P.items.release();
      P.sync.release();
      P.entries.release();
      P.n_entries = 0;
    }
  }
}

template <typename SVT>
void FactorBank::autotune_panel(const SVT& sets, int max_nrhs, cudaStream_t st, int reps, int flow_mode) {
  using T = typename std::conditional<std::is_same<SVT, IlSetsViewF>::value, float, double>::type;
  const int rpl = panel_rpl(sets, max_nrhs);
  cudaEvent_t e0, e1;
  PECS_CUDA(cudaEventCreate(&e0));
  PECS_CUDA(cudaEventCreate(&e1));
  for (int pass = 0; pass < 2; ++pass)
    for (PanelPlan& L : pass == 0 ? pfwd_ : pbwd_)
      L.tuned = panel_default_option<T>(L, max_nrhs, rpl, tune_, parts_ld_);
  auto time_sweep = [&]() {
    const int per_sweep = kernel_launches_per_solve();
    float best = 1e30f;
    solve_panel(sets, max_nrhs, st);  // warm-up
    tune_launches_ += per_sweep;
    for (int r = 0; r < reps; ++r) {
      PECS_CUDA(cudaEventRecord(e0, st));
      solve_panel(sets, max_nrhs, st);
      PECS_CUDA(cudaEventRecord(e1, st));
      PECS_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      PECS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, ms);
      tune_launches_ += per_sweep;
    }
    return best;
  };
  float best_sweep = time_sweep();
  for (int pass = 0; pass < 2; ++pass) {
    for (PanelPlan& L : pass == 0 ? pfwd_ : pbwd_) {
      const PanelOption keep = L.tuned;
      PanelOption best = keep;
      for (const PanelOption& o : panel_options<T>(L, max_nrhs, rpl, parts_ld_)) {
        if (o.kind == keep.kind && o.cap_idx == keep.cap_idx && o.rpl == keep.rpl) continue;
        L.tuned = o;
        float ms;
        try {
          ms = time_sweep();
        } catch (const PecsError& err) {
          if (err.code != PECS_E_ARG) throw;
          continue;  // the option's staging does not fit in shared memory
        }
        if (ms < best_sweep) {
          best_sweep = ms;
          best = o;
        }
      }
      L.tuned = best;
    }
  }
  // the flow sweep (one persistent launch per direction) at each valid
  // right-hand-sides-per-lane count, against the tuned level sweep
  int best_flow = -1;
  float best_flow_ms = 1e30f;
  for (int c = 0; c < (int)flow_cfg_.size() && flow_mode >= 0; ++c) {
    if (!flow_ok(sets, max_nrhs, c)) continue;
    flow_sel_ = c;
    const float ms = time_sweep();
    flow_sel_ = -1;
    if (std::getenv("PECS_TUNE_LOG"))  // diagnostic: every flow configuration's sweep time
      std::fprintf(stderr, "flow top %d kc %d rpl %d: %.4f ms (levels %.4f ms)\n", flow_cfg_[c].top,
                   flow_cfg_[c].kc, flow_cfg_[c].rpl, ms, best_sweep);
    if (flow_error() != 0)
      throw PecsError(PECS_E_CUDA, "flow sweep: a wait for a node's inputs ran out");
    if (ms < best_flow_ms) {
      best_flow_ms = ms;
      best_flow = c;
    }
  }
  if (best_flow >= 0 && (flow_mode > 0 || best_flow_ms < best_sweep)) {
    best_sweep = best_flow_ms;
    flow_sel_ = best_flow;
  }
  release_unused_flow();
  tuned_ms_ = best_sweep;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

std::vector<double> FactorBank::time_levels(const IlSetsViewF& sets, int max_nrhs, cudaStream_t st,
                                            int reps) const {
  if (!panel_ || prec_ == PECS_PREC_FP64) throw PecsError(PECS_E_STATE, "level timing needs an FP32 panel bank");
  const int rpl = panel_rpl(sets, max_nrhs);
  const BankView B = view();
  const int nl = (int)(pfwd_.size() + pbwd_.size());
  std::vector<cudaEvent_t> ev(nl + 1);
  for (auto& e : ev) PECS_CUDA(cudaEventCreate(&e));
  std::vector<double> ms(nl, 0.0);
  for (int r = 0; r <= reps; ++r) {
    int l = 0;
    PECS_CUDA(cudaEventRecord(ev[0], st));
    for (int pass = 0; pass < 2; ++pass)
      for (const PanelPlan& L : pass == 0 ? pfwd_ : pbwd_) {
        launch_panel_level<float, IlSetsViewF>(pass == 0, B, sets, L, max_nrhs, rpl, tune_, parts_ld_, st);
        PECS_CUDA(cudaEventRecord(ev[++l], st));
      }
    PECS_CUDA(cudaEventSynchronize(ev[nl]));
    if (r == 0) continue;
    for (int k = 0; k < nl; ++k) {
      float t = 0.f;
      PECS_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      ms[k] += t / reps;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return ms;
}

void FactorBank::autotune(const IlSetsViewF& sets, int max_nrhs, cudaStream_t st, int reps, int flow_mode) {
  if (!panel_ || prec_ == PECS_PREC_FP64) throw PecsError(PECS_E_STATE, "autotune needs an FP32 panel bank");
  autotune_panel(sets, max_nrhs, st, reps, flow_mode);
}

void FactorBank::autotune(const IlSetsView& sets, int max_nrhs, cudaStream_t st, int reps, int flow_mode) {
  if (!panel_ || prec_ != PECS_PREC_FP64) throw PecsError(PECS_E_STATE, "autotune needs an FP64 panel bank");
  autotune_panel(sets, max_nrhs, st, reps, flow_mode);
}

void FactorBank::solve(const IlSetsViewF& sets, int max_nrhs, cudaStream_t st) const {
  if (!panel_ || prec_ == PECS_PREC_FP64)
    throw PecsError(PECS_E_STATE, "float solve vectors need a panel bank with FP32 factors");
  solve_panel(sets, max_nrhs, st);
}

}  // namespace pecs
