// Dense FP64 kernels for the multifrontal fronts (see dense.hpp).
#include "dense.hpp"

#include <algorithm>
#include <cmath>
#include <exception>
#include <utility>

namespace pecs {
namespace dense {

Team::Team(int n) : n_(std::max(1, n)) {
  th_.reserve(n_ - 1);
  try {
    for (int i = 1; i < n_; ++i) th_.emplace_back([this, i]() { worker(i); });
  } catch (...) {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
    throw;
  }
}

void run_threads(int n, const std::function<void(int)>& fn) {
  std::vector<std::thread> th;
  th.reserve(n > 1 ? n - 1 : 0);
  std::exception_ptr err;
  try {
    for (int t = 1; t < n; ++t) th.emplace_back(fn, t);
    fn(0);
  } catch (...) {
    err = std::current_exception();
  }
  for (auto& x : th) x.join();
  if (err) std::rethrow_exception(err);
}

Team::~Team() {
  {
    std::lock_guard<std::mutex> g(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  for (auto& t : th_) t.join();
}

void Team::run(int nt, const std::function<void(int)>& fn) {
  nt = std::max(1, std::min(nt, n_));
  if (nt == 1) {
    fn(0);
    return;
  }
  {
    std::lock_guard<std::mutex> g(mu_);
    job_ = &fn;
    job_nt_ = nt;
    pending_ = nt - 1;
    ++gen_;
  }
  cv_.notify_all();
  fn(0);
  std::unique_lock<std::mutex> lk(mu_);
  done_.wait(lk, [&]() { return pending_ == 0; });
  job_ = nullptr;
}

void Team::worker(int id) {
  long long seen = 0;
  for (;;) {
    const std::function<void(int)>* job;
    int nt;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&]() { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      job = job_;
      nt = job_nt_;
    }
    if (id < nt) {
      (*job)(id);
      std::lock_guard<std::mutex> g(mu_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
}

namespace {

constexpr int MR = 4;      // micro-tile rows
constexpr int NR = 8;      // micro-tile columns
constexpr int KC = 256;    // K block (packed strips stay in L1/L2)
constexpr int MC = 64;     // rows of A packed per block
constexpr int NC = 1024;   // columns of B packed per block
constexpr int kBase = 64;  // triangular inverses: scalar below this size
constexpr int NB = 64;     // LU block-column width
constexpr int kTrmmBase = 128;  // triangular products: dense GEMM below this size
constexpr double kWorkPerThread = 2.5e5;  // multiply-adds that justify one more thread

int team_size(const Team* team) { return team ? team->size() : 1; }

// Runs fn(begin, end) over [0, n) in at most nt contiguous ranges whose
// boundaries are multiples of grain.
void parallel_ranges(int n, Team* team, int nt, int grain, const std::function<void(int, int)>& fn) {
  const int chunks = (n + grain - 1) / grain;
  nt = std::max(1, std::min({nt, chunks, team_size(team)}));
  if (nt == 1) {
    fn(0, n);
    return;
  }
  team->run(nt, [&](int t) {
    const int c0 = (int)((long long)chunks * t / nt), c1 = (int)((long long)chunks * (t + 1) / nt);
    const int b = std::min(n, c0 * grain), e = std::min(n, c1 * grain);
    if (b < e) fn(b, e);
  });
}

int threads_for(double work, const Team* team) {
  return (int)std::max(1.0, std::min((double)team_size(team), work / kWorkPerThread));
}

// Packs A[0:mc, 0:kc] * alpha into MR-row strips: Ap[strip][k][MR], zero-padded.
void pack_a(int mc, int kc, double alpha, const double* A, int lda, double* Ap) {
  for (int i0 = 0; i0 < mc; i0 += MR) {
    const int mr = std::min(MR, mc - i0);
    for (int k = 0; k < kc; ++k) {
      double* d = Ap + (size_t)k * MR;
      for (int r = 0; r < mr; ++r) d[r] = alpha * A[(size_t)(i0 + r) * lda + k];
      for (int r = mr; r < MR; ++r) d[r] = 0.0;
    }
    Ap += (size_t)kc * MR;
  }
}

// Packs B[0:kc, 0:nc] into NR-column strips: Bp[strip][k][NR], zero-padded.
void pack_b(int kc, int nc, const double* B, int ldb, double* Bp) {
  for (int j0 = 0; j0 < nc; j0 += NR) {
    const int nr = std::min(NR, nc - j0);
    for (int k = 0; k < kc; ++k) {
      const double* s = B + (size_t)k * ldb + j0;
      double* d = Bp + (size_t)k * NR;
      for (int q = 0; q < nr; ++q) d[q] = s[q];
      for (int q = nr; q < NR; ++q) d[q] = 0.0;
    }
    Bp += (size_t)kc * NR;
  }
}

// C[0:mr, 0:nr] += a-strip * b-strip over kc.
inline void micro(int kc, const double* __restrict a, const double* __restrict b, double* C, int ldc,
                  int mr, int nr) {
  double c[MR][NR];
  for (int r = 0; r < MR; ++r)
    for (int q = 0; q < NR; ++q) c[r][q] = 0.0;
  for (int k = 0; k < kc; ++k) {
    const double* ak = a + (size_t)k * MR;
    const double* bk = b + (size_t)k * NR;
    for (int r = 0; r < MR; ++r) {
      const double ar = ak[r];
      for (int q = 0; q < NR; ++q) c[r][q] += ar * bk[q];
    }
  }
  if (mr == MR && nr == NR) {
    for (int r = 0; r < MR; ++r)
      for (int q = 0; q < NR; ++q) C[(size_t)r * ldc + q] += c[r][q];
  } else {
    for (int r = 0; r < mr; ++r)
      for (int q = 0; q < nr; ++q) C[(size_t)r * ldc + q] += c[r][q];
  }
}

void gemm_serial(int M, int N, int K, double alpha, const double* A, int lda, const double* B,
                 int ldb, double* C, int ldc) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  thread_local std::vector<double> Ap, Bp;
  const int ncmax = std::min(NC, (N + NR - 1) / NR * NR);
  const int mcmax = std::min(MC, (M + MR - 1) / MR * MR);
  const int kcmax = std::min(KC, K);
  if (Bp.size() < (size_t)kcmax * ncmax) Bp.resize((size_t)kcmax * ncmax);
  if (Ap.size() < (size_t)kcmax * mcmax) Ap.resize((size_t)kcmax * mcmax);
  for (int jc = 0; jc < N; jc += NC) {
    const int nc = std::min(NC, N - jc);
    for (int pc = 0; pc < K; pc += KC) {
      const int kc = std::min(KC, K - pc);
      pack_b(kc, nc, B + (size_t)pc * ldb + jc, ldb, Bp.data());
      for (int ic = 0; ic < M; ic += MC) {
        const int mc = std::min(MC, M - ic);
        pack_a(mc, kc, alpha, A + (size_t)ic * lda + pc, lda, Ap.data());
        for (int jr = 0; jr < nc; jr += NR) {
          const double* bs = Bp.data() + (size_t)(jr / NR) * kc * NR;
          for (int ir = 0; ir < mc; ir += MR)
            micro(kc, Ap.data() + (size_t)(ir / MR) * kc * MR, bs,
                  C + (size_t)(ic + ir) * ldc + jc + jr, ldc, std::min(MR, mc - ir),
                  std::min(NR, nc - jr));
        }
      }
    }
  }
}

void inv_unit_lower_base(int n, const double* L, int ldl, double* X, int ldx) {
  for (int r = 0; r < n; ++r) {
    double* xr = X + (size_t)r * ldx;
    for (int c = 0; c < n; ++c) xr[c] = 0.0;
    xr[r] = 1.0;
    const double* lr = L + (size_t)r * ldl;
    for (int t = 0; t < r; ++t) {
      const double l = lr[t];
      if (l == 0.0) continue;
      const double* xt = X + (size_t)t * ldx;
      for (int c = 0; c <= t; ++c) xr[c] -= l * xt[c];
    }
  }
}

void inv_upper_base(int n, const double* U, int ldu, double* Y, int ldy) {
  for (int r = n - 1; r >= 0; --r) {
    const double* ur = U + (size_t)r * ldu;
    double* yr = Y + (size_t)r * ldy;
    for (int c = 0; c < n; ++c) yr[c] = 0.0;
    const double dinv = 1.0 / ur[r];
    yr[r] = dinv;
    for (int t = r + 1; t < n; ++t) {
      const double u = ur[t];
      if (u == 0.0) continue;
      const double* yt = Y + (size_t)t * ldy;
      for (int c = t; c < n; ++c) yr[c] -= u * dinv * yt[c];
    }
  }
}

int split_point(int n) { return std::max(kBase / 2, (n / 2 + 7) / 8 * 8); }

// Recursive LU of the block column [c0, c0+nc) over rows [c0, f), pivots among
// rows [c0, s); everything right of the block column is left untouched except
// for whole-row swaps.
int panel_lu(int f, int s, double* A, int lda, int* perm, int c0, int nc, double tiny,
             double* bad_pivot, Team* team) {
  if (nc == 1) {
    const int col = c0;
    int piv = col;
    double best = std::fabs(A[(size_t)col * lda + col]);
    for (int r = col + 1; r < s; ++r) {
      const double v = std::fabs(A[(size_t)r * lda + col]);
      if (v > best) {
        best = v;
        piv = r;
      }
    }
    if (!(best > tiny) || !std::isfinite(best)) {
      *bad_pivot = best;
      return col;
    }
    if (piv != col) {
      std::swap_ranges(A + (size_t)col * lda, A + (size_t)col * lda + f, A + (size_t)piv * lda);
      std::swap(perm[col], perm[piv]);
    }
    const double inv = 1.0 / A[(size_t)col * lda + col];
    for (int r = col + 1; r < f; ++r) A[(size_t)r * lda + col] *= inv;
    return -1;
  }
  const int n1 = nc / 2, n2 = nc - n1, c1 = c0 + n1;
  int bad = panel_lu(f, s, A, lda, perm, c0, n1, tiny, bad_pivot, team);
  if (bad >= 0) return bad;
  // rows c0..c1-1, columns c1..c0+nc-1 <- L11^-1 (unit lower) applied
  for (int r = c0 + 1; r < c1; ++r) {
    double* rr = A + (size_t)r * lda + c1;
    for (int t = c0; t < r; ++t) {
      const double l = A[(size_t)r * lda + t];
      if (l == 0.0) continue;
      const double* tr = A + (size_t)t * lda + c1;
      for (int c = 0; c < n2; ++c) rr[c] -= l * tr[c];
    }
  }
  gemm(f - c1, n2, n1, -1.0, A + (size_t)c1 * lda + c0, lda, A + (size_t)c0 * lda + c1, lda,
       A + (size_t)c1 * lda + c1, lda, team);
  return panel_lu(f, s, A, lda, perm, c1, n2, tiny, bad_pivot, team);
}

}  // namespace

void gemm(int M, int N, int K, double alpha, const double* A, int lda, const double* B, int ldb,
          double* C, int ldc, Team* team) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  const int nt = threads_for((double)M * N * K, team);
  if (nt <= 1) {
    gemm_serial(M, N, K, alpha, A, lda, B, ldb, C, ldc);
    return;
  }
  // split the longer output dimension; every element keeps its K order
  if (M >= N)
    parallel_ranges(M, team, nt, MR, [&](int r0, int r1) {
      gemm_serial(r1 - r0, N, K, alpha, A + (size_t)r0 * lda, lda, B, ldb, C + (size_t)r0 * ldc, ldc);
    });
  else
    parallel_ranges(N, team, nt, NR, [&](int c0, int c1) {
      gemm_serial(M, c1 - c0, K, alpha, A, lda, B + c0, ldb, C + c0, ldc);
    });
}

void trmm(bool left, bool lower, int M, int N, double alpha, const double* T, int ldt,
          const double* B, int ldb, double* C, int ldc, Team* team) {
  if (M <= 0 || N <= 0) return;
  const int n = left ? M : N;
  if (n <= kTrmmBase) {
    if (left)
      gemm(M, N, M, alpha, T, ldt, B, ldb, C, ldc, team);
    else
      gemm(M, N, N, alpha, B, ldb, T, ldt, C, ldc, team);
    return;
  }
  const int p = split_point(n), r = n - p;
  const double* T11 = T;
  const double* T12 = T + p;
  const double* T21 = T + (size_t)p * ldt;
  const double* T22 = T + (size_t)p * ldt + p;
  if (left) {
    // rows of C: [0, p) and [p, M)
    const double* B1 = B;
    const double* B2 = B + (size_t)p * ldb;
    double* C1 = C;
    double* C2 = C + (size_t)p * ldc;
    if (lower) {  // C1 += T11 B1; C2 += T21 B1 + T22 B2
      trmm(true, true, p, N, alpha, T11, ldt, B1, ldb, C1, ldc, team);
      gemm(r, N, p, alpha, T21, ldt, B1, ldb, C2, ldc, team);
      trmm(true, true, r, N, alpha, T22, ldt, B2, ldb, C2, ldc, team);
    } else {      // C1 += T11 B1 + T12 B2; C2 += T22 B2
      trmm(true, false, p, N, alpha, T11, ldt, B1, ldb, C1, ldc, team);
      gemm(p, N, r, alpha, T12, ldt, B2, ldb, C1, ldc, team);
      trmm(true, false, r, N, alpha, T22, ldt, B2, ldb, C2, ldc, team);
    }
  } else {
    // columns of C: [0, p) and [p, N)
    const double* B1 = B;
    const double* B2 = B + p;
    double* C1 = C;
    double* C2 = C + p;
    if (lower) {  // C1 += B1 T11 + B2 T21; C2 += B2 T22
      trmm(false, true, M, p, alpha, T11, ldt, B1, ldb, C1, ldc, team);
      gemm(M, p, r, alpha, B2, ldb, T21, ldt, C1, ldc, team);
      trmm(false, true, M, r, alpha, T22, ldt, B2, ldb, C2, ldc, team);
    } else {      // C1 += B1 T11; C2 += B1 T12 + B2 T22
      trmm(false, false, M, p, alpha, T11, ldt, B1, ldb, C1, ldc, team);
      gemm(M, r, p, alpha, B1, ldb, T12, ldt, C2, ldc, team);
      trmm(false, false, M, r, alpha, T22, ldt, B2, ldb, C2, ldc, team);
    }
  }
}

void inv_unit_lower(int n, const double* L, int ldl, double* X, int ldx, Team* team) {
  if (n <= kBase) {
    inv_unit_lower_base(n, L, ldl, X, ldx);
    return;
  }
  // L = [La 0; Lb Lc]  ->  L^-1 = [La^-1 0; -Lc^-1 Lb La^-1  Lc^-1]
  const int n1 = split_point(n), n2 = n - n1;
  inv_unit_lower(n1, L, ldl, X, ldx, team);
  inv_unit_lower(n2, L + (size_t)n1 * ldl + n1, ldl, X + (size_t)n1 * ldx + n1, ldx, team);
  for (int r = 0; r < n1; ++r)
    for (int c = n1; c < n; ++c) X[(size_t)r * ldx + c] = 0.0;
  std::vector<double> T((size_t)n2 * n1, 0.0);
  trmm(false, true, n2, n1, 1.0, X, ldx, L + (size_t)n1 * ldl, ldl, T.data(), n1, team);
  double* Xb = X + (size_t)n1 * ldx;
  for (int r = 0; r < n2; ++r)
    for (int c = 0; c < n1; ++c) Xb[(size_t)r * ldx + c] = 0.0;
  trmm(true, true, n2, n1, -1.0, X + (size_t)n1 * ldx + n1, ldx, T.data(), n1, Xb, ldx, team);
}

void inv_upper(int n, const double* U, int ldu, double* Y, int ldy, Team* team) {
  if (n <= kBase) {
    inv_upper_base(n, U, ldu, Y, ldy);
    return;
  }
  // U = [Ua Ub; 0 Uc]  ->  U^-1 = [Ua^-1  -Ua^-1 Ub Uc^-1; 0 Uc^-1]
  const int n1 = split_point(n), n2 = n - n1;
  inv_upper(n1, U, ldu, Y, ldy, team);
  inv_upper(n2, U + (size_t)n1 * ldu + n1, ldu, Y + (size_t)n1 * ldy + n1, ldy, team);
  for (int r = n1; r < n; ++r)
    for (int c = 0; c < n1; ++c) Y[(size_t)r * ldy + c] = 0.0;
  std::vector<double> T((size_t)n1 * n2, 0.0);
  trmm(false, false, n1, n2, 1.0, Y + (size_t)n1 * ldy + n1, ldy, U + n1, ldu, T.data(), n2, team);
  double* Yb = Y + n1;
  for (int r = 0; r < n1; ++r)
    for (int c = 0; c < n2; ++c) Yb[(size_t)r * ldy + c] = 0.0;
  trmm(true, false, n1, n2, -1.0, Y, ldy, T.data(), n2, Yb, ldy, team);
}

int lu_front(int f, int s, double* A, int lda, int* perm, double tiny, double* bad_pivot,
             Team* team) {
  for (int t = 0; t < s; ++t) perm[t] = t;
  for (int k0 = 0; k0 < s; k0 += NB) {
    const int k1 = std::min(s, k0 + NB), kb = k1 - k0;
    const int bad = panel_lu(f, s, A, lda, perm, k0, kb, tiny, bad_pivot, team);
    if (bad >= 0) return bad;
    if (k1 == f) continue;
    // U block row: rows k0..k1-1, columns k1..f-1 <- L_kk^-1 (unit lower) applied
    parallel_ranges(f - k1, team, threads_for(0.5 * kb * kb * (double)(f - k1), team), 64,
                    [&](int c0, int c1) {
                      for (int r = k0 + 1; r < k1; ++r) {
                        double* rr = A + (size_t)r * lda + k1;
                        for (int t = k0; t < r; ++t) {
                          const double l = A[(size_t)r * lda + t];
                          if (l == 0.0) continue;
                          const double* tr = A + (size_t)t * lda + k1;
                          for (int c = c0; c < c1; ++c) rr[c] -= l * tr[c];
                        }
                      }
                    });
    // trailing update of every row below the block column, all remaining columns
    gemm(f - k1, f - k1, kb, -1.0, A + (size_t)k1 * lda + k0, lda, A + (size_t)k0 * lda + k1, lda,
         A + (size_t)k1 * lda + k1, lda, team);
  }
  return -1;
}

}  // namespace dense
}  // namespace pecs
