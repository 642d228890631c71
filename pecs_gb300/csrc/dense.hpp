// Dense FP64 kernels for the multifrontal factorisation's fronts (host).
//
// All matrices are row-major with an explicit leading dimension.  The GEMM
// packs K x N panels of B and M x K panels of A into register-tile strips and
// runs a fixed-size micro-kernel; the per-element summation order depends
// only on the K blocking, never on the thread count, so results are the same
// for any number of threads.  Plain C++ (no intrinsics): the compiler
// vectorises the micro-kernel on x86-64 and aarch64 alike.
#pragma once

#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace pecs {
namespace dense {

// A fixed group of threads that runs data-parallel jobs: run(nt, fn) calls
// fn(t) for t in [0, nt) (nt <= size()), the caller itself taking t = 0, and
// returns when every part is done.  fn must not throw.
class Team {
 public:
  explicit Team(int n);
  ~Team();
  Team(const Team&) = delete;
  Team& operator=(const Team&) = delete;
  int size() const { return n_; }
  void run(int nt, const std::function<void(int)>& fn);

 private:
  void worker(int id);
  int n_;
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int job_nt_ = 0, pending_ = 0;
  long long gen_ = 0;
  bool stop_ = false;
};

// Runs fn(t) for t in [0, n) on n threads (the caller takes t = 0) and joins
// them; if starting a thread fails, joins the started ones and rethrows.
void run_threads(int n, const std::function<void(int)>& fn);

// C[M x N] += alpha * A[M x K] * B[K x N]; threads from `team` (may be null).
void gemm(int M, int N, int K, double alpha, const double* A, int lda, const double* B, int ldb,
          double* C, int ldc, Team* team);

// C += alpha * T * B (left) or C += alpha * B * T (right), T triangular
// (lower or upper; its other triangle must hold zeros, which the blocks below
// the recursion's base size multiply through).  C is M x N; T is M x M (left)
// or N x N (right).  About half a GEMM's work.
void trmm(bool left, bool lower, int M, int N, double alpha, const double* T, int ldt,
          const double* B, int ldb, double* C, int ldc, Team* team);

// X = L^{-1} for a unit lower-triangular L (n x n, strictly lower part read
// from L); X's strictly upper part is set to zero.
void inv_unit_lower(int n, const double* L, int ldl, double* X, int ldx, Team* team);

// Y = U^{-1} for an upper-triangular U (n x n, upper part incl. the diagonal
// read from U); Y's strictly lower part is set to zero.
void inv_upper(int n, const double* U, int ldu, double* Y, int ldy, Team* team);

// In-place LU with partial pivoting of the first s columns of the f x f
// front A (rows 0..s-1 are the pivot candidates, rows s..f-1 are only
// eliminated): P A[:, 0:s] = [L11; L21] U11, A[0:s, s:f] <- L11^{-1} P A12,
// A[s:f, s:f] <- A22 - L21 U12.  Row swaps are applied to whole rows and
// recorded in perm (perm[t] = original row now at row t).  Returns the index
// of the first column whose pivot magnitude is not above tiny (or is not
// finite) and stores that magnitude in *bad_pivot, or returns -1.
int lu_front(int f, int s, double* A, int lda, int* perm, double tiny, double* bad_pivot,
             Team* team);

}  // namespace dense
}  // namespace pecs
