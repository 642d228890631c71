// Checks of the front kernels in pecs_gb300/csrc/dense.cpp, compiled and run
// by test_dense_host.py.  Prints one line per check and exits non-zero on the
// first failure.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dense.hpp"

using namespace pecs::dense;

static uint64_t rng_state = 88172645463325252ULL;
static double urand() {  // xorshift64, uniform in [-1, 1)
  rng_state ^= rng_state << 13;
  rng_state ^= rng_state >> 7;
  rng_state ^= rng_state << 17;
  return (double)(rng_state >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

static int fail(const char* what, double v) {
  std::printf("FAIL %s %.3e\n", what, v);
  return 1;
}

// max |P A0 - [L; L21] [U11 U12] - [0 0; 0 S]| / max |A0| for the output of lu_front
static double lu_error(int f, int s, const std::vector<double>& A0, const std::vector<double>& A,
                       const std::vector<int>& perm) {
  double e = 0.0, nrm = 0.0;
  for (int i = 0; i < f; ++i) {
    const int src = i < s ? perm[i] : i;
    for (int j = 0; j < f; ++j) {
      double v = (i >= s && j >= s) ? A[(size_t)i * f + j] : 0.0;
      const int kmax = std::min(std::min(i, j) + 1, s);
      for (int k = 0; k < kmax; ++k) {
        const double l = k == i ? 1.0 : A[(size_t)i * f + k];
        v += l * A[(size_t)k * f + j];
      }
      e = std::max(e, std::fabs(v - A0[(size_t)src * f + j]));
      nrm = std::max(nrm, std::fabs(A0[(size_t)src * f + j]));
    }
  }
  return e / nrm;
}

int main() {
  Team t1(1), t4(4);
  // GEMM against the naive triple loop
  {
    const int M = 77, N = 131, K = 300;
    std::vector<double> A(M * K), B(K * N), C(M * N), R;
    for (auto& x : A) x = urand();
    for (auto& x : B) x = urand();
    for (auto& x : C) x = urand();
    R = C;
    gemm(M, N, K, -1.0, A.data(), K, B.data(), N, C.data(), N, &t4);
    double e = 0.0;
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < N; ++j) {
        double s = R[i * N + j];
        for (int k = 0; k < K; ++k) s -= A[i * K + k] * B[k * N + j];
        e = std::max(e, std::fabs(s - C[i * N + j]));
      }
    std::printf("gemm %.3e\n", e);
    if (!(e < 1e-12)) return fail("gemm", e);
  }
  // triangular products (all four forms) against the naive loop
  for (int left = 0; left < 2; ++left)
    for (int lower = 0; lower < 2; ++lower) {
      const int M = 301, N = 277, n = left ? M : N;
      std::vector<double> T((size_t)n * n, 0.0), B((size_t)M * N), C((size_t)M * N), R;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          if (lower ? j <= i : j >= i) T[(size_t)i * n + j] = urand();
      for (auto& x : B) x = urand();
      for (auto& x : C) x = urand();
      R = C;
      std::vector<double> C1 = C;
      trmm(left, lower, M, N, -1.0, T.data(), n, B.data(), N, C.data(), N, &t4);
      trmm(left, lower, M, N, -1.0, T.data(), n, B.data(), N, C1.data(), N, &t1);
      if (C != C1) return fail("trmm differs between 1 and 4 threads", 1.0);
      double e = 0.0;
      for (int i = 0; i < M; ++i)
        for (int j = 0; j < N; ++j) {
          double s = R[(size_t)i * N + j];
          for (int k = 0; k < n; ++k)
            s -= left ? T[(size_t)i * n + k] * B[(size_t)k * N + j]
                      : B[(size_t)i * N + k] * T[(size_t)k * n + j];
          e = std::max(e, std::fabs(s - C[(size_t)i * N + j]));
        }
      std::printf("trmm left=%d lower=%d %.3e\n", left, lower, e);
      if (!(e < 1e-12)) return fail("trmm", e);
    }
  const int sizes[][2] = {{1, 1}, {5, 3}, {65, 65}, {200, 130}, {700, 450}};
  for (const auto& fs : sizes) {
    const int f = fs[0], s = fs[1];
    std::vector<double> A0((size_t)f * f);
    for (auto& x : A0) x = urand();
    std::vector<double> A1 = A0, A4 = A0;
    std::vector<int> p1(s), p4(s);
    double bad = 0.0;
    if (lu_front(f, s, A1.data(), f, p1.data(), 1e-300, &bad, &t1) != -1) return fail("lu pivot", bad);
    if (lu_front(f, s, A4.data(), f, p4.data(), 1e-300, &bad, &t4) != -1) return fail("lu pivot", bad);
    if (std::memcmp(A1.data(), A4.data(), A1.size() * sizeof(double)) != 0 || p1 != p4)
      return fail("lu differs between 1 and 4 threads", 1.0);
    const double e = lu_error(f, s, A0, A4, p4);
    // inverses of the triangular factors
    std::vector<double> X((size_t)s * s), Y((size_t)s * s), X1((size_t)s * s), Y1((size_t)s * s);
    inv_unit_lower(s, A4.data(), f, X.data(), s, &t4);
    inv_upper(s, A4.data(), f, Y.data(), s, &t4);
    inv_unit_lower(s, A4.data(), f, X1.data(), s, &t1);
    inv_upper(s, A4.data(), f, Y1.data(), s, &t1);
    if (X != X1 || Y != Y1) return fail("inverses differ between 1 and 4 threads", 1.0);
    double ex = 0.0, ey = 0.0;
    for (int i = 0; i < s; ++i)
      for (int j = 0; j < s; ++j) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < s; ++k) {
          const double l = k == i ? 1.0 : (k < i ? A4[(size_t)i * f + k] : 0.0);
          a += l * X[(size_t)k * s + j];
          const double u = k >= i ? A4[(size_t)i * f + k] : 0.0;
          b += u * Y[(size_t)k * s + j];
        }
        ex = std::max(ex, std::fabs(a - (i == j)));
        ey = std::max(ey, std::fabs(b - (i == j)));
      }
    std::printf("front %d+%d lu %.3e Linv %.3e Uinv %.3e\n", s, f - s, e, ex, ey);
    if (!(e < 1e-12)) return fail("lu", e);
    if (!(ex < 1e-10) || !(ey < 1e-10)) return fail("inverse", std::max(ex, ey));
  }
  // a front whose fully-summed rows are rank deficient: the pivot check fires
  {
    const int f = 150, s = 100;
    std::vector<double> A((size_t)f * f);
    for (auto& x : A) x = urand();
    for (int r = 0; r < s; ++r) A[(size_t)r * f + 70] = 2.0 * A[(size_t)r * f + 3];
    std::vector<int> p(s);
    double bad = -1.0;
    const int col = lu_front(f, s, A.data(), f, p.data(), 1e-10, &bad, &t4);
    std::printf("singular column %d pivot %.3e\n", col, bad);
    if (col != 70) return fail("singular column not found", (double)col);
  }
  std::printf("OK\n");
  return 0;
}
