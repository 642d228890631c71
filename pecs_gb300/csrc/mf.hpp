// Multifrontal sparse LU with nested-dissection ordering, laid out for GEMV
// application on the GPU.
//
// Replaces SparseDirectUMFPACK::initialize / vmult as used by
// Carrier::set_solver / solve (source/Carrier.cpp:26-40) and
// PoissonData::set_solver / solve (source/Poisson.cpp:90-105).
//
// Ordering: dofs are grouped into "nodes".  Class-0 dofs (cell-local blocks
// that do not couple to class-0 dofs of other cells -- the LDG currents) form
// one leaf node per cell and are eliminated first.  The remaining dofs are
// ordered by geometric nested dissection over mesh cells on the quotient graph
// of the Schur complement left after the class-0 elimination; dofs with a zero
// diagonal (the mixed-method potential) are moved to the last node that holds
// a dof of their row, so that every fully-summed block is nonsingular without
// delayed pivots.
//
// Numerics: each node's front F = [F11 F12; F21 F22] (s own dofs, m update
// dofs) is factored with partial pivoting among its s fully-summed rows:
// P F11 = L11 U11, U12 = L11^-1 P F12, L21 = F21 U11^-1, S = F22 - L21 U12.
// What the solve needs is stored as two dense row-major blocks per node:
//   Gf = [L11^-1 P ; L21 L11^-1 P]         ((s+m) x s)  forward
//   Hb = [U11^-1 | -U11^-1 U12]             (s x (s+m))  backward
// so both sweeps are level-scheduled dense GEMVs (no sequential triangular
// substitution inside a node).
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "problem.hpp"

namespace pecs {

struct MfNode {
  int s = 0, m = 0;
  std::vector<int> own;  // global dofs, in front order (slot r <-> own[r])
  std::vector<int> upd;  // global dofs of the update set, ascending elimination position
  int parent = -1;
  std::vector<int> children;
  int height = 0, depth = 0;
  bool cls0 = false;
};

struct MfFactor {
  int n = 0;
  std::vector<MfNode> nodes;  // elimination order (children before parents)
  std::vector<int> pos;       // dof -> elimination position
  std::vector<int> node_of;   // dof -> node
  std::vector<std::vector<double>> Gf, Hb;
  int n_heights = 0, n_depths = 0;
  long long entries() const;  // stored values in Gf + Hb
  int max_front() const;
  double factor_flops = 0.0;
};

// Dense work of one front handed to another device (front.cu): given the
// assembled front Fm (f x f, row-major; s fully-summed rows/columns) and the
// pivot threshold, returns -1 (or the first bad column, with its pivot
// magnitude in *bad) and fills perm (s), Gf (f x s, permuted), Hb (s x f) and
// the Schur complement S (m x m) exactly as the host path defines them.
struct FrontOffload {
  int min_front = 0;  // fronts with at least this many rows go to the device
  void* ctx = nullptr;
  int (*factor)(void* ctx, int f, int s, const double* Fm, double tiny, int* perm, double* bad,
                std::vector<double>& G, std::vector<double>& H, std::vector<double>& S) = nullptr;
};

// The GPU implementation (front.cu) on `device`; fronts of min_front rows and up.
std::shared_ptr<FrontOffload> make_gpu_front_offload(int device, int min_front);

// Ordering + symbolic analysis.  Throws std::runtime_error on invalid input.
MfFactor mf_analyze(const Csr& A, const int* dof_cell, const int* dof_class, int n_cells,
                    const double* cell_xy, int leaf_cells);
// Numeric factorisation (FP64, host; the largest fronts on a device when
// `off` is given).  Throws std::runtime_error("singular ...").
void mf_factorize(MfFactor& F, const Csr& A, int n_threads = 0, const FrontOffload* off = nullptr);
// Host application of the stored factors (diagnostic; the product path runs on the GPU).
void mf_apply_host(const MfFactor& F, const double* b, double* x);

}  // namespace pecs
