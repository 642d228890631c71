// pecs_dropin.hpp -- C++ drop-in classes with the reference's names over the
// pecs C ABI (pecs.h).  Header-only; link against libpecs_gb300.so.
//
// They mirror, member by member, the containers and assembly classes the
// reference's IMEX loop uses (paths relative to the reference project):
//   ChargeCarrierSpace::Carrier      include/Carrier.hpp:38-101, source/Carrier.cpp
//   ChargeCarrierSpace::CarrierPair  include/CarrierPair.hpp:30-110, source/CarrierPair.cpp
//   Poisson::PoissonData             include/Poisson.hpp:26-84, source/Poisson.cpp
//   Assembly::AssemblyScratch, Assembly::{Poisson,DriftDiffusion}::CopyData
//                                    include/Assembly.hpp:46-283
//   LDG_System::LDG                  include/LDG.hpp:189-290, source/LDG.cpp:40-678
//   MixedPoisson::MixedFEM           include/MixedFEM.hpp:165-172, source/MixedFEM.cpp:29-164
// with deal.II types replaced by plain containers: the system matrix is a CSR
// triple, vectors are std::vector<double>, a cell iterator is a CellIterator
// (the cell's size, face boundary ids, material id, dof indices and
// neighbours), and the FEValues of the scratch are the library's element
// tables.  set_solver() factorises once
// (UMFPACK's initialize), solve() applies the factors on the GPU (UMFPACK's
// vmult).  Errors throw std::runtime_error, which the reference's main()
// already catches as std::exception (source/main/main.cpp:28-39).
#pragma once
#include <algorithm>
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "pecs.h"

namespace pecs_dropin {

inline void check(int code) {
  if (code != PECS_OK) throw std::runtime_error(std::string("pecs: ") + pecs_last_error());
}

struct SparseMatrix {  // CSR (the role of dealii::SparseMatrix<double>)
  int n = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
  // A(i, j) += v; the entry must be in the sparsity pattern (columns sorted
  // per row), as for dealii::SparseMatrix::add
  void add(int i, int j, double v) {
    if (i < 0 || i >= n) throw std::runtime_error("pecs: row out of range");
    const int* b = col.data() + rowptr[i];
    const int* e = col.data() + rowptr[i + 1];
    const int* p = std::lower_bound(b, e, j);
    if (p == e || *p != j)
      throw std::runtime_error("pecs: entry (" + std::to_string(i) + ", " + std::to_string(j) +
                               ") not in the sparsity pattern");
    val[p - col.data()] += v;
  }
  void set_zero() { std::fill(val.begin(), val.end(), 0.0); }
};

// What the reference's assembly reads from a DoFHandler cell iterator.
struct CellIterator {
  pecs_cell geometry{};              // hx, hy, boundary_id[4] (-1 interior), material_id
  std::vector<int> dof_indices;      // cell->get_dof_indices
  int neighbor[4] = {-1, -1, -1, -1};  // neighbouring cell per face (index into the cell list)
};

// Mesh information the nested-dissection ordering needs: the cell owning each
// dof, cell centres, and (for the LDG systems) which dofs are cell-local
// currents.  deal.II callers fill it from DoFHandler::active_cell_iterator.
struct DofMap {
  std::vector<int> dof_cell;
  std::vector<int> dof_class;  // empty = all class 1
  std::vector<double> cell_xy;
};

class DirectSolver {  // SparseDirectUMFPACK replacement
 public:
  DirectSolver() = default;
  DirectSolver(const DirectSolver&) = delete;
  DirectSolver& operator=(const DirectSolver&) = delete;
  ~DirectSolver() { pecs_lu_destroy(lu_); }
  void initialize(const SparseMatrix& A, const DofMap& m, int precision = PECS_PREC_FP64) {
    pecs_lu_destroy(lu_);
    lu_ = nullptr;
    check(pecs_lu_factor(A.n, A.rowptr.data(), A.col.data(), A.val.data(), m.dof_cell.data(),
                         m.dof_class.empty() ? nullptr : m.dof_class.data(),
                         (int)(m.cell_xy.size() / 2), m.cell_xy.data(), precision, 0, &lu_));
    n_ = A.n;
    A_ = &A;
  }
  // x = A^-1 b on the GPU, then one refinement step with an FP64 residual on
  // the host: the step UMFPACK's default control takes when deal.II's
  // SparseDirectUMFPACK::solve / vmult hands it the matrix
  void vmult(std::vector<double>& x, const std::vector<double>& b) const {
    if (!lu_) throw std::runtime_error("pecs: solver not initialised");
    if ((int)b.size() != n_) throw std::runtime_error("pecs: rhs size mismatch");
    x.resize(n_);
    std::vector<double> r(n_), d(n_);
    check(pecs_lu_solve(lu_, 1, b.data(), x.data()));
    for (int i = 0; i < n_; ++i) {
      double s = b[i];
      for (int p = A_->rowptr[i]; p < A_->rowptr[i + 1]; ++p) s -= A_->val[p] * x[A_->col[p]];
      r[i] = s;
    }
    check(pecs_lu_solve(lu_, 1, r.data(), d.data()));
    for (int i = 0; i < n_; ++i) x[i] += d[i];
  }

 private:
  pecs_lu* lu_ = nullptr;
  const SparseMatrix* A_ = nullptr;  // the factored matrix (kept alive by its owner)
  int n_ = 0;
};

namespace ChargeCarrierSpace {

struct Carrier {
  void set_name(const std::string& s) { name = s; }
  void set_solver() { solver.initialize(system_matrix, dof_map); }  // Carrier.cpp:26-32
  void solve() { solver.vmult(solution, system_rhs); }              // Carrier.cpp:34-40
  std::string name;
  SparseMatrix system_matrix;
  std::vector<double> system_rhs;
  std::vector<double> solution;
  DirectSolver solver;
  DofMap dof_map;
  double scaled_mobility = 1.0;
  double charge_number = 0.0;
};

struct CarrierPair {
  void set_name(const std::string& s) { material_name = s; }
  // CarrierPair::print_dofs / read_dofs (CarrierPair.cpp:89-121): the
  // solution of each carrier as "<name>.dofs" in the layout of deal.II's
  // Vector::block_write -- the size in ASCII decimal, '\n', '[', the raw
  // doubles, ']' -- so restart files move between the two codes.
  void print_dofs() const {
    for (const Carrier* c : {&carrier_1, &carrier_2}) {
      std::ofstream out(c->name + ".dofs", std::ios::binary);
      const std::string head = std::to_string(c->solution.size()) + "\n[";
      out.write(head.data(), (std::streamsize)head.size());
      out.write(reinterpret_cast<const char*>(c->solution.data()),
                (std::streamsize)(c->solution.size() * sizeof(double)));
      out.put(']');
      if (!out) throw std::runtime_error("pecs: cannot write " + c->name + ".dofs");
    }
  }
  void read_dofs() {
    for (Carrier* c : {&carrier_1, &carrier_2}) {
      std::ifstream in(c->name + ".dofs", std::ios::binary);
      std::size_t n = 0;
      char open = 0, close = 0;
      in >> n;
      in.get();  // '\n'
      in.get(open);
      c->solution.resize(n);
      in.read(reinterpret_cast<char*>(c->solution.data()), (std::streamsize)(n * sizeof(double)));
      in.get(close);
      if (!in || open != '[' || close != ']')
        throw std::runtime_error("pecs: cannot read " + c->name + ".dofs");
    }
  }
  Carrier carrier_1, carrier_2;
  SparseMatrix mass_matrix;
  double penalty = 1.0;
  double delta_t = 0.0;
  double material_permittivity = 1.0;
  std::string material_name;
};

}  // namespace ChargeCarrierSpace

namespace Poisson {

struct PoissonData {
  void set_solver() { solver.initialize(system_matrix, dof_map); }  // Poisson.cpp:90-96
  void solve() {                                                    // Poisson.cpp:98-105
    solver.vmult(solution, system_rhs);
    for (int d : constrained_dofs) solution[d] = 0.0;  // constraints.distribute (homogeneous)
  }
  SparseMatrix system_matrix;
  std::vector<double> system_rhs, solution;
  std::vector<int> constrained_dofs;
  DirectSolver solver;
  DofMap dof_map;
};

}  // namespace Poisson

// ---- assembly scratch and copy data (include/Assembly.hpp:46-283) -----------
namespace Assembly {

// The reference's scratch holds FEValues objects and per-qp buffers for the
// Poisson and carrier elements; here the element tables live in the library
// and the scratch keeps the element choice and the local block sizes.
struct AssemblyScratch {
  AssemblyScratch(int degree_, int poisson_pairing_ = 0) : degree(degree_), poisson_pairing(poisson_pairing_) {
    check(pecs_element_sizes(degree, poisson_pairing, &carrier_dofs_per_cell, &poisson_rt_dofs,
                             &poisson_phi_dofs));
  }
  int degree, poisson_pairing;
  int carrier_dofs_per_cell = 0, poisson_rt_dofs = 0, poisson_phi_dofs = 0;
};

struct FullMatrix {  // dealii::FullMatrix<double>, row-major
  int m = 0;
  std::vector<double> v;
  void reinit(int n) {
    m = n;
    v.assign((size_t)n * n, 0.0);
  }
  double operator()(int i, int j) const { return v[(size_t)i * m + j]; }
  double* data() { return v.data(); }
};

namespace Poisson {
struct CopyData {
  explicit CopyData(const AssemblyScratch& s) {
    const int n = s.poisson_rt_dofs + s.poisson_phi_dofs;
    local_rhs.assign(n, 0.0);
    local_matrix.reinit(n);
    local_dof_indices.assign(n, 0);
  }
  std::vector<double> local_rhs;
  FullMatrix local_matrix;
  std::vector<int> local_dof_indices;
};
}  // namespace Poisson

namespace DriftDiffusion {
struct CopyData {
  explicit CopyData(const AssemblyScratch& s) {
    const int n = s.carrier_dofs_per_cell;
    local_carrier_1_rhs.assign(n, 0.0);
    local_carrier_2_rhs.assign(n, 0.0);
    for (FullMatrix* M : {&local_matrix_1, &local_matrix_2, &local_mass_matrix, &vi_ui_matrix,
                          &vi_ue_matrix, &ve_ui_matrix, &ve_ue_matrix})
      M->reinit(n);
    local_dof_indices.assign(n, 0);
    local_neighbor_dof_indices.assign(n, 0);
  }
  std::vector<double> local_carrier_1_rhs, local_carrier_2_rhs;
  FullMatrix local_matrix_1, local_matrix_2, local_mass_matrix;
  FullMatrix vi_ui_matrix, vi_ue_matrix, ve_ui_matrix, ve_ue_matrix;
  std::vector<int> local_dof_indices, local_neighbor_dof_indices;
};
}  // namespace DriftDiffusion

}  // namespace Assembly

// ---- LDG system assembly (include/LDG.hpp:189-290) ----------------------------
namespace LDG_System {

inline void add_local(SparseMatrix& A, const std::vector<int>& rows, const std::vector<int>& cols,
                      const Assembly::FullMatrix& M) {
  for (int i = 0; i < M.m; ++i)
    for (int j = 0; j < M.m; ++j) {
      const double v = M(i, j);
      if (v != 0.0) A.add(rows[i], cols[j], v);
    }
}

struct LDG {
  // LDG.cpp:40-83
  void assemble_local_LDG_mass_matrix(const CellIterator& cell, Assembly::AssemblyScratch& scratch,
                                      Assembly::DriftDiffusion::CopyData& data, const double& delta_t) {
    data.local_dof_indices = cell.dof_indices;
    check(pecs_ldg_local_mass_matrix(scratch.degree, &cell.geometry, delta_t, data.local_mass_matrix.data()));
  }
  // LDG.cpp:85-281
  void assemble_local_LDG_cell_and_bc_terms(const CellIterator& cell, Assembly::AssemblyScratch& scratch,
                                            Assembly::DriftDiffusion::CopyData& data,
                                            const double& scaled_mobility_1, const double& scaled_mobility_2,
                                            const double& delta_t, const double& transient_or_steady,
                                            const double& penalty) {
    data.local_dof_indices = cell.dof_indices;
    check(pecs_ldg_local_cell_and_bc_terms(scratch.degree, &cell.geometry, scaled_mobility_1,
                                           scaled_mobility_2, delta_t, transient_or_steady, penalty,
                                           data.local_matrix_1.data(), data.local_matrix_2.data()));
  }
  // LDG.cpp:429-622, for the face `face` of the cell the data's
  // local_dof_indices belong to, with the neighbour across it
  void assemble_local_flux_terms(const CellIterator& cell, int face, const CellIterator& neighbor,
                                 Assembly::AssemblyScratch& scratch, Assembly::DriftDiffusion::CopyData& data,
                                 const double& penalty) {
    data.local_dof_indices = cell.dof_indices;
    data.local_neighbor_dof_indices = neighbor.dof_indices;
    check(pecs_ldg_local_flux_terms(scratch.degree, &cell.geometry, face, &neighbor.geometry, penalty,
                                    data.vi_ui_matrix.data(), data.vi_ue_matrix.data(),
                                    data.ve_ui_matrix.data(), data.ve_ue_matrix.data()));
  }
  // LDG.cpp:624-678: the four blocks into both carriers' matrices
  void distribute_local_fluxes_to_global(ChargeCarrierSpace::CarrierPair& carrier_pair,
                                         Assembly::DriftDiffusion::CopyData& data) {
    for (ChargeCarrierSpace::Carrier* c : {&carrier_pair.carrier_1, &carrier_pair.carrier_2}) {
      add_local(c->system_matrix, data.local_dof_indices, data.local_dof_indices, data.vi_ui_matrix);
      add_local(c->system_matrix, data.local_dof_indices, data.local_neighbor_dof_indices, data.vi_ue_matrix);
      add_local(c->system_matrix, data.local_neighbor_dof_indices, data.local_dof_indices, data.ve_ui_matrix);
      add_local(c->system_matrix, data.local_neighbor_dof_indices, data.local_neighbor_dof_indices,
                data.ve_ue_matrix);
    }
  }
  // LDG.cpp:283-426: every interior face once, from its lower-numbered cell
  void assemble_flux_terms(const std::vector<CellIterator>& cells, ChargeCarrierSpace::CarrierPair& carrier_pair,
                           Assembly::AssemblyScratch& scratch) {
    Assembly::DriftDiffusion::CopyData data(scratch);
    for (int K = 0; K < (int)cells.size(); ++K)
      for (int f = 0; f < 4; ++f) {
        const int nb = cells[K].neighbor[f];
        if (nb <= K) continue;
        assemble_local_flux_terms(cells[K], f, cells[nb], scratch, data, carrier_pair.penalty);
        distribute_local_fluxes_to_global(carrier_pair, data);
      }
  }
};

}  // namespace LDG_System

// ---- mixed Poisson assembly (include/MixedFEM.hpp:165-172) ---------------------
namespace MixedPoisson {

struct MixedFEM {
  void assemble_local_Poisson_matrix(const CellIterator& cell, Assembly::AssemblyScratch& scratch,
                                     Assembly::Poisson::CopyData& data, const double& semi_permittivity,
                                     const double& elec_permittivity, const double& scaled_debye_length) {
    data.local_dof_indices = cell.dof_indices;
    check(pecs_mixed_local_poisson_matrix(scratch.degree, scratch.poisson_pairing, &cell.geometry,
                                          semi_permittivity, elec_permittivity, scaled_debye_length,
                                          data.local_matrix.data()));
  }
};

}  // namespace MixedPoisson

}  // namespace pecs_dropin
