// pecs_dropin.hpp -- C++ drop-in classes with the reference's names over the
// pecs C ABI (pecs.h).  Header-only; link against libpecs_gb300.so.
//
// They mirror, member by member, the containers the reference's IMEX loop
// uses (paths relative to the reference project):
//   ChargeCarrierSpace::Carrier      include/Carrier.hpp:38-101, source/Carrier.cpp
//   ChargeCarrierSpace::CarrierPair  include/CarrierPair.hpp:30-110, source/CarrierPair.cpp
//   Poisson::PoissonData             include/Poisson.hpp:26-84, source/Poisson.cpp
// with deal.II types replaced by plain containers: the system matrix is a CSR
// triple, vectors are std::vector<double>.  set_solver() factorises once
// (UMFPACK's initialize), solve() applies the factors on the GPU (UMFPACK's
// vmult).  Errors throw std::runtime_error, which the reference's main()
// already catches as std::exception (source/main/main.cpp:28-39).
#pragma once
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
  }
  void vmult(std::vector<double>& x, const std::vector<double>& b) const {
    if (!lu_) throw std::runtime_error("pecs: solver not initialised");
    if ((int)b.size() != n_) throw std::runtime_error("pecs: rhs size mismatch");
    x.resize(n_);
    check(pecs_lu_solve(lu_, 1, b.data(), x.data()));
  }

 private:
  pecs_lu* lu_ = nullptr;
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

}  // namespace pecs_dropin
