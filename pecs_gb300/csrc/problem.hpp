// Host-side setup of a PECS half-cell problem: meshes, DoF maps, the fixed
// LDG and mixed-Poisson matrices, and the time-independent parts of the
// right-hand sides.  This is the work deal.II does once before the IMEX loop
// (SolarCellProblem::setup_dofs, setup_mappings, assemble_Poisson_matrix,
// assemble_LDG_system; source/SolarCell.cpp:105-121, 156-932).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pecs.h"
#include "fe.hpp"

namespace pecs {

struct Csr {
  int n = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
  long long nnz() const { return (long long)col.size(); }
};

// COO -> CSR with sorted columns and summed duplicates; exact zeros are dropped.
Csr coo_to_csr(int n, const std::vector<int>& r, const std::vector<int>& c,
               const std::vector<double>& v);

// Rectilinear structured grid; cells numbered i + nx*j.
struct Grid {
  int nx = 0, ny = 0;
  std::vector<double> xs, ys;
  int bc[4] = {0, 0, 0, 0};
  // cells with i >= split take bc2's id (where > 0) on their outer faces: the
  // Poisson mesh over the electrolyte; split < 0: one id per side
  int split = -1;
  int bc2[4] = {0, 0, 0, 0};
  std::vector<int> material;  // 0 semiconductor, 2 electrolyte
  int nc() const { return nx * ny; }
  int face_bid(int K, int f) const;  // -1 for interior faces
  void geom(int K, double& x0, double& y0, double& hx, double& hy) const;
};

struct CarrierSystem {
  Grid grid;
  int ndofs = 0;
  Csr A[2];   // carrier_1, carrier_2 system matrices
  Csr M;      // (1/dt) mass matrix
  std::vector<int> dof_cell, dof_class;
  std::vector<double> cell_xy;
};

struct PoissonSystem {
  Grid grid;
  int ndofs = 0, n_rt_total = 0;
  std::vector<int> l2g;  // nc * (n_rt + n_phi)
  std::vector<char> constrained;
  Csr A;
  std::vector<int> dof_cell;
  std::vector<double> cell_xy;
};

// Everything the device needs, built once on the host.
struct Setup {
  std::vector<pecs_params> inst;  // per instance
  int k = 1, n1 = 4, n_rt = 4, n_phi = 1, Q = 9, nq1 = 3;
  bool full = true;
  CarrierTables ct;
  PoissonTables pt;
  CarrierSystem semi, elec;
  PoissonSystem pois;
  std::vector<int> s2p, e2p;               // carrier cell -> Poisson cell
  std::vector<int> iface_semi, iface_elec; // paired interface cells (semi right face, elec left face)
  // time-independent right-hand-side parts, [inst][ndofs] per field
  std::vector<std::vector<double>> bconst[5];
  // interface equilibria n_e, p_e at the semi face qp: [inst][iface*nq1 + q]
  std::vector<std::vector<double>> iface_ne, iface_pe;
  // Schottky equilibria at semi boundary face qp: [inst][(K*4+f)*nq1+q] (only if used)
  bool has_schottky = false;
  std::vector<std::vector<double>> schottky_ne, schottky_pe;
  // initial state per instance (projected profiles), [inst][field][ndofs]
  std::vector<std::vector<double>> init[4];

  explicit Setup(const std::vector<pecs_params>& p);
  void compute_instances(const std::vector<pecs_params>& p);
  // recompute the per-instance data of instance s from inst[s] (its cell
  // loops split over `threads` host threads)
  void compute_instance(int s, int threads = 1);
  // the per-instance data of one parameter set, computed apart from the
  // slots (reads only the shared setup: safe beside other threads' calls),
  // and its move into slot s
  struct InstanceData {
    std::vector<double> bconst[5], init[4], iface_ne, iface_pe, schottky_ne, schottky_pe;
  };
  void compute_instance_data(const pecs_params& p, InstanceData& d, int threads = 1) const;
  void store_instance(int s, InstanceData&& d);
  // the same for several instances, on the host threads
  void compute_instances_at(const std::vector<int>& slots);
};

// Validates a parameter set; returns an empty string when it is usable.
std::string validate_params(const pecs_params* p, int n_inst);

}  // namespace pecs
