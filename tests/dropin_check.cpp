// Drives the C++ drop-in classes (include/pecs_dropin.hpp) the way the
// reference's SolarCellProblem drives its own: the LDG and mixed matrices are
// assembled cell by cell through LDG_System::LDG and MixedPoisson::MixedFEM
// into CSR patterns (SolarCell.cpp:377-417, 822-932), then the carrier and
// Poisson solvers are set up and applied through Carrier::set_solver/solve and
// PoissonData::set_solver/solve (SolarCell.cpp:1733-1756).
//
//   dropin_check assemble <degree> <pairing>
//       CPU: the assembled matrices must equal the library's own setup
//       (pecs_get_matrix of a host-only context) to 1e-14; prints "assemble ok".
//   dropin_check solve <degree> <pairing> <outdir>
//       GPU: solves the electron and Poisson systems for fixed right-hand sides
//       and writes b, x (raw doubles) and the CSR matrices for the caller's check.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <string>
#include <vector>

#include "pecs_dropin.hpp"

using namespace pecs_dropin;

static pecs_params half_cell(int degree, int pairing) {
  pecs_params p{};
  p.degree = degree;
  p.full_system = 1;
  p.nx_semi = 4;
  p.nx_elec = 4;
  p.ny = 4;
  p.x_semi0 = 0.0;
  p.x_semi1 = 1.0;
  p.x_elec1 = 2.0;
  p.height = 1.0;
  const int bs[4] = {PECS_DIRICHLET, PECS_INTERFACE, PECS_NEUMANN, PECS_NEUMANN};
  const int be[4] = {PECS_INTERFACE, PECS_DIRICHLET, PECS_NEUMANN, PECS_NEUMANN};
  const int bp[4] = {PECS_DIRICHLET, PECS_DIRICHLET, PECS_NEUMANN, PECS_NEUMANN};
  for (int f = 0; f < 4; ++f) {
    p.bc_semi[f] = bs[f];
    p.bc_elec[f] = be[f];
    p.bc_poisson[f] = bp[f];
  }
  p.lambda2 = 1e-2;
  p.eps_semi = 1.0;
  p.eps_elec = 1.5;
  const double mu[4] = {1.0, 0.5, 2.0, 1.0};
  for (int c = 0; c < 4; ++c) p.mu[c] = mu[c];
  p.dt = 1e-3;
  p.penalty = 1.0;
  p.k_et = p.k_ht = 1e-2;
  p.junction_x = 0.5;
  p.nd[0] = p.nd[1] = 1.0;
  p.n_eq[0] = p.n_eq[1] = 1.0;
  p.p_eq[0] = p.p_eq[1] = 1e-4;
  p.r_eq = p.o_eq = 1.0;
  p.gen_kind = 2;
  p.G0 = 1.0;
  p.alpha = 5.0;
  p.srh = 1;
  p.tau_n = p.tau_p = 1.0;
  p.n_i = 1e-2;
  p.grading = 3.0;  // graded cells: every cell size differs along x
  p.poisson_pairing = pairing;
  return p;
}

static SparseMatrix library_matrix(pecs_ctx* ctx, int which) {
  SparseMatrix A;
  long long nnz = 0;
  check(pecs_get_matrix(ctx, which, &A.n, &nnz, nullptr, nullptr, nullptr));
  A.rowptr.resize(A.n + 1);
  A.col.resize(nnz);
  A.val.resize(nnz);
  check(pecs_get_matrix(ctx, which, nullptr, nullptr, A.rowptr.data(), A.col.data(), A.val.data()));
  return A;
}

// cells of one mesh with their geometry, face ids and neighbours; ids of the
// outer faces come from bc (left, right, bottom, top) and, past column split,
// from bc2 where bc2 > 0 (the Poisson mesh over the electrolyte)
static std::vector<CellIterator> mesh_cells(pecs_ctx* ctx, int mesh, const int* bc, const int* bc2, int split,
                                            int material_left, int material_right) {
  int nx = 0, ny = 0;
  check(pecs_get_mesh(ctx, mesh, &nx, &ny, nullptr, nullptr));
  std::vector<double> xs(nx + 1), ys(ny + 1);
  check(pecs_get_mesh(ctx, mesh, nullptr, nullptr, xs.data(), ys.data()));
  std::vector<CellIterator> cells(nx * ny);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      CellIterator& c = cells[i + nx * j];
      c.geometry.hx = xs[i + 1] - xs[i];
      c.geometry.hy = ys[j + 1] - ys[j];
      const bool right_part = split > 0 && i >= split;
      c.geometry.material_id = right_part ? material_right : material_left;
      auto outer = [&](int f) { return (right_part && bc2 && bc2[f] > 0) ? bc2[f] : bc[f]; };
      c.geometry.boundary_id[0] = i == 0 ? outer(0) : -1;
      c.geometry.boundary_id[1] = i == nx - 1 ? outer(1) : -1;
      c.geometry.boundary_id[2] = j == 0 ? outer(2) : -1;
      c.geometry.boundary_id[3] = j == ny - 1 ? outer(3) : -1;
      c.neighbor[0] = i > 0 ? i - 1 + nx * j : -1;
      c.neighbor[1] = i < nx - 1 ? i + 1 + nx * j : -1;
      c.neighbor[2] = j > 0 ? i + nx * (j - 1) : -1;
      c.neighbor[3] = j < ny - 1 ? i + nx * (j + 1) : -1;
    }
  return cells;
}

static void carrier_dofs(std::vector<CellIterator>& cells, int n1) {
  const int nc = (int)cells.size();
  for (int K = 0; K < nc; ++K) {
    cells[K].dof_indices.resize(3 * n1);
    for (int comp = 0; comp < 3; ++comp)
      for (int a = 0; a < n1; ++a) cells[K].dof_indices[comp * n1 + a] = comp * nc * n1 + K * n1 + a;
  }
}

// the library's Poisson numbering: [vertical faces | horizontal faces | interior RT | Phi]
static std::vector<char> poisson_dofs(std::vector<CellIterator>& cells, int nx, int ny, int kp, int nphi) {
  const int nc = nx * ny, nint = 2 * kp * (kp - 1), nxd = kp * (kp + 1);
  const int off_h = (nx + 1) * ny * kp, off_i = off_h + nx * (ny + 1) * kp, off_phi = off_i + nc * nint;
  std::vector<char> constrained(off_phi + nc * nphi, 0);
  for (int K = 0; K < nc; ++K) {
    const int i = K % nx, j = K / nx;
    std::vector<int>& d = cells[K].dof_indices;
    d.assign(2 * nxd + nphi, 0);
    int cnt = 0;
    for (int b = 0; b < kp; ++b)
      for (int a = 0; a <= kp; ++a)
        d[a + (kp + 1) * b] = a == 0 ? (i + (nx + 1) * j) * kp + b
                              : a == kp ? (i + 1 + (nx + 1) * j) * kp + b
                                        : off_i + K * nint + cnt++;
    for (int b = 0; b <= kp; ++b)
      for (int a = 0; a < kp; ++a)
        d[nxd + a + kp * b] = b == 0 ? off_h + (i + nx * j) * kp + a
                              : b == kp ? off_h + (i + nx * (j + 1)) * kp + a
                                        : off_i + K * nint + cnt++;
    for (int a = 0; a < nphi; ++a) d[2 * nxd + a] = off_phi + K * nphi + a;
    // zero D.n on Neumann faces (Poisson.cpp:32-49)
    const pecs_cell& g = cells[K].geometry;
    for (int b = 0; b < kp; ++b) {
      if (g.boundary_id[0] == PECS_NEUMANN) constrained[d[0 + (kp + 1) * b]] = 1;
      if (g.boundary_id[1] == PECS_NEUMANN) constrained[d[kp + (kp + 1) * b]] = 1;
    }
    for (int a = 0; a < kp; ++a) {
      if (g.boundary_id[2] == PECS_NEUMANN) constrained[d[nxd + a]] = 1;
      if (g.boundary_id[3] == PECS_NEUMANN) constrained[d[nxd + a + kp * kp]] = 1;
    }
  }
  return constrained;
}

static double rel_diff(const SparseMatrix& A, const SparseMatrix& B) {
  if (A.n != B.n || A.col != B.col) return 1e300;
  double num = 0.0, den = 0.0;
  for (size_t p = 0; p < A.val.size(); ++p) {
    num = std::max(num, std::fabs(A.val[p] - B.val[p]));
    den = std::max(den, std::fabs(B.val[p]));
  }
  return num / den;
}

template <typename T>
static void write(const std::string& path, const std::vector<T>& v) {
  std::ofstream o(path, std::ios::binary);
  o.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

static void write_csr(const std::string& stem, const SparseMatrix& A) {
  write(stem + "_rowptr.bin", A.rowptr);
  write(stem + "_col.bin", A.col);
  write(stem + "_val.bin", A.val);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: dropin_check assemble|solve <degree> <pairing> [outdir]\n");
    return 2;
  }
  const std::string mode = argv[1];
  const int degree = std::atoi(argv[2]), pairing = std::atoi(argv[3]);
  try {
    pecs_params P = half_cell(degree, pairing);
    pecs_options o;
    pecs_default_options(&o);
    o.host_setup_only = 1;
    pecs_ctx* ctx = nullptr;
    check(pecs_create(&P, 1, &o, &ctx));
    const int n1 = (degree + 1) * (degree + 1);
    Assembly::AssemblyScratch scratch(degree, pairing);
    // ---- semiconductor carrier pair: cell, boundary and flux terms
    std::vector<CellIterator> semi = mesh_cells(ctx, PECS_MESH_SEMI, P.bc_semi, nullptr, 0, 0, 0);
    carrier_dofs(semi, n1);
    ChargeCarrierSpace::CarrierPair pair;
    pair.penalty = P.penalty;
    pair.delta_t = P.dt;
    pair.carrier_1.system_matrix = library_matrix(ctx, PECS_MAT_N);
    pair.carrier_2.system_matrix = library_matrix(ctx, PECS_MAT_P);
    pair.mass_matrix = library_matrix(ctx, PECS_MAT_MASS_SEMI);
    const SparseMatrix An = pair.carrier_1.system_matrix, Ap = pair.carrier_2.system_matrix,
                       M = pair.mass_matrix;
    pair.carrier_1.system_matrix.set_zero();
    pair.carrier_2.system_matrix.set_zero();
    pair.mass_matrix.set_zero();
    LDG_System::LDG ldg;
    Assembly::DriftDiffusion::CopyData dd(scratch);
    for (const CellIterator& c : semi) {
      ldg.assemble_local_LDG_mass_matrix(c, scratch, dd, pair.delta_t);
      LDG_System::add_local(pair.mass_matrix, dd.local_dof_indices, dd.local_dof_indices, dd.local_mass_matrix);
      ldg.assemble_local_LDG_cell_and_bc_terms(c, scratch, dd, P.mu[0], P.mu[1], P.dt, 1.0, pair.penalty);
      LDG_System::add_local(pair.carrier_1.system_matrix, dd.local_dof_indices, dd.local_dof_indices,
                            dd.local_matrix_1);
      LDG_System::add_local(pair.carrier_2.system_matrix, dd.local_dof_indices, dd.local_dof_indices,
                            dd.local_matrix_2);
    }
    ldg.assemble_flux_terms(semi, pair, scratch);
    // ---- Poisson: mixed matrix, constrained rows and columns condensed
    int pnx = 0, pny = 0;
    check(pecs_get_mesh(ctx, PECS_MESH_POISSON, &pnx, &pny, nullptr, nullptr));
    std::vector<CellIterator> pc = mesh_cells(ctx, PECS_MESH_POISSON, P.bc_poisson, P.bc_poisson_elec,
                                              P.nx_semi, 0, 2);
    const std::vector<char> constrained = poisson_dofs(pc, pnx, pny, scratch.degree + pairing,
                                                       scratch.poisson_phi_dofs);
    Poisson::PoissonData pois;
    pois.system_matrix = library_matrix(ctx, PECS_MAT_POISSON);
    const SparseMatrix AP = pois.system_matrix;
    pois.system_matrix.set_zero();
    MixedPoisson::MixedFEM mixed;
    Assembly::Poisson::CopyData pd(scratch);
    for (const CellIterator& c : pc) {
      mixed.assemble_local_Poisson_matrix(c, scratch, pd, P.eps_semi, P.eps_elec, P.lambda2);
      const int nl = pd.local_matrix.m;
      for (int a = 0; a < nl; ++a)
        for (int b = 0; b < nl; ++b) {
          const int ga = pd.local_dof_indices[a], gb = pd.local_dof_indices[b];
          // the library's pattern holds the non-zero couplings only
          if (constrained[ga] || constrained[gb] || pd.local_matrix(a, b) == 0.0) continue;
          pois.system_matrix.add(ga, gb, pd.local_matrix(a, b));
        }
    }
    for (int d = 0; d < (int)constrained.size(); ++d)
      if (constrained[d]) {
        pois.system_matrix.add(d, d, 1.0);
        pois.constrained_dofs.push_back(d);
      }
    const double eN = rel_diff(pair.carrier_1.system_matrix, An), eP = rel_diff(pair.carrier_2.system_matrix, Ap),
                 eM = rel_diff(pair.mass_matrix, M), ePo = rel_diff(pois.system_matrix, AP);
    std::printf("electrons %.3e holes %.3e mass %.3e poisson %.3e\n", eN, eP, eM, ePo);
    if (!(eN < 1e-14 && eP < 1e-14 && eM < 1e-14 && ePo < 1e-14)) {
      std::fprintf(stderr, "assembled matrices differ from the library's\n");
      return 1;
    }
    if (mode == "assemble") {
      std::printf("assemble ok\n");
      pecs_destroy(ctx);
      return 0;
    }
    // ---- solves on the GPU through set_solver / solve
    const std::string out = argc > 4 ? argv[4] : ".";
    ChargeCarrierSpace::Carrier& el = pair.carrier_1;
    const int nc = (int)semi.size();
    el.dof_map.dof_class.assign(3 * nc * n1, 1);
    el.dof_map.dof_cell.resize(3 * nc * n1);
    for (int K = 0; K < nc; ++K)
      for (int comp = 0; comp < 3; ++comp)
        for (int a = 0; a < n1; ++a) {
          el.dof_map.dof_cell[comp * nc * n1 + K * n1 + a] = K;
          el.dof_map.dof_class[comp * nc * n1 + K * n1 + a] = comp < 2 ? 0 : 1;
        }
    el.dof_map.cell_xy.resize(2 * nc);
    {
      int nx = 0, ny = 0;
      check(pecs_get_mesh(ctx, PECS_MESH_SEMI, &nx, &ny, nullptr, nullptr));
      std::vector<double> xs(nx + 1), ys(ny + 1);
      check(pecs_get_mesh(ctx, PECS_MESH_SEMI, nullptr, nullptr, xs.data(), ys.data()));
      for (int K = 0; K < nc; ++K) {
        el.dof_map.cell_xy[2 * K] = 0.5 * (xs[K % nx] + xs[K % nx + 1]);
        el.dof_map.cell_xy[2 * K + 1] = 0.5 * (ys[K / nx] + ys[K / nx + 1]);
      }
    }
    std::mt19937_64 rng(17);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    el.system_rhs.resize(el.system_matrix.n);
    for (double& v : el.system_rhs) v = U(rng);
    el.set_solver();
    el.solve();
    // Poisson: dofs owned by the cell of their first appearance
    const int npc = (int)pc.size();
    pois.dof_map.dof_cell.assign(pois.system_matrix.n, -1);
    pois.dof_map.cell_xy.resize(2 * npc);
    {
      std::vector<double> xs(pnx + 1), ys(pny + 1);
      check(pecs_get_mesh(ctx, PECS_MESH_POISSON, nullptr, nullptr, xs.data(), ys.data()));
      for (int K = 0; K < npc; ++K) {
        pois.dof_map.cell_xy[2 * K] = 0.5 * (xs[K % pnx] + xs[K % pnx + 1]);
        pois.dof_map.cell_xy[2 * K + 1] = 0.5 * (ys[K / pnx] + ys[K / pnx + 1]);
        for (int d : pc[K].dof_indices)
          if (pois.dof_map.dof_cell[d] < 0) pois.dof_map.dof_cell[d] = K;
      }
    }
    pois.system_rhs.resize(pois.system_matrix.n);
    for (int d = 0; d < pois.system_matrix.n; ++d) pois.system_rhs[d] = constrained[d] ? 0.0 : U(rng);
    pois.set_solver();
    pois.solve();
    write_csr(out + "/carrier_A", el.system_matrix);
    write_csr(out + "/poisson_A", pois.system_matrix);
    write(out + "/carrier_b.bin", el.system_rhs);
    write(out + "/carrier_x.bin", el.solution);
    write(out + "/poisson_b.bin", pois.system_rhs);
    write(out + "/poisson_x.bin", pois.solution);
    std::printf("solve ok\n");
    pecs_destroy(ctx);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
