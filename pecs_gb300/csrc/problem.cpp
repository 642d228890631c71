// Host-side setup of the PECS problem (see problem.hpp).
#include "problem.hpp"

#include "dense.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <sstream>
#include <thread>
#include <stdexcept>
#include <tuple>

namespace pecs {

Csr coo_to_csr(int n, const std::vector<int>& r, const std::vector<int>& c,
               const std::vector<double>& v) {
  Csr A;
  A.n = n;
  std::vector<int> cnt(n + 1, 0);
  for (int x : r) cnt[x + 1]++;
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> pos(cnt.begin(), cnt.end() - 1);
  std::vector<int> cc(r.size());
  std::vector<double> vv(r.size());
  for (size_t t = 0; t < r.size(); ++t) {
    int p = pos[r[t]]++;
    cc[p] = c[t];
    vv[p] = v[t];
  }
  A.rowptr.assign(n + 1, 0);
  std::vector<std::pair<int, double>> row;
  for (int i = 0; i < n; ++i) {
    row.clear();
    for (int p = cnt[i]; p < cnt[i + 1]; ++p) row.emplace_back(cc[p], vv[p]);
    std::stable_sort(row.begin(), row.end(),
                     [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
                       return a.first < b.first;
                     });
    for (size_t t = 0; t < row.size();) {
      int col = row[t].first;
      double s = 0.0;
      while (t < row.size() && row[t].first == col) s += row[t++].second;
      if (s == 0.0) continue;  // structural zeros of the flux pattern are not stored
      A.col.push_back(col);
      A.val.push_back(s);
    }
    A.rowptr[i + 1] = (int)A.col.size();
  }
  return A;
}

int Grid::face_bid(int K, int f) const {
  int i = K % nx, j = K / nx;
  const bool outer = (f == kLeft && i == 0) || (f == kRight && i == nx - 1) ||
                     (f == kBottom && j == 0) || (f == kTop && j == ny - 1);
  if (!outer) return -1;
  if (split >= 0 && i >= split && bc2[f] > 0) return bc2[f];
  return bc[f];
}

void Grid::geom(int K, double& x0, double& y0, double& hx, double& hy) const {
  int i = K % nx, j = K / nx;
  x0 = xs[i];
  y0 = ys[j];
  hx = xs[i + 1] - xs[i];
  hy = ys[j + 1] - ys[j];
}

// Cell boundaries along one axis.  grading <= 1: uniform, with the arithmetic
// of numpy.linspace (x0 + i*step, last point exact).  grading > 1: widths
// shrinking by q = grading^(1/(n-1)) per cell toward x1 (fine_at_x1) or toward
// x0, so widest / narrowest = grading; normalised prefix sums of the widths.
static std::vector<double> axis_coords(double x0, double x1, int n, double grading,
                                       bool fine_at_x1) {
  std::vector<double> xs(n + 1);
  if (!(grading > 1.0)) {
    const double sx = (x1 - x0) / n;
    for (int i = 0; i <= n; ++i) xs[i] = x0 + i * sx;
  } else {
    const double q = std::pow(grading, 1.0 / (n - 1));
    std::vector<double> w(n);
    w[0] = 1.0;
    for (int i = 1; i < n; ++i) w[i] = w[i - 1] / q;
    if (!fine_at_x1) std::reverse(w.begin(), w.end());
    std::vector<double> S(n + 1, 0.0);
    for (int i = 0; i < n; ++i) S[i + 1] = S[i] + w[i];
    for (int i = 0; i <= n; ++i) xs[i] = x0 + (x1 - x0) * (S[i] / S[n]);
  }
  xs[n] = x1;
  return xs;
}

// One carrier region: graded along x toward the interface, uniform along y.
static Grid region(double x0, double x1, double y0, double y1, int nx, int ny, const int* bc,
                   int material, double grading, bool fine_at_x1) {
  Grid g;
  g.nx = nx;
  g.ny = ny;
  g.xs = axis_coords(x0, x1, nx, grading, fine_at_x1);
  g.ys = axis_coords(y0, y1, ny, 1.0, false);
  for (int f = 0; f < 4; ++f) g.bc[f] = bc[f];
  g.material.assign(g.nc(), material);
  return g;
}

// ---------------------------------------------------------------------------
// Coefficient functions (reference: source/InitialConditions.cpp,
// Generation.cpp:29-44, BiasValues.cpp:11-31,75-94, SolarCell.hpp:86-98)
// ---------------------------------------------------------------------------
static inline double pw(double x, const double v[2], double xj) { return x < xj ? v[0] : v[1]; }

static double generation(const pecs_params& P, double x, double y) {
  if (P.gen_kind == 0) return 0.0;
  if (P.gen_kind == 1) return P.alpha * P.G0 * std::exp(P.alpha * (y - P.height));
  return P.G0 * std::exp(-P.alpha * (P.x_semi1 - x));
}

static double potential_dirichlet(const pecs_params& P, double x, double /*y*/) {
  return x == 0.0 ? (P.phi_bi - P.phi_app) : 0.0;
}

static double carrier_bc(const pecs_params& P, int field, double x, double /*y*/) {
  switch (field) {
    case 0: return pw(x, P.n_eq, P.junction_x);
    case 1: return pw(x, P.p_eq, P.junction_x);
    case 2: return P.r_eq;
    default: return P.o_eq;
  }
}

static double initial_profile(const pecs_params& P, int field, double x, double y) {
  if (P.ic_kind == 1 && field == 0) return pw(x, P.nd, P.junction_x);
  if (P.ic_kind == 1 && field == 1) return pw(x, P.na, P.junction_x);
  return carrier_bc(P, field, x, y);
}

// ---------------------------------------------------------------------------
// Local matrices
// ---------------------------------------------------------------------------
namespace {

struct DofVals {  // values of one carrier local dof at points
  const double *px, *py, *v;
};

// Carrier local dof i in [0, 3 n1): component and node.
inline void carrier_comp(int i, int n1, int& comp, int& a) {
  comp = i / n1;
  a = i % n1;
}

// assemble_local_LDG_cell_and_bc_terms (source/LDG.cpp:85-281) on an
// axis-aligned hx*hy cell.
std::vector<double> ldg_cell_matrix(const CarrierTables& ct, double hx, double hy, double mu,
                                    double dt, double tos, double pen_h, const int bids[4]) {
  const int n1 = ct.n1, nd = 3 * n1, Q = ct.Q, nq = ct.nq1;
  std::vector<double> A(nd * nd, 0.0);
  for (int i = 0; i < nd; ++i) {
    int ci, a;
    carrier_comp(i, n1, ci, a);
    for (int j = 0; j < nd; ++j) {
      int cj, b;
      carrier_comp(j, n1, cj, b);
      double s = 0.0;
      for (int q = 0; q < Q; ++q) {
        double JxW = ct.qw[q] * hx * hy;
        double phia = ct.phi[a * Q + q], phib = ct.phi[b * Q + q];
        double dxa = ct.dphi_x[a * Q + q] / hx, dya = ct.dphi_y[a * Q + q] / hy;
        double t = 0.0;
        // (tos/dt) v u
        if (ci == 2 && cj == 2) t += (tos / dt) * phia * phib;
        // (1/mu) p . q
        if (ci == cj && ci < 2) t += (1.0 / mu) * phia * phib;
        // - div(p) u
        if (cj == 2) {
          if (ci == 0) t -= dxa * phib;
          if (ci == 1) t -= dya * phib;
        }
        // - grad(v) . q
        if (ci == 2) {
          if (cj == 0) t -= dxa * phib;
          if (cj == 1) t -= dya * phib;
        }
        s += t * JxW;
      }
      A[i * nd + j] = s;
    }
  }
  for (int f = 0; f < 4; ++f) {
    int bid = bids[f];
    if (bid < 0) continue;
    double flen = (f == kLeft || f == kRight) ? hy : hx;
    const double nx_ = kFaceNormal[f][0], ny_ = kFaceNormal[f][1];
    for (int i = 0; i < nd; ++i) {
      int ci, a;
      carrier_comp(i, n1, ci, a);
      for (int j = 0; j < nd; ++j) {
        int cj, b;
        carrier_comp(j, n1, cj, b);
        double s = 0.0;
        for (int q = 0; q < nq; ++q) {
          double Jf = ct.fw[q] * flen;
          double fa = ct.fphi[(f * n1 + a) * nq + q], fb = ct.fphi[(f * n1 + b) * nq + q];
          if (bid == kDirichlet) {
            // v (n.q + pen/h u)
            if (ci != 2) continue;
            double nq_ = (cj == 0 ? nx_ * fb : 0.0) + (cj == 1 ? ny_ * fb : 0.0);
            double uj = (cj == 2) ? fb : 0.0;
            s += fa * (nq_ + pen_h * uj) * Jf;
          } else {
            // (p.n) u
            if (cj != 2) continue;
            double pn = (ci == 0 ? nx_ * fa : 0.0) + (ci == 1 ? ny_ * fa : 0.0);
            s += pn * fb * Jf;
          }
        }
        A[i * nd + j] += s;
      }
    }
  }
  return A;
}

// assemble_local_flux_terms (source/LDG.cpp:429-622); minus = left/bottom cell.
void ldg_flux_blocks(const CarrierTables& ct, int fminus, int fplus, double flen, double pen_h,
                     std::vector<double> blk[4]) {
  const int n1 = ct.n1, nd = 3 * n1, nq = ct.nq1;
  const double nx_ = kFaceNormal[fminus][0], ny_ = kFaceNormal[fminus][1];
  const double beta = 1.0 / std::sqrt(2.0);  // beta = (1,1)/|(1,1)|
  // per side, per dof: p.n, v, beta.p at face qp
  auto vals = [&](int f, int i, int q, double& pn, double& v, double& bp) {
    int c, a;
    carrier_comp(i, n1, c, a);
    double ph = ct.fphi[(f * n1 + a) * nq + q];
    double px = c == 0 ? ph : 0.0, py = c == 1 ? ph : 0.0;
    pn = px * nx_ + py * ny_;
    v = c == 2 ? ph : 0.0;
    bp = beta * px + beta * py;
  };
  const int sides[4][2] = {{fminus, fminus}, {fminus, fplus}, {fplus, fminus}, {fplus, fplus}};
  const double sh[4] = {+1, +1, -1, -1}, sb[4] = {+1, -1, -1, +1}, sp[4] = {+1, -1, -1, +1};
  for (int t = 0; t < 4; ++t) {
    blk[t].assign(nd * nd, 0.0);
    int ft = sides[t][0], fr = sides[t][1];
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) {
        double s = 0.0;
        for (int q = 0; q < nq; ++q) {
          double tpn, tv, tbp, rpn, rv, rbp;
          vals(ft, i, q, tpn, tv, tbp);
          vals(fr, j, q, rpn, rv, rbp);
          double Jf = ct.fw[q] * flen;
          double e = 0.5 * sh[t] * (tpn * rv + tv * rpn) + sb[t] * (tbp * rv - tv * rbp) +
                     sp[t] * pen_h * tv * rv;
          s += e * Jf;
        }
        blk[t][i * nd + j] = s;
      }
  }
}

// MixedFEM::assemble_local_Poisson_matrix (source/MixedFEM.cpp:29-164).
std::vector<double> poisson_cell_matrix(const PoissonTables& pt, const CarrierTables& ct, double hx,
                                        double hy, double eps, double lambda2) {
  const int nr = pt.n_rt, np = pt.n_phi, nd = nr + np, Q = ct.Q;
  std::vector<double> A(nd * nd, 0.0);
  for (int i = 0; i < nd; ++i)
    for (int j = 0; j < nd; ++j) {
      double s = 0.0;
      for (int q = 0; q < Q; ++q) {
        double JxW = ct.qw[q] * hx * hy;
        double t = 0.0;
        if (i < nr && j < nr)
          t = (1.0 / eps) * (pt.psi_x[i * Q + q] * pt.psi_x[j * Q + q] +
                             pt.psi_y[i * Q + q] * pt.psi_y[j * Q + q]);
        else if (i < nr && j >= nr)
          t = -(pt.div_x[i * Q + q] / hx + pt.div_y[i * Q + q] / hy) * pt.phi[(j - nr) * Q + q];
        else if (i >= nr && j < nr)
          t = -lambda2 * pt.phi[(i - nr) * Q + q] *
              (pt.div_x[j * Q + q] / hx + pt.div_y[j * Q + q] / hy);
        s += t * JxW;
      }
      A[i * nd + j] = s;
    }
  return A;
}

}  // namespace

// ---------------------------------------------------------------------------
std::string validate_params(const pecs_params* p, int n_inst) {
  std::ostringstream e;
  if (!p) return "params is NULL";
  if (n_inst < 1) return "n_inst must be >= 1";
  const pecs_params& a = p[0];
  if (a.degree < 1 || a.degree > 2) e << "degree must be 1 or 2; ";
  if (a.poisson_pairing != 0 && a.poisson_pairing != 1) e << "poisson_pairing must be 0 or 1; ";
  if (a.nx_semi < 2 || a.ny < 2 || (a.full_system && a.nx_elec < 2)) e << "mesh too small; ";
  if (a.nx_semi > 4096 || a.ny > 4096 || a.nx_elec > 4096) e << "mesh too large; ";
  if (!(a.dt > 0) || !(a.lambda2 > 0) || !(a.eps_semi > 0) || (a.full_system && !(a.eps_elec > 0)))
    e << "dt, lambda2 and permittivities must be > 0; ";
  for (int c = 0; c < 4; ++c)
    if (!(a.mu[c] > 0)) e << "mobilities must be > 0; ";
  if (!(a.x_semi1 > a.x_semi0) || !(a.height > 0) || (a.full_system && !(a.x_elec1 > a.x_semi1)))
    e << "bad geometry; ";
  if (!(a.grading >= 0.0 && a.grading <= 1e4)) e << "grading must be in [0, 1e4]; ";
  for (int f = 0; f < 4; ++f) {
    if (a.bc_semi[f] < 0 || a.bc_semi[f] > 3 || a.bc_elec[f] < 0 || a.bc_elec[f] > 3 ||
        a.bc_poisson[f] < 0 || a.bc_poisson[f] > 3 || a.bc_poisson_elec[f] < -1 ||
        a.bc_poisson_elec[f] > 3)
      e << "bad boundary id; ";
  }
  for (int i = 1; i < n_inst; ++i) {
    const pecs_params& b = p[i];
    std::string diff;
    auto chk = [&](bool eq, const char* name) {
      if (!eq) diff += std::string(diff.empty() ? "" : ", ") + name;
    };
    chk(a.degree == b.degree, "degree");
    chk(a.poisson_pairing == b.poisson_pairing, "poisson_pairing");
    chk(a.full_system == b.full_system, "full_system");
    chk(a.nx_semi == b.nx_semi && a.nx_elec == b.nx_elec && a.ny == b.ny, "cell counts");
    chk(a.x_semi0 == b.x_semi0 && a.x_semi1 == b.x_semi1 && a.x_elec1 == b.x_elec1 && a.height == b.height,
        "geometry");
    chk(a.lambda2 == b.lambda2, "lambda2");
    chk(a.eps_semi == b.eps_semi && a.eps_elec == b.eps_elec, "permittivities");
    chk(a.dt == b.dt, "dt");
    chk(a.penalty == b.penalty, "penalty");
    chk(a.grading == b.grading || (!(a.grading > 1.0) && !(b.grading > 1.0)), "grading");
    chk(std::memcmp(a.mu, b.mu, sizeof(a.mu)) == 0, "mobilities");
    chk(std::memcmp(a.bc_semi, b.bc_semi, sizeof(a.bc_semi)) == 0 &&
            std::memcmp(a.bc_elec, b.bc_elec, sizeof(a.bc_elec)) == 0 &&
            std::memcmp(a.bc_poisson, b.bc_poisson, sizeof(a.bc_poisson)) == 0 &&
            std::memcmp(a.bc_poisson_elec, b.bc_poisson_elec, sizeof(a.bc_poisson_elec)) == 0,
        "boundary ids");
    if (!diff.empty()) {
      e << "instance " << i << " differs from instance 0 in a matrix-defining field (" << diff << "); ";
      break;
    }
  }
  return e.str();
}

// Carrier system matrices straight into CSR.  Row (K, i) couples to the dofs
// of K and of its face neighbours; a row's columns are sorted by dof index
// (component, then cell, then node) and exact zeros are not stored.  Each
// entry of the diagonal block sums its terms in the order: cell matrix, face
// below (K is its plus side), face on the left (plus side), face on the right
// (minus side), face above (minus side) -- the order of the reference's
// cell loop followed by its face loop over cells in index order.
static void assemble_carrier(CarrierSystem& S, const CarrierTables& ct, const pecs_params& P,
                             double mu1, double mu2) {
  const Grid& g = S.grid;
  const int n1 = ct.n1, nd = 3 * n1, nc = g.nc(), nx = g.nx, ny = g.ny;
  S.ndofs = 3 * nc * n1;
  auto dof = [&](int K, int i) { return (i / n1) * nc * n1 + K * n1 + (i % n1); };
  // cell matrices (assemble_local_LDG_cell_and_bc_terms, source/LDG.cpp:85-281),
  // shared between cells of equal size and boundary ids
  std::map<std::tuple<double, double, int, int, int, int>, std::vector<double>> cache[2];
  std::vector<const std::vector<double>*> cellA[2];
  cellA[0].resize(nc);
  cellA[1].resize(nc);
  std::vector<int> mr, mc;
  std::vector<double> mv;
  for (int K = 0; K < nc; ++K) {
    double x0, y0, hx, hy;
    g.geom(K, x0, y0, hx, hy);
    int bids[4];
    for (int f = 0; f < 4; ++f) bids[f] = g.face_bid(K, f);
    double diam = std::sqrt(hx * hx + hy * hy);
    auto key = std::make_tuple(hx, hy, bids[0], bids[1], bids[2], bids[3]);
    for (int s = 0; s < 2; ++s) {
      auto it = cache[s].find(key);
      if (it == cache[s].end())
        it = cache[s].emplace(key, ldg_cell_matrix(ct, hx, hy, s == 0 ? mu1 : mu2, P.dt, 1.0,
                                                   P.penalty / diam, bids))
                 .first;
      cellA[s][K] = &it->second;
    }
    // (1/dt) mass, source/LDG.cpp:40-83
    for (int a = 0; a < n1; ++a)
      for (int b = 0; b < n1; ++b) {
        double s = 0.0;
        for (int q = 0; q < ct.Q; ++q)
          s += (1.0 / P.dt) * ct.phi[a * ct.Q + q] * ct.phi[b * ct.Q + q] * ct.qw[q] * hx * hy;
        mr.push_back(dof(K, 2 * n1 + a));
        mc.push_back(dof(K, 2 * n1 + b));
        mv.push_back(s);
      }
  }
  // interior-face blocks (assemble_flux_terms, source/LDG.cpp:283-426): for the
  // face of K in direction dir (0: right, 1: top), blocks (K,K), (K,nb), (nb,K),
  // (nb,nb); equal for both carriers
  std::map<std::tuple<int, double, double>, std::vector<std::vector<double>>> fcache;
  std::vector<const std::vector<std::vector<double>>*> faceB(2 * (size_t)nc, nullptr);
  for (int K = 0; K < nc; ++K) {
    const int i = K % nx, j = K / nx;
    for (int dir = 0; dir < 2; ++dir) {
      if (dir == 0 ? i >= nx - 1 : j >= ny - 1) continue;
      const int nb = dir == 0 ? K + 1 : K + nx;
      const int fm = dir == 0 ? kRight : kTop, fp = dir == 0 ? kLeft : kBottom;
      double x0, y0, hx, hy, x1, y1, hx1, hy1;
      g.geom(K, x0, y0, hx, hy);
      g.geom(nb, x1, y1, hx1, hy1);
      double flen = dir == 0 ? hy : hx;
      double h = std::min(std::sqrt(hx * hx + hy * hy), std::sqrt(hx1 * hx1 + hy1 * hy1));
      auto key = std::make_tuple(fm, flen, h);
      auto it = fcache.find(key);
      if (it == fcache.end()) {
        std::vector<double> blk[4];
        ldg_flux_blocks(ct, fm, fp, flen, P.penalty / h, blk);
        it = fcache.emplace(key, std::vector<std::vector<double>>(blk, blk + 4)).first;
      }
      faceB[2 * (size_t)K + dir] = &it->second;
    }
  }
  // rows, cell range by cell range; per thread one buffer per (carrier, component)
  struct Part {
    std::vector<int> len[2][3], col[2][3];
    std::vector<double> val[2][3];
  };
  unsigned hc = std::thread::hardware_concurrency();
  const int nt = (int)std::max(1u, std::min({hc, 16u, (unsigned)std::max(1, nc / 64)}));
  std::vector<Part> parts(nt);
  auto work = [&](int t) {
    const int K0 = (int)((long long)nc * t / nt), K1 = (int)((long long)nc * (t + 1) / nt);
    Part& pt = parts[t];
    std::vector<double> blk[5];
    for (auto& b : blk) b.resize((size_t)nd * nd);
    for (int K = K0; K < K1; ++K) {
      const int i = K % nx, j = K / nx;
      int cells[5], nb = 0;
      if (j > 0) cells[nb++] = K - nx;
      if (i > 0) cells[nb++] = K - 1;
      cells[nb++] = K;
      if (i < nx - 1) cells[nb++] = K + 1;
      if (j < ny - 1) cells[nb++] = K + nx;
      for (int s = 0; s < 2; ++s) {
        for (int c = 0; c < nb; ++c) {
          const int C = cells[c];
          double* B = blk[c].data();
          if (C == K) {
            const std::vector<double>& A = *cellA[s][K];
            for (int e = 0; e < nd * nd; ++e) B[e] = 0.0 + A[e];
            if (j > 0) {
              const std::vector<double>& F = (*faceB[2 * (size_t)(K - nx) + 1])[3];
              for (int e = 0; e < nd * nd; ++e) B[e] += F[e];
            }
            if (i > 0) {
              const std::vector<double>& F = (*faceB[2 * (size_t)(K - 1) + 0])[3];
              for (int e = 0; e < nd * nd; ++e) B[e] += F[e];
            }
            if (i < nx - 1) {
              const std::vector<double>& F = (*faceB[2 * (size_t)K + 0])[0];
              for (int e = 0; e < nd * nd; ++e) B[e] += F[e];
            }
            if (j < ny - 1) {
              const std::vector<double>& F = (*faceB[2 * (size_t)K + 1])[0];
              for (int e = 0; e < nd * nd; ++e) B[e] += F[e];
            }
          } else {
            const std::vector<double>* F;
            if (C == K + 1) F = &(*faceB[2 * (size_t)K + 0])[1];
            else if (C == K + nx) F = &(*faceB[2 * (size_t)K + 1])[1];
            else if (C == K - 1) F = &(*faceB[2 * (size_t)(K - 1) + 0])[2];
            else F = &(*faceB[2 * (size_t)(K - nx) + 1])[2];
            for (int e = 0; e < nd * nd; ++e) B[e] = 0.0 + (*F)[e];
          }
        }
        for (int r = 0; r < nd; ++r) {
          const int rc = r / n1;
          int cnt = 0;
          for (int comp = 0; comp < 3; ++comp)
            for (int c = 0; c < nb; ++c) {
              const double* B = blk[c].data() + (size_t)r * nd + comp * n1;
              const int base = comp * nc * n1 + cells[c] * n1;
              for (int a = 0; a < n1; ++a) {
                if (B[a] == 0.0) continue;  // structural zeros of the flux pattern are not stored
                pt.col[s][rc].push_back(base + a);
                pt.val[s][rc].push_back(B[a]);
                ++cnt;
              }
            }
          pt.len[s][rc].push_back(cnt);
        }
      }
    }
  };
  dense::run_threads(nt, work);
  for (int s = 0; s < 2; ++s) {
    Csr& A = S.A[s];
    A.n = S.ndofs;
    A.rowptr.assign(S.ndofs + 1, 0);
    size_t nnz = 0;
    for (auto& pt : parts)
      for (int rc = 0; rc < 3; ++rc) nnz += pt.col[s][rc].size();
    A.col.reserve(nnz);
    A.val.reserve(nnz);
    // rows of component rc, cell K, node a sit at rc*nc*n1 + K*n1 + a; within a
    // part they were produced cell by cell, node by node (r = rc*n1 + a)
    int row = 0;
    for (int rc = 0; rc < 3; ++rc)
      for (auto& pt : parts) {
        A.col.insert(A.col.end(), pt.col[s][rc].begin(), pt.col[s][rc].end());
        A.val.insert(A.val.end(), pt.val[s][rc].begin(), pt.val[s][rc].end());
        for (int l : pt.len[s][rc]) {
          A.rowptr[row + 1] = A.rowptr[row] + l;
          ++row;
        }
        std::vector<int>().swap(pt.col[s][rc]);
        std::vector<double>().swap(pt.val[s][rc]);
      }
  }
  S.M = coo_to_csr(S.ndofs, mr, mc, mv);
  S.dof_cell.resize(S.ndofs);
  S.dof_class.resize(S.ndofs);
  for (int K = 0; K < nc; ++K)
    for (int i = 0; i < nd; ++i) {
      S.dof_cell[dof(K, i)] = K;
      S.dof_class[dof(K, i)] = (i < 2 * n1) ? 0 : 1;
    }
  S.cell_xy.resize(2 * nc);
  for (int K = 0; K < nc; ++K) {
    double x0, y0, hx, hy;
    g.geom(K, x0, y0, hx, hy);
    S.cell_xy[2 * K] = x0 + 0.5 * hx;
    S.cell_xy[2 * K + 1] = y0 + 0.5 * hy;
  }
}

static void setup_poisson(PoissonSystem& S, const PoissonTables& pt, const CarrierTables& ct,
                          const pecs_params& P) {
  const Grid& g = S.grid;
  const int k = pt.k, nx = g.nx, ny = g.ny, nc = g.nc();
  const int nloc = pt.n_rt + pt.n_phi;
  const int nvert = (nx + 1) * ny, nhor = nx * (ny + 1), nint = 2 * k * (k - 1);
  const int off_h = nvert * k, off_i = off_h + nhor * k, off_phi = off_i + nc * nint;
  S.n_rt_total = off_phi;
  S.ndofs = off_phi + nc * pt.n_phi;
  S.l2g.assign(nc * nloc, 0);
  const int nxd = k * (k + 1);
  for (int K = 0; K < nc; ++K) {
    int i = K % nx, j = K / nx, cnt = 0;
    for (int b = 0; b < k; ++b)
      for (int a = 0; a <= k; ++a) {
        int loc = a + (k + 1) * b;
        int gdof;
        if (a == 0)
          gdof = (i + (nx + 1) * j) * k + b;
        else if (a == k)
          gdof = (i + 1 + (nx + 1) * j) * k + b;
        else
          gdof = off_i + K * nint + cnt++;
        S.l2g[K * nloc + loc] = gdof;
      }
    for (int b = 0; b <= k; ++b)
      for (int a = 0; a < k; ++a) {
        int loc = nxd + a + k * b;
        int gdof;
        if (b == 0)
          gdof = off_h + (i + nx * j) * k + a;
        else if (b == k)
          gdof = off_h + (i + nx * (j + 1)) * k + a;
        else
          gdof = off_i + K * nint + cnt++;
        S.l2g[K * nloc + loc] = gdof;
      }
    for (int a = 0; a < pt.n_phi; ++a) S.l2g[K * nloc + pt.n_rt + a] = off_phi + K * pt.n_phi + a;
  }
  // zero D.n on Neumann faces (source/Poisson.cpp:32-49)
  S.constrained.assign(S.ndofs, 0);
  for (int K = 0; K < nc; ++K)
    for (int f = 0; f < 4; ++f)
      if (g.face_bid(K, f) == kNeumann)
        for (int loc : pt.face_dofs[f]) S.constrained[S.l2g[K * nloc + loc]] = 1;
  // matrix
  std::vector<int> r, c;
  std::vector<double> v;
  std::map<std::tuple<double, double, double>, std::vector<double>> cache;
  for (int K = 0; K < nc; ++K) {
    double x0, y0, hx, hy;
    g.geom(K, x0, y0, hx, hy);
    double eps = (g.material[K] == 0 || g.material[K] == 1) ? P.eps_semi : P.eps_elec;
    auto key = std::make_tuple(hx, hy, eps);
    auto it = cache.find(key);
    if (it == cache.end())
      it = cache.emplace(key, poisson_cell_matrix(pt, ct, hx, hy, eps, P.lambda2)).first;
    const std::vector<double>& A = it->second;
    for (int a = 0; a < nloc; ++a) {
      int ga = S.l2g[K * nloc + a];
      if (S.constrained[ga]) continue;
      for (int b = 0; b < nloc; ++b) {
        int gb = S.l2g[K * nloc + b];
        if (S.constrained[gb]) continue;
        r.push_back(ga);
        c.push_back(gb);
        v.push_back(A[a * nloc + b]);
      }
    }
  }
  for (int d = 0; d < S.ndofs; ++d)
    if (S.constrained[d]) {
      r.push_back(d);
      c.push_back(d);
      v.push_back(1.0);
    }
  S.A = coo_to_csr(S.ndofs, r, c, v);
  // dof -> owning cell: faces to the left/bottom neighbour, cell dofs to the cell
  S.dof_cell.assign(S.ndofs, -1);
  for (int K = 0; K < nc; ++K) {
    int i = K % nx, j = K / nx;
    for (int loc = 0; loc < nloc; ++loc) {
      int gd = S.l2g[K * nloc + loc];
      int owner = K;
      bool is_left = false, is_bottom = false;
      for (int t : pt.face_dofs[kLeft]) is_left |= (t == loc);
      for (int t : pt.face_dofs[kBottom]) is_bottom |= (t == loc);
      if (is_left && i > 0) owner = K - 1;
      if (is_bottom && j > 0) owner = K - nx;
      if (S.dof_cell[gd] < 0) S.dof_cell[gd] = owner;
    }
  }
  S.cell_xy.resize(2 * nc);
  for (int K = 0; K < nc; ++K) {
    double x0, y0, hx, hy;
    g.geom(K, x0, y0, hx, hy);
    S.cell_xy[2 * K] = x0 + 0.5 * hx;
    S.cell_xy[2 * K + 1] = y0 + 0.5 * hy;
  }
}

Setup::Setup(const std::vector<pecs_params>& p)
    : inst(p), ct(p[0].degree), pt(p[0].degree + p[0].poisson_pairing, ct) {
  const pecs_params& P = p[0];
  k = P.degree;
  n1 = ct.n1;
  n_rt = pt.n_rt;
  n_phi = pt.n_phi;
  Q = ct.Q;
  nq1 = ct.nq1;
  full = P.full_system != 0;
  semi.grid = region(P.x_semi0, P.x_semi1, 0.0, P.height, P.nx_semi, P.ny, P.bc_semi, 0, P.grading,
                     true);
  if (full)
    elec.grid = region(P.x_semi1, P.x_elec1, 0.0, P.height, P.nx_elec, P.ny, P.bc_elec, 2, P.grading,
                       false);
  // Poisson mesh: merged triangulation (Grid.cpp:320-336)
  Grid& pg = pois.grid;
  pg.nx = P.nx_semi + (full ? P.nx_elec : 0);
  pg.ny = P.ny;
  pg.xs = semi.grid.xs;
  if (full) pg.xs.insert(pg.xs.end(), elec.grid.xs.begin() + 1, elec.grid.xs.end());
  pg.ys = semi.grid.ys;
  for (int f = 0; f < 4; ++f) pg.bc[f] = P.bc_poisson[f];
  if (full) {
    pg.split = P.nx_semi;
    for (int f = 0; f < 4; ++f) pg.bc2[f] = P.bc_poisson_elec[f];
  }
  pg.material.resize(pg.nc());
  for (int K = 0; K < pg.nc(); ++K) pg.material[K] = (K % pg.nx) < P.nx_semi ? 0 : 2;

  assemble_carrier(semi, ct, P, P.mu[0], P.mu[1]);
  if (full) assemble_carrier(elec, ct, P, P.mu[2], P.mu[3]);
  setup_poisson(pois, pt, ct, P);

  // setup_mappings (SolarCell.cpp:156-372): identical cell centres
  s2p.resize(semi.grid.nc());
  for (int K = 0; K < semi.grid.nc(); ++K) s2p[K] = (K % semi.grid.nx) + pg.nx * (K / semi.grid.nx);
  if (full) {
    e2p.resize(elec.grid.nc());
    for (int K = 0; K < elec.grid.nc(); ++K)
      e2p[K] = (K % elec.grid.nx) + P.nx_semi + pg.nx * (K / elec.grid.nx);
    for (int j = 0; j < P.ny; ++j) {
      int Ks = (semi.grid.nx - 1) + semi.grid.nx * j;
      int Ke = 0 + elec.grid.nx * j;
      if (semi.grid.face_bid(Ks, kRight) == kInterface && elec.grid.face_bid(Ke, kLeft) == kInterface) {
        iface_semi.push_back(Ks);
        iface_elec.push_back(Ke);
      }
    }
  }
  for (int K = 0; K < semi.grid.nc(); ++K)
    for (int f = 0; f < 4; ++f)
      if (semi.grid.face_bid(K, f) == kSchottky) has_schottky = true;

  compute_instances(p);
}


// Per-instance data: time-independent RHS parts, interface/Schottky
// equilibria and the projected initial state.  Only fields that do not enter
// the matrices may differ between instances (validate_params checks that).
void Setup::compute_instances(const std::vector<pecs_params>& p) {
  inst = p;
  const int ninst = (int)p.size();
  for (int fld = 0; fld < 5; ++fld) bconst[fld].assign(ninst, {});
  iface_ne.assign(ninst, {});
  iface_pe.assign(ninst, {});
  schottky_ne.assign(ninst, {});
  schottky_pe.assign(ninst, {});
  for (int fld = 0; fld < 4; ++fld) init[fld].assign(ninst, {});
  std::vector<int> all(ninst);
  for (int s = 0; s < ninst; ++s) all[s] = s;
  compute_instances_at(all);
}

// The listed instances' data on the host threads (each instance writes only
// its own slots and reads the shared setup, so the results do not depend on
// the thread count); instances are handed out one at a time.
// Fewer instances than threads (a streamed sweep refilling a slot or two):
// each instance's cell loops are split over the threads instead.
void Setup::compute_instances_at(const std::vector<int>& slots) {
  const int n = (int)slots.size();
  if (n == 0) return;
  const unsigned hc = std::thread::hardware_concurrency();
  const int hw = std::max(1, (int)(hc ? hc : 1));
  if (n < hw) {
    for (int t = 0; t < n; ++t) compute_instance(slots[t], hw);
    return;
  }
  std::atomic<int> next{0};
  dense::run_threads(hw, [&](int) {
    for (int t = next.fetch_add(1); t < n; t = next.fetch_add(1)) compute_instance(slots[t]);
  });
}

namespace {
// fn(first, last) over [0, n) in `threads` contiguous ranges (one when small)
void par_range(int n, int threads, const std::function<void(int, int)>& fn) {
  if (threads <= 1 || n < 512) {
    fn(0, n);
    return;
  }
  const int chunk = (n + threads - 1) / threads;
  dense::run_threads(threads, [&](int t) {
    const int a = t * chunk, b = std::min(n, a + chunk);
    if (a < b) fn(a, b);
  });
}
}  // namespace

void Setup::compute_instance(int s, int threads) {
  InstanceData d;
  compute_instance_data(inst[s], d, threads);
  store_instance(s, std::move(d));
}

void Setup::store_instance(int s, InstanceData&& d) {
  for (int f = 0; f < 5; ++f) bconst[f][s] = std::move(d.bconst[f]);
  for (int f = 0; f < 4; ++f) init[f][s] = std::move(d.init[f]);
  iface_ne[s] = std::move(d.iface_ne);
  iface_pe[s] = std::move(d.iface_pe);
  schottky_ne[s] = std::move(d.schottky_ne);
  schottky_pe[s] = std::move(d.schottky_pe);
}

void Setup::compute_instance_data(const pecs_params& Pi, InstanceData& d, int threads) const {
  const int nloc = n_rt + n_phi;
  std::vector<double> g1, w1;
  gauss01(k + 1, g1, w1);
  {
    for (int reg = 0; reg < (full ? 2 : 1); ++reg) {
      const CarrierSystem& CS = reg == 0 ? semi : elec;
      const Grid& g = CS.grid;
      const int nc = g.nc();
      for (int cc = 0; cc < 2; ++cc) {
        int fld = 2 * reg + cc;
        std::vector<double> b(CS.ndofs, 0.0);
        // every cell writes only its own rows of b
        par_range(nc, threads, [&](int K0, int K1) {
        for (int K = K0; K < K1; ++K) {
          double x0, y0, hx, hy;
          g.geom(K, x0, y0, hx, hy);
          double diam = std::sqrt(hx * hx + hy * hy);
          if (reg == 0 && Pi.gen_kind != 0) {
            for (int a = 0; a < n1; ++a) {
              double sacc = 0.0;
              for (int q = 0; q < Q; ++q) {
                double X = x0 + hx * ct.qx[q], Y = y0 + hy * ct.qy[q];
                sacc += ct.phi[a * Q + q] * generation(Pi, X, Y) * ct.qw[q] * hx * hy;
              }
              b[2 * nc * n1 + K * n1 + a] += sacc;
            }
          }
          for (int f = 0; f < 4; ++f) {
            if (g.face_bid(K, f) != kDirichlet) continue;
            double flen = (f == kLeft || f == kRight) ? hy : hx;
            for (int i = 0; i < 3 * n1; ++i) {
              int ci = i / n1, a = i % n1;
              double sacc = 0.0;
              for (int q = 0; q < nq1; ++q) {
                double X, Y;
                if (f == kLeft) { X = x0; Y = y0 + hy * ct.fq[q]; }
                else if (f == kRight) { X = x0 + hx; Y = y0 + hy * ct.fq[q]; }
                else if (f == kBottom) { X = x0 + hx * ct.fq[q]; Y = y0; }
                else { X = x0 + hx * ct.fq[q]; Y = y0 + hy; }
                double ph = ct.fphi[(f * n1 + a) * nq1 + q];
                double pn = (ci == 0 ? kFaceNormal[f][0] * ph : 0.0) + (ci == 1 ? kFaceNormal[f][1] * ph : 0.0);
                double vv = ci == 2 ? ph : 0.0;
                sacc += (-pn + (Pi.penalty / diam) * vv) * carrier_bc(Pi, fld, X, Y) * ct.fw[q] * flen;
              }
              b[ci * nc * n1 + K * n1 + a] += sacc;
            }
          }
        }
        });
        d.bconst[fld] = std::move(b);
        // initial conditions: L2 projection with QGauss(k+1) (SolarCell.cpp:1996-2021)
        std::vector<double> u(CS.ndofs, 0.0);
        {
          const int m = k + 1, nq = (int)g1.size();
          auto nodes = dgq_nodes(k);
          std::vector<std::vector<double>> L(nq), dL(nq);
          for (int q = 0; q < nq; ++q) lagrange1d(nodes, g1[q], L[q], dL[q]);
          std::vector<double> Mref(n1 * n1, 0.0);
          for (int a = 0; a < n1; ++a)
            for (int bb = 0; bb < n1; ++bb)
              for (int qy_ = 0; qy_ < nq; ++qy_)
                for (int qx_ = 0; qx_ < nq; ++qx_)
                  Mref[a * n1 + bb] += L[qx_][a % m] * L[qy_][a / m] * L[qx_][bb % m] * L[qy_][bb / m] *
                                       w1[qx_] * w1[qy_];
          par_range(nc, threads, [&](int K0, int K1) {
          for (int K = K0; K < K1; ++K) {
            double x0, y0, hx, hy;
            g.geom(K, x0, y0, hx, hy);
            std::vector<double> rhs(n1, 0.0);
            for (int a = 0; a < n1; ++a)
              for (int qy_ = 0; qy_ < nq; ++qy_)
                for (int qx_ = 0; qx_ < nq; ++qx_)
                  rhs[a] += L[qx_][a % m] * L[qy_][a / m] *
                            initial_profile(Pi, fld, x0 + hx * g1[qx_], y0 + hy * g1[qy_]) * w1[qx_] *
                            w1[qy_];
            // solve Mref c = rhs (Gaussian elimination with partial pivoting)
            std::vector<double> M = Mref;
            std::vector<double> c = rhs;
            for (int col = 0; col < n1; ++col) {
              int piv = col;
              for (int rr = col + 1; rr < n1; ++rr)
                if (std::fabs(M[rr * n1 + col]) > std::fabs(M[piv * n1 + col])) piv = rr;
              if (piv != col) {
                for (int cc2 = 0; cc2 < n1; ++cc2) std::swap(M[col * n1 + cc2], M[piv * n1 + cc2]);
                std::swap(c[col], c[piv]);
              }
              for (int rr = col + 1; rr < n1; ++rr) {
                double f = M[rr * n1 + col] / M[col * n1 + col];
                for (int cc2 = col; cc2 < n1; ++cc2) M[rr * n1 + cc2] -= f * M[col * n1 + cc2];
                c[rr] -= f * c[col];
              }
            }
            for (int rr = n1 - 1; rr >= 0; --rr) {
              double sacc = c[rr];
              for (int cc2 = rr + 1; cc2 < n1; ++cc2) sacc -= M[rr * n1 + cc2] * c[cc2];
              c[rr] = sacc / M[rr * n1 + rr];
            }
            for (int a = 0; a < n1; ++a) u[2 * nc * n1 + K * n1 + a] = c[a];
          }
          });
        }
        d.init[fld] = std::move(u);
      }
    }
    // Poisson constant part: doping on semiconductor cells + Dirichlet potential
    std::vector<double> bP(pois.ndofs, 0.0);
    const Grid& g = pois.grid;
    for (int K = 0; K < g.nc(); ++K) {
      double x0, y0, hx, hy;
      g.geom(K, x0, y0, hx, hy);
      if (g.material[K] == 0) {
        for (int a = 0; a < n_phi; ++a) {
          double sacc = 0.0;
          for (int q = 0; q < Q; ++q) {
            double X = x0 + hx * ct.qx[q];
            double dop = pw(X, Pi.nd, Pi.junction_x) - pw(X, Pi.na, Pi.junction_x);
            sacc += pt.phi[a * Q + q] * dop * ct.qw[q] * hx * hy;
          }
          bP[pois.l2g[K * nloc + n_rt + a]] += -sacc;
        }
      }
      for (int f = 0; f < 4; ++f) {
        if (g.face_bid(K, f) != kDirichlet) continue;
        double flen = (f == kLeft || f == kRight) ? hy : hx;
        for (int i = 0; i < n_rt; ++i) {
          double sacc = 0.0;
          for (int q = 0; q < nq1; ++q) {
            double X, Y;
            if (f == kLeft) { X = x0; Y = y0 + hy * ct.fq[q]; }
            else if (f == kRight) { X = x0 + hx; Y = y0 + hy * ct.fq[q]; }
            else if (f == kBottom) { X = x0 + hx * ct.fq[q]; Y = y0; }
            else { X = x0 + hx * ct.fq[q]; Y = y0 + hy; }
            sacc += pt.fpsi_n[(f * n_rt + i) * nq1 + q] * potential_dirichlet(Pi, X, Y) * ct.fw[q] * flen;
          }
          bP[pois.l2g[K * nloc + i]] += -sacc;
        }
      }
    }
    for (int d = 0; d < pois.ndofs; ++d)
      if (pois.constrained[d]) bP[d] = 0.0;
    d.bconst[4] = std::move(bP);
    // interface equilibria at the semiconductor face qp
    if (full) {
      std::vector<double> ne(iface_semi.size() * nq1), pe(iface_semi.size() * nq1);
      for (size_t t = 0; t < iface_semi.size(); ++t) {
        double x0, y0, hx, hy;
        semi.grid.geom(iface_semi[t], x0, y0, hx, hy);
        for (int q = 0; q < nq1; ++q) {
          double X = x0 + hx, Y = y0 + hy * ct.fq[q];
          ne[t * nq1 + q] = carrier_bc(Pi, 0, X, Y);
          pe[t * nq1 + q] = carrier_bc(Pi, 1, X, Y);
        }
      }
      d.iface_ne = std::move(ne);
      d.iface_pe = std::move(pe);
    }
    if (has_schottky) {
      const Grid& gs = semi.grid;
      std::vector<double> ne(gs.nc() * 4 * nq1, 0.0), pe(gs.nc() * 4 * nq1, 0.0);
      for (int K = 0; K < gs.nc(); ++K) {
        double x0, y0, hx, hy;
        gs.geom(K, x0, y0, hx, hy);
        for (int f = 0; f < 4; ++f) {
          if (gs.face_bid(K, f) != kSchottky) continue;
          for (int q = 0; q < nq1; ++q) {
            double X, Y;
            if (f == kLeft) { X = x0; Y = y0 + hy * ct.fq[q]; }
            else if (f == kRight) { X = x0 + hx; Y = y0 + hy * ct.fq[q]; }
            else if (f == kBottom) { X = x0 + hx * ct.fq[q]; Y = y0; }
            else { X = x0 + hx * ct.fq[q]; Y = y0 + hy; }
            ne[(K * 4 + f) * nq1 + q] = carrier_bc(Pi, 0, X, Y);
            pe[(K * 4 + f) * nq1 + q] = carrier_bc(Pi, 1, X, Y);
          }
        }
      }
      d.schottky_ne = std::move(ne);
      d.schottky_pe = std::move(pe);
    }
  }
}

}  // namespace pecs

// ---------------------------------------------------------------------------
// Element matrices for the drop-in assembly classes (host only): what the
// reference's local assembly members compute for one cell, on the library's
// element tables.  Matrices are row-major; carrier local dofs are
// [J_x (n1) | J_y (n1) | u (n1)], n1 = (k+1)^2; Poisson local dofs
// [D_x | D_y | Phi] of the nodal RT basis (fe.hpp).
// ---------------------------------------------------------------------------
namespace pecs {
void set_error_external(const std::string& m);
}

namespace {

bool cell_ok(const pecs_cell* c, std::string& err) {
  if (!c) {
    err = "cell is NULL";
    return false;
  }
  if (!(c->hx > 0.0) || !(c->hy > 0.0) || !std::isfinite(c->hx) || !std::isfinite(c->hy)) {
    err = "cell sizes must be positive and finite";
    return false;
  }
  for (int f = 0; f < 4; ++f)
    if (c->boundary_id[f] < -1 || c->boundary_id[f] > 3) {
      err = "boundary ids must be -1 (interior) or 0..3";
      return false;
    }
  return true;
}

int fail(const std::string& m) {
  pecs::set_error_external(m);
  return PECS_E_ARG;
}

}  // namespace

extern "C" {

int pecs_ldg_local_mass_matrix(int degree, const pecs_cell* cell, double delta_t, double* out) {
  using namespace pecs;
  std::string err;
  if (degree < 1 || degree > 2) return fail("degree must be 1 or 2");
  if (!cell_ok(cell, err)) return fail(err);
  if (!(delta_t > 0.0) || !out) return fail("delta_t must be > 0 and out not NULL");
  CarrierTables ct(degree);
  const int n1 = ct.n1, nd = 3 * n1;
  std::fill(out, out + nd * nd, 0.0);
  for (int a = 0; a < n1; ++a)
    for (int b = 0; b < n1; ++b) {
      double s = 0.0;
      for (int q = 0; q < ct.Q; ++q)
        s += (1.0 / delta_t) * ct.phi[a * ct.Q + q] * ct.phi[b * ct.Q + q] * ct.qw[q] * cell->hx * cell->hy;
      out[(2 * n1 + a) * nd + 2 * n1 + b] = s;
    }
  return PECS_OK;
}

int pecs_ldg_local_cell_and_bc_terms(int degree, const pecs_cell* cell, double mobility_1,
                                     double mobility_2, double delta_t, double transient_or_steady,
                                     double penalty, double* out_1, double* out_2) {
  using namespace pecs;
  std::string err;
  if (degree < 1 || degree > 2) return fail("degree must be 1 or 2");
  if (!cell_ok(cell, err)) return fail(err);
  if (!(mobility_1 > 0.0) || !(mobility_2 > 0.0) || !(delta_t > 0.0) || !out_1 || !out_2)
    return fail("mobilities and delta_t must be > 0, outputs not NULL");
  CarrierTables ct(degree);
  const double diam = std::sqrt(cell->hx * cell->hx + cell->hy * cell->hy);  // cell->diameter()
  const std::vector<double> A1 = ldg_cell_matrix(ct, cell->hx, cell->hy, mobility_1, delta_t,
                                                 transient_or_steady, penalty / diam, cell->boundary_id);
  const std::vector<double> A2 = ldg_cell_matrix(ct, cell->hx, cell->hy, mobility_2, delta_t,
                                                 transient_or_steady, penalty / diam, cell->boundary_id);
  std::copy(A1.begin(), A1.end(), out_1);
  std::copy(A2.begin(), A2.end(), out_2);
  return PECS_OK;
}

int pecs_ldg_local_flux_terms(int degree, const pecs_cell* cell, int face, const pecs_cell* neighbor,
                              double penalty, double* vi_ui, double* vi_ue, double* ve_ui, double* ve_ue) {
  using namespace pecs;
  std::string err;
  if (degree < 1 || degree > 2) return fail("degree must be 1 or 2");
  if (!cell_ok(cell, err) || !cell_ok(neighbor, err)) return fail(err);
  if (face < 0 || face > 3) return fail("face must be 0..3");
  if (!vi_ui || !vi_ue || !ve_ui || !ve_ue) return fail("outputs must not be NULL");
  CarrierTables ct(degree);
  const double flen = (face == kLeft || face == kRight) ? cell->hy : cell->hx;
  const double h = std::min(std::sqrt(cell->hx * cell->hx + cell->hy * cell->hy),
                            std::sqrt(neighbor->hx * neighbor->hx + neighbor->hy * neighbor->hy));
  std::vector<double> blk[4];
  ldg_flux_blocks(ct, face, face ^ 1, flen, penalty / h, blk);
  double* outs[4] = {vi_ui, vi_ue, ve_ui, ve_ue};
  for (int t = 0; t < 4; ++t) std::copy(blk[t].begin(), blk[t].end(), outs[t]);
  return PECS_OK;
}

int pecs_mixed_local_poisson_matrix(int degree, int poisson_pairing, const pecs_cell* cell,
                                    double semi_permittivity, double elec_permittivity,
                                    double scaled_debye_length, double* out) {
  using namespace pecs;
  std::string err;
  if (degree < 1 || degree > 2) return fail("degree must be 1 or 2");
  if (poisson_pairing != 0 && poisson_pairing != 1) return fail("poisson_pairing must be 0 or 1");
  if (!cell_ok(cell, err)) return fail(err);
  if (!out || !(semi_permittivity > 0.0) || !(elec_permittivity > 0.0) || !(scaled_debye_length > 0.0))
    return fail("permittivities and the Debye length must be > 0, out not NULL");
  CarrierTables ct(degree);
  PoissonTables pt(degree + poisson_pairing, ct);
  // material ids 0, 1: semiconductor; 2, 3: electrolyte (MixedFEM.hpp:226-236)
  const double eps = cell->material_id <= 1 ? semi_permittivity : elec_permittivity;
  const std::vector<double> A = poisson_cell_matrix(pt, ct, cell->hx, cell->hy, eps, scaled_debye_length);
  std::copy(A.begin(), A.end(), out);
  return PECS_OK;
}

int pecs_element_sizes(int degree, int poisson_pairing, int* carrier_dofs, int* poisson_rt_dofs,
                       int* poisson_phi_dofs) {
  if (degree < 1 || degree > 2) return fail("degree must be 1 or 2");
  if (poisson_pairing != 0 && poisson_pairing != 1) return fail("poisson_pairing must be 0 or 1");
  const int kp = degree + poisson_pairing;
  if (carrier_dofs) *carrier_dofs = 3 * (degree + 1) * (degree + 1);
  if (poisson_rt_dofs) *poisson_rt_dofs = 2 * kp * (kp + 1);
  if (poisson_phi_dofs) *poisson_phi_dofs = kp * kp;
  return PECS_OK;
}

}  // extern "C"
