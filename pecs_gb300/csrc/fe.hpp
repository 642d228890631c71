// Reference-element tables for the PECS carrier and Poisson spaces.
//
// Carrier space: FESystem(FE_DGQ(k)^2, FE_DGQ(k)) (source/SolarCell.cpp:30-31 of
// the reference): Lagrange basis on k+1 equidistant nodes per direction,
// lexicographic (x fastest).  Local dofs [J_x (n1) | J_y (n1) | u (n1)].
//
// Poisson space: RT_{k-1} x DGQ_{k-1} (source/SolarCell.cpp:23-24).  The RT
// space is spanned by a tensor-product nodal basis: the normal component uses
// k+1 equidistant nodes (so the coefficients at the two end nodes live on the
// faces and are shared between neighbouring cells), the tangential one k nodes
// at (i+1/2)/k.  Local dofs [D_x (k(k+1)) | D_y (k(k+1)) | Phi (k^2)].
//
// Quadrature: QGauss(k+2) on cells and faces (source/SolarCell.cpp:402-403).
#pragma once
#include <cmath>
#include <stdexcept>
#include <vector>

namespace pecs {

enum BoundaryId { kInterface = 0, kDirichlet = 1, kNeumann = 2, kSchottky = 3 };
enum FaceNo { kLeft = 0, kRight = 1, kBottom = 2, kTop = 3 };
static const double kFaceNormal[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};

// Gauss-Legendre rule on [0,1] (Newton iteration on P_n).
inline void gauss01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int m = 2; m <= n; ++m) {
        double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
        p0 = p1;
        p1 = p2;
      }
      double pn = (n == 1) ? z : p1;
      double pm = (n == 1) ? 1.0 : p0;
      dp = n * (z * pn - pm) / (z * z - 1.0);
      double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    // recompute derivative at the converged root
    double p0 = 1.0, p1 = z;
    for (int m = 2; m <= n; ++m) {
      double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
      p0 = p1;
      p1 = p2;
    }
    double pn = (n == 1) ? z : p1;
    double pm = (n == 1) ? 1.0 : p0;
    dp = n * (z * pn - pm) / (z * z - 1.0);
    // roots come out in descending order; store ascending on [0,1]
    x[n - 1 - i] = 0.5 * (z + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Lagrange polynomials on `nodes`: values/derivatives at point t.
inline void lagrange1d(const std::vector<double>& nodes, double t, std::vector<double>& val,
                       std::vector<double>& der) {
  const int m = (int)nodes.size();
  val.assign(m, 1.0);
  der.assign(m, 0.0);
  for (int a = 0; a < m; ++a) {
    double denom = 1.0;
    for (int b = 0; b < m; ++b)
      if (b != a) denom *= (nodes[a] - nodes[b]);
    double v = 1.0;
    for (int b = 0; b < m; ++b)
      if (b != a) v *= (t - nodes[b]);
    double d = 0.0;
    for (int c = 0; c < m; ++c) {
      if (c == a) continue;
      double term = 1.0;
      for (int b = 0; b < m; ++b)
        if (b != a && b != c) term *= (t - nodes[b]);
      d += term;
    }
    val[a] = v / denom;
    der[a] = d / denom;
  }
}

inline std::vector<double> dgq_nodes(int k) {
  if (k == 0) return {0.5};
  std::vector<double> n(k + 1);
  for (int i = 0; i <= k; ++i) n[i] = double(i) / k;
  return n;
}

// Tables of the carrier element on the unit square.
struct CarrierTables {
  int k = 0, n1 = 0, nq1 = 0, Q = 0;
  std::vector<double> qx, qy, qw;      // cell qp (x fastest)
  std::vector<double> phi, dphi_x, dphi_y;  // [a*Q + q]
  std::vector<double> fq, fw;          // face rule on [0,1]
  std::vector<double> fphi;            // [(f*n1 + a)*nq1 + q]

  explicit CarrierTables(int k_, int nq1_ = -1) : k(k_) {
    nq1 = nq1_ > 0 ? nq1_ : k + 2;
    const int m = k + 1;
    n1 = m * m;
    Q = nq1 * nq1;
    std::vector<double> g, w;
    gauss01(nq1, g, w);
    fq = g;
    fw = w;
    auto nodes = dgq_nodes(k);
    std::vector<std::vector<double>> L(nq1), dL(nq1);
    for (int q = 0; q < nq1; ++q) lagrange1d(nodes, g[q], L[q], dL[q]);
    qx.resize(Q);
    qy.resize(Q);
    qw.resize(Q);
    for (int qy_ = 0; qy_ < nq1; ++qy_)
      for (int qx_ = 0; qx_ < nq1; ++qx_) {
        int q = qx_ + nq1 * qy_;
        qx[q] = g[qx_];
        qy[q] = g[qy_];
        qw[q] = w[qx_] * w[qy_];
      }
    phi.assign(n1 * Q, 0.0);
    dphi_x.assign(n1 * Q, 0.0);
    dphi_y.assign(n1 * Q, 0.0);
    for (int ay = 0; ay < m; ++ay)
      for (int ax = 0; ax < m; ++ax) {
        int a = ax + m * ay;
        for (int qy_ = 0; qy_ < nq1; ++qy_)
          for (int qx_ = 0; qx_ < nq1; ++qx_) {
            int q = qx_ + nq1 * qy_;
            phi[a * Q + q] = L[qx_][ax] * L[qy_][ay];
            dphi_x[a * Q + q] = dL[qx_][ax] * L[qy_][ay];
            dphi_y[a * Q + q] = L[qx_][ax] * dL[qy_][ay];
          }
      }
    std::vector<double> L0, L1, tmp;
    lagrange1d(nodes, 0.0, L0, tmp);
    lagrange1d(nodes, 1.0, L1, tmp);
    fphi.assign(4 * n1 * nq1, 0.0);
    for (int ay = 0; ay < m; ++ay)
      for (int ax = 0; ax < m; ++ax) {
        int a = ax + m * ay;
        for (int q = 0; q < nq1; ++q) {
          fphi[(kLeft * n1 + a) * nq1 + q] = L0[ax] * L[q][ay];
          fphi[(kRight * n1 + a) * nq1 + q] = L1[ax] * L[q][ay];
          fphi[(kBottom * n1 + a) * nq1 + q] = L[q][ax] * L0[ay];
          fphi[(kTop * n1 + a) * nq1 + q] = L[q][ax] * L1[ay];
        }
      }
  }
};

// Tables of the RT_{k-1} x DGQ_{k-1} element on the unit square.
struct PoissonTables {
  int k = 0, n_rt = 0, n_phi = 0, Q = 0, nq1 = 0;
  std::vector<double> psi_x, psi_y, div_x, div_y;  // [i*Q + q]
  std::vector<double> phi;                         // [a*Q + q]
  std::vector<double> fpsi_n;                      // [(f*n_rt + i)*nq1 + q] outward normal comp.
  std::vector<std::vector<int>> face_dofs;         // per face, local RT dofs on it
  std::vector<int> interior_dofs;

  PoissonTables(int k_, const CarrierTables& ct) : k(k_) {
    nq1 = ct.nq1;
    Q = ct.Q;
    const std::vector<double>& g = ct.fq;
    std::vector<double> nn(k + 1), tn(k);
    for (int i = 0; i <= k; ++i) nn[i] = double(i) / k;
    for (int i = 0; i < k; ++i) tn[i] = (i + 0.5) / k;
    std::vector<std::vector<double>> Ln(nq1), dLn(nq1), Lt(nq1), dLt(nq1);
    for (int q = 0; q < nq1; ++q) {
      lagrange1d(nn, g[q], Ln[q], dLn[q]);
      lagrange1d(tn, g[q], Lt[q], dLt[q]);
    }
    std::vector<double> Ln0, Ln1, tmp;
    lagrange1d(nn, 0.0, Ln0, tmp);
    lagrange1d(nn, 1.0, Ln1, tmp);
    const int nxd = k * (k + 1);
    n_rt = 2 * nxd;
    psi_x.assign(n_rt * Q, 0.0);
    psi_y.assign(n_rt * Q, 0.0);
    div_x.assign(n_rt * Q, 0.0);
    div_y.assign(n_rt * Q, 0.0);
    fpsi_n.assign(4 * n_rt * nq1, 0.0);
    face_dofs.assign(4, {});
    for (int b = 0; b < k; ++b)
      for (int a = 0; a <= k; ++a) {
        int i = a + (k + 1) * b;
        for (int qy_ = 0; qy_ < nq1; ++qy_)
          for (int qx_ = 0; qx_ < nq1; ++qx_) {
            int q = qx_ + nq1 * qy_;
            psi_x[i * Q + q] = Ln[qx_][a] * Lt[qy_][b];
            div_x[i * Q + q] = dLn[qx_][a] * Lt[qy_][b];
          }
        for (int q = 0; q < nq1; ++q) {
          fpsi_n[(kLeft * n_rt + i) * nq1 + q] = -Ln0[a] * Lt[q][b];
          fpsi_n[(kRight * n_rt + i) * nq1 + q] = Ln1[a] * Lt[q][b];
        }
        if (a == 0)
          face_dofs[kLeft].push_back(i);
        else if (a == k)
          face_dofs[kRight].push_back(i);
        else
          interior_dofs.push_back(i);
      }
    for (int b = 0; b <= k; ++b)
      for (int a = 0; a < k; ++a) {
        int i = nxd + a + k * b;
        for (int qy_ = 0; qy_ < nq1; ++qy_)
          for (int qx_ = 0; qx_ < nq1; ++qx_) {
            int q = qx_ + nq1 * qy_;
            psi_y[i * Q + q] = Lt[qx_][a] * Ln[qy_][b];
            div_y[i * Q + q] = Lt[qx_][a] * dLn[qy_][b];
          }
        for (int q = 0; q < nq1; ++q) {
          fpsi_n[(kBottom * n_rt + i) * nq1 + q] = -Lt[q][a] * Ln0[b];
          fpsi_n[(kTop * n_rt + i) * nq1 + q] = Lt[q][a] * Ln1[b];
        }
        if (b == 0)
          face_dofs[kBottom].push_back(i);
        else if (b == k)
          face_dofs[kTop].push_back(i);
        else
          interior_dofs.push_back(i);
      }
    const int kp = k - 1;
    auto pn = dgq_nodes(kp);
    n_phi = (kp + 1) * (kp + 1);
    phi.assign(n_phi * Q, 0.0);
    std::vector<std::vector<double>> Lp(nq1), dLp(nq1);
    for (int q = 0; q < nq1; ++q) lagrange1d(pn, g[q], Lp[q], dLp[q]);
    for (int ay = 0; ay <= kp; ++ay)
      for (int ax = 0; ax <= kp; ++ax) {
        int a = ax + (kp + 1) * ay;
        for (int qy_ = 0; qy_ < nq1; ++qy_)
          for (int qx_ = 0; qx_ < nq1; ++qx_) phi[a * Q + qx_ + nq1 * qy_] = Lp[qx_][ax] * Lp[qy_][ay];
      }
  }
};

}  // namespace pecs
