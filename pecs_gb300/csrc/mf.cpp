// Multifrontal LU: ordering, symbolic analysis, numeric factorisation (see mf.hpp).
#include "mf.hpp"

#include "dense.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <thread>

namespace pecs {

long long MfFactor::entries() const {
  long long e = 0;
  for (const MfNode& nd : nodes) e += 2LL * nd.s * (nd.s + nd.m);
  return e;
}

int MfFactor::max_front() const {
  int f = 0;
  for (const MfNode& nd : nodes) f = std::max(f, nd.s + nd.m);
  return f;
}

namespace {

struct Pattern {  // symmetric structure of A + A^T (nonzero values only) without the diagonal
  std::vector<int> ptr, idx;
};

Pattern symmetric_pattern(const Csr& A) {
  const int n = A.n;
  std::vector<int> cnt(n + 1, 0);
  for (int i = 0; i < n; ++i)
    for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; ++p) {
      int k = A.col[p];
      if (k == i || A.val[p] == 0.0) continue;
      cnt[i + 1]++;
      cnt[k + 1]++;
    }
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> idx(cnt[n]);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; ++p) {
      int k = A.col[p];
      if (k == i || A.val[p] == 0.0) continue;
      idx[fill[i]++] = k;
      idx[fill[k]++] = i;
    }
  Pattern P;
  P.ptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    auto b = idx.begin() + cnt[i], e = idx.begin() + cnt[i + 1];
    std::sort(b, e);
    auto u = std::unique(b, e);
    for (auto it = b; it != u; ++it) P.idx.push_back(*it);
    P.ptr[i + 1] = (int)P.idx.size();
  }
  return P;
}

struct NdCtx {
  const std::vector<std::vector<int>>* adj;
  const double* xy;
  int leaf;
  std::vector<std::vector<int>> groups;  // postorder
  std::vector<int> mark;
};

void nested_dissection(NdCtx& C, std::vector<int> cells) {
  if ((int)cells.size() <= C.leaf) {
    C.groups.push_back(std::move(cells));
    return;
  }
  double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
  for (int c : cells) {
    xmin = std::min(xmin, C.xy[2 * c]);
    xmax = std::max(xmax, C.xy[2 * c]);
    ymin = std::min(ymin, C.xy[2 * c + 1]);
    ymax = std::max(ymax, C.xy[2 * c + 1]);
  }
  const int ax = (xmax - xmin >= ymax - ymin) ? 0 : 1;
  const double ext = std::max(xmax - xmin, ymax - ymin);
  const double tol = 1e-9 * (ext > 0 ? ext : 1.0);
  std::vector<double> keys;
  keys.reserve(cells.size());
  for (int c : cells) keys.push_back(C.xy[2 * c + ax]);
  std::vector<double> vals = keys;
  std::sort(vals.begin(), vals.end());
  std::vector<double> uv;
  for (double v : vals)
    if (uv.empty() || v - uv.back() > tol) uv.push_back(v);
  const double m = uv[uv.size() / 2];
  std::vector<int> L, S, R;
  for (size_t t = 0; t < cells.size(); ++t) {
    if (keys[t] < m - tol)
      L.push_back(cells[t]);
    else if (keys[t] > m + tol)
      R.push_back(cells[t]);
    else
      S.push_back(cells[t]);
  }
  // separator fix-up: L cells adjacent to R join S
  for (int c : R) C.mark[c] = 2;
  std::vector<int> L2;
  for (int c : L) {
    bool touch = false;
    for (int nb : (*C.adj)[c])
      if (C.mark[nb] == 2) {
        touch = true;
        break;
      }
    if (touch)
      S.push_back(c);
    else
      L2.push_back(c);
  }
  for (int c : R) C.mark[c] = 0;
  if (!L2.empty()) nested_dissection(C, std::move(L2));
  if (!R.empty()) nested_dissection(C, std::move(R));
  std::sort(S.begin(), S.end());
  C.groups.push_back(std::move(S));
}

}  // namespace

MfFactor mf_analyze(const Csr& A, const int* dof_cell, const int* dof_class, int n_cells,
                    const double* cell_xy, int leaf_cells) {
  const int n = A.n;
  if (n <= 0) throw std::runtime_error("empty matrix");
  if ((int)A.rowptr.size() != n + 1) throw std::runtime_error("bad rowptr");
  for (int i = 0; i < n; ++i) {
    if (A.rowptr[i + 1] < A.rowptr[i]) throw std::runtime_error("rowptr not monotone");
    if (dof_cell[i] < 0 || dof_cell[i] >= n_cells) throw std::runtime_error("dof_cell out of range");
  }
  for (int p = 0; p < A.rowptr[n]; ++p)
    if (A.col[p] < 0 || A.col[p] >= n) throw std::runtime_error("column index out of range");
  if (leaf_cells <= 0) leaf_cells = 8;
  auto cls = [&](int i) { return dof_class ? dof_class[i] : 1; };
  Pattern P = symmetric_pattern(A);
  // class-0 validation
  for (int i = 0; i < n; ++i) {
    if (cls(i) != 0) continue;
    for (int p = P.ptr[i]; p < P.ptr[i + 1]; ++p) {
      int k = P.idx[p];
      if (cls(k) == 0 && dof_cell[k] != dof_cell[i])
        throw std::runtime_error("class-0 dofs of different cells are coupled");
    }
  }
  // dofs per cell by class
  std::vector<std::vector<int>> c0(n_cells), c1(n_cells);
  for (int i = 0; i < n; ++i) (cls(i) == 0 ? c0 : c1)[dof_cell[i]].push_back(i);
  // reduced quotient graph over cells (class-1 couplings + fill of class-0 elimination)
  std::vector<std::vector<int>> adj(n_cells);
  auto add_edge = [&](int a, int b) {
    if (a == b) return;
    adj[a].push_back(b);
    adj[b].push_back(a);
  };
  for (int i = 0; i < n; ++i) {
    if (cls(i) == 0) continue;
    for (int p = P.ptr[i]; p < P.ptr[i + 1]; ++p) {
      int k = P.idx[p];
      if (cls(k) != 0) add_edge(dof_cell[i], dof_cell[k]);
    }
  }
  std::vector<int> nb;
  for (int L = 0; L < n_cells; ++L) {
    if (c0[L].empty()) continue;
    nb.clear();
    for (int i : c0[L])
      for (int p = P.ptr[i]; p < P.ptr[i + 1]; ++p) {
        int k = P.idx[p];
        if (cls(k) != 0) nb.push_back(dof_cell[k]);
      }
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    for (size_t a = 0; a < nb.size(); ++a)
      for (size_t b = a + 1; b < nb.size(); ++b) add_edge(nb[a], nb[b]);
  }
  for (auto& v : adj) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  // nested dissection over cells that own class-1 dofs
  NdCtx C;
  C.adj = &adj;
  C.xy = cell_xy;
  C.leaf = leaf_cells;
  C.mark.assign(n_cells, 0);
  std::vector<int> cells1;
  for (int c = 0; c < n_cells; ++c)
    if (!c1[c].empty()) cells1.push_back(c);
  if (!cells1.empty()) nested_dissection(C, cells1);

  MfFactor F;
  F.n = n;
  F.node_of.assign(n, -1);
  std::vector<char> is_c0;
  for (int L = 0; L < n_cells; ++L) {
    if (c0[L].empty()) continue;
    for (int i : c0[L]) F.node_of[i] = (int)is_c0.size();
    is_c0.push_back(1);
  }
  for (auto& g : C.groups) {
    if (g.empty()) continue;
    int id = (int)is_c0.size();
    for (int c : g)
      for (int i : c1[c]) F.node_of[i] = id;
    is_c0.push_back(0);
  }
  const int nn0 = (int)is_c0.size();
  // zero-diagonal dofs move to the latest node holding a dof of their row
  std::vector<double> diag(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; ++p)
      if (A.col[p] == i) diag[i] += A.val[p];
  std::vector<int> moved = F.node_of;
  for (int i = 0; i < n; ++i) {
    if (cls(i) == 0 || diag[i] != 0.0) continue;
    int t = F.node_of[i];
    for (int p = P.ptr[i]; p < P.ptr[i + 1]; ++p) t = std::max(t, F.node_of[P.idx[p]]);
    moved[i] = t;
  }
  F.node_of = moved;
  std::vector<std::vector<int>> own(nn0);
  for (int i = 0; i < n; ++i) own[F.node_of[i]].push_back(i);
  // drop empty nodes, renumber
  std::vector<int> remap(nn0, -1);
  for (int j = 0; j < nn0; ++j)
    if (!own[j].empty()) {
      remap[j] = (int)F.nodes.size();
      MfNode nd;
      nd.own = own[j];
      nd.s = (int)nd.own.size();
      nd.cls0 = is_c0[j] != 0;
      F.nodes.push_back(std::move(nd));
    }
  for (int i = 0; i < n; ++i) F.node_of[i] = remap[F.node_of[i]];
  F.pos.assign(n, -1);
  int cnt = 0;
  for (auto& nd : F.nodes)
    for (int i : nd.own) F.pos[i] = cnt++;
  // symbolic factorisation
  const int N = (int)F.nodes.size();
  std::vector<int> stamp(n, -1);
  for (int j = 0; j < N; ++j) {
    MfNode& nd = F.nodes[j];
    const int hi = F.pos[nd.own.back()];
    std::vector<int> U;
    for (int i : nd.own)
      for (int p = P.ptr[i]; p < P.ptr[i + 1]; ++p) {
        int k = P.idx[p];
        if (F.pos[k] > hi && stamp[k] != j) {
          stamp[k] = j;
          U.push_back(k);
        }
      }
    for (int c : nd.children)
      for (int k : F.nodes[c].upd)
        if (F.pos[k] > hi && stamp[k] != j) {
          stamp[k] = j;
          U.push_back(k);
        }
    std::sort(U.begin(), U.end(), [&](int a, int b) { return F.pos[a] < F.pos[b]; });
    nd.upd = std::move(U);
    nd.m = (int)nd.upd.size();
    if (nd.m > 0) {
      nd.parent = F.node_of[nd.upd[0]];
      F.nodes[nd.parent].children.push_back(j);
    }
    int h = 0;
    for (int c : nd.children) h = std::max(h, F.nodes[c].height + 1);
    nd.height = h;
    F.n_heights = std::max(F.n_heights, h + 1);
  }
  for (int j = N - 1; j >= 0; --j) {
    MfNode& nd = F.nodes[j];
    nd.depth = nd.parent < 0 ? 0 : F.nodes[nd.parent].depth + 1;
    F.n_depths = std::max(F.n_depths, nd.depth + 1);
  }
  return F;
}

namespace {

// Factor one node's front.  Returns the update matrix S (m x m).
std::vector<double> factor_node(MfFactor& F, int j, const Csr& A, const Csr& AT,
                                std::vector<std::vector<double>>& Sstore, std::vector<int>& fpos,
                                double& flops, dense::Team* team, const FrontOffload* off) {
  MfNode& nd = F.nodes[j];
  const int s = nd.s, m = nd.m, f = s + m;
  std::vector<double> Fm((size_t)f * f, 0.0);
  for (int t = 0; t < s; ++t) fpos[nd.own[t]] = t;
  for (int t = 0; t < m; ++t) fpos[nd.upd[t]] = s + t;
  const int lo = F.pos[nd.own.front()], hi = F.pos[nd.own.back()];
  for (int t = 0; t < s; ++t) {
    const int i = nd.own[t];
    for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; ++p) {
      int k = A.col[p];
      if (F.pos[k] < lo || A.val[p] == 0.0) continue;  // explicit zeros carry no structure
      int c = fpos[k];
      if (c < 0) throw std::runtime_error("symbolic structure mismatch (row)");
      Fm[(size_t)t * f + c] += A.val[p];
    }
    for (int p = AT.rowptr[i]; p < AT.rowptr[i + 1]; ++p) {
      int k = AT.col[p];  // A(k, i)
      if (F.pos[k] <= hi || AT.val[p] == 0.0) continue;
      int r = fpos[k];
      if (r < 0) throw std::runtime_error("symbolic structure mismatch (col)");
      Fm[(size_t)r * f + t] += AT.val[p];
    }
  }
  for (int c : nd.children) {
    const MfNode& ch = F.nodes[c];
    std::vector<double>& S = Sstore[c];
    const int mc = ch.m;
    std::vector<int> map(mc);
    for (int a = 0; a < mc; ++a) {
      map[a] = fpos[ch.upd[a]];
      if (map[a] < 0) throw std::runtime_error("extend-add structure mismatch");
    }
    for (int a = 0; a < mc; ++a) {
      double* row = &Fm[(size_t)map[a] * f];
      const double* srow = &S[(size_t)a * mc];
      for (int b = 0; b < mc; ++b) row[map[b]] += srow[b];
    }
    std::vector<double>().swap(S);
  }
  // partial pivoting LU on the first s columns, pivots among the s fully-summed rows
  std::vector<int> perm(s);
  double colmax_all = 0.0;
  for (size_t t = 0; t < (size_t)s * f; ++t) colmax_all = std::max(colmax_all, std::fabs(Fm[t]));
  double bad = 0.0;
  if (off && off->factor && f >= off->min_front) {
    // the same factorisation on the device
    std::vector<double> S;
    const int bc = off->factor(off->ctx, f, s, Fm.data(), 1e-14 * colmax_all, perm.data(), &bad, F.Gf[j],
                               F.Hb[j], S);
    if (bc >= 0) {
      std::ostringstream e;
      e << "singular pivot " << bad << " at node " << j << " column " << bc << " (front " << s << "+" << m
        << ")";
      throw std::runtime_error(e.str());
    }
    for (int col = 0; col < s; ++col) flops += 2.0 * (double)(f - col - 1) * (double)(f - col - 1);
    flops += 2.0 * s * s * (double)(s + m);
    for (int t = 0; t < s; ++t) fpos[nd.own[t]] = -1;
    for (int t = 0; t < m; ++t) fpos[nd.upd[t]] = -1;
    return S;
  }
  const int badcol = dense::lu_front(f, s, Fm.data(), f, perm.data(), 1e-14 * colmax_all, &bad, team);
  if (badcol >= 0) {
    std::ostringstream e;
    e << "singular pivot " << bad << " at node " << j << " column " << badcol << " (front " << s
      << "+" << m << ")";
    throw std::runtime_error(e.str());
  }
  for (int col = 0; col < s; ++col) flops += 2.0 * (double)(f - col - 1) * (double)(f - col - 1);
  // update matrix
  std::vector<double> S((size_t)m * m);
  for (int a = 0; a < m; ++a)
    std::copy_n(&Fm[(size_t)(s + a) * f + s], m, &S[(size_t)a * m]);
  // Gf = [L11^-1 P ; L21 L11^-1 P]
  std::vector<double> X((size_t)f * s, 0.0);
  dense::inv_unit_lower(s, Fm.data(), f, X.data(), s, team);
  dense::trmm(false, true, m, s, 1.0, X.data(), s, &Fm[(size_t)s * f], f, &X[(size_t)s * s], s, team);
  std::vector<double>& G = F.Gf[j];
  G.assign((size_t)f * s, 0.0);
  for (int r = 0; r < f; ++r)
    for (int t = 0; t < s; ++t) G[(size_t)r * s + perm[t]] = X[(size_t)r * s + t];
  std::vector<double>().swap(X);
  // Hb = [U11^-1 | -U11^-1 U12]
  std::vector<double>& H = F.Hb[j];
  H.assign((size_t)s * f, 0.0);
  dense::inv_upper(s, Fm.data(), f, H.data(), f, team);
  dense::trmm(true, false, s, m, -1.0, H.data(), f, &Fm[s], f, &H[s], f, team);
  for (int t = 0; t < s; ++t) fpos[nd.own[t]] = -1;
  for (int t = 0; t < m; ++t) fpos[nd.upd[t]] = -1;
  flops += 2.0 * s * s * (double)(s + m);
  return S;
}

Csr transpose(const Csr& A) {
  Csr T;
  T.n = A.n;
  T.rowptr.assign(A.n + 1, 0);
  for (int p = 0; p < A.rowptr[A.n]; ++p) T.rowptr[A.col[p] + 1]++;
  for (int i = 0; i < A.n; ++i) T.rowptr[i + 1] += T.rowptr[i];
  T.col.resize(A.col.size());
  T.val.resize(A.val.size());
  std::vector<int> fill(T.rowptr.begin(), T.rowptr.end() - 1);
  for (int i = 0; i < A.n; ++i)
    for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; ++p) {
      int q = fill[A.col[p]]++;
      T.col[q] = i;
      T.val[q] = A.val[p];
    }
  return T;
}

}  // namespace

void mf_factorize(MfFactor& F, const Csr& A, int n_threads, const FrontOffload* off) {
  const int N = (int)F.nodes.size();
  Csr AT = transpose(A);
  F.Gf.assign(N, {});
  F.Hb.assign(N, {});
  std::vector<std::vector<double>> Sstore(N);
  if (n_threads <= 0) {
    unsigned hc = std::thread::hardware_concurrency();
    n_threads = (int)std::max(1u, std::min(hc, 16u));
  }
  // nodes of equal height are independent: factor them in parallel, height by
  // height.  Wide levels run one node per thread; narrow levels (the top of the
  // tree, few large fronts) give each node a team that shares its dense work.
  std::vector<std::vector<int>> by_h(F.n_heights);
  for (int j = 0; j < N; ++j) by_h[F.nodes[j].height].push_back(j);
  double flops = 0.0;
  std::string err;
  std::mutex mu;
  for (auto& lvl : by_h) {
    const int L = (int)lvl.size();
    const int nt = std::min(n_threads, L);
    const int per_node = std::max(1, n_threads / std::max(1, L));
    std::atomic<size_t> next(0);
    auto worker = [&]() {
      std::vector<int> fpos(F.n, -1);
      std::unique_ptr<dense::Team> team;
      if (per_node > 1) team.reset(new dense::Team(per_node));
      double fl = 0.0;
      for (;;) {
        size_t t = next.fetch_add(1);
        if (t >= lvl.size()) break;
        int j = lvl[t];
        try {
          Sstore[j] = factor_node(F, j, A, AT, Sstore, fpos, fl, team.get(), off);
        } catch (const std::exception& e) {
          std::lock_guard<std::mutex> g(mu);
          if (err.empty()) err = e.what();
        }
      }
      std::lock_guard<std::mutex> g(mu);
      flops += fl;
    };
    dense::run_threads(std::max(1, nt), [&](int) { worker(); });
    if (!err.empty()) throw std::runtime_error(err);
  }
  F.factor_flops = flops;
}

void mf_apply_host(const MfFactor& F, const double* b, double* x) {
  const int N = (int)F.nodes.size();
  std::vector<std::vector<double>> w(N);
  std::vector<double> y(F.n, 0.0);
  std::vector<int> fpos(F.n, -1);
  for (int j = 0; j < N; ++j) {
    const MfNode& nd = F.nodes[j];
    const int s = nd.s, m = nd.m;
    for (int t = 0; t < s; ++t) fpos[nd.own[t]] = t;
    for (int t = 0; t < m; ++t) fpos[nd.upd[t]] = s + t;
    std::vector<double> d(s), cu(m, 0.0);
    for (int t = 0; t < s; ++t) d[t] = b[nd.own[t]];
    for (int c : nd.children) {
      const MfNode& ch = F.nodes[c];
      for (int a = 0; a < ch.m; ++a) {
        int p = fpos[ch.upd[a]];
        if (p < s)
          d[p] -= w[c][a];
        else
          cu[p - s] += w[c][a];
      }
      std::vector<double>().swap(w[c]);
    }
    const std::vector<double>& G = F.Gf[j];
    for (int r = 0; r < s; ++r) {
      double acc = 0.0;
      for (int c2 = 0; c2 < s; ++c2) acc += G[(size_t)r * s + c2] * d[c2];
      y[nd.own[r]] = acc;
    }
    w[j].assign(m, 0.0);
    for (int r = 0; r < m; ++r) {
      double acc = cu[r];
      for (int c2 = 0; c2 < s; ++c2) acc += G[(size_t)(s + r) * s + c2] * d[c2];
      w[j][r] = acc;
    }
    for (int t = 0; t < s; ++t) fpos[nd.own[t]] = -1;
    for (int t = 0; t < m; ++t) fpos[nd.upd[t]] = -1;
  }
  for (int j = N - 1; j >= 0; --j) {
    const MfNode& nd = F.nodes[j];
    const int s = nd.s, m = nd.m, f = s + m;
    std::vector<double> v(f);
    for (int t = 0; t < s; ++t) v[t] = y[nd.own[t]];
    for (int t = 0; t < m; ++t) v[s + t] = x[nd.upd[t]];
    const std::vector<double>& H = F.Hb[j];
    for (int r = 0; r < s; ++r) {
      double acc = 0.0;
      for (int c2 = 0; c2 < f; ++c2) acc += H[(size_t)r * f + c2] * v[c2];
      x[nd.own[r]] = acc;
    }
  }
}

}  // namespace pecs
