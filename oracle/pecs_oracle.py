"""FP64 CPU restatement of the PECS per-time-step drift-diffusion--Poisson path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function cites the reference routine it restates (paths relative to the
reference project).  Meshes are rectilinear (tensor-product) grids of
axis-aligned rectangles, which covers the uniform meshes the benchmark
configurations use; the reference's trapezoidal nanowire meshes and hanging
nodes are not restated.

Conventions shared with the GPU library (they only fix a basis / numbering,
the discrete solutions are basis independent):

* carrier element = FESystem(FE_DGQ(k)^2, FE_DGQ(k)) (source/SolarCell.cpp:30-31):
  Lagrange basis on equidistant nodes, lexicographic; local dofs
  ``[J_x (n1) | J_y (n1) | u (n1)]`` with ``n1=(k+1)^2``; global numbering is
  component-wise (DoFRenumbering::component_wise, source/CarrierPair.cpp:33):
  ``comp*Nc*n1 + cell*n1 + a``.
* Poisson element = RT_{k-1} x DGQ_{k-1} (source/SolarCell.cpp:23-24).  The RT
  space is spanned by a tensor-product nodal basis (normal direction: k+1
  equidistant nodes incl. the faces; tangential: k nodes (i+1/2)/k), so face
  coefficients are shared between neighbours (H(div) conformity).  Global
  numbering ``[vertical-face dofs | horizontal-face dofs | interior RT | Phi]``.
* cells are numbered lexicographically (i + nx*j); on an interior face the
  "minus" cell is the left/bottom one, which is what deal.II's lower-index rule
  (source/LDG.cpp:375-377) gives on these meshes (cell indices after global
  refinement are Morton ordered, monotone in x and in y).
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# boundary ids, include/SolarCell.hpp:314-324 (Interface is deal.II's default 0)
INTERFACE, DIRICHLET, NEUMANN, SCHOTTKY = 0, 1, 2, 3
# deal.II face numbering of a quadrilateral
LEFT, RIGHT, BOTTOM, TOP = 0, 1, 2, 3
FACE_NORMALS = np.array([[-1.0, 0.0], [1.0, 0.0], [0.0, -1.0], [0.0, 1.0]])

# ---------------------------------------------------------------------------
# 1-D building blocks
# ---------------------------------------------------------------------------


def gauss01(n: int):
    """n-point Gauss-Legendre rule on [0,1] (deal.II QGauss<1>(n))."""
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def lagrange1d(nodes: np.ndarray, x: np.ndarray):
    """Values and derivatives of the Lagrange polynomials on ``nodes`` at ``x``.

    Returns (val, der) with shape (len(nodes), len(x)).
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    m = len(nodes)
    val = np.ones((m, len(x)))
    der = np.zeros((m, len(x)))
    for a in range(m):
        others = [b for b in range(m) if b != a]
        denom = np.prod([nodes[a] - nodes[b] for b in others]) if others else 1.0
        for b in others:
            val[a] *= (x - nodes[b])
        # derivative: sum over dropped factor
        for c in others:
            term = np.ones(len(x))
            for b in others:
                if b != c:
                    term = term * (x - nodes[b])
            der[a] += term
        val[a] /= denom
        der[a] /= denom
    return val, der


def dgq_nodes(k: int) -> np.ndarray:
    """Support points of FE_DGQ(k) on [0,1] (equidistant; k=0 -> centre)."""
    if k == 0:
        return np.array([0.5])
    return np.linspace(0.0, 1.0, k + 1)


# ---------------------------------------------------------------------------
# Reference-element tables
# ---------------------------------------------------------------------------


@dataclass
class CarrierElement:
    """Tables of FESystem(FE_DGQ(k)^dim, FE_DGQ(k)) on the unit square.

    Restates what deal.II FEValues provides for the carrier space
    (include/Assembly.hpp:46-283 holds the FEValues objects).
    """

    k: int
    n1: int
    nq1: int
    # cell quadrature (x fastest)
    qx: np.ndarray
    qy: np.ndarray
    qw: np.ndarray
    phi: np.ndarray      # (n1, Q)
    dphi_x: np.ndarray   # d/dxi  (n1, Q)
    dphi_y: np.ndarray   # d/deta (n1, Q)
    fq: np.ndarray       # face quadrature points on [0,1] (nq1,)
    fw: np.ndarray
    fphi: np.ndarray     # (4, n1, nq1) values on each face

    @staticmethod
    def make(k: int, nq1: Optional[int] = None) -> "CarrierElement":
        nq1 = k + 2 if nq1 is None else nq1
        g, w = gauss01(nq1)
        nodes = dgq_nodes(k)
        L, dL = lagrange1d(nodes, g)
        m = k + 1
        n1 = m * m
        Q = nq1 * nq1
        qx = np.tile(g, nq1)
        qy = np.repeat(g, nq1)
        qw = np.tile(w, nq1) * np.repeat(w, nq1)
        phi = np.zeros((n1, Q))
        dx = np.zeros((n1, Q))
        dy = np.zeros((n1, Q))
        for ay in range(m):
            for ax in range(m):
                a = ax + m * ay
                phi[a] = np.tile(L[ax], nq1) * np.repeat(L[ay], nq1)
                dx[a] = np.tile(dL[ax], nq1) * np.repeat(L[ay], nq1)
                dy[a] = np.tile(L[ax], nq1) * np.repeat(dL[ay], nq1)
        L0, _ = lagrange1d(nodes, np.array([0.0]))
        L1, _ = lagrange1d(nodes, np.array([1.0]))
        fphi = np.zeros((4, n1, nq1))
        for ay in range(m):
            for ax in range(m):
                a = ax + m * ay
                fphi[LEFT, a] = L0[ax, 0] * L[ay]
                fphi[RIGHT, a] = L1[ax, 0] * L[ay]
                fphi[BOTTOM, a] = L[ax] * L0[ay, 0]
                fphi[TOP, a] = L[ax] * L1[ay, 0]
        return CarrierElement(k, n1, nq1, qx, qy, qw, phi, dx, dy, g, w, fphi)


@dataclass
class PoissonElement:
    """Tables of RT_{k-1} x DGQ_{k-1} on the unit square (nodal RT basis).

    Local dofs: ``[D_x (k(k+1)) | D_y (k(k+1)) | Phi (k^2)]``.
    D_x dof (a,b) -> index a + (k+1) b, normal node a in xi, tangential b in eta.
    D_y dof (a,b) -> index k(k+1) + a + k b, tangential a in xi, normal b in eta.
    """

    k: int
    n_rt: int
    n_phi: int
    psi_x: np.ndarray    # (n_rt, Q) x-component of RT basis at cell qp
    psi_y: np.ndarray
    div_x: np.ndarray    # d/dxi part of divergence (for D_x functions) (n_rt, Q)
    div_y: np.ndarray    # d/deta part (for D_y functions)
    phi: np.ndarray      # (n_phi, Q)
    fpsi_n: np.ndarray   # (4, n_rt, nq1): outward-normal component on each face
    face_dofs: list      # face -> list of local RT dof indices on it
    interior_dofs: list

    @staticmethod
    def make(k: int, ce: CarrierElement) -> "PoissonElement":
        g = ce.fq
        nq1 = ce.nq1
        nn = np.linspace(0.0, 1.0, k + 1)            # normal nodes
        tn = (np.arange(k) + 0.5) / k                 # tangential nodes
        Ln, dLn = lagrange1d(nn, g)
        Lt, _ = lagrange1d(tn, g)
        Ln0, _ = lagrange1d(nn, np.array([0.0]))
        Ln1, _ = lagrange1d(nn, np.array([1.0]))
        nx_ = k * (k + 1)
        n_rt = 2 * nx_
        Q = nq1 * nq1
        psi_x = np.zeros((n_rt, Q))
        psi_y = np.zeros((n_rt, Q))
        div_x = np.zeros((n_rt, Q))
        div_y = np.zeros((n_rt, Q))
        fpsi_n = np.zeros((4, n_rt, nq1))
        face_dofs = [[], [], [], []]
        interior = []
        for b in range(k):
            for a in range(k + 1):
                i = a + (k + 1) * b
                psi_x[i] = np.tile(Ln[a], nq1) * np.repeat(Lt[b], nq1)
                div_x[i] = np.tile(dLn[a], nq1) * np.repeat(Lt[b], nq1)
                fpsi_n[LEFT, i] = -Ln0[a, 0] * Lt[b]
                fpsi_n[RIGHT, i] = Ln1[a, 0] * Lt[b]
                if a == 0:
                    face_dofs[LEFT].append(i)
                elif a == k:
                    face_dofs[RIGHT].append(i)
                else:
                    interior.append(i)
        for b in range(k + 1):
            for a in range(k):
                i = nx_ + a + k * b
                psi_y[i] = np.tile(Lt[a], nq1) * np.repeat(Ln[b], nq1)
                div_y[i] = np.tile(Lt[a], nq1) * np.repeat(dLn[b], nq1)
                fpsi_n[BOTTOM, i] = -Lt[a] * Ln0[b, 0]
                fpsi_n[TOP, i] = Lt[a] * Ln1[b, 0]
                if b == 0:
                    face_dofs[BOTTOM].append(i)
                elif b == k:
                    face_dofs[TOP].append(i)
                else:
                    interior.append(i)
        kp = k - 1
        pn = dgq_nodes(kp)
        Lp, _ = lagrange1d(pn, g)
        n_phi = (kp + 1) ** 2
        phi = np.zeros((n_phi, Q))
        for ay in range(kp + 1):
            for ax in range(kp + 1):
                phi[ax + (kp + 1) * ay] = np.tile(Lp[ax], nq1) * np.repeat(Lp[ay], nq1)
        return PoissonElement(k, n_rt, n_phi, psi_x, psi_y, div_x, div_y, phi,
                              fpsi_n, face_dofs, interior)


# ---------------------------------------------------------------------------
# Rectilinear grids (restates Grid_Maker::Grid, source/Grid.cpp:44-133,
# 340-503, for axis-aligned rectangles)
# ---------------------------------------------------------------------------


@dataclass
class RectGrid:
    xs: np.ndarray   # (nx+1,) column edges
    ys: np.ndarray   # (ny+1,) row edges
    bc: tuple        # boundary id of (left, right, bottom, top) sides
    material: np.ndarray = None  # (nc,) 0 semiconductor, 2 electrolyte (include/Grid.hpp:150-156)
    # cells with i >= split take bc2's id (where > 0) on their outer faces: the
    # Poisson mesh over the electrolyte, whose sides may change id at the
    # interface (Grid.cpp:377-431); split < 0: one id per side
    split: int = -1
    bc2: tuple = (0, 0, 0, 0)

    @property
    def nx(self):
        return len(self.xs) - 1

    @property
    def ny(self):
        return len(self.ys) - 1

    @property
    def nc(self):
        return self.nx * self.ny

    def cell_ij(self):
        K = np.arange(self.nc)
        return K % self.nx, K // self.nx

    def cell_geom(self):
        i, j = self.cell_ij()
        x0 = self.xs[i]
        y0 = self.ys[j]
        hx = self.xs[i + 1] - x0
        hy = self.ys[j + 1] - y0
        return x0, y0, hx, hy

    def face_bid(self, K: int, f: int) -> Optional[int]:
        """Boundary id of face f of cell K, None for an interior face."""
        i, j = K % self.nx, K // self.nx
        outer = ((f == LEFT and i == 0) or (f == RIGHT and i == self.nx - 1)
                 or (f == BOTTOM and j == 0) or (f == TOP and j == self.ny - 1))
        if not outer:
            return None
        if self.split >= 0 and i >= self.split and self.bc2[f] > 0:
            return self.bc2[f]
        return self.bc[f]


def uniform_grid(x0, x1, y0, y1, nx, ny, bc, material=0) -> RectGrid:
    g = RectGrid(np.linspace(x0, x1, nx + 1), np.linspace(y0, y1, ny + 1), tuple(bc))
    g.material = np.full(g.nc, material, dtype=np.int64)
    return g


def graded_coords(x0: float, x1: float, n: int, grading: float, fine_at_x1: bool) -> np.ndarray:
    """n + 1 points on [x0, x1] whose cell widths shrink by the constant factor
    q = grading^(1/(n-1)) toward x1 (fine_at_x1) or toward x0: widest/narrowest
    = grading.  grading <= 1 gives numpy.linspace's points."""
    if not grading > 1.0:
        return np.linspace(x0, x1, n + 1)
    q = grading ** (1.0 / (n - 1))
    w = np.empty(n)
    w[0] = 1.0
    for i in range(1, n):
        w[i] = w[i - 1] / q
    if not fine_at_x1:
        w = w[::-1].copy()
    S = np.concatenate([[0.0], np.cumsum(w)])
    xs = x0 + (x1 - x0) * (S / S[n])
    xs[n] = x1
    return xs


def region_grid(x0, x1, y0, y1, nx, ny, bc, grading, fine_at_x1, material=0) -> RectGrid:
    g = RectGrid(graded_coords(x0, x1, nx, grading, fine_at_x1), np.linspace(y0, y1, ny + 1),
                 tuple(bc))
    g.material = np.full(g.nc, material, dtype=np.int64)
    return g


# ---------------------------------------------------------------------------
# Parameters (already-scaled, restates the role of ParameterSpace::Parameters,
# include/Parameters.hpp:27-289; the benchmark configurations override the
# reference's hard-coded profiles through the *_kind switches)
# ---------------------------------------------------------------------------


@dataclass
class Params:
    degree: int = 1
    full_system: bool = True
    nx_semi: int = 16
    nx_elec: int = 16
    ny: int = 16
    x_semi0: float = 0.0
    x_semi1: float = 1.0
    x_elec1: float = 2.0
    height: float = 1.0
    bc_semi: tuple = (DIRICHLET, INTERFACE, NEUMANN, NEUMANN)
    bc_elec: tuple = (INTERFACE, DIRICHLET, NEUMANN, NEUMANN)
    bc_poisson: tuple = (DIRICHLET, DIRICHLET, NEUMANN, NEUMANN)
    lambda2: float = 1e-2        # scaled Debye length^2 (Parameters.hpp:198-205)
    eps_semi: float = 1.0
    eps_elec: float = 1.5
    mu: tuple = (1.0, 1.0, 1.0, 1.0)   # electrons, holes, reductants, oxidants
    dt: float = 1e-3
    penalty: float = 1.0         # SolarCell.cpp:1944-1945
    k_et: float = 1e-2
    k_ht: float = 1e-2
    # doping / equilibrium profiles: value_left for x < junction_x else value_right
    junction_x: float = 0.5
    nd: tuple = (1.0, 1.0)
    na: tuple = (0.0, 0.0)
    n_eq: tuple = (1.0, 1.0)
    p_eq: tuple = (1e-4, 1e-4)
    r_eq: float = 1.0
    o_eq: float = 1.0
    ic_kind: int = 0             # 0: equilibrium densities, 1: doping profile
    gen_kind: int = 2            # 0 off, 1 reference alpha*G0*exp(alpha*(y-H)), 2 G0*exp(-alpha*(x1-x))
    G0: float = 1.0
    alpha: float = 5.0
    srh: bool = True
    tau_n: float = 1.0
    tau_p: float = 1.0
    n_i: float = 1e-2
    phi_bi: float = 0.0
    phi_app: float = 0.0
    s_n: float = 0.0             # Schottky recombination velocities (SolarCell.cpp:1386-1401)
    s_p: float = 0.0
    # widest / narrowest cell width of each region along x, cells narrowing
    # geometrically toward the interface x = x_semi1 (<= 1: uniform).  A
    # boundary layer on a tensor-product mesh, in place of the reference's
    # local refinement with hanging nodes (Grid.cpp:71-111).
    grading: float = 1.0
    # full system: ids of the Poisson mesh's outer faces over the electrolyte
    # (left unused, right, bottom, top); entries <= 0 take bc_poisson's id
    bc_poisson_elec: tuple = (0, 0, 0, 0)
    # Poisson element: 0 = RT_{k-1} x DGQ_{k-1}, the reference's pairing
    # (source/SolarCell.cpp:23-24); 1 = RT_k x DGQ_k, the pairing the benchmark
    # configurations name
    poisson_pairing: int = 0

    def copy(self, **kw) -> "Params":
        return dataclasses.replace(self, **kw)


def reference_params(n_refine: int = 4, degree: int = 1, **kw) -> Params:
    """Reference-faithful physics (what the reference code hard-codes): constant equilibria
    2, 0, 30, 29 (source/InitialConditions.cpp:5-82), SRH returning 0
    (include/SolarCell.hpp:86-98), generation alpha*G0*exp(alpha*(y-H))
    (source/Generation.cpp:29-44), potential data Phi_bi - Phi_app on x==0
    (source/BiasValues.cpp:11-31,75-94)."""
    n = 2 ** n_refine
    p = Params(degree=degree, nx_semi=n, nx_elec=n, ny=n, nd=(2.0, 2.0), na=(0.0, 0.0),
               n_eq=(2.0, 2.0), p_eq=(0.0, 0.0), r_eq=30.0, o_eq=29.0, ic_kind=0,
               gen_kind=1, srh=False, bc_semi=(DIRICHLET, INTERFACE, DIRICHLET, DIRICHLET),
               bc_elec=(INTERFACE, DIRICHLET, DIRICHLET, DIRICHLET),
               bc_poisson=(DIRICHLET, DIRICHLET, DIRICHLET, DIRICHLET))
    return p.copy(**kw)


def pn_junction_params(**kw) -> Params:
    """Semiconductor-only p-n junction, unit square, 16x16, k=1, 100 steps."""
    n_i = 1e-2
    p = Params(degree=1, full_system=False, nx_semi=16, nx_elec=0, ny=16,
               bc_semi=(DIRICHLET, DIRICHLET, NEUMANN, NEUMANN),
               bc_poisson=(DIRICHLET, DIRICHLET, NEUMANN, NEUMANN),
               lambda2=1e-2, eps_semi=1.0, mu=(1.0, 1.0, 1.0, 1.0), dt=1e-3,
               junction_x=0.5, nd=(1.0, 0.0), na=(0.0, 1.0),
               n_eq=(1.0, n_i * n_i), p_eq=(n_i * n_i, 1.0), ic_kind=1,
               gen_kind=0, srh=True, tau_n=1.0, tau_p=1.0, n_i=n_i,
               phi_bi=math.log(1.0 * 1.0 / (n_i * n_i)), phi_app=0.0,
               k_et=0.0, k_ht=0.0)
    return p.copy(**kw)


def half_cell_params(n_refine: int = 6, **kw) -> Params:
    """Coupled half cell: semi [0,1]^2, electrolyte [1,2]x[0,1], 2^r x 2^r each."""
    n_i = 1e-2
    n = 2 ** n_refine
    p = Params(degree=1, full_system=True, nx_semi=n, nx_elec=n, ny=n,
               lambda2=1e-2, eps_semi=1.0, eps_elec=1.5, dt=1e-3,
               nd=(1.0, 1.0), na=(0.0, 0.0), n_eq=(1.0, 1.0), p_eq=(n_i * n_i, n_i * n_i),
               r_eq=1.0, o_eq=1.0, ic_kind=0, gen_kind=2, G0=1.0, alpha=5.0,
               srh=True, tau_n=1.0, tau_p=1.0, n_i=n_i, k_et=1e-2, k_ht=1e-2,
               phi_bi=0.0, phi_app=0.0)
    return p.copy(**kw)


# ---------------------------------------------------------------------------
# Coefficient functions (source/InitialConditions.cpp, Generation.cpp,
# BiasValues.cpp, include/SolarCell.hpp:86-98)
# ---------------------------------------------------------------------------


def _pw(x, pair, xj):
    return np.where(x < xj, pair[0], pair[1]).astype(np.float64)


def donor(P: Params, x, y):
    return _pw(x, P.nd, P.junction_x)


def acceptor(P: Params, x, y):
    return _pw(x, P.na, P.junction_x)


def n_equilibrium(P: Params, x, y):
    return _pw(x, P.n_eq, P.junction_x)


def p_equilibrium(P: Params, x, y):
    return _pw(x, P.p_eq, P.junction_x)


def generation(P: Params, x, y):
    """Generation<dim>::value (source/Generation.cpp:29-44) or the config form."""
    if P.gen_kind == 0:
        return np.zeros_like(x)
    if P.gen_kind == 1:
        return P.alpha * P.G0 * np.exp(P.alpha * (y - P.height))
    return P.G0 * np.exp(-P.alpha * (P.x_semi1 - x))


def srh(P: Params, n, p):
    """SRH_Recombination (include/SolarCell.hpp:86-98; documented formula
    include/SolarCell.hpp:71-77).  Zero in reference-faithful mode."""
    if not P.srh:
        return np.zeros_like(n)
    ni = P.n_i
    return (ni * ni - n * p) / (P.tau_n * (n + ni) + P.tau_p * (p + ni))


def potential_dirichlet(P: Params, x, y):
    """Built_In_Bias - Applied_Bias (source/BiasValues.cpp:11-31, 75-94):
    non-zero only where x == 0 exactly; Bulk_Bias is identically 0."""
    return np.where(x == 0.0, P.phi_bi - P.phi_app, 0.0)


# ---------------------------------------------------------------------------
# Discretisation object
# ---------------------------------------------------------------------------


@dataclass
class CarrierSpace:
    grid: RectGrid
    ce: CarrierElement
    nc: int
    n1: int
    ndofs: int

    def dofs(self, K):
        """Global dofs of cell(s) K -> array (..., 3*n1), local order [Jx|Jy|u]."""
        K = np.asarray(K)
        n1 = self.n1
        a = np.arange(n1)
        blocks = [c * self.nc * n1 + K[..., None] * n1 + a for c in range(3)]
        return np.concatenate(blocks, axis=-1)

    def u_dofs(self, K):
        K = np.asarray(K)
        return 2 * self.nc * self.n1 + K[..., None] * self.n1 + np.arange(self.n1)


@dataclass
class PoissonSpace:
    grid: RectGrid
    pe: PoissonElement
    nc: int
    n_rt: int
    ndofs: int
    l2g: np.ndarray    # (nc, n_rt + n_phi)
    constrained: np.ndarray  # bool (ndofs,)


def make_carrier_space(grid: RectGrid, k: int) -> CarrierSpace:
    ce = CarrierElement.make(k)
    return CarrierSpace(grid, ce, grid.nc, ce.n1, 3 * grid.nc * ce.n1)


def make_poisson_space(grid: RectGrid, k: int, ce: CarrierElement) -> PoissonSpace:
    """DoF distribution of RT_{k-1} x DGQ_{k-1} plus the zero D.n constraints on
    Neumann faces (PoissonData::setup_dofs, source/Poisson.cpp:18-69)."""
    pe = PoissonElement.make(k, ce)
    nx, ny, nc = grid.nx, grid.ny, grid.nc
    nvert = (nx + 1) * ny
    nhor = nx * (ny + 1)
    nint = 2 * k * (k - 1)
    off_h = nvert * k
    off_i = off_h + nhor * k
    off_phi = off_i + nc * nint
    n_rt_total = off_phi
    ndofs = off_phi + nc * pe.n_phi
    l2g = np.zeros((nc, pe.n_rt + pe.n_phi), dtype=np.int64)
    i_, j_ = grid.cell_ij()
    nxd = k * (k + 1)
    for K in range(nc):
        i, j = i_[K], j_[K]
        # D_x dofs
        cnt_int = 0
        for b in range(k):
            for a in range(k + 1):
                loc = a + (k + 1) * b
                if a == 0:
                    l2g[K, loc] = (i + (nx + 1) * j) * k + b
                elif a == k:
                    l2g[K, loc] = (i + 1 + (nx + 1) * j) * k + b
                else:
                    l2g[K, loc] = off_i + K * nint + cnt_int
                    cnt_int += 1
        for b in range(k + 1):
            for a in range(k):
                loc = nxd + a + k * b
                if b == 0:
                    l2g[K, loc] = off_h + (i + nx * j) * k + a
                elif b == k:
                    l2g[K, loc] = off_h + (i + nx * (j + 1)) * k + a
                else:
                    l2g[K, loc] = off_i + K * nint + cnt_int
                    cnt_int += 1
        for a in range(pe.n_phi):
            l2g[K, pe.n_rt + a] = off_phi + K * pe.n_phi + a
    constrained = np.zeros(ndofs, dtype=bool)
    for K in range(nc):
        for f in range(4):
            if grid.face_bid(K, f) == NEUMANN:
                constrained[l2g[K, pe.face_dofs[f]]] = True
    return PoissonSpace(grid, pe, nc, n_rt_total, ndofs, l2g, constrained)


# ---------------------------------------------------------------------------
# Matrix assembly
# ---------------------------------------------------------------------------


def _carrier_point_tables(ce: CarrierElement, hx: float, hy: float):
    """Per local dof: (px, py, v, divp, gvx, gvy) at the cell qp for a hx*hy cell."""
    n1, Q = ce.phi.shape
    z = np.zeros((n1, Q))
    px = np.concatenate([ce.phi, z, z])
    py = np.concatenate([z, ce.phi, z])
    v = np.concatenate([z, z, ce.phi])
    divp = np.concatenate([ce.dphi_x / hx, ce.dphi_y / hy, z])
    gvx = np.concatenate([z, z, ce.dphi_x / hx])
    gvy = np.concatenate([z, z, ce.dphi_y / hy])
    return px, py, v, divp, gvx, gvy


def _carrier_face_tables(ce: CarrierElement, f: int):
    n1, nq = ce.fphi.shape[1:]
    z = np.zeros((n1, nq))
    fp = ce.fphi[f]
    px = np.concatenate([fp, z, z])
    py = np.concatenate([z, fp, z])
    v = np.concatenate([z, z, fp])
    return px, py, v


def ldg_local_cell_matrix(ce, hx, hy, mu, dt, tos, pen_h, bids):
    """assemble_local_LDG_cell_and_bc_terms (source/LDG.cpp:85-281) for one
    rectangle with boundary ids ``bids`` (None for interior faces)."""
    px, py, v, divp, gvx, gvy = _carrier_point_tables(ce, hx, hy)
    JxW = ce.qw * hx * hy
    A = ((tos / dt) * (v * JxW) @ v.T
         + (1.0 / mu) * ((px * JxW) @ px.T + (py * JxW) @ py.T)
         - (divp * JxW) @ v.T
         - ((gvx * JxW) @ px.T + (gvy * JxW) @ py.T))
    for f in range(4):
        bid = bids[f]
        if bid is None:
            continue
        fpx, fpy, fv = _carrier_face_tables(ce, f)
        nvec = FACE_NORMALS[f]
        flen = hy if f in (LEFT, RIGHT) else hx
        Jf = ce.fw * flen
        pn = fpx * nvec[0] + fpy * nvec[1]
        if bid == DIRICHLET:
            # v (n.q + pen/h u)
            A += (fv * Jf) @ (pn + pen_h * fv).T
        elif bid in (INTERFACE, NEUMANN, SCHOTTKY):
            # (p.n) u
            A += (pn * Jf) @ fv.T
        else:
            raise ValueError(bid)
    return A


def ldg_local_flux_matrices(ce, fminus, fplus, flen, pen_h):
    """assemble_local_flux_terms (source/LDG.cpp:429-622): the four interior
    face blocks; beta=(1,1)/sqrt(2) enters as beta.p (LDG.cpp:455-458)."""
    mpx, mpy, mv = _carrier_face_tables(ce, fminus)
    ppx, ppy, pv = _carrier_face_tables(ce, fplus)
    nvec = FACE_NORMALS[fminus]
    beta = np.array([1.0, 1.0]) / math.sqrt(2.0)
    Jf = ce.fw * flen
    mpn = mpx * nvec[0] + mpy * nvec[1]
    ppn = ppx * nvec[0] + ppy * nvec[1]
    mbp = mpx * beta[0] + mpy * beta[1]
    pbp = ppx * beta[0] + ppy * beta[1]

    def blk(tp_n, tv, tbp, rv, rp_n, rbp, s_half, s_beta, s_pen):
        # s_half*0.5*(p_i.n u_j + v_i n.q_j) + s_beta*((beta.p_i) u_j - v_i (beta.q_j)) + s_pen*pen v_i u_j
        return ((tp_n * Jf) @ rv.T * (0.5 * s_half) + (tv * Jf) @ rp_n.T * (0.5 * s_half)
                + s_beta * ((tbp * Jf) @ rv.T - (tv * Jf) @ rbp.T)
                + s_pen * pen_h * (tv * Jf) @ rv.T)

    vi_ui = blk(mpn, mv, mbp, mv, mpn, mbp, +1, +1, +1)
    vi_ue = blk(mpn, mv, mbp, pv, ppn, pbp, +1, -1, -1)
    ve_ui = blk(ppn, pv, pbp, mv, mpn, mbp, -1, -1, -1)
    ve_ue = blk(ppn, pv, pbp, pv, ppn, pbp, -1, +1, +1)
    return vi_ui, vi_ue, ve_ui, ve_ue


def assemble_ldg_matrices(cs: CarrierSpace, mu: float, dt: float, penalty: float, tos: float = 1.0):
    """assemble_LDG_system (source/SolarCell.cpp:822-932): system matrix of one
    carrier and the (1/dt) mass matrix (source/LDG.cpp:40-83)."""
    g, ce = cs.grid, cs.ce
    x0, y0, hx, hy = g.cell_geom()
    diam = np.sqrt(hx * hx + hy * hy)     # cell->diameter() of a rectangle
    rows, cols, vals = [], [], []
    mrows, mcols, mvals = [], [], []
    cache = {}
    for K in range(g.nc):
        bids = tuple(g.face_bid(K, f) for f in range(4))
        key = (hx[K], hy[K], bids)
        if key not in cache:
            cache[key] = ldg_local_cell_matrix(ce, hx[K], hy[K], mu, dt, tos, penalty / diam[K], bids)
        A = cache[key]
        d = cs.dofs(K)
        rows.append(np.repeat(d, len(d)))
        cols.append(np.tile(d, len(d)))
        vals.append(A.ravel())
        # mass (1/dt) int v u
        ud = cs.u_dofs(K)
        Mloc = (1.0 / dt) * (ce.phi * (ce.qw * hx[K] * hy[K])) @ ce.phi.T
        mrows.append(np.repeat(ud, len(ud)))
        mcols.append(np.tile(ud, len(ud)))
        mvals.append(Mloc.ravel())
    # interior faces: minus = left/bottom
    fcache = {}
    nx, ny = g.nx, g.ny
    for K in range(g.nc):
        i, j = K % nx, K // nx
        for (fm, fp, nb, ok) in ((RIGHT, LEFT, K + 1, i < nx - 1), (TOP, BOTTOM, K + nx, j < ny - 1)):
            if not ok:
                continue
            flen = hy[K] if fm == RIGHT else hx[K]
            h = min(diam[K], diam[nb])
            key = (fm, flen, h)
            if key not in fcache:
                fcache[key] = ldg_local_flux_matrices(ce, fm, fp, flen, penalty / h)
            vi_ui, vi_ue, ve_ui, ve_ue = fcache[key]
            dm, dp = cs.dofs(K), cs.dofs(nb)
            for (B, r, c) in ((vi_ui, dm, dm), (vi_ue, dm, dp), (ve_ui, dp, dm), (ve_ue, dp, dp)):
                rows.append(np.repeat(r, len(c)))
                cols.append(np.tile(c, len(r)))
                vals.append(B.ravel())
    n = cs.ndofs
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    M = sp.csr_matrix((np.concatenate(mvals), (np.concatenate(mrows), np.concatenate(mcols))), shape=(n, n))
    A.sum_duplicates()
    M.sum_duplicates()
    return A, M


def poisson_local_matrix(pe: PoissonElement, ce: CarrierElement, hx, hy, eps, lambda2):
    """MixedFEM::assemble_local_Poisson_matrix (source/MixedFEM.cpp:29-164):
    p.(1/eps)D - div(p) Phi - lambda^2 v div(D)."""
    JxW = ce.qw * hx * hy
    n_rt, n_phi = pe.n_rt, pe.n_phi
    div = pe.div_x / hx + pe.div_y / hy
    Z = np.zeros((n_rt + n_phi, n_rt + n_phi))
    Z[:n_rt, :n_rt] = (1.0 / eps) * ((pe.psi_x * JxW) @ pe.psi_x.T + (pe.psi_y * JxW) @ pe.psi_y.T)
    Z[:n_rt, n_rt:] = -(div * JxW) @ pe.phi.T
    Z[n_rt:, :n_rt] = -lambda2 * (pe.phi * JxW) @ div.T
    return Z


def assemble_poisson_matrix(ps: PoissonSpace, ce: CarrierElement, eps_semi, eps_elec, lambda2):
    """assemble_Poisson_matrix (source/SolarCell.cpp:377-406) with the zero
    D.n constraints applied as deal.II's distribute_local_to_global does
    (constrained rows/columns eliminated, unit diagonal)."""
    g, pe = ps.grid, ps.pe
    x0, y0, hx, hy = g.cell_geom()
    rows, cols, vals = [], [], []
    cache = {}
    for K in range(g.nc):
        eps = eps_semi if g.material[K] in (0, 1) else eps_elec
        key = (hx[K], hy[K], eps)
        if key not in cache:
            cache[key] = poisson_local_matrix(pe, ce, hx[K], hy[K], eps, lambda2)
        d = ps.l2g[K]
        rows.append(np.repeat(d, len(d)))
        cols.append(np.tile(d, len(d)))
        vals.append(cache[key].ravel())
    n = ps.ndofs
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    A.sum_duplicates()
    return apply_constraints(A, ps.constrained)


def apply_constraints(A: sp.csr_matrix, constrained: np.ndarray) -> sp.csr_matrix:
    if not constrained.any():
        return A
    keep = sp.diags((~constrained).astype(np.float64))
    A = (keep @ A @ keep).tocsr()
    A = A + sp.diags(constrained.astype(np.float64))
    A = A.tocsr()
    A.eliminate_zeros()
    A.sort_indices()
    return A


# ---------------------------------------------------------------------------
# Problem: meshes, maps, constant RHS parts, time loop
# ---------------------------------------------------------------------------


class Problem:
    """Restates SOLARCELL::SolarCellProblem::run_full_system's setup and IMEX
    loop (source/SolarCell.cpp:1898-2095)."""

    def __init__(self, P: Params):
        self.P = P
        k = P.degree
        self.semi_grid = region_grid(P.x_semi0, P.x_semi1, 0.0, P.height, P.nx_semi, P.ny,
                                     P.bc_semi, P.grading, True, material=0)
        self.semi = make_carrier_space(self.semi_grid, k)
        ce = self.semi.ce
        self.ce = ce
        if P.full_system:
            self.elec_grid = region_grid(P.x_semi1, P.x_elec1, 0.0, P.height, P.nx_elec, P.ny,
                                         P.bc_elec, P.grading, False, material=2)
            self.elec = make_carrier_space(self.elec_grid, k)
            xs = np.concatenate([self.semi_grid.xs, self.elec_grid.xs[1:]])
            pg = RectGrid(xs, self.semi_grid.ys.copy(), tuple(P.bc_poisson), split=P.nx_semi,
                          bc2=tuple(P.bc_poisson_elec))
            ci, cj = pg.cell_ij()
            pg.material = np.where(ci < P.nx_semi, 0, 2)
        else:
            self.elec_grid = None
            self.elec = None
            pg = RectGrid(self.semi_grid.xs.copy(), self.semi_grid.ys.copy(), tuple(P.bc_poisson))
            pg.material = np.zeros(pg.nc, dtype=np.int64)
        self.poisson_grid = pg
        self.pois = make_poisson_space(pg, k + P.poisson_pairing, ce)
        # carrier cell -> Poisson cell maps (setup_mappings, SolarCell.cpp:264-372)
        si, sj = self.semi_grid.cell_ij()
        self.s2p = si + pg.nx * sj
        if P.full_system:
            ei, ej = self.elec_grid.cell_ij()
            self.e2p = (ei + P.nx_semi) + pg.nx * ej
            # interface pairing (SolarCell.cpp:160-259): semi right face <-> elec left face
            self.iface_semi = np.array([K for K in range(self.semi_grid.nc)
                                        if self.semi_grid.face_bid(K, RIGHT) == INTERFACE])
            self.iface_elec = np.array([K for K in range(self.elec_grid.nc)
                                        if self.elec_grid.face_bid(K, LEFT) == INTERFACE])
            assert len(self.iface_semi) == len(self.iface_elec)
        self._assemble_matrices()
        self._precompute_rhs_tables()

    # -- setup ---------------------------------------------------------------
    def _assemble_matrices(self):
        P = self.P
        self.A_n, self.M_semi = assemble_ldg_matrices(self.semi, P.mu[0], P.dt, P.penalty)
        self.A_p, _ = assemble_ldg_matrices(self.semi, P.mu[1], P.dt, P.penalty)
        if P.full_system:
            self.A_r, self.M_elec = assemble_ldg_matrices(self.elec, P.mu[2], P.dt, P.penalty)
            self.A_o, _ = assemble_ldg_matrices(self.elec, P.mu[3], P.dt, P.penalty)
        self.A_P = assemble_poisson_matrix(self.pois, self.ce, P.eps_semi, P.eps_elec, P.lambda2)
        self._lu = {}

    def lu(self, name):
        """SparseDirectUMFPACK::initialize restated by scipy's sparse LU
        (Carrier.cpp:26-32, Poisson.cpp:90-96).  The LDG carrier matrices have
        a symmetric pattern (flux sparsity, CarrierPair.cpp:44-48), for which
        UMFPACK's default strategy is its symmetric one: a fill-reducing
        ordering of A + A^T and diagonal pivots preferred down to a relative
        tolerance of 0.001.  SuperLU's symmetric mode with the same tolerance
        does that (a third of COLAMD's fill here).  The mixed Poisson matrix
        keeps COLAMD with partial pivoting (its potential block has a zero
        diagonal)."""
        if name not in self._lu:
            A = getattr(self, "A_" + name).tocsc()
            if name == "P":
                self._lu[name] = spla.splu(A, permc_spec="COLAMD")
            else:
                self._lu[name] = spla.splu(A, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.001,
                                           options=dict(SymmetricMode=True))
        return self._lu[name]

    def lu_solve(self, name, b):
        """SparseDirectUMFPACK::solve / vmult (Carrier.cpp:34-40,
        Poisson.cpp:98-105): deal.II hands UMFPACK the matrix with the
        factors, and UMFPACK's default control then refines the solution (up
        to UMFPACK_IRSTEP = 2 steps, stopping once the componentwise backward
        error max_i |b - A x|_i / (|A| |x| + |b|)_i is at machine precision).
        Restated with FP64 residuals."""
        lu = self.lu(name)
        A = getattr(self, "A_" + name)
        if not hasattr(self, "_absA"):
            self._absA = {}
        if name not in self._absA:
            self._absA[name] = abs(A).tocsr()
        x = lu.solve(b)
        for _ in range(2):
            r = b - A @ x
            den = self._absA[name] @ np.abs(x) + np.abs(b)
            omega = np.max(np.abs(r)[den > 0] / den[den > 0]) if np.any(den > 0) else 0.0
            if omega <= np.finfo(np.float64).eps:
                break
            x = x + lu.solve(r)
        return x

    def _cell_points(self, grid):
        x0, y0, hx, hy = grid.cell_geom()
        ce = self.ce
        X = x0[:, None] + hx[:, None] * ce.qx[None, :]
        Y = y0[:, None] + hy[:, None] * ce.qy[None, :]
        JxW = (hx * hy)[:, None] * ce.qw[None, :]
        return X, Y, JxW

    def _face_points(self, grid, K, f):
        x0, y0, hx, hy = grid.cell_geom()
        g = self.ce.fq
        if f == LEFT:
            X, Y, L = np.full_like(g, x0[K]), y0[K] + hy[K] * g, hy[K]
        elif f == RIGHT:
            X, Y, L = np.full_like(g, x0[K] + hx[K]), y0[K] + hy[K] * g, hy[K]
        elif f == BOTTOM:
            X, Y, L = x0[K] + hx[K] * g, np.full_like(g, y0[K]), hx[K]
        else:
            X, Y, L = x0[K] + hx[K] * g, np.full_like(g, y0[K] + hy[K]), hx[K]
        return X, Y, self.ce.fw * L

    def _precompute_rhs_tables(self):
        """Time-independent parts of the carrier and Poisson right-hand sides:
        generation and Dirichlet data (SolarCell.cpp:1146-1264, 1572-1629,
        583-684, 762-813), plus the qp tables used every step."""
        P, ce = self.P, self.ce
        self.sX, self.sY, self.sJxW = self._cell_points(self.semi_grid)
        # carrier constant parts
        self.bconst = {}
        regions = [("semi", self.semi, self.semi_grid, ("n", "p"))]
        if P.full_system:
            regions.append(("elec", self.elec, self.elec_grid, ("r", "o")))
        for (rname, cs, grid, names) in regions:
            X, Y, JxW = self._cell_points(grid)
            x0, y0, hx, hy = grid.cell_geom()
            diam = np.sqrt(hx * hx + hy * hy)
            for cname in names:
                b = np.zeros(cs.ndofs)
                if rname == "semi":
                    G = generation(P, X, Y)
                    ud = cs.u_dofs(np.arange(grid.nc))
                    np.add.at(b, ud, np.einsum("aq,kq->ka", ce.phi, G * JxW))
                for K in range(grid.nc):
                    for f in range(4):
                        if grid.face_bid(K, f) != DIRICHLET:
                            continue
                        fx, fy, Jf = self._face_points(grid, K, f)
                        uD = self._bc_value(cname, fx, fy)
                        fpx, fpy, fv = _carrier_face_tables(ce, f)
                        nvec = FACE_NORMALS[f]
                        pn = fpx * nvec[0] + fpy * nvec[1]
                        loc = (-pn + (P.penalty / diam[K]) * fv) @ (uD * Jf)
                        np.add.at(b, cs.dofs(K), loc)
                self.bconst[cname] = b
        # Poisson constant part: doping (semi cells) + Dirichlet potential faces
        ps, pe = self.pois, self.pois.pe
        bP = np.zeros(ps.ndofs)
        pX, pY, pJxW = self._cell_points(self.poisson_grid)
        semi_cells = np.nonzero(self.poisson_grid.material == 0)[0]
        dop = donor(P, pX, pY) - acceptor(P, pX, pY)
        loc = -np.einsum("aq,kq->ka", pe.phi, (dop * pJxW)[semi_cells])
        np.add.at(bP, ps.l2g[semi_cells, pe.n_rt:], loc)
        pg = self.poisson_grid
        for K in range(pg.nc):
            for f in range(4):
                if pg.face_bid(K, f) != DIRICHLET:
                    continue
                fx, fy, Jf = self._face_points(pg, K, f)
                phiD = potential_dirichlet(P, fx, fy)
                loc = -(pe.fpsi_n[f] @ (phiD * Jf))
                np.add.at(bP, ps.l2g[K, :pe.n_rt], loc)
        bP[ps.constrained] = 0.0
        self.bconst["P"] = bP
        # interface equilibria at the semi face qp
        if P.full_system:
            self.iface_pts = [self._face_points(self.semi_grid, K, RIGHT) for K in self.iface_semi]

    def _bc_value(self, cname, x, y):
        P = self.P
        if cname == "n":
            return n_equilibrium(P, x, y)
        if cname == "p":
            return p_equilibrium(P, x, y)
        if cname == "r":
            return np.full_like(x, P.r_eq)
        return np.full_like(x, P.o_eq)

    # -- state -----------------------------------------------------------------
    def initial_state(self):
        """Initial conditions (SolarCell.cpp:1996-2034): L2 projection of the
        equilibrium (or doping) profiles onto DGQ_k, zero currents; then the
        initial Poisson solve."""
        P, ce = self.P, self.ce
        st = {}
        names = [("n", self.semi, self.semi_grid), ("p", self.semi, self.semi_grid)]
        if P.full_system:
            names += [("r", self.elec, self.elec_grid), ("o", self.elec, self.elec_grid)]
        g1, w1 = gauss01(P.degree + 1)
        L, _ = lagrange1d(dgq_nodes(P.degree), g1)
        m = P.degree + 1
        Q = len(g1) ** 2
        phiq = np.zeros((m * m, Q))
        for ay in range(m):
            for ax in range(m):
                phiq[ax + m * ay] = np.tile(L[ax], len(g1)) * np.repeat(L[ay], len(g1))
        wq = np.tile(w1, len(g1)) * np.repeat(w1, len(g1))
        Mref = (phiq * wq) @ phiq.T
        for (cname, cs, grid) in names:
            x0, y0, hx, hy = grid.cell_geom()
            X = x0[:, None] + hx[:, None] * np.tile(g1, len(g1))[None, :]
            Y = y0[:, None] + hy[:, None] * np.repeat(g1, len(g1))[None, :]
            if P.ic_kind == 1 and cname in ("n", "p"):
                f = donor(P, X, Y) if cname == "n" else acceptor(P, X, Y)
            else:
                f = self._bc_value(cname, X, Y)
            rhs = (f * wq) @ phiq.T            # (nc, n1)
            coef = np.linalg.solve(Mref, rhs.T).T
            u = np.zeros(cs.ndofs)
            u[cs.u_dofs(np.arange(grid.nc))] = coef
            st[cname] = u
        st["P"] = self.solve_poisson(self.poisson_rhs(st))
        return st

    def densities_at_qp(self, cs, u):
        U = u[cs.u_dofs(np.arange(cs.nc))]      # (nc, n1)
        return U @ self.ce.phi                  # (nc, Q)

    def field_at_qp(self, phiP, cells_p):
        """D (the RT part of the Poisson solution) at the carrier qp of the
        matching Poisson cells (the ElectricField extractor,
        SolarCell.cpp:1139-1141)."""
        pe, ps = self.pois.pe, self.pois
        Dl = phiP[ps.l2g[cells_p, :pe.n_rt]]     # (nc, n_rt)
        return Dl @ pe.psi_x, Dl @ pe.psi_y

    # -- per-step assembly ----------------------------------------------------
    def carrier_rhs(self, st):
        """assemble_semiconductor_rhs / assemble_electrolyte_rhs
        (SolarCell.cpp:1037-1726) for all carriers."""
        P, ce = self.P, self.ce
        out = {}
        regs = [("semi", self.semi, self.semi_grid, self.s2p, ("n", "p"), (-1.0, 1.0), P.eps_semi,
                 self.M_semi)]
        if P.full_system:
            regs.append(("elec", self.elec, self.elec_grid, self.e2p, ("r", "o"), (-1.0, 1.0),
                         P.eps_elec, self.M_elec))
        dens = {}
        for (rname, cs, grid, c2p, names, charges, eps, M) in regs:
            X, Y, JxW = self._cell_points(grid)
            Ex, Ey = self.field_at_qp(st["P"], c2p)
            uq = [self.densities_at_qp(cs, st[c]) for c in names]
            dens[names[0]], dens[names[1]] = uq
            K = np.arange(grid.nc)
            for ci, cname in enumerate(names):
                b = M @ st[cname] + self.bconst[cname]
                # drift: q/eps (p_i . D) u_old
                w = charges[ci] / eps * uq[ci] * JxW
                rx = np.einsum("aq,kq->ka", ce.phi, Ex * w)
                ry = np.einsum("aq,kq->ka", ce.phi, Ey * w)
                n1, nc = cs.n1, cs.nc
                b[0 * nc * n1:1 * nc * n1] += rx.ravel()
                b[1 * nc * n1:2 * nc * n1] += ry.ravel()
                if rname == "semi" and P.srh:
                    R = srh(P, uq[0], uq[1])
                    b[cs.u_dofs(K)] += np.einsum("aq,kq->ka", ce.phi, R * JxW)
                out[cname] = b
        if P.full_system:
            self._interface_terms(st, out)
        if P.s_n != 0.0 or P.s_p != 0.0:
            self._schottky_terms(st, out)
        return out

    def _interface_terms(self, st, out):
        """Interface Robin transfer (SolarCell.cpp:1265-1347, 1630-1716)."""
        P, ce = self.P, self.ce
        fs = ce.fphi[RIGHT]    # semi side test functions on its interface face
        fe = ce.fphi[LEFT]
        for idx, (Ks, Ke) in enumerate(zip(self.iface_semi, self.iface_elec)):
            fx, fy, Jf = self.iface_pts[idx]
            n = st["n"][self.semi.u_dofs(Ks)] @ fs
            p = st["p"][self.semi.u_dofs(Ks)] @ fs
            r = st["r"][self.elec.u_dofs(Ke)] @ fe
            o = st["o"][self.elec.u_dofs(Ke)] @ fe
            ne = n_equilibrium(P, fx, fy)
            pe_ = p_equilibrium(P, fx, fy)
            tn = -P.k_et * (n - ne) * o * Jf
            tp = +P.k_ht * (p - pe_) * r * Jf
            out["n"][self.semi.u_dofs(Ks)] += fs @ tn
            out["p"][self.semi.u_dofs(Ks)] += fs @ tp
            cur = fe @ (tn + tp)
            out["r"][self.elec.u_dofs(Ke)] += cur
            out["o"][self.elec.u_dofs(Ke)] -= cur

    def _schottky_terms(self, st, out):
        """Schottky faces (SolarCell.cpp:1348-1404)."""
        P, ce, g = self.P, self.ce, self.semi_grid
        for K in range(g.nc):
            for f in range(4):
                if g.face_bid(K, f) != SCHOTTKY:
                    continue
                fx, fy, Jf = self._face_points(g, K, f)
                ft = ce.fphi[f]
                n = st["n"][self.semi.u_dofs(K)] @ ft
                p = st["p"][self.semi.u_dofs(K)] @ ft
                out["n"][self.semi.u_dofs(K)] += ft @ (-P.s_n * (n - n_equilibrium(P, fx, fy)) * Jf)
                out["p"][self.semi.u_dofs(K)] += ft @ (+P.s_p * (p - p_equilibrium(P, fx, fy)) * Jf)

    def poisson_rhs(self, st):
        """assemble_Poisson_rhs (SolarCell.cpp:430-815): -(v, N_D-N_A + sum q_i u_i)
        on semiconductor cells, -(v, sum q_i u_i) on electrolyte cells, plus the
        constant Dirichlet part."""
        P, pe, ps = self.P, self.pois.pe, self.pois
        b = self.bconst["P"].copy()
        regs = [(self.semi, self.semi_grid, self.s2p, ("n", "p"))]
        if P.full_system:
            regs.append((self.elec, self.elec_grid, self.e2p, ("r", "o")))
        for (cs, grid, c2p, names) in regs:
            X, Y, JxW = self._cell_points(grid)
            rho = -self.densities_at_qp(cs, st[names[0]]) + self.densities_at_qp(cs, st[names[1]])
            loc = -np.einsum("aq,kq->ka", pe.phi, rho * JxW)
            np.add.at(b, ps.l2g[c2p, pe.n_rt:], loc)
        b[ps.constrained] = 0.0
        return b

    def solve_poisson(self, b):
        """PoissonData::solve (Poisson.cpp:98-105): LU apply, then distribute
        (homogeneous constraints -> 0)."""
        x = self.lu_solve("P", b)
        x[self.pois.constrained] = 0.0
        return x

    def step(self, st):
        """One IMEX step (SolarCell.cpp:2055-2080)."""
        rhs = self.carrier_rhs(st)
        new = {}
        for c in ("n", "p", "r", "o"):
            if c in rhs:
                new[c] = self.lu_solve(c, rhs[c])
        new["P"] = self.solve_poisson(self.poisson_rhs(new))
        return new

    # -- observables ------------------------------------------------------------
    def interface_current(self, st) -> float:
        """I_Sigma = int_Sigma [k_et (n-n_e) o - k_ht (p-p_e) r] ds, the same
        integrand as SolarCell.cpp:1692-1705 with v == 1."""
        if not self.P.full_system:
            return 0.0
        P, ce = self.P, self.ce
        tot = 0.0
        for idx, (Ks, Ke) in enumerate(zip(self.iface_semi, self.iface_elec)):
            fx, fy, Jf = self.iface_pts[idx]
            n = st["n"][self.semi.u_dofs(Ks)] @ ce.fphi[RIGHT]
            p = st["p"][self.semi.u_dofs(Ks)] @ ce.fphi[RIGHT]
            r = st["r"][self.elec.u_dofs(Ke)] @ ce.fphi[LEFT]
            o = st["o"][self.elec.u_dofs(Ke)] @ ce.fphi[LEFT]
            tot += np.sum((P.k_et * (n - n_equilibrium(P, fx, fy)) * o
                           - P.k_ht * (p - p_equilibrium(P, fx, fy)) * r) * Jf)
        return float(tot)

    def field_names(self):
        return ("n", "p", "r", "o", "P") if self.P.full_system else ("n", "p", "P")

    @staticmethod
    def rel_change(new, old, names) -> float:
        """max over fields of ||new-old||_2 / ||new||_2 (steady-state test)."""
        r = 0.0
        for c in names:
            den = np.linalg.norm(new[c])
            r = max(r, np.linalg.norm(new[c] - old[c]) / (den if den > 0 else 1.0))
        return r

    def run(self, n_steps: int, st=None, tol: float = 0.0):
        """March n_steps (or until the relative change <= tol if tol > 0)."""
        st = self.initial_state() if st is None else st
        taken = 0
        last = math.inf
        for _ in range(n_steps):
            new = self.step(st)
            taken += 1
            if tol > 0.0:
                last = self.rel_change(new, st, self.field_names())
            st = new
            if tol > 0.0 and last <= tol:
                break
        return st, taken, last


__all__ = [n for n in dir() if not n.startswith("_")]
