"""The reference's known-answer tests, restated on the oracle.

TEST INFRASTRUCTURE ONLY.

* ``poisson_mixed_errors`` -- the mixed-FEM half of ``test_steady_state``
  (source/SolarCell.cpp:2749-2860, tests/Poisson_test.cpp): manufactured
  Phi = cos(2 pi y) - sin(2 pi x) - x on the unit square, Dirichlet x=0,1,
  zero D.n on y=0,1 (Grid.cpp:464-503), lambda^2 = eps = 1
  (Parameters.hpp:88-107).  Analytic data: source/test_functions.cpp:13-93.
* ``ldg_imex_errors`` -- ``test_transient`` (source/SolarCell.cpp:2865-2965,
  tests/IMEX_LDG_test.cpp): u = e^{-t} + cos 2 pi x + cos 2 pi y, fixed field
  E = (1,0) (LDG.cpp:856-858), dt = h^{k+1}, t_end = 1, Dirichlet x=0,
  Interface data on x=1, Neumann y=0,1 (Grid.cpp:531-568).  Analytic data:
  source/test_functions.cpp:99-220, initial condition 1 + cos(2 pi x)cos(2 pi y)
  (test_functions.cpp:429-440).

The reference only prints its convergence tables; the rates asserted in
``tests/`` are the theoretical ones for these elements.

Both studies solve with scipy's sparse LU unless ``solver`` is given: a
factory ``solver(A, space, kind)`` (kind "poisson" or "carrier") returning a
function b -> x, through which the tests run the same studies on the
library's multifrontal solver.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse.linalg as spla

from .pecs_oracle import (BOTTOM, DIRICHLET, FACE_NORMALS, INTERFACE, LEFT, NEUMANN, RIGHT, TOP,
                          _carrier_face_tables, assemble_ldg_matrices, assemble_poisson_matrix,
                          dgq_nodes, gauss01, lagrange1d, make_carrier_space, make_poisson_space,
                          region_grid, CarrierElement, PoissonElement)

TWO_PI = 2.0 * math.pi


def _face_points(grid, K, f, g, w):
    x0, y0, hx, hy = grid.cell_geom()
    if f == LEFT:
        return np.full_like(g, x0[K]), y0[K] + hy[K] * g, w * hy[K]
    if f == RIGHT:
        return np.full_like(g, x0[K] + hx[K]), y0[K] + hy[K] * g, w * hy[K]
    if f == BOTTOM:
        return x0[K] + hx[K] * g, np.full_like(g, y0[K]), w * hx[K]
    return x0[K] + hx[K] * g, np.full_like(g, y0[K] + hy[K]), w * hx[K]


def _fine_rule(nq=8):
    g, w = gauss01(nq)
    return np.tile(g, nq), np.repeat(g, nq), np.tile(w, nq) * np.repeat(w, nq)


def _scipy_solver(A, space, kind):
    lu = spla.splu(A.tocsc())
    return lu.solve


def poisson_mixed_errors(n_refine: int, k: int = 1, solver=None, grading: float = 1.0):
    """Returns (h, ||Phi-Phi_h||_L2, ||D-D_h||_L2).  grading > 1: cells graded
    along x toward x = 1 (widest/narrowest = grading)."""
    n = 2 ** n_refine
    grid = region_grid(0.0, 1.0, 0.0, 1.0, n, n, (DIRICHLET, DIRICHLET, NEUMANN, NEUMANN), grading,
                       True)
    ce = CarrierElement.make(k)
    ps = make_poisson_space(grid, k, ce)
    pe = ps.pe
    A = assemble_poisson_matrix(ps, ce, 1.0, 1.0, 1.0)
    b = np.zeros(ps.ndofs)
    x0, y0, hx, hy = grid.cell_geom()
    X = x0[:, None] + hx[:, None] * ce.qx
    Y = y0[:, None] + hy[:, None] * ce.qy
    JxW = (hx * hy)[:, None] * ce.qw
    f = 4 * math.pi ** 2 * (np.cos(TWO_PI * Y) - np.sin(TWO_PI * X))
    np.add.at(b, ps.l2g[:, pe.n_rt:], -np.einsum("aq,kq->ka", pe.phi, f * JxW))
    for K in range(grid.nc):
        for fc in range(4):
            if grid.face_bid(K, fc) != DIRICHLET:
                continue
            fx, fy, Jf = _face_points(grid, K, fc, ce.fq, ce.fw)
            gD = np.cos(TWO_PI * fy) - np.sin(TWO_PI * fx) - fx
            np.add.at(b, ps.l2g[K, :pe.n_rt], -(pe.fpsi_n[fc] @ (gD * Jf)))
    b[ps.constrained] = 0.0
    sol = (solver or _scipy_solver)(A, ps, "poisson")(b)
    sol[ps.constrained] = 0.0
    # errors on a fine Gauss rule
    qx, qy, qw = _fine_rule()
    fce = CarrierElement.make(k, nq1=8)
    fpe = PoissonElement.make(k, fce)
    Xf = x0[:, None] + hx[:, None] * qx
    Yf = y0[:, None] + hy[:, None] * qy
    Wf = (hx * hy)[:, None] * qw
    loc = sol[ps.l2g]
    Dx = loc[:, :pe.n_rt] @ fpe.psi_x
    Dy = loc[:, :pe.n_rt] @ fpe.psi_y
    Ph = loc[:, pe.n_rt:] @ fpe.phi
    Pt = np.cos(TWO_PI * Yf) - np.sin(TWO_PI * Xf) - Xf
    Dxt = 1 + TWO_PI * np.cos(TWO_PI * Xf)
    Dyt = TWO_PI * np.sin(TWO_PI * Yf)
    e_phi = math.sqrt(np.sum((Ph - Pt) ** 2 * Wf))
    e_D = math.sqrt(np.sum(((Dx - Dxt) ** 2 + (Dy - Dyt) ** 2) * Wf))
    return math.sqrt(2.0) / n, e_phi, e_D


def ldg_imex_errors(n_refine: int, k: int = 1, t_end: float = 1.0, solver=None,
                    grading: float = 1.0):
    """Returns (h, ||u-u_h||_L2, ||J-J_h||_L2, n_steps) at the final time.
    grading > 1: cells graded along x toward x = 1."""
    n = 2 ** n_refine
    grid = region_grid(0.0, 1.0, 0.0, 1.0, n, n, (DIRICHLET, INTERFACE, NEUMANN, NEUMANN), grading,
                       True)
    cs = make_carrier_space(grid, k)
    ce = cs.ce
    h = math.sqrt(2.0) / n
    dt = h ** (k + 1)
    penalty = 1.0
    A, M = assemble_ldg_matrices(cs, 1.0, dt, penalty, tos=1.0)
    solve = (solver or _scipy_solver)(A, cs, "carrier")
    x0, y0, hx, hy = grid.cell_geom()
    diam = np.sqrt(hx ** 2 + hy ** 2)
    X = x0[:, None] + hx[:, None] * ce.qx
    Y = y0[:, None] + hy[:, None] * ce.qy
    JxW = (hx * hy)[:, None] * ce.qw
    nc, n1 = cs.nc, cs.n1
    allK = np.arange(nc)
    # initial condition: projection with QGauss(k+1) of 1 + cos(2pi x)cos(2pi y)
    g1, w1 = gauss01(k + 1)
    L, _ = lagrange1d(dgq_nodes(k), g1)
    m = k + 1
    phiq = np.zeros((m * m, len(g1) ** 2))
    for ay in range(m):
        for ax in range(m):
            phiq[ax + m * ay] = np.tile(L[ax], len(g1)) * np.repeat(L[ay], len(g1))
    wq = np.tile(w1, len(g1)) * np.repeat(w1, len(g1))
    Xi = x0[:, None] + hx[:, None] * np.tile(g1, len(g1))
    Yi = y0[:, None] + hy[:, None] * np.repeat(g1, len(g1))
    f0 = 1 + np.cos(TWO_PI * Xi) * np.cos(TWO_PI * Yi)
    coef = np.linalg.solve((phiq * wq) @ phiq.T, ((f0 * wq) @ phiq.T).T).T
    u = np.zeros(cs.ndofs)
    u[cs.u_dofs(allK)] = coef
    bfaces = [(K, f, grid.face_bid(K, f)) for K in range(nc) for f in range(4)
              if grid.face_bid(K, f) in (DIRICHLET, INTERFACE)]
    time = 0.0
    steps = 0
    while time < t_end:
        # assemble_local_test_transient_rhs (source/LDG.cpp:820-990) at the old time
        b = M @ u
        uq = u[cs.u_dofs(allK)] @ ce.phi
        fval = (-math.exp(-time) + TWO_PI ** 2 * np.cos(TWO_PI * X) + TWO_PI ** 2 * np.cos(TWO_PI * Y)
                + TWO_PI * np.sin(TWO_PI * X))
        b[cs.u_dofs(allK)] += np.einsum("aq,kq->ka", ce.phi, fval * JxW)
        # - (p . E) u_old with E = (1, 0): only J_x tests
        b[0:nc * n1] += -np.einsum("aq,kq->ka", ce.phi, uq * JxW).ravel()
        for (K, f, bid) in bfaces:
            fx, fy, Jf = _face_points(grid, K, f, ce.fq, ce.fw)
            fpx, fpy, fv = _carrier_face_tables(ce, f)
            if bid == DIRICHLET:
                gD = math.exp(-time) + np.cos(TWO_PI * fx) + np.cos(TWO_PI * fy)
                pn = fpx * FACE_NORMALS[f][0] + fpy * FACE_NORMALS[f][1]
                b[cs.dofs(K)] += (-pn + (penalty / diam[K]) * fv) @ (gD * Jf)
            else:
                I = -math.exp(-time) - np.cos(TWO_PI * fy) - 1.0
                b[cs.dofs(K)] += -(fv @ (I * Jf))
        u = solve(b)
        time += dt
        steps += 1
    qx, qy, qw = _fine_rule()
    fce = CarrierElement.make(k, nq1=8)
    Xf = x0[:, None] + hx[:, None] * qx
    Yf = y0[:, None] + hy[:, None] * qy
    Wf = (hx * hy)[:, None] * qw
    uh = u[cs.u_dofs(allK)] @ fce.phi
    jx = u[0:nc * n1].reshape(nc, n1) @ fce.phi
    jy = u[nc * n1:2 * nc * n1].reshape(nc, n1) @ fce.phi
    ut = math.exp(-time) + np.cos(TWO_PI * Xf) + np.cos(TWO_PI * Yf)
    jxt = TWO_PI * np.sin(TWO_PI * Xf) - ut
    jyt = TWO_PI * np.sin(TWO_PI * Yf)
    e_u = math.sqrt(np.sum((uh - ut) ** 2 * Wf))
    e_j = math.sqrt(np.sum(((jx - jxt) ** 2 + (jy - jyt) ** 2) * Wf))
    return h, e_u, e_j, steps


def rates(errors):
    """log2 reduction rates between consecutive refinements (as the reference's
    ConvergenceTable::evaluate_convergence_rates prints them)."""
    return [math.log2(errors[i] / errors[i + 1]) for i in range(len(errors) - 1)]
