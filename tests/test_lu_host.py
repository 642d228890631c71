"""Nested-dissection multifrontal LU (the pecs_lu_* drop-in for
SparseDirectUMFPACK as used by Carrier/PoissonData) checked on the host:
ordering, symbolic analysis and factorisation applied by the diagnostic
host sweep against scipy's sparse direct solve."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
import pecs_gb300 as pg


def _maps_carrier(pb, cs):
    nc, n1 = cs.nc, cs.n1
    dof_cell = np.concatenate([np.repeat(np.arange(nc), n1)] * 3)
    dof_class = np.concatenate([np.zeros(2 * nc * n1, int), np.ones(nc * n1, int)])
    x0, y0, hx, hy = cs.grid.cell_geom()
    xy = np.stack([x0 + hx / 2, y0 + hy / 2], 1)
    return dof_cell, dof_class, xy


def _maps_poisson(pb):
    ps = pb.pois
    g = ps.grid
    nloc = ps.l2g.shape[1]
    dof_cell = -np.ones(ps.ndofs, int)
    for K in range(g.nc):
        for d in ps.l2g[K]:
            if dof_cell[d] < 0:
                dof_cell[d] = K
    x0, y0, hx, hy = g.cell_geom()
    return dof_cell, np.stack([x0 + hx / 2, y0 + hy / 2], 1)


@pytest.mark.parametrize("P", [oracle.half_cell_params(n_refine=3), oracle.pn_junction_params(),
                               oracle.reference_params(2, 2),
                               # fronts of a few hundred dofs: blocked LU, recursive inverses
                               oracle.half_cell_params(n_refine=4, degree=2)])
def test_host_factorisation_matches_scipy(pecs_lib, P):
    pb = oracle.Problem(P)
    rng = np.random.default_rng(0)
    dc, cl, xy = _maps_carrier(pb, pb.semi)
    for use_class in (True, False):
        lu = pg.LU(pb.A_n, dc, xy, cl if use_class else None)
        b = rng.standard_normal(pb.A_n.shape[0])
        x = lu.host_apply(b)
        ref = spla.spsolve(pb.A_n.tocsc(), b)
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-11
    dcp, xyp = _maps_poisson(pb)
    lu = pg.LU(pb.A_P, dcp, xyp)
    b = pb.poisson_rhs(pb.initial_state())
    x = lu.host_apply(b)
    ref = spla.spsolve(pb.A_P.tocsc(), b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-12
    st = lu.stats()
    assert st["levels"] >= 2 and st["entries"] > 0


def test_class0_coupling_is_rejected(pecs_lib):
    pb = oracle.Problem(oracle.half_cell_params(n_refine=2))
    dc, cl, xy = _maps_carrier(pb, pb.semi)
    bad = np.zeros_like(cl)   # every dof "cell-local": u dofs couple across cells
    with pytest.raises(pg.PecsError):
        pg.LU(pb.A_n, dc, xy, bad)


def test_singular_matrix_is_rejected(pecs_lib):
    n = 8
    A = sp.csr_matrix(np.ones((n, n)))
    with pytest.raises(pg.PecsError) as ei:
        pg.LU(A, np.zeros(n, int), np.array([[0.5, 0.5]]))
    assert ei.value.code == pg._ffi.PECS_E_SINGULAR


def test_bad_arguments_are_rejected(pecs_lib):
    A = sp.identity(4, format="csr")
    with pytest.raises(pg.PecsError):
        pg.LU(A, np.array([0, 1, 2, 9]), np.zeros((4, 2)))
