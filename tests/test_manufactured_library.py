"""The reference's manufactured-solution studies -- tests/Poisson_test.cpp
(mixed RT x DGQ Poisson) and tests/IMEX_LDG_test.cpp (LDG-IMEX transient),
analytic data source/test_functions.cpp:13-220 -- run with the library's
multifrontal solver in place of scipy's: on the host (the stored factors
applied by the diagnostic host sweep) and on the GPU (pecs_lu_solve, the
level-scheduled sweeps).  The convergence rates must be the elements' rates,
and every error must equal the one the scipy-solved study gives."""
import numpy as np
import pytest

import pecs_gb300 as pg
from oracle.manufactured import ldg_imex_errors, poisson_mixed_errors, rates


def _carrier_maps(cs):
    nc, n1 = cs.nc, cs.n1
    dof_cell = np.concatenate([np.repeat(np.arange(nc), n1)] * 3)
    dof_class = np.concatenate([np.zeros(2 * nc * n1, int), np.ones(nc * n1, int)])
    x0, y0, hx, hy = cs.grid.cell_geom()
    return dof_cell, dof_class, np.stack([x0 + hx / 2, y0 + hy / 2], 1)


def _poisson_maps(ps):
    dof_cell = -np.ones(ps.ndofs, int)
    for K in range(ps.grid.nc):
        for d in ps.l2g[K]:
            if dof_cell[d] < 0:
                dof_cell[d] = K
    x0, y0, hx, hy = ps.grid.cell_geom()
    return dof_cell, np.stack([x0 + hx / 2, y0 + hy / 2], 1)


def _library_solver(where):
    def factory(A, space, kind):
        if kind == "carrier":
            dc, cl, xy = _carrier_maps(space)
            lu = pg.LU(A, dc, xy, cl)
        else:
            dc, xy = _poisson_maps(space)
            lu = pg.LU(A, dc, xy)
        return lu.host_apply if where == "host" else lu.solve
    return factory


def _poisson_study(where):
    for k, levels, phi_rate, d_rate in ((1, range(2, 6), 1.0, 2.0), (2, range(1, 5), 2.0, 3.0)):
        E = [poisson_mixed_errors(n, k, solver=_library_solver(where)) for n in levels]
        R = [poisson_mixed_errors(n, k) for n in levels]
        for e, r in zip(E, R):
            np.testing.assert_allclose(e[1:], r[1:], rtol=1e-8)
        assert rates([e[1] for e in E])[-1] == pytest.approx(phi_rate, abs=0.1)
        assert rates([e[2] for e in E])[-1] == pytest.approx(d_rate, abs=0.15)


def _ldg_study(where):
    E = [ldg_imex_errors(n, 1, solver=_library_solver(where)) for n in range(2, 5)]
    R = [ldg_imex_errors(n, 1) for n in range(2, 5)]
    for e, r in zip(E, R):
        assert e[3] == r[3]
        np.testing.assert_allclose(e[1:3], r[1:3], rtol=1e-8)
    assert rates([e[1] for e in E])[-1] == pytest.approx(2.0, abs=0.15)   # u: O(h^{k+1})
    assert rates([e[2] for e in E])[-1] == pytest.approx(1.0, abs=0.15)   # J: O(h^k)


def test_mixed_poisson_study_host_factors(pecs_lib):
    _poisson_study("host")


def test_ldg_imex_study_host_factors(pecs_lib):
    _ldg_study("host")


@pytest.mark.gpu
def test_mixed_poisson_study_gpu(pecs_lib):
    _poisson_study("device")


@pytest.mark.gpu
def test_ldg_imex_study_gpu(pecs_lib):
    _ldg_study("device")
