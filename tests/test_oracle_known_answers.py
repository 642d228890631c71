"""Pins the CPU oracle against the reference's own known-answer tests: the
manufactured-solution convergence studies of tests/Poisson_test.cpp (mixed
RT x DGQ Poisson) and tests/IMEX_LDG_test.cpp (LDG-IMEX transient).  The
reference prints these tables without recording numbers, so the assertion is
on the rates the elements must reach."""
import pytest

from oracle.manufactured import ldg_imex_errors, poisson_mixed_errors, rates


@pytest.mark.parametrize("k,levels,phi_rate,d_rate", [
    (1, range(2, 6), 1.0, 2.0),   # DGQ0 potential O(h); RT0 flux (x/y-separable solution) O(h^2)
    (2, range(1, 5), 2.0, 3.0),   # DGQ1 potential O(h^2); RT1 flux O(h^3)
    (3, range(1, 5), 3.0, 4.0),   # DGQ2 potential O(h^3); RT2 flux O(h^4): the RT_k x DGQ_k
                                  # pairing of the configurations at LDG degree 2
])
def test_mixed_poisson_convergence(k, levels, phi_rate, d_rate):
    E = [poisson_mixed_errors(n, k) for n in levels]
    r_phi = rates([e[1] for e in E])
    r_d = rates([e[2] for e in E])
    assert r_phi[-1] == pytest.approx(phi_rate, abs=0.1)
    assert r_d[-1] == pytest.approx(d_rate, abs=0.15)
    assert all(e1[1] > e2[1] for e1, e2 in zip(E, E[1:]))


def test_ldg_imex_convergence():
    E = [ldg_imex_errors(n, 1) for n in range(2, 5)]
    r_u = rates([e[1] for e in E])
    r_j = rates([e[2] for e in E])
    assert r_u[-1] == pytest.approx(2.0, abs=0.15)   # u: O(h^{k+1})
    assert r_j[-1] == pytest.approx(1.0, abs=0.15)   # J: O(h^k)
    assert E[-1][1] < 1.2e-2


@pytest.mark.parametrize("k,levels,phi_rate,d_rate", [(1, range(3, 6), 1.0, 2.0),
                                                      (2, range(2, 5), 2.0, 3.0)])
def test_mixed_poisson_convergence_graded(k, levels, phi_rate, d_rate):
    """Cells graded 4:1 along x (non-square, non-uniform): the element rates
    still hold, which pins the oracle's per-cell geometry."""
    E = [poisson_mixed_errors(n, k, grading=4.0) for n in levels]
    assert rates([e[1] for e in E])[-1] == pytest.approx(phi_rate, abs=0.15)
    assert rates([e[2] for e in E])[-1] == pytest.approx(d_rate, abs=0.2)


def test_ldg_imex_convergence_graded():
    E = [ldg_imex_errors(n, 1, grading=4.0) for n in range(2, 5)]
    assert rates([e[1] for e in E])[-1] == pytest.approx(2.0, abs=0.2)
    assert rates([e[2] for e in E])[-1] == pytest.approx(1.0, abs=0.2)
