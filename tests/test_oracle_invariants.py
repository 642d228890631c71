"""Structural invariants of the reference's scheme, checked on the oracle
(they pin it where no recorded numbers exist):

* the electrolyte's interface terms: r gains exactly what o loses
  (r += current, o -= current, SolarCell.cpp:1692-1712);
* charge balance across the interface: with v = 1 (the DGQ basis sums to
  one) what the semiconductor's n and p take from the interface equals what
  the electrolyte's r receives (SolarCell.cpp:1289-1345 against 1630-1716);
* the interface transfer enters the density rows only, never the currents';
* a uniform equilibrium with no generation, recombination, transfer or
  field stays put: densities constant, currents and potential zero."""
import numpy as np
import pytest

import oracle


def _interface_parts(P, steps=5):
    """Carrier RHS parts that the interface transfer adds, at a state
    reached after a few steps (densities non-uniform), and the full RHS
    (the parts are differences of full right-hand sides, so their rounding
    is that of the full entries)."""
    pb = oracle.Problem(P)
    st, _, _ = pb.run(steps)
    with_t = pb.carrier_rhs(st)
    without = oracle.Problem(P.copy(k_et=0.0, k_ht=0.0)).carrier_rhs(st)
    return pb, {f: with_t[f] - without[f] for f in with_t}, with_t


@pytest.mark.parametrize("k", [1, 2])
def test_interface_transfer_balances(k):
    P = oracle.half_cell_params(n_refine=2 if k == 2 else 3, degree=k, k_et=0.05, k_ht=0.03)
    pb, d, full = _interface_parts(P)
    cs, ce = pb.semi, pb.elec
    us = cs.u_dofs(np.arange(cs.nc)).ravel()
    ue = ce.u_dofs(np.arange(ce.nc)).ravel()
    assert np.abs(d["r"]).max() > 0
    eps = np.finfo(float).eps
    # r += current, o -= current: negatives of each other
    np.testing.assert_allclose(d["r"], -d["o"], rtol=0,
                               atol=4 * eps * max(np.abs(full["r"]).max(), np.abs(full["o"]).max()))
    # what leaves the semiconductor arrives in the electrolyte
    total_semi = d["n"][us].sum() + d["p"][us].sum()
    bound = 8 * eps * (np.abs(full["n"][us]).sum() + np.abs(full["p"][us]).sum()
                       + np.abs(full["r"][ue]).sum())
    assert abs(total_semi - d["r"][ue].sum()) <= bound
    assert bound < 1e-3 * abs(d["r"][ue].sum())    # the check is not vacuous
    # only density rows see the transfer
    for f, cs_ in (("n", cs), ("p", cs), ("r", ce), ("o", ce)):
        assert np.all(d[f][:2 * cs_.nc * cs_.n1] == 0.0), f


@pytest.mark.parametrize("k", [1, 2])
def test_uniform_equilibrium_is_preserved(k):
    Q = oracle.half_cell_params(n_refine=2, degree=k, gen_kind=0, srh=False, k_et=0.0, k_ht=0.0,
                                nd=(1.0, 1.0), na=(0.0, 0.0), n_eq=(1.0, 1.0), p_eq=(0.0, 0.0),
                                r_eq=1.0, o_eq=1.0, phi_bi=0.0, phi_app=0.0)
    pb = oracle.Problem(Q)
    s0 = pb.initial_state()
    s, _, _ = pb.run(5)
    for f, cs_ in (("n", pb.semi), ("r", pb.elec), ("o", pb.elec)):
        u = cs_.u_dofs(np.arange(cs_.nc)).ravel()
        np.testing.assert_allclose(s[f][u], 1.0, rtol=0, atol=1e-10)
        assert np.abs(s[f][:2 * cs_.nc * cs_.n1]).max() < 1e-9, f   # currents
        assert np.abs(s[f] - s0[f]).max() < 1e-10, f
    assert np.abs(s["p"]).max() == 0.0
    assert np.abs(s["P"]).max() < 1e-12
