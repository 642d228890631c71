"""Host logic of the learned warm start (pecs_gb300/learned.py), on the CPU:
the parameter draws and their normalisation, the mapping of a draw to an
instance (which must share the base's matrices), where the predicted
quantities sit in the state vectors (against the oracle's DoF layout), the
block-scaled POD fit, and the committed model file."""
import os

import numpy as np
import pytest

import oracle
import pecs_gb300 as pg
from helpers import to_lib
from pecs_gb300 import learned as L
from pecs_gb300.sweep import matrix_key

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_draws_follow_their_distributions():
    a = L.sample(40000, seed=3)
    assert a.shape == (40000, 6)
    np.testing.assert_array_equal(a, L.sample(40000, seed=3))
    assert not np.array_equal(a, L.sample(40000, seed=4))
    for j, (lo, hi, lg) in enumerate(L.RANGES):
        v = a[:, j]
        assert v.min() >= lo and v.max() <= hi, L.NAMES[j]
        # uniform on [lo, hi] (in log for the log-uniform ones): mean within 4 sigma
        x = np.log(v) if lg else v
        a0, b0 = (np.log(lo), np.log(hi)) if lg else (lo, hi)
        sigma = (b0 - a0) / np.sqrt(12.0 * len(x))
        assert abs(x.mean() - 0.5 * (a0 + b0)) < 4 * sigma, L.NAMES[j]


def test_normalisation_maps_each_range_onto_minus_one_one():
    lo = np.array([[r[0] for r in L.RANGES]])
    hi = np.array([[r[1] for r in L.RANGES]])
    np.testing.assert_allclose(L.normalize(lo), -1.0, atol=1e-6)
    np.testing.assert_allclose(L.normalize(hi), 1.0, atol=1e-6)
    x = L.normalize(L.sample(1000, seed=1))
    assert x.dtype == np.float32 and x.min() >= -1 - 1e-6 and x.max() <= 1 + 1e-6


def test_instances_share_the_base_matrices(pecs_lib):
    base = pg.half_cell(n_refine=2)
    th = L.sample(5, seed=9)
    ps = [L.instance_params(t, base) for t in th]
    for t, p in zip(th, ps):
        assert matrix_key(p) == matrix_key(base)
        assert p.phi_app == t[0] and p.G0 == t[1] and p.alpha == t[2]
        assert p.nd == (t[3], t[3]) and p.n_eq == (t[3], t[3])
        np.testing.assert_allclose(p.p_eq, (base.n_i ** 2 / t[3],) * 2)
        assert p.tau_n == p.tau_p == t[4] and p.k_et == p.k_ht == t[5]
    pg.Context([base] + ps, host_setup_only=True).close()


@pytest.mark.parametrize("P", [oracle.half_cell_params(n_refine=2),
                               oracle.half_cell_params(n_refine=2, degree=2)], ids=["k1", "k2"])
def test_layout_matches_the_dof_layout(pecs_lib, P):
    ctx = pg.Context(to_lib(P), host_setup_only=True)
    lay = L.Layout.of(ctx)
    pb = oracle.Problem(P)
    cs, ps = pb.semi, pb.pois
    u = np.sort(cs.u_dofs(np.arange(cs.nc)).ravel())
    np.testing.assert_array_equal(u, np.arange(lay.u_off, lay.u_off + lay.n_u))
    phi = np.sort(np.unique(ps.l2g[:, ps.pe.n_rt:]))
    np.testing.assert_array_equal(phi, np.arange(lay.phi_off, lay.phi_off + lay.n_phi))
    assert lay.nd_poisson == ps.ndofs and lay.phi_off + lay.n_phi == ps.ndofs
    st = pb.initial_state()
    y = L.fields_to_targets(st["n"], st["p"], st["P"], lay)
    assert y.shape == (lay.n_out,)
    np.testing.assert_allclose(y[:lay.n_u], np.log(np.maximum(st["n"][u], L.DENSITY_FLOOR)))
    np.testing.assert_array_equal(y[2 * lay.n_u:], st["P"][phi])


def test_pod_fit_reproduces_low_rank_snapshots():
    torch = pytest.importorskip("torch")
    lay = L.Layout(nd_carrier=30, n_u=10, u_off=20, nd_poisson=12, n_phi=5, phi_off=7)
    rng = np.random.default_rng(0)
    r = 4
    Y = torch.from_numpy(rng.standard_normal((50, r)) @ rng.standard_normal((r, lay.n_out))
                         * np.r_[np.full(20, 3.0), np.full(5, 0.01)] + 7.0)
    op = L.NeuralOperator.__new__(L.NeuralOperator)   # the POD part only: no network
    op.rank = 6
    T = op.fit_basis(Y, lay)
    V = op.basis
    np.testing.assert_allclose((V.T @ V).numpy(), np.eye(op.rank), atol=1e-12)
    assert T.shape == (50, op.rank) and T.dtype == torch.float32
    np.testing.assert_allclose(op.targets(Y).numpy(), T.numpy(), rtol=1e-6, atol=1e-6)
    # rank-4 data: the basis spans it, so decoding the coefficients gives Y back
    C = (Y - op.mean) / op.scale @ V
    back = op.mean + op.scale * (C @ V.T)
    np.testing.assert_allclose(back.numpy(), Y.numpy(), rtol=0, atol=1e-9)
    # block scaling: each block of the scaled snapshots has unit standard deviation
    Z = (Y - op.mean) / op.scale
    for a, b in ((0, 10), (10, 20), (20, 25)):
        assert abs(float(Z[:, a:b].std()) - 1.0) < 1e-12


def test_committed_model_file_is_consistent():
    d = np.load(os.path.join(ROOT, "pecs_gb300", "models", "warmstart_ref6.npz"))
    widths = [int(w) for w in d["widths"]]
    assert widths[0] == 6 and widths[-1] == int(d["rank"])
    n_params = sum(a * b + b for a, b in zip(widths[:-1], widths[1:]))
    assert d["params"].shape == (n_params,) and np.all(np.isfinite(d["params"]))
    # the half cell at the model's refinement, k = 1: 2 density blocks + the potential
    n = 2 ** int(d["refine"])
    n_u, n_phi = n * n * 4, 2 * n * n
    n_out = 2 * n_u + n_phi
    assert d["mean"].shape == d["scale"].shape == (n_out,)
    assert d["basis"].shape == (n_out, int(d["rank"])) and d["cscale"].shape == (int(d["rank"]),)
    assert np.all(d["scale"] > 0) and np.all(d["cscale"] > 0)


def test_stream_order_longest_lifetime_first_results_in_row_order():
    """stream_warm_sweep hands the points to the stream longest carrier
    lifetime first and returns every result in the caller's row order."""
    import pecs_gb300 as pg
    th = L.sample(10, seed=3)

    class FakeStream:
        def sweep_stream(self, params, max_steps, tol, check_every, init_n=None, init_p=None,
                         want_fields=False):
            taus = np.array([p.tau_n for p in params])
            assert np.all(np.diff(taus) <= 0)  # longest lifetime first
            fin = {0: np.repeat(taus, 3), 4: np.repeat(-taus, 2)} if want_fields else None
            return (taus * 100).astype(np.int32), taus.copy(), fin

    steps, fb, cur, fin = L.stream_warm_sweep(FakeStream(), None, th, pg.half_cell(n_refine=2),
                                              want_fields=True)
    assert np.allclose(cur, th[:, 4])
    assert np.array_equal(steps, (th[:, 4] * 100).astype(np.int32))
    assert np.allclose(fin[0].reshape(10, 3), th[:, 4:5]) and np.allclose(fin[4].reshape(10, 2), -th[:, 4:5])
    assert np.all(fb)
    # order=False keeps the rows' order
    class Plain(FakeStream):
        def sweep_stream(self, params, *a, **k):
            return np.arange(len(params), dtype=np.int32), np.zeros(len(params)), None
    s2, _, _, _ = L.stream_warm_sweep(Plain(), None, th, pg.half_cell(n_refine=2), order=False)
    assert np.array_equal(s2, np.arange(10))
