"""Failure detection on the GPU path.  Every failure is made on the host: a NaN
written into a state vector through pecs_set_state, a warm-start vector full
of NaN handed to a streamed sweep, and learned predictions poisoned with NaN
or absurd densities.  No kernel is made to fault, trap or hang: the device
only ever computes on finite-sized, in-bounds data that happens to hold NaN,
and the library reports it through its error codes."""
import numpy as np
import pytest

import pecs_gb300 as pg
from pecs_gb300 import learned as L

pytestmark = pytest.mark.gpu


def _base():
    return pg.half_cell(3)


def test_nan_state_is_reported_and_the_context_stays_usable(pecs_lib):
    base = _base()
    Ps = [base, base.copy(phi_app=0.2)]
    clean = pg.Context(Ps)
    clean.initialize()
    clean.run_to_steady_state(40, 0.0, 10)
    ctx = pg.Context(Ps)
    ctx.initialize()
    v = ctx.get_state(pg.FIELD_N, 1)
    v[v.size - 5] = np.nan
    ctx.set_state(pg.FIELD_N, v, 1)
    with pytest.raises(pg.PecsError) as e:
        ctx.run_to_steady_state(40, 0.0, 10)
    assert e.value.code == pg._ffi.PECS_E_NONFINITE
    assert "instance 1" in str(e.value)
    # the other instance marched on untouched
    for f in ctx.fields():
        a, b = ctx.get_state(f, 0), clean.get_state(f, 0)
        assert np.max(np.abs(a - b)) <= 1e-14 * np.max(np.abs(b)), f
    # the context is still usable: a fresh start gives the clean result
    ctx.initialize()
    ctx.run_to_steady_state(40, 0.0, 10)
    for i in range(2):
        for f in ctx.fields():
            a, b = ctx.get_state(f, i), clean.get_state(f, i)
            assert np.max(np.abs(a - b)) <= 1e-14 * np.max(np.abs(b)), (i, f)


def test_streamed_point_with_a_nan_start_is_marked_and_the_others_are_unchanged(pecs_lib):
    torch = pytest.importorskip("torch")
    base = _base()
    thetas = L.sample(6, seed=31)
    params = [L.instance_params(t, base) for t in thetas]
    ctx = pg.Context([base] * 4)
    steps0, cur0, _ = ctx.sweep_stream(params, 3000, 1e-8, 25)
    bad = torch.full((ctx.ndofs[pg.FIELD_N],), float("nan"), dtype=torch.float64, device="cuda")
    init_n = [0] * len(params)
    init_n[2] = bad.data_ptr()
    steps1, cur1, _ = ctx.sweep_stream(params, 3000, 1e-8, 25, init_n=init_n)
    assert steps1[2] < 0
    for k in range(len(params)):
        if k == 2:
            continue
        assert steps1[k] == steps0[k] > 0
        assert abs(cur1[k] - cur0[k]) <= 1e-13 * abs(cur0[k])


class _PoisonedOperator:
    """Stands in for the trained operator: rows 0-1 predict NaN densities, row
    2 densities of 1e30, row 3 the plain method's own steady state (a perfect
    prediction)."""

    def __init__(self, good_n, good_p):
        self.good = (good_n, good_p)

    def predict_vectors(self, X, lay):
        import torch
        out = []
        for g in self.good:
            v = torch.zeros(X.shape[0], lay.nd_carrier, dtype=torch.float64, device="cuda")
            v[0:2, lay.u_off:lay.u_off + lay.n_u] = float("nan")
            v[2, lay.u_off:lay.u_off + lay.n_u] = 1e30
            v[3] = g
            out.append(v)
        return tuple(out)


def test_poisoned_predictions_fall_back_to_the_standard_start(pecs_lib):
    torch = pytest.importorskip("torch")
    base = _base()
    thetas = L.sample(4, seed=77)
    ctx = pg.Context([base] * 4)
    lay = L.Layout.of(ctx)
    # order=False: the stand-in operator poisons rows by their position in
    # the batch it is given, so the points keep the rows' order
    steps_p, _, cur_p, fin = L.stream_warm_sweep(ctx, None, thetas, base, 3000, 1e-8, 25,
                                                 want_fields=True, order=False)
    nd = lay.nd_carrier
    gn = torch.from_numpy(fin[pg.FIELD_N].reshape(4, nd)[3].copy()).cuda()
    gp = torch.from_numpy(fin[pg.FIELD_P].reshape(4, nd)[3].copy()).cuda()
    gn[:lay.u_off] = 0.0       # a prediction carries densities only
    gp[:lay.u_off] = 0.0
    op = _PoisonedOperator(gn, gp)
    steps_w, fb, cur_w, _ = L.stream_warm_sweep(ctx, op, thetas, base, 3000, 1e-8, 25, order=False)
    assert list(fb) == [True, True, True, False]
    for k in range(3):   # fallbacks: exactly the plain march, plus the two probe steps
        assert steps_w[k] == steps_p[k] + 2
        assert abs(cur_w[k] - cur_p[k]) <= 1e-13 * abs(cur_p[k])
    assert 0 < steps_w[3] < steps_p[3]
    # the batch variant takes the same decisions
    steps_b, fb_b, cur_b = L.warm_started_sweep(ctx, op, thetas, base, 3000, 1e-8, 25)
    assert list(fb_b) == [True, True, True, False]
    assert np.all(np.isfinite(cur_b))


def test_lifetime_order_changes_only_the_schedule(pecs_lib):
    """Streaming the points longest lifetime first changes which slot runs
    which point and when, not the points' results: the same steps and
    currents, in the caller's row order, as the rows' own order."""
    base = _base()
    thetas = L.sample(8, seed=78)
    ctx = pg.Context([base] * 4)
    s0, f0, c0, _ = L.stream_warm_sweep(ctx, None, thetas, base, 3000, 1e-8, 25, order=False)
    s1, f1, c1, _ = L.stream_warm_sweep(ctx, None, thetas, base, 3000, 1e-8, 25, order=True)
    assert np.array_equal(s0, s1) and np.array_equal(f0, f1)
    assert np.allclose(c1, c0, rtol=1e-13, atol=0.0)
