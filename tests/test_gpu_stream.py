"""Streamed I-V sweeps (pecs_sweep_stream): points marched through a
context's slots, each slot refilled as soon as its point converges or reaches
the step cap.  Every point must end exactly where the same point ends when it
is marched in an ordinary batch of the same context (the per-instance
arithmetic does not depend on what the other slots hold), and warm starts
passed as device vectors must act like states set through the stage API."""
import numpy as np
import pytest

import pecs_gb300 as pg
from pecs_gb300 import learned as L

pytestmark = pytest.mark.gpu


def _points(n, seed, refine=3):
    base = pg.half_cell(n_refine=refine)
    return [L.instance_params(t, base) for t in L.sample(n, seed)]


def _batch_reference(ctx, pts, max_steps, tol, check_every):
    """The same points in ordinary batches of ctx.n_inst (padded)."""
    B = ctx.n_inst
    steps, cur, fields = [], [], {f: [] for f in ctx.fields()}
    for b0 in range(0, len(pts), B):
        rows = pts[b0:b0 + B]
        pad = rows + [rows[-1]] * (B - len(rows))
        ctx.set_instances(pad)
        ctx.initialize()
        s, _ = ctx.run_to_steady_state(max_steps, tol, check_every)
        c = ctx.interface_current()
        for k in range(len(rows)):
            steps.append(int(s[k]))
            cur.append(c[k])
            for f in ctx.fields():
                fields[f].append(ctx.get_state(f, k).copy())
    return np.array(steps), np.array(cur), fields


@pytest.mark.parametrize("n_slots,precision", [(4, pg.PREC_FP64), (40, pg.PREC_FP64),
                                               (40, pg.PREC_FP32_MIXED)])
def test_stream_matches_batches(pecs_lib, n_slots, precision):
    # a cap low enough that some points stop at it, and uneven convergence so
    # that slots are refilled at different steps
    n_pts, max_steps, tol, every = int(2.5 * n_slots), 900, 1e-6, 10
    pts = _points(n_pts, seed=11)
    ctx = pg.Context(pts[:n_slots], precision=precision)
    steps, cur, fin = ctx.sweep_stream(pts, max_steps, tol, every, want_fields=True)
    ref_steps, ref_cur, ref_fields = _batch_reference(ctx, pts, max_steps, tol, every)
    assert (steps == max_steps).any() and (steps < max_steps).any()
    np.testing.assert_array_equal(steps, ref_steps)
    tol_f = 1e-13 if precision == pg.PREC_FP64 else 1e-9
    for f in ctx.fields():
        nd = ctx.ndofs[f]
        for k in range(n_pts):
            a = fin[f][k * nd:(k + 1) * nd]
            b = ref_fields[f][k]
            assert np.linalg.norm(a - b) <= tol_f * max(np.linalg.norm(b), 1e-300), (f, k)
    np.testing.assert_allclose(cur, ref_cur, rtol=tol_f, atol=0)


def test_stream_warm_start_vectors(pecs_lib):
    """Device initial densities for some points: the stream must reproduce
    a batch whose states were set through set_state_device."""
    import torch
    n_slots, n_pts, max_steps, tol, every = 4, 9, 700, 1e-6, 10
    pts = _points(n_pts, seed=5)
    ctx = pg.Context(pts[:n_slots])
    # the "prediction": each point's own standard initial densities, scaled
    lay = L.Layout.of(ctx)
    warm = {}
    for k in (1, 4, 8):
        ctx.set_instances([pts[k]] * n_slots)
        ctx.initialize()
        vs = []
        for f, fac in ((pg.FIELD_N, 1.02), (pg.FIELD_P, 0.98)):
            v = torch.from_numpy(ctx.get_state(f, 0)).cuda()
            v[lay.u_off:lay.u_off + lay.n_u] *= fac
            vs.append(v)
        warm[k] = tuple(vs)
    init_n = [warm[k][0].data_ptr() if k in warm else 0 for k in range(n_pts)]
    init_p = [warm[k][1].data_ptr() if k in warm else 0 for k in range(n_pts)]
    steps, cur, fin = ctx.sweep_stream(pts, max_steps, tol, every, init_n=init_n, init_p=init_p,
                                       want_fields=True)
    for k in range(n_pts):
        ctx.set_instances([pts[k]] * n_slots)
        ctx.initialize()
        if k in warm:
            ctx.set_state_device(pg.FIELD_N, 0, warm[k][0].data_ptr())
            ctx.set_state_device(pg.FIELD_P, 0, warm[k][1].data_ptr())
            ctx.assemble_poisson_rhs()
            ctx.solve_poisson()
        s, _ = ctx.run_to_steady_state(max_steps, tol, every)
        assert int(steps[k]) == int(s[0]), k
        for f in ctx.fields():
            a = fin[f][k * ctx.ndofs[f]:(k + 1) * ctx.ndofs[f]]
            b = ctx.get_state(f, 0)
            assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(b), (f, k)
