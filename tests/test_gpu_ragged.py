"""Ragged I-V sweeps (the batched sweep with uneven instances): points with different
refinement levels and degrees are grouped by their meshes and streamed through
one context per group; every point must end exactly where it ends alone."""
import numpy as np
import pytest

import pecs_gb300 as pg
from pecs_gb300.sweep import matrix_key, ragged_sweep

pytestmark = pytest.mark.gpu


def test_ragged_sweep_matches_single_instances(pecs_lib):
    rng = np.random.default_rng(3)
    pts = []
    for _ in range(10):
        r = int(rng.integers(2, 4))          # refinement 2 or 3
        k = int(rng.integers(1, 3))          # degree 1 or 2
        pts.append(pg.half_cell(n_refine=r, degree=k, phi_app=float(rng.uniform(-0.5, 0.5)),
                              G0=float(rng.uniform(0.5, 2.0))))
    steps, cur, fields = ragged_sweep(pts, slots=3, max_steps=400, tol=1e-6, check_every=10,
                                      want_fields=True)
    gsize = {}
    for p in pts:
        gsize[matrix_key(p)] = gsize.get(matrix_key(p), 0) + 1
    for i, p in enumerate(pts):
        # the reference runs the point alone in a context with as many slots
        # as its group got (same kernels), padded with copies of itself
        ctx = pg.Context([p] * min(3, gsize[matrix_key(p)]))
        ctx.initialize()
        s, _ = ctx.run_to_steady_state(400, 1e-6, 10)
        assert int(steps[i]) == int(s[0]), i
        c = ctx.interface_current()[0]
        assert abs(cur[i] - c) <= 1e-12 * abs(c)
        for f in ctx.fields():
            b = ctx.get_state(f, 0)
            assert np.linalg.norm(fields[i][f] - b) <= 1e-13 * np.linalg.norm(b), (i, f)
