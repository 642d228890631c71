"""Large degree-2 meshes: the half cell at refinement 7 (16,384 cells per
region, 442,368 dofs per carrier, 393,984 Poisson dofs) and, when
PECS_LARGE_TESTS=1, refinement 8 (1,769,472 dofs per carrier, 1,574,400
Poisson dofs), at the applied biases -0.3, 0 and 0.3 batched as three
instances, with FP32 factors refined against FP64 residuals.  The oracle
cannot march these sizes in seconds, so the checks are size-independent:
every solve's FP64 relative residual reaches the 1e-12 target, and the
FP32-refined trajectory agrees with the FP64-factor trajectory."""
import os
import time

import numpy as np
import pytest

import pecs_gb300 as pg

pytestmark = pytest.mark.gpu

BIASES = (-0.3, 0.0, 0.3)


def _instances(refine):
    return [pg.half_cell(n_refine=refine, degree=2, phi_app=b) for b in BIASES]


def _march(refine, precision, steps, **opts):
    t0 = time.perf_counter()
    ctx = pg.Context(_instances(refine), precision=precision, **opts)
    setup = time.perf_counter() - t0
    ctx.initialize()
    ctx.step(1)
    ctx.synchronize()
    t1 = time.perf_counter()
    ctx.step(steps - 1)
    ctx.synchronize()
    per_step = (time.perf_counter() - t1) / max(1, steps - 1)
    res = (ctx.solve_residual(0), ctx.solve_residual(1))
    states = [ctx.state(i) for i in range(len(BIASES))]
    cur = ctx.interface_current()
    print(f"refine {refine} k=2 precision {precision} {opts}: setup {setup:.1f} s, "
          f"{1e3 * per_step:.1f} ms per step (3 instances), residuals {res}")
    ctx.close()
    return res, states, cur


def test_refine7_k2_fp32_refined_matches_fp64(pecs_lib):
    steps = 4
    res64, st64, cur64 = _march(7, pg.PREC_FP64, steps)
    res32, st32, cur32 = _march(7, pg.PREC_FP32_IR, steps)
    # measured on GB300: FP64 factors (explicit inverse blocks) 3.1e-13
    # carrier / 9.8e-12 Poisson -- the mixed Poisson system's conditioning
    # grows with refinement and degree; FP32 factors + 2 FP64-residual sweeps
    # 4.6e-15 / 4.9e-13, the 1e-12 target of the FP32 variant
    assert max(res64) < 1e-10
    assert max(res32) < 1e-12
    worst = 0.0
    for i in range(len(BIASES)):
        for f, ref in st64[i].items():
            assert np.all(np.isfinite(st32[i][f]))
            err = np.linalg.norm(st32[i][f] - ref) / np.linalg.norm(ref)
            worst = max(worst, err)
            # measured 5.2e-9: the FP64-factor solve's own error (its residual
            # is 20x the refined one's) dominates the difference
            assert err < 5e-8, (i, f, err)
    print(f"FP32-refined vs FP64 trajectory after {steps} steps: {worst:.3e} (fields), "
          f"{np.max(np.abs(cur32 / cur64 - 1)):.3e} (currents)")
    np.testing.assert_allclose(cur32, cur64, rtol=5e-8, atol=0)
    # the bias reaches the solution: the potential differs between instances
    phi = [st64[i]["P"] for i in range(len(BIASES))]
    assert np.linalg.norm(phi[0] - phi[2]) > 1e-6 * np.linalg.norm(phi[1])


@pytest.mark.parametrize("refine", [7, pytest.param(8, marks=pytest.mark.skipif(
    os.environ.get("PECS_LARGE_TESTS") != "1", reason="refinement 8 with k=2: PECS_LARGE_TESTS=1"))])
def test_setup_with_gpu_fronts_matches_host_setup(pecs_lib, refine):
    """The factorisation with the large fronts on the GPU (the default) gives
    the trajectory of the all-host factorisation; prints both setup times."""
    times, states = {}, {}
    for label, mf in (("gpu fronts", 0), ("host", -1)):
        t0 = time.perf_counter()
        ctx = pg.Context(_instances(refine), precision=pg.PREC_FP64, gpu_factor_min_front=mf)
        times[label] = time.perf_counter() - t0
        ctx.initialize()
        ctx.step(2)
        states[label] = [ctx.state(i) for i in range(len(BIASES))]
        ctx.close()
    print(f"refine {refine} k=2 setup: {times['gpu fronts']:.1f} s with the large fronts on the GPU, "
          f"{times['host']:.1f} s on the host")
    for a, b in zip(states["gpu fronts"], states["host"]):
        for f in b:
            assert np.linalg.norm(a[f] - b[f]) / np.linalg.norm(b[f]) < 1e-11, f


@pytest.mark.skipif(os.environ.get("PECS_LARGE_TESTS") != "1",
                    reason="refinement 8 with k=2 takes minutes of host setup; PECS_LARGE_TESTS=1")
def test_refine8_k2_fp32_refined_residuals(pecs_lib):
    # two refinement sweeps reach 1.8e-14 (carrier) / 1.2e-12 (Poisson) at
    # this size on GB300; a third brings the Poisson solve under the target
    res, st, cur = _march(8, pg.PREC_FP32_IR, 3, ir_max_iters=3)
    assert max(res) < 1e-12
    for s in st:
        for v in s.values():
            assert np.all(np.isfinite(v))
    assert np.all(np.isfinite(cur))
