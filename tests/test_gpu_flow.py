"""Flow sweeps (solve.cu, k_panel_flow): one persistent launch per sweep
direction, each node started as soon as its children (forward) or its parent
(backward) have finished.  Forced on and off on the same batches: FP64
trajectories agree to rounding and with the oracle; the mixed mode is as
accurate as with level-by-level sweeps; a wait that runs out (armed on the
host) is reported, writes NaN, and leaves the context usable."""
import ctypes as C
import time

import numpy as np
import pytest

import oracle
import pecs_gb300 as pg
from helpers import rel_err, to_lib
from test_gpu_parity import STEP_TOL, _compare_state, _panel_instances

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_inst,refine", [(40, 3), (64, 5)], ids=["80rhs_ref3", "128rhs_ref5"])
def test_flow_sweep_fp64_matches_levels_and_oracle(pecs_lib, n_inst, refine):
    Ps = _panel_instances(n_inst, oracle.half_cell_params(n_refine=refine))
    flow = pg.Context([to_lib(P) for P in Ps], flow_sweep=1)
    lev = pg.Context([to_lib(P) for P in Ps], flow_sweep=-1)
    assert flow.info().flow_rpl[0] > 0 and lev.info().flow_rpl[0] == 0
    for c in (flow, lev):
        c.initialize()
        c.step(3)
    for i in range(n_inst):
        for f in flow.fields():
            assert rel_err(flow.get_state(f, i), lev.get_state(f, i)) < 1e-12, (i, f)
    st, _, _ = oracle.Problem(Ps[0]).run(3)
    _compare_state(flow, st, STEP_TOL, inst=0)


def test_flow_sweep_mixed_as_accurate_as_levels(pecs_lib):
    """64 instances at refinement 4 in the batched throughput mode: carrier
    (128 RHS) and Poisson (64 RHS) banks both on flow sweeps; distance to the
    FP64 trajectory no larger than the level sweeps' (within rounding), and
    solve residuals at the mixed mode's level."""
    Ps = _panel_instances(64, oracle.half_cell_params(n_refine=4))
    ref = pg.Context([to_lib(P) for P in Ps])
    flow = pg.Context([to_lib(P) for P in Ps], precision=pg.PREC_FP32_MIXED, flow_sweep=1)
    lev = pg.Context([to_lib(P) for P in Ps], precision=pg.PREC_FP32_MIXED, flow_sweep=-1)
    assert list(flow.info().flow_rpl) != [0, 0] and list(lev.info().flow_rpl) == [0, 0]
    for c in (ref, flow, lev):
        c.initialize()
        c.step(10)
    for f in ref.fields():
        e_flow = max(rel_err(flow.get_state(f, i), ref.get_state(f, i)) for i in range(64))
        e_lev = max(rel_err(lev.get_state(f, i), ref.get_state(f, i)) for i in range(64))
        print(f, e_flow, e_lev)
        assert e_flow < 1e-6 and e_flow <= max(4 * e_lev, 1e-9), (f, e_flow, e_lev)
    assert max(flow.solve_residual(0), flow.solve_residual(1)) < 1e-10


def test_flow_wait_runs_out_and_is_reported(pecs_lib):
    """The first factor's root counter is set far below its target before a
    forward flow sweep: its waits run out after their poll limit, the sweep
    writes NaN and sets the bank's error flag, which the host reads; the next
    sweeps start from zeroed counters and the context's trajectory is that of
    a context that never stalled."""
    Ps = _panel_instances(64, oracle.half_cell_params(n_refine=3))
    ctx = pg.Context([to_lib(P) for P in Ps], flow_sweep=1)
    lev = pg.Context([to_lib(P) for P in Ps], flow_sweep=-1)
    assert ctx.info().flow_rpl[0] > 0
    ctx.initialize()
    flag = C.c_int(-1)
    t0 = time.perf_counter()
    pg._ffi.check(pg.lib().pecs_debug_flow_stall(ctx._h, 0, C.byref(flag)))
    dt = time.perf_counter() - t0
    print("stalled sweep", dt, "s")
    assert flag.value == 1 and dt < 30.0
    pg._ffi.check(pg.lib().pecs_debug_flow_stall(ctx._h, 0, C.byref(flag)))
    assert flag.value == 1
    for c in (ctx, lev):
        c.initialize()
        c.step(3)
    for i in range(64):
        for f in ctx.fields():
            x = ctx.get_state(f, i)
            assert np.all(np.isfinite(x))
            assert rel_err(x, lev.get_state(f, i)) < 1e-12


@pytest.mark.parametrize("P", [oracle.half_cell_params(n_refine=5), oracle.half_cell_params(n_refine=3, degree=2)],
                         ids=["ref5_k1", "ref3_k2"])
def test_rows_flow_fp64_single_instance_matches_levels_and_oracle(pecs_lib, P):
    """The plain single-instance FP64 path (two carrier and one Poisson
    right-hand sides: the few-RHS kernels) with its sweeps as one persistent
    launch per direction: equal to the level launches to 1e-12 and to the
    oracle's trajectory within the step tolerance."""
    lib_p = to_lib(P)
    flow = pg.Context(lib_p, flow_sweep=1)
    lev = pg.Context(lib_p, flow_sweep=-1)
    assert flow.info().flow_top[0] > 0 and flow.info().solve_launches[0] == 2
    assert lev.info().flow_top[0] == 0
    for c in (flow, lev):
        c.initialize()
        c.step(10)
    for f in flow.fields():
        assert rel_err(flow.get_state(f), lev.get_state(f)) < 1e-12, f
    st, _, _ = oracle.Problem(P).run(10)
    _compare_state(flow, st, STEP_TOL)


def test_rows_flow_wait_runs_out_and_is_reported(pecs_lib):
    """As test_flow_wait_runs_out_and_is_reported, for the few-RHS flow sweep:
    the stalled root's rows are written as NaN, the flag is raised, and the
    context's next trajectory equals the level path's."""
    lib_p = to_lib(oracle.half_cell_params(n_refine=4))
    ctx = pg.Context(lib_p, flow_sweep=1)
    lev = pg.Context(lib_p, flow_sweep=-1)
    ctx.initialize()
    flag = C.c_int(-1)
    pg._ffi.check(pg.lib().pecs_debug_flow_stall(ctx._h, 0, C.byref(flag)))
    assert flag.value == 1
    for c in (ctx, lev):
        c.initialize()
        c.step(3)
    for f in ctx.fields():
        x = ctx.get_state(f)
        assert np.all(np.isfinite(x))
        assert rel_err(x, lev.get_state(f)) < 1e-12
