"""Multi-rank I-V sweep sharding over gloo (world size 2, CPU): every instance
is computed exactly once, on the rank that owns its slice, and the gathered
results come back in global order on every rank."""
import multiprocessing as mp
import os
import socket

import pytest

from pecs_gb300.sweep import distributed_sweep, shard


def test_shard_covers_everything_once():
    for n in (0, 1, 5, 64, 65):
        for w in (1, 2, 3, 8):
            seen = [i for r in range(w) for i in shard(n, w, r)]
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_matrix_key_groups_points_by_their_matrices(pecs_lib):
    """Points share a context exactly when the library accepts them in one:
    the grouping key of ragged sweeps covers every matrix-defining field,
    grading and boundary layouts included."""
    import pecs_gb300 as pg
    from pecs_gb300.sweep import MATRIX_FIELDS, matrix_key
    base = pg.half_cell(n_refine=2)
    same = [base.copy(phi_app=0.3), base.copy(G0=2.0, alpha=3.0), base.copy(tau_n=0.5, k_et=1e-3)]
    other = [base.copy(grading=4.0), pg.boundary_layout(base, insulated=True),
             pg.boundary_layout(base, schottky=True), base.copy(ny=8), base.copy(dt=2e-3),
             base.copy(degree=2)]
    for p in same:
        assert matrix_key(p) == matrix_key(base)
        pg.Context([base, p], host_setup_only=True).close()
    for p in other:
        assert matrix_key(p) != matrix_key(base)
        with pytest.raises(pg.PecsError):
            pg.Context([base, p], host_setup_only=True)
    assert set(MATRIX_FIELDS) <= set(base.__dataclass_fields__)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    params = [{"bias": -0.5 + i / max(1, n - 1)} for i in range(n)]
    calls = []

    def compute(ps):
        calls.extend(p["bias"] for p in ps)
        return [(p["bias"], rank) for p in ps]

    out = distributed_sweep(params, compute)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, calls, out))


@pytest.mark.parametrize("n", [5, 8])
def test_gloo_two_ranks(n):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    all_calls = sorted(b for _, calls, _ in res for b in calls)
    assert len(all_calls) == n  # each instance computed once
    for rank, calls, out in res:
        assert [o[0] for o in out] == [-0.5 + i / max(1, n - 1) for i in range(n)]
        owners = [o[1] for o in out]
        assert owners == sorted(owners)  # contiguous slices
        assert set(owners) == {0, 1}


def test_without_process_group_runs_locally():
    out = distributed_sweep([1, 2, 3], lambda ps: [p * 2 for p in ps])
    assert out == [2, 4, 6]


def _setup_result(ps):
    """Per-instance setup on the host (a host_setup_only library context for
    this rank's slice): the constant right-hand-side parts of every field and
    the projected initial electron density."""
    import numpy as np
    import pecs_gb300 as pg
    ctx = pg.Context(ps, host_setup_only=True)
    out = []
    for i in range(len(ps)):
        v = [ctx.setup_vector(pg.SETUP_CONST_RHS, f, i) for f in range(5)]
        v.append(ctx.setup_vector(pg.SETUP_INITIAL, pg.FIELD_N, i))
        out.append(np.concatenate(v))
    ctx.close()
    return out


def _setup_worker(rank, world, port, n, q):
    import torch.distributed as dist

    import pecs_gb300 as pg
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    base = pg.half_cell(n_refine=2)
    params = [base.copy(phi_app=-0.5 + i / (n - 1), G0=0.5 + 0.25 * i, nd=(1.0 + 0.1 * i,) * 2,
                        n_eq=(1.0 + 0.1 * i,) * 2) for i in range(n)]
    out = distributed_sweep(params, _setup_result)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_gloo_two_ranks_build_library_contexts(pecs_lib):
    """Each of two gloo ranks builds a host-only library context for its slice
    of instances; the gathered per-instance setup vectors equal those of one
    process that builds every instance itself."""
    import numpy as np

    import pecs_gb300 as pg
    n = 5
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_setup_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    base = pg.half_cell(n_refine=2)
    params = [base.copy(phi_app=-0.5 + i / (n - 1), G0=0.5 + 0.25 * i, nd=(1.0 + 0.1 * i,) * 2,
                        n_eq=(1.0 + 0.1 * i,) * 2) for i in range(n)]
    want = _setup_result(params)
    for _, out in res:
        assert len(out) == n
        for a, b in zip(out, want):
            np.testing.assert_array_equal(a, b)
    # the instances really differ (each rank computed different data)
    assert not np.array_equal(want[0], want[-1])


class _FakeContext:
    """Stands in for pecs_gb300.api.Context in ragged_sweep: steps, current
    and a two-entry field per point derived from the point's parameters."""
    made, closed = [], []
    fail_degree = None

    def __init__(self, pts, precision=None, **kw):
        self.ndofs = {0: 2}
        _FakeContext.made.append(self)

    def sweep_stream(self, pts, max_steps, tol, check_every, want_fields=False):
        import time

        import numpy as np
        time.sleep(0.01)
        if _FakeContext.fail_degree is not None and pts[0].degree == _FakeContext.fail_degree:
            raise RuntimeError("group failed")
        steps = np.array([int(round(p.phi_app * 1000)) for p in pts])
        cur = np.array([p.G0 for p in pts])
        fin = {0: np.concatenate([[p.G0, p.ny] for p in pts])} if want_fields else None
        return steps, cur, fin

    def close(self):
        _FakeContext.closed.append(self)


def test_ragged_sweep_concurrent_groups_on_host(pecs_lib, monkeypatch):
    """Grouping, result order and clean-up of ragged_sweep, serial and
    concurrent, with a fake context: the same results in point order either
    way, every context closed, and a group's error raised after all the
    contexts are closed."""
    import numpy as np

    import pecs_gb300 as pg
    import pecs_gb300.api as api
    from pecs_gb300.sweep import ragged_sweep
    monkeypatch.setattr(api, "Context", _FakeContext)
    pts = [pg.half_cell(n_refine=2 + i % 2, degree=1 + (i // 2) % 2, phi_app=0.01 * i, G0=1.0 + i)
           for i in range(11)]
    res = {}
    for conc in (False, True):
        _FakeContext.made, _FakeContext.closed = [], []
        res[conc] = ragged_sweep(pts, slots=2, want_fields=True, concurrent=conc)
        assert len(_FakeContext.made) == 4 and len(_FakeContext.closed) == 4
    for conc in (False, True):
        steps, cur, fields = res[conc]
        assert list(steps) == [10 * i for i in range(11)]
        assert list(cur) == [1.0 + i for i in range(11)]
        assert [list(f[0]) for f in fields] == [[1.0 + i, p.ny] for i, p in enumerate(pts)]
    for conc in (False, True):
        steps, cur, fields = ragged_sweep([], want_fields=True, concurrent=conc)
        assert len(steps) == len(cur) == len(fields) == 0
    _FakeContext.made, _FakeContext.closed = [], []
    _FakeContext.fail_degree = 2
    try:
        with pytest.raises(RuntimeError, match="group failed"):
            ragged_sweep(pts, concurrent=True)
    finally:
        _FakeContext.fail_degree = None
    assert len(_FakeContext.closed) == len(_FakeContext.made) == 4
