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
