"""pecs_lu_solve_device_noalloc: the solve for callers that cannot allocate
device memory at solve time (their own pool owns the GPU's memory, or they
must stay inside a fixed memory budget).  Its sweeps keep their scratch in a
fixed file-scope device array instead of handle-owned memory.  Checked
through the C ABI against the allocating entry point pecs_lu_solve_device, on
two calls in a row (the array keeps the previous call's contents), and for
its size limits.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import oracle
import pecs_gb300 as pg
from test_lu_host import _maps_carrier, _maps_poisson

pytestmark = pytest.mark.gpu

TOL = 1e-12   # same kernels on the same factors: agreement to rounding


def _noalloc(lu, nrhs, b_ptr, x_ptr):
    return pg.lib().pecs_lu_solve_device_noalloc(lu._h, nrhs, C.c_void_p(b_ptr), C.c_void_p(x_ptr),
                                                 C.c_void_p(0))


def _rel(a, b):
    return float((a - b).norm() / b.norm())


@pytest.mark.parametrize("system", ["carrier", "poisson"])
def test_noalloc_matches_allocating_solve_twice(pecs_lib, system):
    torch = pytest.importorskip("torch")
    pb = oracle.Problem(oracle.half_cell_params(n_refine=4))
    if system == "carrier":
        dc, cl, xy = _maps_carrier(pb, pb.semi)
        lu = pg.LU(pb.A_n, dc, xy, cl)
        n = pb.A_n.shape[0]
    else:
        dc, xy = _maps_poisson(pb)
        lu = pg.LU(pb.A_P, dc, xy)
        n = pb.A_P.shape[0]
    nrhs = 2
    gen = torch.Generator(device="cuda").manual_seed(7)
    for call in range(2):   # two calls in a row share the static scratch
        b = torch.randn(nrhs, n, dtype=torch.float64, device="cuda", generator=gen)
        x_ref = torch.zeros_like(b)
        lu.solve_device(b.data_ptr(), x_ref.data_ptr(), nrhs=nrhs)   # allocating entry point
        x = torch.full_like(b, float("nan"))
        pg._ffi.check(_noalloc(lu, nrhs, b.data_ptr(), x.data_ptr()))
        torch.cuda.synchronize()
        assert torch.isfinite(x).all()
        assert _rel(x, x_ref) < TOL, (call, _rel(x, x_ref))


def test_noalloc_limits_and_preconditions(pecs_lib):
    torch = pytest.importorskip("torch")
    pb = oracle.Problem(oracle.half_cell_params(n_refine=6))
    dc, cl, xy = _maps_carrier(pb, pb.semi)
    lu = pg.LU(pb.A_n, dc, xy, cl)
    n = pb.A_n.shape[0]
    b = torch.ones(8, n, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    # factors not yet on the device: refused, nothing allocated
    assert _noalloc(lu, 1, b.data_ptr(), x.data_ptr()) == pg._ffi.PECS_E_STATE
    lu.solve_device(b.data_ptr(), x.data_ptr(), nrhs=1)
    # more right-hand sides than the scratch holds: a clear error
    code = _noalloc(lu, 8, b.data_ptr(), x.data_ptr())
    assert code == pg._ffi.PECS_E_ARG
    assert b"scratch" in pg.lib().pecs_last_error()
    assert _noalloc(lu, 9, b.data_ptr(), x.data_ptr()) == pg._ffi.PECS_E_ARG
    # one right-hand side of this size fits
    x1 = torch.zeros(n, dtype=torch.float64, device="cuda")
    x2 = torch.zeros(n, dtype=torch.float64, device="cuda")
    lu.solve_device(b[0].data_ptr(), x1.data_ptr(), nrhs=1)
    pg._ffi.check(_noalloc(lu, 1, b[0].data_ptr(), x2.data_ptr()))
    assert _rel(x2, x1) < TOL


def _block_diagonal(n_cells, first_single=False):
    """2x2 blocks, one per cell, coupled to nothing else (first_single: the
    first cell has a 1x1 block).  No node of the factor has an update set, and
    the sweeps keep one update-vector slot per right-hand side all the same,
    so a solve needs exactly nrhs * (n + 1) doubles of scratch."""
    import scipy.sparse as sp
    rng = np.random.default_rng(11)
    blocks = list(rng.uniform(-1.0, 1.0, (n_cells, 2, 2)) + 3.0 * np.eye(2))
    sizes = [2] * n_cells
    if first_single:
        blocks[0] = np.array([[2.5]])
        sizes[0] = 1
    A = sp.block_diag(blocks, format="csr")
    dof_cell = np.repeat(np.arange(n_cells, dtype=np.int32), sizes)
    xy = np.stack([np.arange(n_cells) + 0.5, np.full(n_cells, 0.5)], axis=1)
    return A, dof_cell, xy


def test_noalloc_fills_scratch_exactly_on_a_caller_stream_without_allocating(pecs_lib):
    """nrhs * (n + 1) equal to the scratch's 2^20 doubles is accepted, one dof
    more is refused; the call runs on the caller's stream and the device's
    free memory is the same before and after it."""
    torch = pytest.importorskip("torch")
    cap = 1 << 20
    nrhs = 8
    A, dc, xy = _block_diagonal(cap // nrhs // 2, first_single=True)
    n = A.shape[0]
    assert nrhs * (n + 1) == cap
    lu = pg.LU(A, dc, xy)
    gen = torch.Generator(device="cuda").manual_seed(3)
    b = torch.randn(nrhs, n, dtype=torch.float64, device="cuda", generator=gen)
    x_ref = torch.zeros_like(b)
    lu.solve_device(b.data_ptr(), x_ref.data_ptr(), nrhs=nrhs)    # uploads the factors
    x = torch.full_like(b, float("nan"))
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        pg._ffi.check(pg.lib().pecs_lu_solve_device_noalloc(
            lu._h, nrhs, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
            C.c_void_p(stream.cuda_stream)))
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert _rel(x, x_ref) < TOL
    # the exact answer of the first blocks, checked on the host
    bh, xh = b.cpu().numpy(), x.cpu().numpy()
    np.testing.assert_allclose(xh[:, 0], bh[:, 0] / 2.5, rtol=1e-14)
    for c in range(1, 5):
        i = 2 * c - 1
        blk = A[i:i + 2, i:i + 2].toarray()
        np.testing.assert_allclose(xh[:, i:i + 2], np.linalg.solve(blk, bh[:, i:i + 2].T).T,
                                   rtol=1e-12, atol=1e-14)
    # one dof more than fits: refused before any device work
    A2, dc2, xy2 = _block_diagonal(cap // nrhs // 2)
    lu2 = pg.LU(A2, dc2, xy2)
    b2 = torch.ones(nrhs, A2.shape[0], dtype=torch.float64, device="cuda")
    x2 = torch.zeros_like(b2)
    lu2.solve_device(b2.data_ptr(), x2.data_ptr(), nrhs=1)
    assert _noalloc(lu2, nrhs, b2.data_ptr(), x2.data_ptr()) == pg._ffi.PECS_E_ARG
    assert b"scratch" in pg.lib().pecs_last_error()
    assert _noalloc(lu2, nrhs - 1, b2.data_ptr(), x2.data_ptr()) == pg._ffi.PECS_OK
