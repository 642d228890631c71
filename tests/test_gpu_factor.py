"""FP64 factorisation of the largest fronts on the GPU (front.cu): the stored
factor values (Gf, Hb of every node) must equal the host's to 1e-12, for the
LDG carrier and the mixed Poisson matrices at degrees 1 and 2, and a time
trajectory on GPU-factored matrices must match the one on host-factored
matrices.  Small fronts are sent to the GPU here (a low row threshold) so that
small meshes exercise every part: panel LU with pivoting, the row-block
triangular solves, the trailing updates and the triangular inverses."""
import numpy as np
import pytest

import oracle
import pecs_gb300 as pg
from test_lu_host import _maps_carrier, _maps_poisson

pytestmark = pytest.mark.gpu


def _values(A, maps, min_front):
    old = pg.lib().pecs_lu_set_gpu_factor_min_front(min_front)
    try:
        lu = pg.LU(A, *maps)
        return lu, lu.factor_values()
    finally:
        pg.lib().pecs_lu_set_gpu_factor_min_front(old)


@pytest.mark.parametrize("P,which", [(oracle.half_cell_params(n_refine=5), "carrier"),
                                     (oracle.half_cell_params(n_refine=5), "poisson"),
                                     (oracle.half_cell_params(n_refine=3, degree=2), "carrier"),
                                     (oracle.half_cell_params(n_refine=3, degree=2), "poisson"),
                                     (oracle.half_cell_params(n_refine=3, degree=2, poisson_pairing=1),
                                      "poisson")],
                         ids=["r5_carrier", "r5_poisson", "r3_k2_carrier", "r3_k2_poisson", "r3_k2_rt2_poisson"])
def test_gpu_fronts_equal_host_fronts(pecs_lib, P, which):
    pb = oracle.Problem(P)
    if which == "carrier":
        dc, cl, xy = _maps_carrier(pb, pb.semi)
        A, maps = pb.A_n, (dc, xy, cl)
    else:
        dc, xy = _maps_poisson(pb)
        A, maps = pb.A_P, (dc, xy)
    lu_h, vh = _values(A, maps, -1)    # every front on the host
    lu_g, vg = _values(A, maps, 64)    # fronts of 64 rows and more on the GPU
    assert lu_g.stats()["max_front"] >= 64
    assert vh.shape == vg.shape
    err = np.max(np.abs(vg - vh)) / np.max(np.abs(vh))
    assert err < 1e-12, err
    rng = np.random.default_rng(2)
    b = rng.standard_normal(A.shape[0])
    xg = lu_g.solve(b)
    assert np.linalg.norm(A @ xg - b) / np.linalg.norm(b) < 1e-10


def test_trajectory_on_gpu_factored_matrices(pecs_lib):
    """A context whose fronts of 128 rows and more were factored on the GPU
    marches the same trajectory as one factored on the host."""
    P = oracle.half_cell_params(n_refine=5)
    lib_p = pg.Params(**{k: getattr(P, k) for k in P.__dataclass_fields__})
    a = pg.Context(lib_p, gpu_factor_min_front=128)
    b = pg.Context(lib_p, gpu_factor_min_front=-1)
    for c in (a, b):
        c.initialize()
        c.step(20)
    for f in a.fields():
        x, y = a.get_state(f), b.get_state(f)
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-11, f
