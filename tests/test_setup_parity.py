"""The library's host setup (meshes, DoF maps, LDG and mixed matrices) against
the oracle's restatement of SolarCellProblem's setup (SolarCell.cpp:377-932,
LDG.cpp:40-678, MixedFEM.cpp:29-164).  Runs on the CPU via host_setup_only."""
import numpy as np
import pytest

import oracle
import pecs_gb300 as pg
from helpers import to_lib, with_layout

CASES = [
    ("pn_junction", oracle.pn_junction_params()),
    ("halfcell_r3", oracle.half_cell_params(n_refine=3)),
    ("reference_r3_k1", oracle.reference_params(3, 1)),
    ("reference_r2_k2", oracle.reference_params(2, 2)),
    ("halfcell_r2_k2_mu", oracle.half_cell_params(n_refine=2, degree=2, mu=(1.0, 0.5, 2.0, 1.0))),
    # non-square cells, graded meshes (finest at the interface)
    ("halfcell_8x16", oracle.half_cell_params(n_refine=3, ny=16)),
    ("halfcell_r3_graded", oracle.half_cell_params(n_refine=3, grading=8.0)),
    ("halfcell_r2_k2_graded", oracle.half_cell_params(n_refine=2, degree=2, ny=8, grading=4.0)),
    ("pn_junction_graded", oracle.pn_junction_params(grading=5.0)),
    # the configurations' RT_k x DGQ_k Poisson pairing
    ("halfcell_r3_rt1", oracle.half_cell_params(n_refine=3, poisson_pairing=1)),
    ("halfcell_r2_k2_rt2", oracle.half_cell_params(n_refine=2, degree=2, poisson_pairing=1)),
    ("pn_junction_rt1_graded", oracle.pn_junction_params(poisson_pairing=1, grading=3.0)),
]


def _cmp(A, B):
    D = (A - B).tocsr()
    D.eliminate_zeros()
    scale = max(abs(B).max(), 1e-300)
    return (abs(D).max() if D.nnz else 0.0) / scale


@pytest.mark.parametrize("name,P", CASES, ids=[c[0] for c in CASES])
def test_matrices_match_oracle(pecs_lib, name, P):
    ctx = pg.Context(to_lib(P), host_setup_only=True)
    pb = oracle.Problem(P)
    assert _cmp(ctx.matrix(pg.MAT_N), pb.A_n) < 1e-14
    assert _cmp(ctx.matrix(pg.MAT_P), pb.A_p) < 1e-14
    assert _cmp(ctx.matrix(pg.MAT_POISSON), pb.A_P) < 1e-14
    assert _cmp(ctx.matrix(pg.MAT_MASS_SEMI), pb.M_semi) < 1e-14
    if P.full_system:
        assert _cmp(ctx.matrix(pg.MAT_R), pb.A_r) < 1e-14
        assert _cmp(ctx.matrix(pg.MAT_O), pb.A_o) < 1e-14
        assert _cmp(ctx.matrix(pg.MAT_MASS_ELEC), pb.M_elec) < 1e-14
    info = ctx.info()
    assert list(info.ndofs)[:2] == [pb.semi.ndofs, pb.semi.ndofs]
    assert info.ndofs[4] == pb.pois.ndofs


def test_equal_mobilities_share_one_factor(pecs_lib):
    ctx = pg.Context(pg.half_cell(n_refine=2), host_setup_only=True)
    assert ctx.info().n_distinct_carrier_factors == 2
    ctx = pg.Context(pg.half_cell(n_refine=2, mu=(1.0, 0.5, 1.0, 1.0)), host_setup_only=True)
    assert ctx.info().n_distinct_carrier_factors == 3


def test_invalid_params_are_rejected(pecs_lib):
    with pytest.raises(pg.PecsError):
        pg.Context(pg.half_cell(n_refine=2, degree=3), host_setup_only=True)
    with pytest.raises(pg.PecsError):
        pg.Context(pg.half_cell(n_refine=2, dt=0.0), host_setup_only=True)
    with pytest.raises(pg.PecsError):
        pg.Context(pg.half_cell(n_refine=2, poisson_pairing=2), host_setup_only=True)
    with pytest.raises(pg.PecsError) as e:   # the pairing defines the Poisson matrix
        pg.Context([pg.half_cell(n_refine=2), pg.half_cell(n_refine=2, poisson_pairing=1)],
                   host_setup_only=True)
    assert "poisson_pairing" in str(e.value)
    a = pg.half_cell(n_refine=2)
    b = pg.half_cell(n_refine=3)
    with pytest.raises(pg.PecsError):
        pg.Context([a, b], host_setup_only=True)
    with pytest.raises(pg.PecsError, match="grading"):
        pg.Context([a, a.copy(grading=4.0)], host_setup_only=True)
    with pytest.raises(pg.PecsError, match="grading"):
        pg.Context(a.copy(grading=-2.0), host_setup_only=True)
    # 0 and 1 both mean uniform
    pg.Context([a.copy(grading=0.0), a.copy(grading=1.0)], host_setup_only=True)


def _reference_id(mesh, x, y, P, insulated, schottky):
    """The id the reference's Grid::make_grids gives the outer face with centre
    (x, y) of a mesh ("semi", "elec", "poisson"): make_Dirichlet_boundaries
    (Grid.cpp:343-373) on faces at x = 0, x = L, y = 0, y = H (the
    semiconductor-electrolyte faces keep the default Interface id), then
    make_Neumann_boundaries (Grid.cpp:377-431), then make_Schottky_boundaries
    (Grid.cpp:434-461, semiconductor and Poisson meshes only)."""
    L = P.x_elec1 if P.full_system else P.x_semi1
    H = P.height
    bid = oracle.INTERFACE
    if x == 0.0 or x == L or y == 0.0 or y == H:
        bid = oracle.DIRICHLET
    if insulated:
        if y == H or y == 0.0:
            bid = oracle.NEUMANN if x > P.x_semi1 else oracle.DIRICHLET
        if x == 0.0:
            bid = oracle.NEUMANN
    if schottky and mesh in ("semi", "poisson") and y == H:
        bid = oracle.SCHOTTKY
    return bid


@pytest.mark.parametrize("full", [True, False])
@pytest.mark.parametrize("insulated,schottky", [(False, False), (True, False), (False, True),
                                                (True, True)])
def test_boundary_layouts_follow_the_reference_rules(full, insulated, schottky):
    base = (oracle.half_cell_params(n_refine=2, grading=3.0) if full
            else oracle.pn_junction_params(nx_semi=4, ny=4))
    P = with_layout(base, insulated, schottky)
    pb = oracle.Problem(P)
    meshes = [("semi", pb.semi_grid), ("poisson", pb.poisson_grid)]
    if full:
        meshes.append(("elec", pb.elec_grid))
    for name, g in meshes:
        x0, y0, hx, hy = g.cell_geom()
        for K in range(g.nc):
            for f in range(4):
                bid = g.face_bid(K, f)
                if bid is None:
                    continue
                cx = {oracle.LEFT: x0[K], oracle.RIGHT: x0[K] + hx[K]}.get(f, x0[K] + 0.5 * hx[K])
                cy = {oracle.BOTTOM: y0[K], oracle.TOP: y0[K] + hy[K]}.get(f, y0[K] + 0.5 * hy[K])
                assert bid == _reference_id(name, cx, cy, P, insulated, schottky), (name, K, f)


LAYOUT_CASES = [(ins, sch) for ins in (False, True) for sch in (False, True)]


@pytest.mark.parametrize("insulated,schottky", LAYOUT_CASES)
def test_layout_matrices_match_oracle(pecs_lib, insulated, schottky):
    P = with_layout(oracle.half_cell_params(n_refine=3, s_n=0.5, s_p=0.25), insulated, schottky)
    ctx = pg.Context(to_lib(P), host_setup_only=True)
    pb = oracle.Problem(P)
    for which, ref in ((pg.MAT_N, pb.A_n), (pg.MAT_P, pb.A_p), (pg.MAT_R, pb.A_r),
                       (pg.MAT_O, pb.A_o), (pg.MAT_POISSON, pb.A_P)):
        assert _cmp(ctx.matrix(which), ref) < 1e-14, which


SETUP_VECTOR_CASES = CASES + [
    ("halfcell_bias", oracle.half_cell_params(n_refine=3, phi_bi=0.7, phi_app=0.2)),
    ("insulated_schottky", with_layout(oracle.half_cell_params(n_refine=3, s_n=0.5, phi_bi=0.3),
                                       True, True)),
]


@pytest.mark.parametrize("name,P", SETUP_VECTOR_CASES, ids=[c[0] for c in SETUP_VECTOR_CASES])
def test_constant_rhs_and_initial_state_match_oracle(pecs_lib, name, P):
    """The host-computed per-instance vectors: time-independent RHS parts
    (generation, Dirichlet and Schottky-face data, doping) and the projected
    initial densities, against the oracle's, on the CPU."""
    ctx = pg.Context(to_lib(P), host_setup_only=True)
    pb = oracle.Problem(P)
    fields = {"n": pg.FIELD_N, "p": pg.FIELD_P, "r": pg.FIELD_R, "o": pg.FIELD_O,
              "P": pg.FIELD_POISSON}
    for f, ref in pb.bconst.items():
        v = ctx.setup_vector(pg.SETUP_CONST_RHS, fields[f])
        assert np.abs(v - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1e-300), f
    st = pb.initial_state()
    for f in ("n", "p", "r", "o"):
        if f in st:
            v = ctx.setup_vector(pg.SETUP_INITIAL, fields[f])
            assert np.abs(v - st[f]).max() <= 1e-13 * np.abs(st[f]).max(), f
    with pytest.raises(pg.PecsError):
        ctx.setup_vector(pg.SETUP_INITIAL, pg.FIELD_POISSON)
    with pytest.raises(pg.PecsError):
        ctx.setup_vector(pg.SETUP_CONST_RHS, pg.FIELD_N, inst=1)
    import ctypes
    short = np.zeros(3)
    assert pg.lib().pecs_get_setup_vector(ctx._h, pg.SETUP_CONST_RHS, pg.FIELD_N, 0,
                                          short.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          short.size) != 0
