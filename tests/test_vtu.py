"""Headless VTU output (pecs_gb300/vtu.py): per-cell patches with the
post-processor's fields and scales (PostProcessor.cpp:6-124).  A stand-in
context supplies known state vectors; the file is parsed back."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import pecs_gb300 as pg
from pecs_gb300 import vtu


class FakeCtx:
    """Known state vectors; the meshes come from a host-only library context."""

    def __init__(self, p, vecs):
        self.params = [p]
        self.ndofs = [len(vecs.get(f, [])) for f in range(5)]
        self._v = vecs
        self._host = pg.Context(p, host_setup_only=True)

    def get_state(self, f, inst=0):
        return self._v[f]

    def mesh(self, which):
        return self._host.mesh(which)


def _arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    out = {a.get("Name"): np.array(a.text.split(), dtype=float) for a in piece.iter("DataArray")}
    return piece, out


def test_carrier_patches_and_scaling(tmp_path, pecs_lib):
    p = pg.half_cell(n_refine=1)   # 2x2 cells per region, k = 1
    nc, n1 = 4, 4
    n = np.arange(3 * nc * n1, dtype=float)
    vecs = {pg.FIELD_N: n, pg.FIELD_P: -n}
    ctx = FakeCtx(p, vecs)
    path = tmp_path / "semi.vtu"
    vtu.write_carriers(ctx, str(path), scales=vtu.Scales(density=2.0, current=3.0))
    piece, a = _arrays(path)
    assert piece.get("NumberOfPoints") == str(nc * n1) and piece.get("NumberOfCells") == str(nc)
    np.testing.assert_array_equal(a["Electrons Density"], 2.0 * n[2 * nc * n1:])
    cur = a["Electrons Current"].reshape(-1, 3)
    np.testing.assert_array_equal(cur[:, 0], 3.0 * n[:nc * n1])
    np.testing.assert_array_equal(cur[:, 1], 3.0 * n[nc * n1:2 * nc * n1])
    pts = a["Points"].reshape(-1, 3)
    # cell 1 (i = 1, j = 0) spans x in [0.5, 1], y in [0, 0.5]; nodes x-fastest
    np.testing.assert_allclose(pts[4:8, :2], [[0.5, 0], [1, 0], [0.5, 0.5], [1, 0.5]])
    assert set(a["types"]) == {9.0}


def test_potential_point_data(tmp_path, pecs_lib):
    """k = 1: the potential is DGQ0, one value per cell, written (as DataOut
    writes every quantity) at each of the cell's patch points."""
    p = pg.half_cell(n_refine=1)
    ncp = 8                      # 4 x 2 Poisson cells
    n_rt = 22                    # 10 vertical + 12 horizontal faces, one RT0 dof each
    P = np.concatenate([np.zeros(n_rt), np.arange(ncp, dtype=float)])
    ctx = FakeCtx(p, {pg.FIELD_N: np.zeros(48), pg.FIELD_POISSON: P})
    path = tmp_path / "phi.vtu"
    vtu.write_poisson(ctx, str(path), scales=vtu.Scales(potential=0.5))
    piece, a = _arrays(path)
    assert piece.get("NumberOfCells") == str(ncp) and piece.get("NumberOfPoints") == str(4 * ncp)
    np.testing.assert_array_equal(a["Potential"], 0.5 * np.repeat(np.arange(ncp), 4))
    np.testing.assert_array_equal(a["Field"], 0.0)


@pytest.mark.parametrize("degree,nref", [(1, 1), (2, 1)])
def test_field_D_matches_a_field_in_the_RT_space(tmp_path, pecs_lib, degree, nref):
    """The written "Field" is D evaluated from the RT_{k-1} coefficients: a
    field that RT_{k-1} represents exactly (D_x of degree k in x and k-1 in y,
    D_y the other way round) is put into a Poisson vector through the
    oracle's own dof numbering and must come back at every patch point."""
    import oracle
    from helpers import to_lib
    P = oracle.half_cell_params(n_refine=nref, degree=degree, grading=2.0)
    pb = oracle.Problem(P)
    sp, g = pb.pois, pb.poisson_grid
    k = degree
    fx = lambda x, y: x ** k + (y ** (k - 1) if k > 1 else 0.0) + 0.25   # noqa: E731
    fy = lambda x, y: (x ** (k - 1) if k > 1 else 0.0) - 2.0 * y ** k   # noqa: E731
    v = np.zeros(sp.ndofs)
    nn = np.linspace(0.0, 1.0, k + 1)
    tn = (np.arange(k) + 0.5) / k
    x0, y0, hx, hy = g.cell_geom()
    nxd = k * (k + 1)
    for K in range(g.nc):
        for b in range(k):
            for a in range(k + 1):
                v[sp.l2g[K, a + (k + 1) * b]] = fx(x0[K] + hx[K] * nn[a], y0[K] + hy[K] * tn[b])
        for b in range(k + 1):
            for a in range(k):
                v[sp.l2g[K, nxd + a + k * b]] = fy(x0[K] + hx[K] * tn[a], y0[K] + hy[K] * nn[b])
    lib_p = to_lib(P)
    nd = 3 * pb.semi_grid.nc * (k + 1) ** 2
    ctx = FakeCtx(lib_p, {pg.FIELD_N: np.zeros(nd), pg.FIELD_POISSON: v})
    path = tmp_path / "poisson.vtu"
    vtu.write_poisson(ctx, str(path), scales=vtu.Scales(field=3.0), subdivisions=3)
    _, arr = _arrays(path)
    pts = arr["Points"].reshape(-1, 3)
    F = arr["Field"].reshape(-1, 3)
    np.testing.assert_allclose(F[:, 0], 3.0 * fx(pts[:, 0], pts[:, 1]), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(F[:, 1], 3.0 * fy(pts[:, 0], pts[:, 1]), rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(F[:, 2], 0.0)


def test_reference_scales(pecs_lib):
    """PostProcessor.cpp:11-17: densities unscaled, field 0.2585 / L."""
    s = vtu.Scales.physical(1e-4, 1e16, 1e-12)
    assert s.density == 1.0 and s.potential == 0.02585
    assert abs(s.field - 0.2585 / 1e-4) <= 1e-12 * s.field
    assert abs(s.current - 1.6e-19 * 1e16 * 1e-4 / 1e-12) <= 1e-12 * s.current


def test_graded_mesh_patches_follow_the_cell_edges(tmp_path, pecs_lib):
    """On a mesh graded toward the interface every patch spans its own cell:
    the library's cell edges (pecs_get_mesh) are the oracle's, and the
    written points lie on them."""
    import oracle
    from helpers import to_lib
    P = oracle.half_cell_params(n_refine=2, grading=6.0)
    pb = oracle.Problem(P)
    lib_p = to_lib(P)
    host = pg.Context(lib_p, host_setup_only=True)
    for which, g in ((pg.MESH_SEMI, pb.semi_grid), (pg.MESH_ELEC, pb.elec_grid),
                     (pg.MESH_POISSON, pb.poisson_grid)):
        xs, ys = host.mesh(which)
        np.testing.assert_allclose(xs, g.xs, rtol=0, atol=1e-15)
        np.testing.assert_allclose(ys, g.ys, rtol=0, atol=1e-15)
    nc, n1 = 16, 4
    vecs = {pg.FIELD_N: np.zeros(3 * nc * n1), pg.FIELD_P: np.zeros(3 * nc * n1)}
    path = tmp_path / "graded.vtu"
    vtu.write_carriers(FakeCtx(lib_p, vecs), str(path))
    _, a = _arrays(path)
    pts = a["Points"].reshape(nc, n1, 3)
    x0, y0, hx, hy = pb.semi_grid.cell_geom()
    np.testing.assert_allclose(pts[:, 0, 0], x0, atol=1e-15)
    np.testing.assert_allclose(pts[:, 3, 0], x0 + hx, atol=1e-15)
    np.testing.assert_allclose(pts[:, 3, 1], y0 + hy, atol=1e-15)
    assert hx[3] < hx[0] / 4     # finest next to the interface
    with pytest.raises(pg.PecsError):
        pg.Context(pg.pn_junction(), host_setup_only=True).mesh(pg.MESH_ELEC)
