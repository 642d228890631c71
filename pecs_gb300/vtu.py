"""Headless VTU output of carrier densities, currents and the potential.

Writes what the reference's post-processor writes for a carrier pair and for
the Poisson problem (`source/PostProcessor.cpp:6-124`, used by
`LDG::output_*` `source/LDG.cpp:1135-1290` and `MixedFEM::output_*`
`source/MixedFEM.cpp:297-358`): per carrier "<name> Current" (a vector) and
"<name> Density", scaled by the post-processor's factors, and "Potential".
Like deal.II's DataOut for discontinuous elements, every cell is its own
patch: a DGQ_k cell becomes k x k VTK quads over its (k+1)^2 nodal points, so
values are not averaged between cells.  The file is plain XML (ASCII), which
ParaView and VisIt read.

The densities live in the carrier vectors' u block and the currents in the
J_x / J_y blocks ([J_x | J_y | u], each cells x (k+1)^2, nodes x-fastest);
the potential is the DGQ_{k-1} block of the Poisson vector.  The field D is
not written (its RT basis is not evaluated here).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Sequence

import numpy as np

from . import _ffi as F


@dataclass
class Scales:
    """Post-processor factors (PostProcessor.cpp:11-17): potential 0.02585 V
    (thermal voltage), density = characteristic density, current =
    1.6e-19 * density * length / time.  The defaults (1) write scaled
    values."""
    potential: float = 1.0
    density: float = 1.0
    current: float = 1.0

    @staticmethod
    def physical(characteristic_length: float, characteristic_density: float,
                 characteristic_time: float) -> "Scales":
        return Scales(potential=0.02585, density=characteristic_density,
                      current=1.6e-19 * characteristic_density * characteristic_length
                      / characteristic_time)


def _patches(xs, ys, k):
    """Points (cells*(k+1)^2, 3) and quads (cells*k*k, 4) of per-cell patches
    on the mesh with cell edges xs, ys (cells i + nx*j; graded meshes too)."""
    m = k + 1
    nx, ny = len(xs) - 1, len(ys) - 1
    t = np.linspace(0.0, 1.0, m)
    pts, quads = [], []
    base = 0
    for j in range(ny):
        for i in range(nx):
            X = xs[i] + (xs[i + 1] - xs[i]) * t
            Y = ys[j] + (ys[j + 1] - ys[j]) * t
            for b in range(m):
                for a in range(m):
                    pts.append((X[a], Y[b], 0.0))
            for b in range(k):
                for a in range(k):
                    q = base + a + m * b
                    quads.append((q, q + 1, q + 1 + m, q + m))
            base += m * m
    return np.array(pts), np.array(quads, dtype=np.int64)


def _piece(points, quads, point_data: Dict[str, np.ndarray], cell_data: Dict[str, np.ndarray]) -> str:
    def arr(name, a, ncomp):
        vals = " ".join(f"{v:.17g}" for v in np.asarray(a, dtype=np.float64).ravel())
        return (f'<DataArray type="Float64" Name="{name}" NumberOfComponents="{ncomp}" '
                f'format="ascii">{vals}</DataArray>')
    out = [f'<Piece NumberOfPoints="{len(points)}" NumberOfCells="{len(quads)}">']
    out.append("<PointData>")
    for name, a in point_data.items():
        out.append(arr(name, a, 3 if a.ndim == 2 else 1))
    out.append("</PointData><CellData>")
    for name, a in cell_data.items():
        out.append(arr(name, a, 1))
    out.append("</CellData><Points>")
    out.append(arr("Points", points, 3))
    out.append("</Points><Cells>")
    out.append('<DataArray type="Int64" Name="connectivity" format="ascii">'
               + " ".join(str(v) for v in quads.ravel()) + "</DataArray>")
    out.append('<DataArray type="Int64" Name="offsets" format="ascii">'
               + " ".join(str(4 * (c + 1)) for c in range(len(quads))) + "</DataArray>")
    out.append('<DataArray type="UInt8" Name="types" format="ascii">'
               + " ".join("9" for _ in range(len(quads))) + "</DataArray>")
    out.append("</Cells></Piece>")
    return "".join(out)


def _write(path, pieces: Sequence[str]):
    with open(path, "w") as fh:
        fh.write('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" '
                 'byte_order="LittleEndian" header_type="UInt64">\n<UnstructuredGrid>')
        for pc in pieces:
            fh.write(pc)
        fh.write("</UnstructuredGrid>\n</VTKFile>\n")


def write_carriers(ctx, path: str, inst: int = 0, region: str = "semi",
                   names=("Electrons", "Holes"), scales: Scales = Scales()) -> None:
    """One region's carrier pair (semi: n, p; elec: r, o) as point data on
    per-cell patches."""
    p = ctx.params[inst]
    k = p.degree
    m = k + 1
    n1 = m * m
    xs, ys = ctx.mesh(F.MESH_SEMI if region == "semi" else F.MESH_ELEC)
    nc = (len(xs) - 1) * (len(ys) - 1)
    fields = (F.FIELD_N, F.FIELD_P) if region == "semi" else (F.FIELD_R, F.FIELD_O)
    pts, quads = _patches(xs, ys, k)
    pdata = {}
    for f, name in zip(fields, names):
        v = ctx.get_state(f, inst)
        jx = v[0:nc * n1]
        jy = v[nc * n1:2 * nc * n1]
        u = v[2 * nc * n1:3 * nc * n1]
        pdata[f"{name} Current"] = scales.current * np.stack([jx, jy, np.zeros_like(jx)], axis=1)
        pdata[f"{name} Density"] = scales.density * u
    _write(path, [_piece(pts, quads, pdata, {})])


def write_potential(ctx, path: str, inst: int = 0, scales: Scales = Scales()) -> None:
    """The potential on the Poisson mesh (both regions): DGQ_{k-1}; k = 1
    gives one value per cell (cell data), k >= 2 nodal values per patch."""
    from .learned import Layout
    p = ctx.params[inst]
    k = p.degree
    lay = Layout.of(ctx)
    xs, ys = ctx.mesh(F.MESH_POISSON)
    v = ctx.get_state(F.FIELD_POISSON, inst)
    phi = scales.potential * v[lay.phi_off:lay.phi_off + lay.n_phi]
    if k == 1:
        pts, quads = _patches(xs, ys, 1)
        _write(path, [_piece(pts, quads, {}, {"Potential": phi})])
    else:
        pts, quads = _patches(xs, ys, k - 1)
        _write(path, [_piece(pts, quads, {"Potential": phi}, {})])
