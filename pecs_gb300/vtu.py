"""Headless VTU output of carrier densities, currents, the field D and the potential.

Writes what the reference's post-processor writes (`source/PostProcessor.cpp:
6-124`, used by `LDG::output_rescaled_results` `source/LDG.cpp:1195-1232` and
`MixedFEM::output_rescaled_results` `source/MixedFEM.cpp:297-320`):

* a carrier pair: per carrier "<name> Current" (a vector, times the current
  scale) and "<name> Density" (copied without scaling, PostProcessor.cpp:
  101-107);
* the Poisson problem: "Field", the displacement D (a vector, times the field
  scale 0.2585 / L of PostProcessor.cpp:12) and "Potential" (times the thermal
  voltage 0.02585).

Like deal.II's DataOut with its default `build_patches()` (one subdivision),
every cell is its own patch and every quantity is point data evaluated at the
patch's points, so values are not averaged between cells; `subdivisions`
refines the patches as `build_patches(n)` would.  The file is plain XML
(ASCII), which ParaView and VisIt read.

State layout (the library's, `include/pecs.h`): carrier vectors are
component-wise [J_x | J_y | u], each cells x (k+1)^2 nodal values (DGQ_k on
equidistant nodes, x fastest).  The Poisson vector is [vertical-face RT dofs |
horizontal-face RT dofs | interior RT dofs | Phi (DGQ_{k-1})]: the RT_{k-1}
basis is nodal, its D_x component on k+1 equidistant normal nodes (the two
end nodes on the cell's left and right faces) times k tangential nodes
(i + 1/2) / k, D_y the same with the roles of x and y swapped, and a face's k
coefficients are shared by its two cells.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Sequence

import numpy as np

from . import _ffi as F


@dataclass
class Scales:
    """Post-processor factors (PostProcessor.cpp:11-17).  The defaults (1)
    write scaled values; `physical` gives the reference's: potential 0.02585 V
    (thermal voltage), field 0.2585 / L, current 1.6e-19 * rho * L / T.
    Densities are written unscaled by the reference; `density` is an extra
    factor for callers who want them in cm^-3 (default 1)."""
    potential: float = 1.0
    field: float = 1.0
    current: float = 1.0
    density: float = 1.0

    @staticmethod
    def physical(characteristic_length: float, characteristic_density: float,
                 characteristic_time: float) -> "Scales":
        return Scales(potential=0.02585, field=0.2585 / characteristic_length,
                      current=1.6e-19 * characteristic_density * characteristic_length
                      / characteristic_time, density=1.0)


def _lagrange(nodes, t):
    """Values (len(nodes), len(t)) of the Lagrange polynomials on `nodes` at t."""
    nodes = np.asarray(nodes, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    out = np.ones((len(nodes), len(t)))
    for a, xa in enumerate(nodes):
        for b, xb in enumerate(nodes):
            if a != b:
                out[a] *= (t - xb) / (xa - xb)
    return out


def _patches(xs, ys, s):
    """Points (cells*(s+1)^2, 3) and quads (cells*s*s, 4) of per-cell patches
    with s subdivisions on the mesh with cell edges xs, ys (cells i + nx*j;
    graded meshes too), and the patch points' reference coordinates t."""
    m = s + 1
    nx, ny = len(xs) - 1, len(ys) - 1
    t = np.linspace(0.0, 1.0, m)
    xs, ys = np.asarray(xs), np.asarray(ys)
    X = xs[:-1, None] + (xs[1:] - xs[:-1])[:, None] * t[None, :]     # (nx, m)
    Y = ys[:-1, None] + (ys[1:] - ys[:-1])[:, None] * t[None, :]     # (ny, m)
    px = np.broadcast_to(X[None, :, None, :], (ny, nx, m, m))
    py = np.broadcast_to(Y[:, None, :, None], (ny, nx, m, m))
    pts = np.stack([px.reshape(-1), py.reshape(-1), np.zeros(px.size)], axis=1)
    a, b = np.meshgrid(np.arange(s), np.arange(s))
    q = (a + m * b).reshape(-1)
    local = np.stack([q, q + 1, q + 1 + m, q + m], axis=1)             # (s*s, 4)
    base = (np.arange(nx * ny) * m * m)[:, None, None]
    quads = (base + local[None]).reshape(-1, 4).astype(np.int64)
    return pts, quads, t


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


def _eval_q(coef, deg, t):
    """A DGQ_deg field with per-cell nodal coefficients coef (nc, (deg+1)^2, x
    fastest; equidistant nodes, deg 0: the cell midpoint) at the patch points
    t x t of every cell -> (nc * len(t)^2,), points x fastest."""
    nodes = np.linspace(0.0, 1.0, deg + 1) if deg > 0 else np.array([0.5])
    Lx = _lagrange(nodes, t)                                          # (deg+1, m)
    c = coef.reshape(-1, deg + 1, deg + 1)                            # [cell, b (y), a (x)]
    return np.einsum("cba,ai,bj->cji", c, Lx, Lx).reshape(-1)


def write_carriers(ctx, path: str, inst: int = 0, region: str = "semi",
                   names=("Electrons", "Holes"), scales: Scales = Scales(),
                   subdivisions: int = 1) -> None:
    """One region's carrier pair (semi: n, p; elec: r, o) as point data on
    per-cell patches (LDG::output_rescaled_results, LDG.cpp:1195-1232)."""
    p = ctx.params[inst]
    k = p.degree
    n1 = (k + 1) ** 2
    xs, ys = ctx.mesh(F.MESH_SEMI if region == "semi" else F.MESH_ELEC)
    nc = (len(xs) - 1) * (len(ys) - 1)
    fields = (F.FIELD_N, F.FIELD_P) if region == "semi" else (F.FIELD_R, F.FIELD_O)
    pts, quads, t = _patches(xs, ys, subdivisions)
    pdata = {}
    for f, name in zip(fields, names):
        v = ctx.get_state(f, inst)
        jx = _eval_q(v[0:nc * n1], k, t)
        jy = _eval_q(v[nc * n1:2 * nc * n1], k, t)
        u = _eval_q(v[2 * nc * n1:3 * nc * n1], k, t)
        pdata[f"{name} Current"] = scales.current * np.stack([jx, jy, np.zeros_like(jx)], axis=1)
        pdata[f"{name} Density"] = scales.density * u
    _write(path, [_piece(pts, quads, pdata, {})])


def poisson_field_at(v, nx: int, ny: int, k: int, t) -> np.ndarray:
    """The displacement D of a Poisson vector v (RT_{k-1} x DGQ_{k-1}: k is the
    LDG degree for the reference's pairing, the LDG degree + 1 for RT_k x DGQ_k;
    layout above) at the points t x t of every cell of the nx x ny
    Poisson mesh -> (nc * len(t)^2, 2), points x fastest."""
    nc = nx * ny
    nvert, nhor = (nx + 1) * ny, nx * (ny + 1)
    nint = 2 * k * (k - 1)
    off_h = nvert * k
    off_i = off_h + nhor * k
    nn = np.linspace(0.0, 1.0, k + 1)
    tn = (np.arange(k) + 0.5) / k
    Ln, Lt = _lagrange(nn, t), _lagrange(tn, t)                       # (k+1, m), (k, m)
    j, i = np.divmod(np.arange(nc), nx)
    cells = np.arange(nc)
    # D_x coefficients [cell, b, a]: a normal (x) node 0..k, b tangential (y) node 0..k-1;
    # D_y coefficients [cell, b, a]: b normal (y) node 0..k, a tangential (x) node 0..k-1
    cx = np.zeros((nc, k, k + 1))
    cy = np.zeros((nc, k + 1, k))
    cnt = 0
    for b in range(k):
        cx[:, b, 0] = v[(i + (nx + 1) * j) * k + b]
        cx[:, b, k] = v[(i + 1 + (nx + 1) * j) * k + b]
        for a in range(1, k):
            cx[:, b, a] = v[off_i + cells * nint + cnt]
            cnt += 1
    for b in range(k + 1):
        for a in range(k):
            if b == 0:
                cy[:, b, a] = v[off_h + (i + nx * j) * k + a]
            elif b == k:
                cy[:, b, a] = v[off_h + (i + nx * (j + 1)) * k + a]
            else:
                cy[:, b, a] = v[off_i + cells * nint + cnt]
                cnt += 1
    dx = np.einsum("cba,ai,bj->cji", cx, Ln, Lt).reshape(-1)
    dy = np.einsum("cba,ai,bj->cji", cy, Lt, Ln).reshape(-1)
    return np.stack([dx, dy], axis=1)


def write_poisson(ctx, path: str, inst: int = 0, scales: Scales = Scales(),
                  subdivisions: int = 1) -> None:
    """The Poisson solution on the Poisson mesh (both regions) as
    MixedFEM::output_rescaled_results writes it (MixedFEM.cpp:297-320):
    "Field" (D, a vector) and "Potential", point data on per-cell patches."""
    from .learned import Layout
    p = ctx.params[inst]
    k = p.degree + int(getattr(p, "poisson_pairing", 0))   # RT_{k-1} x DGQ_{k-1}
    lay = Layout.of(ctx)
    xs, ys = ctx.mesh(F.MESH_POISSON)
    nx, ny = len(xs) - 1, len(ys) - 1
    v = ctx.get_state(F.FIELD_POISSON, inst)
    pts, quads, t = _patches(xs, ys, subdivisions)
    phi = _eval_q(v[lay.phi_off:lay.phi_off + lay.n_phi], k - 1, t)
    D = poisson_field_at(v, nx, ny, k, t)
    field = scales.field * np.concatenate([D, np.zeros((D.shape[0], 1))], axis=1)
    _write(path, [_piece(pts, quads, {"Field": field, "Potential": scales.potential * phi}, {})])


# the earlier name of write_poisson
write_potential = write_poisson
