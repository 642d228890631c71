"""SolarCellProblem's output and restart (pecs_gb300/reference_api.py), on
the CPU: print_results writes the files the reference's print_results writes
(Poisson-NNN.vtu and one <pair>NNN.vtu per carrier pair), print_dofs the
four <carrier>.dofs restart files, and read_dofs restarts from them with the
potential recomputed (SolarCell.cpp:1980-2034).  The context is a stand-in
whose states and Poisson solves come from the oracle."""
import os
import xml.etree.ElementTree as ET

import numpy as np

import oracle
import pecs_gb300 as pg
from helpers import FIELD_OF, to_lib
from pecs_gb300.reference_api import SolarCellProblem, block_read

NAMES = {v: k for k, v in FIELD_OF.items()}


class OracleCtx:
    """The part of Context that SolarCellProblem's output and restart use."""

    def __init__(self, P):
        self.P = P
        self.pb = oracle.Problem(P)
        lib_p = to_lib(P)
        self.params = [lib_p]
        self._host = pg.Context(lib_p, host_setup_only=True)
        self.ndofs = list(self._host.info().ndofs)
        self.st = None
        self.calls = []

    def initialize(self):
        self.calls.append("initialize")
        self.st = self.pb.initial_state()

    def get_state(self, f, inst=0):
        return self.st[NAMES[f]].copy()

    def set_state(self, f, v, inst=0):
        self.calls.append(f"set_state {NAMES[f]}")
        self.st[NAMES[f]] = np.asarray(v, dtype=float).copy()

    def assemble_poisson_rhs(self):
        self.calls.append("assemble_poisson_rhs")
        self._bP = self.pb.poisson_rhs(self.st)

    def solve_poisson(self):
        self.calls.append("solve_poisson")
        self.st["P"] = self.pb.solve_poisson(self._bP)

    def mesh(self, which):
        return self._host.mesh(which)


def _problem(ctx):
    sp = SolarCellProblem.__new__(SolarCellProblem)
    sp.sim_params, sp.ctx, sp.time, sp.counter = ctx.params[0], ctx, 0.0, 0
    return sp


def _density(path, name):
    piece = ET.parse(path).getroot().find("UnstructuredGrid/Piece")
    for a in piece.iter("DataArray"):
        if a.get("Name") == name:
            return np.array(a.text.split(), dtype=float)
    raise KeyError(name)


def test_print_results_and_dofs_then_restart(tmp_path, pecs_lib):
    P = oracle.half_cell_params(n_refine=2)
    ctx = OracleCtx(P)
    ctx.st, _, _ = ctx.pb.run(5)
    sp = _problem(ctx)
    sp.print_results(7, str(tmp_path))
    files = sorted(os.listdir(tmp_path))
    assert files == ["Electrolyte-007.vtu", "Poisson-007.vtu", "Semiconductor-007.vtu"]
    nc, n1 = ctx.pb.semi.nc, ctx.pb.semi.n1
    dens = _density(tmp_path / "Semiconductor-007.vtu", "Electrons Density")
    np.testing.assert_array_equal(dens, ctx.st["n"][2 * nc * n1:])
    dens = _density(tmp_path / "Electrolyte-007.vtu", "Oxidants Density")
    np.testing.assert_array_equal(dens, ctx.st["o"][2 * nc * n1:])

    d = tmp_path / "restart"
    d.mkdir()
    sp.print_dofs(str(d))
    assert sorted(os.listdir(d)) == ["Electrons.dofs", "Holes.dofs", "Oxidants.dofs",
                                     "Reductants.dofs"]
    for name, f in (("Electrons", "n"), ("Holes", "p"), ("Reductants", "r"), ("Oxidants", "o")):
        with open(d / (name + ".dofs"), "rb") as fh:
            np.testing.assert_array_equal(block_read(fh), ctx.st[f])

    # restart into a fresh problem: carriers from the files, potential re-solved
    ctx2 = OracleCtx(P)
    sp2 = _problem(ctx2)
    sp2.read_dofs(str(d))
    assert ctx2.calls[0] == "initialize" and ctx2.calls[-2:] == ["assemble_poisson_rhs",
                                                                 "solve_poisson"]
    for f in ("n", "p", "r", "o"):
        np.testing.assert_array_equal(ctx2.st[f], ctx.st[f])
    ref_P = ctx.pb.solve_poisson(ctx.pb.poisson_rhs(ctx.st))
    np.testing.assert_allclose(ctx2.st["P"], ref_P, rtol=0, atol=1e-13 * np.abs(ref_P).max())


def test_semiconductor_only_writes_one_pair(tmp_path, pecs_lib):
    P = oracle.pn_junction_params(nx_semi=4, ny=4)
    ctx = OracleCtx(P)
    ctx.initialize()
    sp = _problem(ctx)
    sp.print_results(0, str(tmp_path))
    sp.print_dofs(str(tmp_path))
    assert sorted(os.listdir(tmp_path)) == ["Electrons.dofs", "Holes.dofs", "Poisson-000.vtu",
                                            "Semiconductor-000.vtu"]
