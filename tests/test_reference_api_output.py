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

    def step(self, n):
        self.calls.append(f"step {n}")
        self.st, _, _ = self.pb.run(n, self.st)


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


def test_run_loop_outputs_and_restart(tmp_path, pecs_lib):
    """The reference's loop: outputs 000..N at the stamps, steps counted by
    float accumulation, restart files at the end; a restart continues the
    output numbers and the time from t_end."""
    P = oracle.half_cell_params(n_refine=2, dt=1e-3)
    ctx = OracleCtx(P)
    sp = _problem(ctx)
    d1 = tmp_path / "first"
    d1.mkdir()
    steps = sp.run(0.010, 3, str(d1))
    # stamps 0.00333.., 0.00666.., 0.01 with time += 1e-3 from 0
    expected, time = [], 0.0
    for stamp in (0.010 / 3, 2 * 0.010 / 3, 0.010):
        n = 0
        while time < stamp:
            time += 1e-3
            n += 1
        expected.append(n)
    assert steps == sum(expected)
    assert [c for c in ctx.calls if c.startswith("step")] == [f"step {n}" for n in expected]
    names = sorted(os.listdir(d1))
    for i in range(4):
        for pair in ("Poisson-", "Semiconductor-", "Electrolyte-"):
            assert f"{pair}{i:03d}.vtu" in names
    assert "Electrons.dofs" in names and "Oxidants.dofs" in names
    ref, _, _ = oracle.Problem(P).run(steps)
    for f in ("n", "p", "r", "o", "P"):
        np.testing.assert_array_equal(ctx.st[f], ref[f])
    # restart: the restart state printed as output 3, then outputs 4..6;
    # time runs from t_end to t_end_2
    ctx2 = OracleCtx(P)
    sp2 = _problem(ctx2)
    d2 = tmp_path / "second"
    d2.mkdir()
    more = sp2.run(0.010, 3, str(d2), restart_from=str(d1), t_end_2=0.016)
    n, time = 0, 0.010
    for stamp in (0.010 + k * 0.006 / 3 for k in (1, 2, 3)):
        while time < stamp:
            time += 1e-3
            n += 1
    assert more == n
    names = sorted(os.listdir(d2))
    assert [f"Poisson-{i:03d}.vtu" for i in range(3, 7)] == [x for x in names if x.startswith("Poisson")]
