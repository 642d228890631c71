"""Host-side mirror of the reference's class surface on the hot path.

Names, methods and their meaning follow the reference (paths relative to the
reference project):

* ``Carrier``      -- ChargeCarrierSpace::Carrier (include/Carrier.hpp:38-101):
  ``set_solver()`` factorises ``system_matrix``; ``solve()`` maps
  ``system_rhs`` to ``solution`` (source/Carrier.cpp:26-40).
* ``CarrierPair``  -- ChargeCarrierSpace::CarrierPair (include/CarrierPair.hpp:30-110):
  ``carrier_1``, ``carrier_2``, ``mass_matrix``, ``penalty``,
  ``material_permittivity``; ``print_dofs``/``read_dofs`` (CarrierPair.cpp:89-121).
* ``PoissonData``  -- Poisson::PoissonData (include/Poisson.hpp:26-84):
  ``set_solver()``, ``solve()`` (LU apply + zero constrained dofs,
  source/Poisson.cpp:90-105).
* ``SolarCellProblem`` -- the IMEX loop driver of
  SOLARCELL::SolarCellProblem::run_full_system (source/SolarCell.cpp:1898-2095)
  with the stage methods it calls each step, ``print_results`` (VTU files,
  SolarCell.cpp:1823-1858) and the end-of-run ``print_dofs`` restart files
  (SolarCell.cpp:2090-2092).

Errors surface as ``PecsError`` (a RuntimeError), as the reference's
exceptions reach ``main``'s ``catch (std::exception&)``.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import _ffi as F
from .api import LU, Context, Params


class Carrier:
    def __init__(self, name: str = "", charge_number: float = 0.0, scaled_mobility: float = 1.0):
        self.name = name
        self.charge_number = charge_number
        self.scaled_mobility = scaled_mobility
        self.system_matrix = None
        self.system_rhs: Optional[np.ndarray] = None
        self.solution: Optional[np.ndarray] = None
        self._lu: Optional[LU] = None
        # the caller's mesh information needed by nested dissection
        self.dof_cell = None
        self.dof_class = None
        self.cell_xy = None

    def set_name(self, name: str):
        self.name = name

    def set_solver(self, precision: int = F.PREC_FP64):
        if self.system_matrix is None or self.dof_cell is None or self.cell_xy is None:
            raise F.PecsError(F.PECS_E_STATE, "system_matrix and mesh maps must be set first")
        self._lu = LU(self.system_matrix, self.dof_cell, self.cell_xy, self.dof_class, precision)

    def solve(self):
        if self._lu is None:
            raise F.PecsError(F.PECS_E_STATE, "set_solver() must be called first")
        self.solution = self._lu.solve(self.system_rhs)


class CarrierPair:
    def __init__(self):
        self.carrier_1 = Carrier()
        self.carrier_2 = Carrier()
        self.mass_matrix = None
        self.penalty = 1.0
        self.delta_t = 0.0
        self.material_permittivity = 1.0
        self.material_name = ""

    def set_name(self, name: str):
        self.material_name = name

    def print_dofs(self, directory: str = "."):
        """Each carrier's solution as "<name>.dofs" (CarrierPair.cpp:89-104)."""
        import os
        for c in (self.carrier_1, self.carrier_2):
            with open(os.path.join(directory, c.name + ".dofs"), "wb") as fh:
                block_write(fh, c.solution)

    def read_dofs(self, directory: str = "."):
        """(CarrierPair.cpp:106-121)"""
        import os
        for c in (self.carrier_1, self.carrier_2):
            with open(os.path.join(directory, c.name + ".dofs"), "rb") as fh:
                c.solution = block_read(fh)


def block_write(fh, v) -> None:
    """The binary vector layout the reference's restart files use (deal.II
    Vector::block_write, called at CarrierPair.cpp:99-102): the size in ASCII
    decimal, a newline, '[', the raw doubles, ']'."""
    a = np.ascontiguousarray(v, dtype=np.float64)
    fh.write(f"{a.size}\n[".encode("ascii"))
    fh.write(a.tobytes())
    fh.write(b"]")


def block_read(fh) -> np.ndarray:
    """Inverse of block_write (deal.II Vector::block_read)."""
    head = b""
    while not head.endswith(b"["):
        ch = fh.read(1)
        if not ch:
            raise ValueError("truncated .dofs header")
        head += ch
    n = int(head[:-1].strip())
    data = fh.read(8 * n)
    if len(data) != 8 * n or fh.read(1) != b"]":
        raise ValueError("truncated or malformed .dofs body")
    return np.frombuffer(data, dtype=np.float64).copy()


class PoissonData(Carrier):
    def __init__(self):
        super().__init__("Poisson")
        self.constrained: Optional[np.ndarray] = None

    def solve(self):
        super().solve()
        if self.constrained is not None:
            self.solution[self.constrained] = 0.0


class SolarCellProblem:
    """The per-step stages of run_full_system on one GPU-resident context."""

    def __init__(self, params: Params, precision: int = F.PREC_FP64):
        self.sim_params = params
        self.ctx = Context(params, precision=precision)
        self.time = 0.0
        self.counter = 0

    # stage names of SolarCell.cpp:2057-2075
    def assemble_semiconductor_rhs(self):
        """Assembles both regions' carrier right-hand sides in one launch; the
        electrolyte call below is then a no-op."""
        self.ctx.assemble_carrier_rhs()
        self._electrolyte_done = True

    def assemble_electrolyte_rhs(self):
        if not getattr(self, "_electrolyte_done", False):
            self.ctx.assemble_carrier_rhs()
        self._electrolyte_done = False

    def solve_full_system(self):
        self.ctx.solve_carriers()

    def assemble_Poisson_rhs(self):  # noqa: N802 (reference name)
        self.ctx.assemble_poisson_rhs()

    def solve_Poisson(self):  # noqa: N802 (reference name)
        self.ctx.solve_poisson()

    # carrier names and pair names the reference sets (SolarCell.cpp:53-81)
    CARRIERS = (("Semiconductor-", F.FIELD_N, "Electrons", F.FIELD_P, "Holes"),
                ("Electrolyte-", F.FIELD_R, "Reductants", F.FIELD_O, "Oxidants"))

    def _pairs(self):
        full = bool(self.sim_params.full_system)
        return self.CARRIERS if full else self.CARRIERS[:1]

    def print_results(self, time_step_number: int, directory: str = ".", scales=None):
        """print_results (SolarCell.cpp:1823-1858): "Poisson-NNN.vtu" and one
        "<pair>NNN.vtu" per carrier pair, as output_rescaled_results names
        them (MixedFEM.cpp:297-320, LDG.cpp:1195-1232; NNN the step number in
        three digits), with the post-processor's scales (vtu.Scales)."""
        import os

        from . import vtu
        sc = scales if scales is not None else vtu.Scales()
        tag = f"{time_step_number:03d}"
        vtu.write_potential(self.ctx, os.path.join(directory, f"Poisson-{tag}.vtu"), scales=sc)
        for (pair, _, name1, _, name2), region in zip(self._pairs(), ("semi", "elec")):
            vtu.write_carriers(self.ctx, os.path.join(directory, f"{pair}{tag}.vtu"), region=region,
                               names=(name1, name2), scales=sc)

    def print_dofs(self, directory: str = "."):
        """The end-of-run restart files (SolarCell.cpp:2090-2092 through
        CarrierPair::print_dofs): "<carrier name>.dofs" per carrier."""
        for _, f1, name1, f2, name2 in self._pairs():
            cp = CarrierPair()
            cp.carrier_1.set_name(name1)
            cp.carrier_2.set_name(name2)
            cp.carrier_1.solution = self.ctx.get_state(f1)
            cp.carrier_2.solution = self.ctx.get_state(f2)
            cp.print_dofs(directory)

    def read_dofs(self, directory: str = "."):
        """Restart (SolarCell.cpp:1980-1995 through CarrierPair::read_dofs):
        the carriers' states from their .dofs files, then the Poisson
        right-hand side and solve for the potential they imply
        (SolarCell.cpp:2032-2034)."""
        self.ctx.initialize()
        for _, f1, name1, f2, name2 in self._pairs():
            cp = CarrierPair()
            cp.carrier_1.set_name(name1)
            cp.carrier_2.set_name(name2)
            cp.read_dofs(directory)
            self.ctx.set_state(f1, cp.carrier_1.solution)
            self.ctx.set_state(f2, cp.carrier_2.solution)
        self.ctx.assemble_poisson_rhs()
        self.ctx.solve_poisson()

    def run(self, t_end: float, number_outputs: int, directory: str = ".",
            restart_from: Optional[str] = None, t_end_2: Optional[float] = None, scales=None) -> int:
        """run_full_system's time loop with its outputs (SolarCell.cpp:1968-2092):
        the initial state (or, with restart_from, the .dofs files there) and
        print_results for it; then for each of number_outputs time stamps the
        IMEX steps while time < stamp, each stamp followed by print_results;
        at the end print_dofs.  Stamps: (k+1) t_end / number_outputs from
        time 0, or on a restart t_end + (k+1) (t_end_2 - t_end) / number_outputs
        from time t_end with output numbers continuing at number_outputs.
        Each interval's steps are counted with the reference's float
        accumulation (time += dt) and marched as one pecs_step call, which
        equals the stage-by-stage loop.  Returns the steps taken."""
        if number_outputs < 1:
            raise ValueError("number_outputs must be >= 1")
        dt = self.sim_params.dt
        if restart_from is None:
            self.ctx.initialize()
            stamps = [(k + 1) * t_end / number_outputs for k in range(number_outputs)]
            number, time = 0, 0.0
        else:
            if t_end_2 is None:
                raise ValueError("a restart needs t_end_2")
            self.read_dofs(restart_from)
            stamps = [t_end + (k + 1) * (t_end_2 - t_end) / number_outputs
                      for k in range(number_outputs)]
            number, time = number_outputs, t_end
        self.print_results(number, directory, scales)
        number += 1
        steps = 0
        for stamp in stamps:
            n = 0
            while time < stamp:
                time += dt
                n += 1
            if n:
                self.ctx.step(n)
            steps += n
            self.print_results(number, directory, scales)
            number += 1
        self.time = time
        self.counter += steps
        self.print_dofs(directory)
        return steps

    def run_full_system(self, n_steps: int, restart_from: Optional[str] = None):
        """n_steps IMEX steps from the initial condition, or, with
        restart_from, from the .dofs files in that directory (the reference's
        restart_status branch, SolarCell.cpp:1980-1995)."""
        if restart_from is None:
            self.ctx.initialize()
        else:
            self.read_dofs(restart_from)
        for _ in range(n_steps):
            self.assemble_semiconductor_rhs()
            self.assemble_electrolyte_rhs()
            self.solve_full_system()
            self.assemble_Poisson_rhs()
            self.solve_Poisson()
            self.time += self.sim_params.dt
            self.counter += 1
        return self.ctx.state()
