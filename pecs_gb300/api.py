"""Python host API over the C ABI: parameters, problem contexts, the drop-in LU.

``Params`` holds already-scaled parameters (the role of
ParameterSpace::Parameters, include/Parameters.hpp:27-289 of the reference);
``Context`` owns one GPU-resident group of instances that share meshes and
matrices; ``LU`` is the externally-assembled direct solver
(SparseDirectUMFPACK's initialize/vmult as used by Carrier/PoissonData).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _ffi as F
from ._ffi import (DIRICHLET, INTERFACE, NEUMANN, SCHOTTKY, FIELD_N, FIELD_O, FIELD_P,
                   FIELD_POISSON, FIELD_R, PREC_FP32_IR, PREC_FP32_MIXED, PREC_FP64, check, lib)


@dataclass
class Params:
    degree: int = 1
    full_system: bool = True
    nx_semi: int = 16
    nx_elec: int = 16
    ny: int = 16
    x_semi0: float = 0.0
    x_semi1: float = 1.0
    x_elec1: float = 2.0
    height: float = 1.0
    bc_semi: tuple = (DIRICHLET, INTERFACE, NEUMANN, NEUMANN)
    bc_elec: tuple = (INTERFACE, DIRICHLET, NEUMANN, NEUMANN)
    bc_poisson: tuple = (DIRICHLET, DIRICHLET, NEUMANN, NEUMANN)
    lambda2: float = 1e-2
    eps_semi: float = 1.0
    eps_elec: float = 1.5
    mu: tuple = (1.0, 1.0, 1.0, 1.0)
    dt: float = 1e-3
    penalty: float = 1.0
    k_et: float = 1e-2
    k_ht: float = 1e-2
    junction_x: float = 0.5
    nd: tuple = (1.0, 1.0)
    na: tuple = (0.0, 0.0)
    n_eq: tuple = (1.0, 1.0)
    p_eq: tuple = (1e-4, 1e-4)
    r_eq: float = 1.0
    o_eq: float = 1.0
    ic_kind: int = 0
    gen_kind: int = 2
    G0: float = 1.0
    alpha: float = 5.0
    srh: bool = True
    tau_n: float = 1.0
    tau_p: float = 1.0
    n_i: float = 1e-2
    phi_bi: float = 0.0
    phi_app: float = 0.0
    s_n: float = 0.0
    s_p: float = 0.0
    grading: float = 1.0  # widest/narrowest cell along x, finest at the interface (1: uniform)
    bc_poisson_elec: tuple = (0, 0, 0, 0)  # Poisson outer-face ids over the electrolyte (<= 0: bc_poisson)
    poisson_pairing: int = 0  # 0: RT_{k-1} x DGQ_{k-1} (the reference's), 1: RT_k x DGQ_k (the configurations')

    def copy(self, **kw) -> "Params":
        return dataclasses.replace(self, **kw)

    def to_c(self) -> F.pecs_params:
        p = F.pecs_params()
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, (tuple, list)):
                arr = getattr(p, f.name)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(p, f.name, int(v) if isinstance(v, bool) else v)
        return p


@dataclass
class PhysicalParams:
    """Physical parameters in the reference's units, as input_file.prm gives
    them (sections computational, mesh, physical, electrons, holes,
    reductants, oxidants of ParameterReader::declare_parameters,
    source/ParameterReader.cpp:29-208).  The defaults are the reference's
    input_file.prm values."""
    time_step: float = 0.05
    mesh_height: float = 1.0
    illuminated: bool = True
    applied_bias: float = 0.0
    built_in_bias: float = 0.41
    schottky_bias: float = 0.0
    characteristic_length: float = 1.0e-4
    characteristic_density: float = 1.0e16
    characteristic_time: float = 1.0e-12
    intrinsic_density: float = 2.564e9
    photon_flux: float = 1.2e17
    absorption_coeff: float = 1.74974e5
    semiconductor_permittivity: float = 11.9
    electrolyte_permittivity: float = 1000.0
    electron_mobility: float = 1350.0
    hole_mobility: float = 480.0
    reductant_mobility: float = 1.0
    oxidant_mobility: float = 1.0
    electron_recombination_time: float = 5e-5
    hole_recombination_time: float = 5e-5
    electron_recombination_velocity: float = 3e5
    hole_recombination_velocity: float = 2.9e5
    electron_transfer_rate: float = 1e-19
    hole_transfer_rate: float = 1e-14

    @classmethod
    def reference(cls) -> "PhysicalParams":
        """The library's copy of the reference's input_file.prm values."""
        c = F.pecs_physical_params()
        lib().pecs_reference_physical_params(C.byref(c))
        return cls(**{f.name: (bool(getattr(c, f.name)) if f.type in (bool, "bool")
                               else getattr(c, f.name)) for f in dataclasses.fields(cls)})

    def to_c(self) -> F.pecs_physical_params:
        c = F.pecs_physical_params()
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            setattr(c, f.name, int(v) if isinstance(v, bool) else float(v))
        return c


# (subsection, key) of the reference's .prm files -> PhysicalParams field
# (source/ParameterReader.cpp:29-208)
_PRM_KEYS = {
    ("computational", "time step size"): "time_step",
    ("mesh", "mesh height"): "mesh_height",
    ("physical", "illumination status"): "illuminated",
    ("physical", "applied bias"): "applied_bias",
    ("physical", "built in bias"): "built_in_bias",
    ("physical", "schottky bias"): "schottky_bias",
    ("physical", "characteristic length"): "characteristic_length",
    ("physical", "characteristic density"): "characteristic_density",
    ("physical", "characteristic time"): "characteristic_time",
    ("physical", "intrinsic density"): "intrinsic_density",
    ("physical", "photon flux"): "photon_flux",
    ("physical", "absorption coefficient"): "absorption_coeff",
    ("physical", "semiconductor permittivity"): "semiconductor_permittivity",
    ("physical", "electrolyte permittivity"): "electrolyte_permittivity",
    ("electrons", "mobility"): "electron_mobility",
    ("electrons", "recombination time"): "electron_recombination_time",
    ("electrons", "recombination velocity"): "electron_recombination_velocity",
    ("electrons", "transfer rate"): "electron_transfer_rate",
    ("holes", "mobility"): "hole_mobility",
    ("holes", "recombination time"): "hole_recombination_time",
    ("holes", "recombination velocity"): "hole_recombination_velocity",
    ("holes", "transfer rate"): "hole_transfer_rate",
    ("reductants", "mobility"): "reductant_mobility",
    ("oxidants", "mobility"): "oxidant_mobility",
}


def read_prm(text: str, base: Optional[PhysicalParams] = None) -> PhysicalParams:
    """Physical parameters from the text of a deal.II ParameterHandler file in
    the layout of the reference's input_file.prm: ``subsection NAME`` ...
    ``end`` blocks of ``set KEY = VALUE`` lines, ``#`` comments.  Entries this
    library does not use (refinements, end times, mesh radii, switches of the
    boundary layout) are skipped; missing entries keep base's value (default:
    the reference's file).  Booleans are ``true``/``false``."""
    out = dataclasses.replace(base) if base is not None else PhysicalParams()
    types = {f.name: f.type for f in dataclasses.fields(PhysicalParams)}
    stack = []
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        word = line.split(None, 1)
        if word[0] == "subsection":
            stack.append(word[1].strip() if len(word) > 1 else "")
        elif word[0] == "end":
            if not stack:
                raise ValueError(f"line {lineno}: 'end' without a subsection")
            stack.pop()
        elif word[0] == "set":
            if len(word) < 2 or "=" not in word[1]:
                raise ValueError(f"line {lineno}: expected 'set KEY = VALUE'")
            key, val = (t.strip() for t in word[1].split("=", 1))
            name = _PRM_KEYS.get((stack[-1] if stack else "", key))
            if name is None:
                continue
            if types[name] in (bool, "bool"):
                if val not in ("true", "false"):
                    raise ValueError(f"line {lineno}: {key} must be true or false")
                setattr(out, name, val == "true")
            else:
                setattr(out, name, float(val))
        else:
            raise ValueError(f"line {lineno}: cannot read {raw!r}")
    if stack:
        raise ValueError(f"subsection {stack[-1]!r} is not closed")
    return out


def scale_params(phys: PhysicalParams, p: Optional[Params] = None):
    """Parameters::parse_and_scale_parameters (include/Parameters.hpp:117-287)
    through pecs_scale_params: returns (p with the scaled physical fields,
    {mobility_scale, rescale_current, rescaled_k_et, rescaled_k_ht,
    schottky_bias}).  Mesh, degree, layout and profile fields of p are kept."""
    c = (p if p is not None else Params()).to_c()
    sc = F.pecs_scales()
    check(lib().pecs_scale_params(C.byref(phys.to_c()), C.byref(c), C.byref(sc)))
    base = p if p is not None else Params()
    kw = {}
    for f in dataclasses.fields(Params):
        v = getattr(c, f.name)
        old = getattr(base, f.name)
        if isinstance(old, tuple):
            kw[f.name] = tuple(v[i] for i in range(len(old)))
        elif isinstance(old, bool):
            kw[f.name] = bool(v)
        else:
            kw[f.name] = v
    scales = {name: getattr(sc, name) for name, _ in F.pecs_scales._fields_}
    return dataclasses.replace(base, **kw), scales


def pn_junction(**kw) -> Params:
    """Semiconductor-only p-n junction on the unit square, 16x16 cells, k=1,
    dt=1e-3, 100 steps, initial densities = doping."""
    n_i = 1e-2
    p = Params(degree=1, full_system=False, nx_semi=16, nx_elec=0, ny=16,
               bc_semi=(DIRICHLET, DIRICHLET, NEUMANN, NEUMANN),
               bc_poisson=(DIRICHLET, DIRICHLET, NEUMANN, NEUMANN),
               lambda2=1e-2, eps_semi=1.0, dt=1e-3, junction_x=0.5, nd=(1.0, 0.0), na=(0.0, 1.0),
               n_eq=(1.0, n_i * n_i), p_eq=(n_i * n_i, 1.0), ic_kind=1, gen_kind=0, srh=True,
               tau_n=1.0, tau_p=1.0, n_i=n_i, phi_bi=math.log(1.0 / (n_i * n_i)), phi_app=0.0,
               k_et=0.0, k_ht=0.0)
    return p.copy(**kw)


def half_cell(n_refine: int = 6, **kw) -> Params:
    """Coupled half cell: semiconductor [0,1]^2 and electrolyte [1,2]x[0,1],
    2^r x 2^r cells each, k=1, G = G0 exp(-alpha (1-x)), dt=1e-3."""
    n_i = 1e-2
    n = 2 ** n_refine
    p = Params(degree=1, full_system=True, nx_semi=n, nx_elec=n, ny=n, lambda2=1e-2,
               eps_semi=1.0, eps_elec=1.5, dt=1e-3, nd=(1.0, 1.0), na=(0.0, 0.0),
               n_eq=(1.0, 1.0), p_eq=(n_i * n_i, n_i * n_i), r_eq=1.0, o_eq=1.0, ic_kind=0,
               gen_kind=2, G0=1.0, alpha=5.0, srh=True, tau_n=1.0, tau_p=1.0, n_i=n_i,
               k_et=1e-2, k_ht=1e-2, phi_bi=0.0, phi_app=0.0)
    return p.copy(**kw)


def boundary_layout(p: Params, insulated: bool = False, schottky: bool = False) -> Params:
    """The reference's boundary layouts (Grid::make_grids, source/Grid.cpp:112-131)
    on a copy of p.  Every outer side is Dirichlet, the semiconductor-electrolyte
    interface keeps the Interface id (make_Dirichlet_boundaries, Grid.cpp:343-373).
    insulated (make_Neumann_boundaries, Grid.cpp:377-431): the left side is
    Neumann, and the top and bottom are Neumann over the electrolyte and
    Dirichlet over the semiconductor -- on the Poisson mesh too, whose top and
    bottom then change id at the interface.  schottky
    (make_Schottky_boundaries, Grid.cpp:434-461): the top side of the
    semiconductor and of the whole Poisson mesh is Schottky; the electrolyte
    mesh keeps its ids."""
    D, N, I, S = DIRICHLET, NEUMANN, INTERFACE, SCHOTTKY
    semi = [D, I if p.full_system else D, D, D]
    elec = [I, D, D, D]
    pois = [D, D, D, D]
    pois_elec = [0, 0, 0, 0]
    if insulated:
        semi[0] = N
        pois[0] = N
        if p.full_system:
            elec[2] = elec[3] = N
            pois_elec[2] = pois_elec[3] = N
    if schottky:
        semi[3] = S
        pois[3] = S
        if p.full_system:
            pois_elec[3] = S
    return p.copy(bc_semi=tuple(semi), bc_elec=tuple(elec), bc_poisson=tuple(pois),
                  bc_poisson_elec=tuple(pois_elec))


def reference_params(n_refine: int = 4, degree: int = 1, **kw) -> Params:
    """Reference-faithful physics: constant equilibria 2, 0, 30, 29, SRH = 0,
    generation alpha*G0*exp(alpha*(y-H)), Dirichlet on every outer side."""
    n = 2 ** n_refine
    p = Params(degree=degree, nx_semi=n, nx_elec=n, ny=n, nd=(2.0, 2.0), na=(0.0, 0.0),
               n_eq=(2.0, 2.0), p_eq=(0.0, 0.0), r_eq=30.0, o_eq=29.0, ic_kind=0, gen_kind=1,
               srh=False, bc_semi=(DIRICHLET, INTERFACE, DIRICHLET, DIRICHLET),
               bc_elec=(INTERFACE, DIRICHLET, DIRICHLET, DIRICHLET),
               bc_poisson=(DIRICHLET, DIRICHLET, DIRICHLET, DIRICHLET))
    return p.copy(**kw)


def default_options(precision: int = PREC_FP64, use_graphs: bool = True, leaf_cells: int = 8,
                    ir_max_iters: int = 0, device: int = 0, host_setup_only: bool = False,
                    panel_chunk: int = 0, panel_min_ctas: int = 0,
                    autotune: bool = True, gpu_factor_min_front: int = 0,
                    flow_sweep: int = 0, increment_solves: bool = False) -> F.pecs_options:
    o = F.pecs_options()
    lib().pecs_default_options(C.byref(o))
    o.precision = precision
    o.use_graphs = int(use_graphs)
    o.leaf_cells = leaf_cells
    o.ir_max_iters = ir_max_iters
    o.device = device
    o.host_setup_only = int(host_setup_only)
    o.panel_chunk = panel_chunk
    o.panel_min_ctas = panel_min_ctas
    o.autotune = int(autotune)
    o.gpu_factor_min_front = gpu_factor_min_front
    o.flow_sweep = flow_sweep
    o.increment_solves = int(increment_solves)
    return o


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Context:
    """A group of instances resident on one GPU (pecs_create)."""

    def __init__(self, params: Sequence[Params] | Params, precision: int = PREC_FP64,
                 use_graphs: bool = True, leaf_cells: int = 8, ir_max_iters: int = 0,
                 device: int = 0, host_setup_only: bool = False, panel_chunk: int = 0,
                 panel_min_ctas: int = 0, autotune: bool = True, gpu_factor_min_front: int = 0,
                 flow_sweep: int = 0, increment_solves: bool = False):
        if isinstance(params, Params):
            params = [params]
        self.params = list(params)
        arr = (F.pecs_params * len(self.params))(*[p.to_c() for p in self.params])
        opt = default_options(precision, use_graphs, leaf_cells, ir_max_iters, device,
                              host_setup_only, panel_chunk, panel_min_ctas, autotune,
                              gpu_factor_min_front, flow_sweep, increment_solves)
        h = C.c_void_p()
        check(lib().pecs_create(arr, len(self.params), C.byref(opt), C.byref(h)))
        self._h = h
        self.n_inst = len(self.params)
        self.full = bool(self.params[0].full_system)
        info = self.info()
        self.ndofs = list(info.ndofs)

    def close(self):
        if getattr(self, "_h", None):
            lib().pecs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> F.pecs_info:
        i = F.pecs_info()
        check(lib().pecs_get_info(self._h, C.byref(i)))
        return i

    def setup_vector(self, kind: int, field: int, inst: int = 0) -> np.ndarray:
        """Host-computed setup vector (SETUP_CONST_RHS or SETUP_INITIAL) of one
        instance and field; also on host_setup_only contexts."""
        out = np.zeros(self.ndofs[field])
        check(lib().pecs_get_setup_vector(self._h, kind, field, inst, _dptr(out), out.size))
        return out

    def mesh(self, which: int):
        """Cell edges (xs, ys) of a mesh (MESH_SEMI, MESH_ELEC, MESH_POISSON);
        cells are numbered i + nx*j."""
        nx, ny = C.c_int(), C.c_int()
        check(lib().pecs_get_mesh(self._h, which, C.byref(nx), C.byref(ny), None, None))
        xs, ys = np.zeros(nx.value + 1), np.zeros(ny.value + 1)
        check(lib().pecs_get_mesh(self._h, which, None, None, _dptr(xs), _dptr(ys)))
        return xs, ys

    def matrix(self, which: int):
        import scipy.sparse as sp
        n = C.c_int()
        nnz = C.c_longlong()
        check(lib().pecs_get_matrix(self._h, which, C.byref(n), C.byref(nnz), None, None, None))
        rp = np.zeros(n.value + 1, dtype=np.int32)
        ci = np.zeros(nnz.value, dtype=np.int32)
        v = np.zeros(nnz.value)
        check(lib().pecs_get_matrix(self._h, which, None, None,
                                    rp.ctypes.data_as(C.POINTER(C.c_int)),
                                    ci.ctypes.data_as(C.POINTER(C.c_int)), _dptr(v)))
        return sp.csr_matrix((v, ci, rp), shape=(n.value, n.value))

    def initialize(self):
        check(lib().pecs_initialize(self._h))

    def get_state(self, field: int, inst: int = 0) -> np.ndarray:
        out = np.zeros(self.ndofs[field])
        check(lib().pecs_get_state(self._h, inst, field, _dptr(out), out.size))
        return out

    def set_state(self, field: int, values: np.ndarray, inst: int = 0):
        v = np.ascontiguousarray(values, dtype=np.float64)
        check(lib().pecs_set_state(self._h, inst, field, _dptr(v), v.size))

    def set_instances(self, params: Sequence[Params]):
        params = list(params)
        arr = (F.pecs_params * len(params))(*[p.to_c() for p in params])
        check(lib().pecs_set_instances(self._h, arr, len(params)))
        self.params = params

    def get_state_device(self, field: int, inst: int, dst_ptr: int):
        check(lib().pecs_get_state_device(self._h, inst, field, C.c_void_p(dst_ptr)))

    def set_state_device(self, field: int, inst: int, src_ptr: int):
        check(lib().pecs_set_state_device(self._h, inst, field, C.c_void_p(src_ptr)))

    def get_rhs(self, field: int, inst: int = 0) -> np.ndarray:
        out = np.zeros(self.ndofs[field])
        check(lib().pecs_get_rhs(self._h, inst, field, _dptr(out), out.size))
        return out

    def fields(self):
        return (FIELD_N, FIELD_P, FIELD_R, FIELD_O, FIELD_POISSON) if self.full else \
            (FIELD_N, FIELD_P, FIELD_POISSON)

    def state(self, inst: int = 0) -> dict:
        names = {FIELD_N: "n", FIELD_P: "p", FIELD_R: "r", FIELD_O: "o", FIELD_POISSON: "P"}
        return {names[f]: self.get_state(f, inst) for f in self.fields()}

    def assemble_carrier_rhs(self):
        check(lib().pecs_assemble_carrier_rhs(self._h))

    def solve_carriers(self):
        check(lib().pecs_solve_carriers(self._h))

    def assemble_poisson_rhs(self):
        check(lib().pecs_assemble_poisson_rhs(self._h))

    def solve_poisson(self):
        check(lib().pecs_solve_poisson(self._h))

    def step(self, n: int = 1):
        check(lib().pecs_step(self._h, n))

    def run_to_steady_state(self, max_steps: int, tol: float, check_every: int = 50):
        steps = np.zeros(self.n_inst, dtype=np.int32)
        rel = np.zeros(self.n_inst)
        check(lib().pecs_run_to_steady_state(self._h, max_steps, tol, check_every,
                                             steps.ctypes.data_as(C.POINTER(C.c_int)), _dptr(rel)))
        return steps, rel

    def probe_step(self) -> np.ndarray:
        """One step of every instance; returns each instance's relative change.
        An instance whose state became non-finite gets +inf instead of raising
        (the warm start's fallback test treats it as the worse start)."""
        steps = np.zeros(self.n_inst, dtype=np.int32)
        rel = np.zeros(self.n_inst)
        code = lib().pecs_run_to_steady_state(self._h, 1, 0.0, 1,
                                              steps.ctypes.data_as(C.POINTER(C.c_int)), _dptr(rel))
        if code == F.PECS_E_NONFINITE:
            rel[steps < 0] = np.inf
        else:
            check(code)
        rel[~np.isfinite(rel)] = np.inf
        return rel

    def last_run_steps(self) -> int:
        return lib().pecs_last_run_steps(self._h)

    def stream(self) -> int:
        return lib().pecs_get_stream(self._h) or 0

    def time_stages(self, reps: int = 10) -> dict:
        """Mean device milliseconds per stage of a time step (pecs_time_stages):
        carrier RHS, carrier solves, Poisson RHS, Poisson solve.  Advances the
        state by reps + 1 steps."""
        ms = (C.c_double * 4)()
        check(lib().pecs_time_stages(self._h, reps, ms))
        return dict(zip(("carrier_rhs", "carrier_solve", "poisson_rhs", "poisson_solve"), list(ms)))

    def time_solve(self, which: int, reps: int = 20) -> float:
        """Mean device milliseconds of one carrier (0) / Poisson (1) solve sweep."""
        ms = C.c_double()
        check(lib().pecs_time_solve(self._h, which, reps, C.byref(ms)))
        return ms.value

    def solve_residual(self, which: int) -> float:
        """Largest relative residual of the latest carrier (0) / Poisson (1) solve."""
        out = C.c_double()
        check(lib().pecs_solve_residual(self._h, which, C.byref(out)))
        return out.value

    def synchronize(self):
        check(lib().pecs_synchronize(self._h))

    def interface_current(self) -> np.ndarray:
        out = np.zeros(self.n_inst)
        check(lib().pecs_interface_current(self._h, _dptr(out)))
        return out

    def iv_sweep(self, max_steps: int, tol: float, check_every: int = 50,
                 init: Optional[dict] = None, want_fields: bool = False):
        """End-to-end I-V sweep through the public API: host initial state in,
        host currents (and optionally fields) out."""
        init_arr = None
        keep = []
        if init is not None:
            ptrs = (C.POINTER(C.c_double) * 5)()
            for f in range(5):
                if self.ndofs[f]:
                    a = np.ascontiguousarray(init[f], dtype=np.float64).reshape(-1)
                    keep.append(a)
                    ptrs[f] = _dptr(a)
            init_arr = ptrs
        cur = np.zeros(self.n_inst)
        steps = np.zeros(self.n_inst, dtype=np.int32)
        finals = None
        fptrs = None
        if want_fields:
            finals = {f: np.zeros(self.n_inst * self.ndofs[f]) for f in range(5) if self.ndofs[f]}
            fptrs = (C.POINTER(C.c_double) * 5)()
            for f, a in finals.items():
                fptrs[f] = _dptr(a)
        check(lib().pecs_iv_sweep(self._h, init_arr, max_steps, tol, check_every, _dptr(cur),
                                  steps.ctypes.data_as(C.POINTER(C.c_int)), fptrs))
        return cur, steps, finals

    def sweep_stream(self, params: Sequence[Params], max_steps: int, tol: float,
                     check_every: int = 50, init_n: Optional[Sequence[int]] = None,
                     init_p: Optional[Sequence[int]] = None, want_fields=False):
        """Streamed I-V sweep (pecs_sweep_stream): every parameter set marched
        to steady state through this context's slots, each slot refilled as
        soon as its point finishes.  init_n / init_p: per point a device
        pointer (int, 0 = built-in initial condition) to a full electron /
        hole vector.  want_fields: False, True (every field) or a list of
        field indices to return.  Returns (steps, currents, fields or None)."""
        n = len(params)
        arr = (F.pecs_params * n)(*[p.to_c() for p in params])
        def ptrs(lst):
            if lst is None:
                return None
            a = (C.c_void_p * n)()
            for k, v in enumerate(lst):
                a[k] = C.c_void_p(int(v)) if v else None
            return a
        steps = np.zeros(n, dtype=np.int32)
        cur = np.zeros(n)
        finals = fptrs = None
        if want_fields:
            sel = range(5) if want_fields is True else want_fields
            finals = {f: np.zeros(n * self.ndofs[f]) for f in sel if self.ndofs[f]}
            fptrs = (C.POINTER(C.c_double) * 5)()
            for f, a in finals.items():
                fptrs[f] = _dptr(a)
        check(lib().pecs_sweep_stream(self._h, n, arr, ptrs(init_n), ptrs(init_p), max_steps, tol,
                                      check_every, steps.ctypes.data_as(C.POINTER(C.c_int)),
                                      _dptr(cur), fptrs))
        return steps, cur, finals


class LU:
    """Drop-in direct solver: factor(set_solver) once, solve() every step."""

    def __init__(self, A, dof_cell: np.ndarray, cell_xy: np.ndarray,
                 dof_class: Optional[np.ndarray] = None, precision: int = PREC_FP64,
                 leaf_cells: int = 8):
        import scipy.sparse as sp
        A = sp.csr_matrix(A)
        A.sort_indices()
        self.n = A.shape[0]
        rp = np.ascontiguousarray(A.indptr, dtype=np.int32)
        ci = np.ascontiguousarray(A.indices, dtype=np.int32)
        v = np.ascontiguousarray(A.data, dtype=np.float64)
        dc = np.ascontiguousarray(dof_cell, dtype=np.int32)
        xy = np.ascontiguousarray(cell_xy, dtype=np.float64).reshape(-1)
        cls = None if dof_class is None else np.ascontiguousarray(dof_class, dtype=np.int32)
        h = C.c_void_p()
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        check(lib().pecs_lu_factor(self.n, ip(rp), ip(ci), _dptr(v), ip(dc),
                                   None if cls is None else ip(cls), xy.size // 2, _dptr(xy),
                                   precision, leaf_cells, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().pecs_lu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, b: np.ndarray) -> np.ndarray:
        b = np.ascontiguousarray(b, dtype=np.float64)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        x = np.zeros_like(b)
        check(lib().pecs_lu_solve(self._h, nrhs, _dptr(b), _dptr(x)))
        return x

    def solve_device(self, b, x, nrhs: int = 1, stream: int = 0):
        """b, x: device pointers (e.g. torch.Tensor.data_ptr()) of nrhs*n doubles."""
        check(lib().pecs_lu_solve_device(self._h, nrhs, C.c_void_p(b), C.c_void_p(x),
                                         C.c_void_p(stream)))

    def factor_values(self) -> np.ndarray:
        """The stored factor values (every node's Gf then Hb), before the
        first solve uploads them (pecs_debug_lu_values)."""
        n = C.c_longlong()
        check(lib().pecs_debug_lu_values(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        check(lib().pecs_debug_lu_values(self._h, _dptr(out), n.value, C.byref(n)))
        return out

    def host_apply(self, b: np.ndarray) -> np.ndarray:
        """Diagnostic host application of the factors (no GPU)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        check(lib().pecs_lu_host_apply(self._h, _dptr(b), _dptr(x)))
        return x

    def stats(self):
        e = C.c_longlong()
        lv = C.c_int()
        nn = C.c_int()
        mf = C.c_int()
        check(lib().pecs_lu_stats(self._h, C.byref(e), C.byref(lv), C.byref(nn), C.byref(mf)))
        return {"entries": e.value, "levels": lv.value, "nodes": nn.value, "max_front": mf.value}
