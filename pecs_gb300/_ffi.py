"""ctypes bindings of the C ABI declared in include/pecs.h and include/pecs_debug.h.

The library must exist (``pecs_gb300._build.build()`` makes it); there is no
fallback implementation -- importing the bindings without it raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from ._build import LIB

PECS_OK = 0
PECS_E_ARG = -1
PECS_E_CUDA = -2
PECS_E_SINGULAR = -3
PECS_E_NONFINITE = -4
PECS_E_STATE = -5
PECS_E_NODEVICE = -6

INTERFACE, DIRICHLET, NEUMANN, SCHOTTKY = 0, 1, 2, 3
FIELD_N, FIELD_P, FIELD_R, FIELD_O, FIELD_POISSON = 0, 1, 2, 3, 4
MAT_N, MAT_P, MAT_R, MAT_O, MAT_POISSON, MAT_MASS_SEMI, MAT_MASS_ELEC = range(7)
SETUP_CONST_RHS, SETUP_INITIAL = 0, 1
MESH_SEMI, MESH_ELEC, MESH_POISSON = 0, 1, 2
PREC_FP64, PREC_FP32_IR, PREC_FP32_MIXED = 0, 1, 2


class pecs_params(C.Structure):
    _fields_ = [
        ("degree", C.c_int), ("full_system", C.c_int),
        ("nx_semi", C.c_int), ("nx_elec", C.c_int), ("ny", C.c_int),
        ("x_semi0", C.c_double), ("x_semi1", C.c_double), ("x_elec1", C.c_double),
        ("height", C.c_double),
        ("bc_semi", C.c_int * 4), ("bc_elec", C.c_int * 4), ("bc_poisson", C.c_int * 4),
        ("lambda2", C.c_double), ("eps_semi", C.c_double), ("eps_elec", C.c_double),
        ("mu", C.c_double * 4), ("dt", C.c_double), ("penalty", C.c_double),
        ("k_et", C.c_double), ("k_ht", C.c_double), ("junction_x", C.c_double),
        ("nd", C.c_double * 2), ("na", C.c_double * 2), ("n_eq", C.c_double * 2),
        ("p_eq", C.c_double * 2), ("r_eq", C.c_double), ("o_eq", C.c_double),
        ("ic_kind", C.c_int), ("gen_kind", C.c_int), ("G0", C.c_double), ("alpha", C.c_double),
        ("srh", C.c_int), ("tau_n", C.c_double), ("tau_p", C.c_double), ("n_i", C.c_double),
        ("phi_bi", C.c_double), ("phi_app", C.c_double), ("s_n", C.c_double), ("s_p", C.c_double),
        ("grading", C.c_double), ("bc_poisson_elec", C.c_int * 4), ("poisson_pairing", C.c_int),
    ]


class pecs_options(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("leaf_cells", C.c_int), ("use_graphs", C.c_int),
        ("ir_max_iters", C.c_int), ("ir_tol", C.c_double), ("device", C.c_int),
        ("host_setup_only", C.c_int), ("panel_chunk", C.c_int), ("panel_min_ctas", C.c_int),
        ("autotune", C.c_int), ("gpu_factor_min_front", C.c_int), ("flow_sweep", C.c_int),
        ("increment_solves", C.c_int),
    ]


class pecs_info(C.Structure):
    _fields_ = [
        ("n_inst", C.c_int), ("ndofs", C.c_int * 5), ("factor_entries", C.c_longlong * 3),
        ("factor_levels", C.c_int * 3), ("factor_nodes", C.c_int * 3),
        ("factor_bytes", C.c_longlong), ("setup_seconds", C.c_double),
        ("n_distinct_carrier_factors", C.c_int), ("launches_per_step", C.c_int),
        ("solve_bytes", C.c_double * 2), ("solve_launches", C.c_int * 2),
        ("setup_launches", C.c_int), ("initialize_launches", C.c_int),
        ("tuned_sweep_ms", C.c_double * 2), ("flow_rpl", C.c_int * 2), ("flow_top", C.c_int * 2),
    ]


class pecs_physical_params(C.Structure):
    _fields_ = [
        ("time_step", C.c_double), ("mesh_height", C.c_double), ("illuminated", C.c_int),
        ("applied_bias", C.c_double), ("built_in_bias", C.c_double), ("schottky_bias", C.c_double),
        ("characteristic_length", C.c_double), ("characteristic_density", C.c_double),
        ("characteristic_time", C.c_double), ("intrinsic_density", C.c_double),
        ("photon_flux", C.c_double), ("absorption_coeff", C.c_double),
        ("semiconductor_permittivity", C.c_double), ("electrolyte_permittivity", C.c_double),
        ("electron_mobility", C.c_double), ("hole_mobility", C.c_double),
        ("reductant_mobility", C.c_double), ("oxidant_mobility", C.c_double),
        ("electron_recombination_time", C.c_double), ("hole_recombination_time", C.c_double),
        ("electron_recombination_velocity", C.c_double), ("hole_recombination_velocity", C.c_double),
        ("electron_transfer_rate", C.c_double), ("hole_transfer_rate", C.c_double),
    ]


class pecs_scales(C.Structure):
    _fields_ = [
        ("mobility_scale", C.c_double), ("rescale_current", C.c_double),
        ("rescaled_k_et", C.c_double), ("rescaled_k_ht", C.c_double), ("schottky_bias", C.c_double),
    ]


class PecsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pecs error {code}: {msg}")
        self.code = code


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

# (name, restype, argtypes)
SIGNATURES = [
    ("pecs_last_error", C.c_char_p, []),
    ("pecs_default_options", None, [C.POINTER(pecs_options)]),
    ("pecs_apply_boundary_layout", C.c_int, [C.POINTER(pecs_params), C.c_int, C.c_int]),
    ("pecs_reference_physical_params", None, [C.POINTER(pecs_physical_params)]),
    ("pecs_scale_params", C.c_int, [C.POINTER(pecs_physical_params), C.POINTER(pecs_params),
                                    C.POINTER(pecs_scales)]),
    ("pecs_get_setup_vector", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                        C.c_longlong]),
    ("pecs_get_mesh", C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("pecs_create", C.c_int, [C.POINTER(pecs_params), C.c_int, C.POINTER(pecs_options), C.POINTER(_vp)]),
    ("pecs_destroy", None, [_vp]),
    ("pecs_get_info", C.c_int, [_vp, C.POINTER(pecs_info)]),
    ("pecs_get_matrix", C.c_int, [_vp, C.c_int, _ip, C.POINTER(C.c_longlong), _ip, _ip, _dp]),
    ("pecs_initialize", C.c_int, [_vp]),
    ("pecs_set_state", C.c_int, [_vp, C.c_int, C.c_int, _dp, C.c_size_t]),
    ("pecs_get_state", C.c_int, [_vp, C.c_int, C.c_int, _dp, C.c_size_t]),
    ("pecs_get_rhs", C.c_int, [_vp, C.c_int, C.c_int, _dp, C.c_size_t]),
    ("pecs_get_state_device", C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    ("pecs_set_state_device", C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    ("pecs_set_instances", C.c_int, [_vp, C.POINTER(pecs_params), C.c_int]),
    ("pecs_assemble_carrier_rhs", C.c_int, [_vp]),
    ("pecs_solve_carriers", C.c_int, [_vp]),
    ("pecs_assemble_poisson_rhs", C.c_int, [_vp]),
    ("pecs_solve_poisson", C.c_int, [_vp]),
    ("pecs_step", C.c_int, [_vp, C.c_int]),
    ("pecs_run_to_steady_state", C.c_int, [_vp, C.c_int, C.c_double, C.c_int, _ip, _dp]),
    ("pecs_interface_current", C.c_int, [_vp, _dp]),
    ("pecs_iv_sweep", C.c_int, [_vp, C.POINTER(_dp), C.c_int, C.c_double, C.c_int, _dp, _ip,
                                C.POINTER(_dp)]),
    ("pecs_sweep_stream", C.c_int, [_vp, C.c_int, C.POINTER(pecs_params), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p), C.c_int, C.c_double, C.c_int, _ip, _dp,
                                    C.POINTER(_dp)]),
    ("pecs_synchronize", C.c_int, [_vp]),
    ("pecs_solve_residual", C.c_int, [_vp, C.c_int, _dp]),
    ("pecs_get_stream", _vp, [_vp]),
    ("pecs_last_run_steps", C.c_int, [_vp]),
    ("pecs_time_solve", C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    ("pecs_time_stages", C.c_int, [_vp, C.c_int, _dp]),
    ("pecs_element_sizes", C.c_int, [C.c_int, C.c_int, _ip, _ip, _ip]),
    ("pecs_ldg_local_mass_matrix", C.c_int, [C.c_int, _vp, C.c_double, _dp]),
    ("pecs_ldg_local_cell_and_bc_terms", C.c_int, [C.c_int, _vp, C.c_double, C.c_double, C.c_double,
                                                   C.c_double, C.c_double, _dp, _dp]),
    ("pecs_ldg_local_flux_terms", C.c_int, [C.c_int, _vp, C.c_int, _vp, C.c_double, _dp, _dp, _dp, _dp]),
    ("pecs_mixed_local_poisson_matrix", C.c_int, [C.c_int, C.c_int, _vp, C.c_double, C.c_double,
                                                  C.c_double, _dp]),
    ("pecs_lu_factor", C.c_int, [C.c_int, _ip, _ip, _dp, _ip, _ip, C.c_int, _dp, C.c_int, C.c_int,
                                 C.POINTER(_vp)]),
    ("pecs_lu_solve", C.c_int, [_vp, C.c_int, _dp, _dp]),
    ("pecs_lu_set_gpu_factor_min_front", C.c_int, [C.c_int]),
    ("pecs_debug_lu_values", C.c_int, [_vp, _dp, C.c_longlong, C.POINTER(C.c_longlong)]),
    ("pecs_lu_solve_device", C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    ("pecs_lu_stats", C.c_int, [_vp, C.POINTER(C.c_longlong), _ip, _ip, _ip]),
    ("pecs_lu_destroy", None, [_vp]),
    ("pecs_lu_solve_device_noalloc", C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    ("pecs_lu_host_apply", C.c_int, [_vp, _dp, _dp]),
    ("pecs_debug_time_levels", C.c_int, [_vp, C.c_int, C.c_int, _dp, C.c_int]),
    ("pecs_debug_flow_stall", C.c_int, [_vp, C.c_int, _ip]),
    ("pecs_mlp_create", C.c_int, [C.c_int, _ip, C.c_ulonglong, C.POINTER(_vp)]),
    ("pecs_mlp_destroy", None, [_vp]),
    ("pecs_mlp_n_params", C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    ("pecs_mlp_get_params", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("pecs_mlp_set_params", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("pecs_mlp_forward", C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    ("pecs_mlp_gradients", C.c_int, [_vp, C.c_int, _vp, _vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("pecs_mlp_train_step", C.c_int, [_vp, C.c_int, _vp, _vp, C.c_float, C.POINTER(C.c_float)]),
    ("pecs_decode", C.c_int, [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("pecs_warm_start_vectors", C.c_int, [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, _vp,
                                          _vp, _vp]),
]

_lib = None


def lib() -> C.CDLL:
    """Load libpecs_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("PECS_GB300_LIB", LIB))
        if not path.exists():
            raise ImportError(f"{path} not found: build it with pecs_gb300._build.build()")
        L = C.CDLL(str(path))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != PECS_OK:
        msg = lib().pecs_last_error()
        raise PecsError(code, msg.decode() if msg else "")
