"""pecs_gb300: GB300-native drift-diffusion--Poisson time step of PECS.

The compute path is libpecs_gb300.so (hand-written CUDA for sm_103a plus C++
host code behind the C ABI in include/pecs.h).  This package only loads and
drives it; there is no Python or CPU implementation of the time step.
"""
from ._build import build, LIB  # noqa: F401
from ._ffi import (DIRICHLET, FIELD_N, FIELD_O, FIELD_P, FIELD_POISSON, FIELD_R,  # noqa: F401
                   INTERFACE, MAT_MASS_ELEC, MAT_MASS_SEMI, MAT_N, MAT_O, MAT_P, MAT_POISSON,
                   MAT_R, NEUMANN, PREC_FP32_IR, PREC_FP32_MIXED, PREC_FP64, SCHOTTKY,
                   SETUP_CONST_RHS, SETUP_INITIAL, MESH_SEMI, MESH_ELEC, MESH_POISSON,
                   PecsError, lib)
from .api import (LU, Context, Params, PhysicalParams, boundary_layout, pn_junction,  # noqa: F401
                  half_cell, read_prm, reference_params, scale_params)
