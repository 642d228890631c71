"""Restatement of the reference's nondimensional scaling, for checking the
library's ``pecs_scale_params``.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Follows ParameterSpace::Parameters::parse_and_scale_parameters
(include/Parameters.hpp:117-287; the scaling itself at 181-243, the physical
constants at 8-11) and the hand-off of the scaled values in the
SolarCellProblem constructor (source/SolarCell.cpp:44-92) and
Generation::set_illuminated_params / set_dark_params
(source/Generation.cpp:8-27).  Plain Python floats, evaluated in the
reference's operation order, so the results are the doubles the reference
computes.
"""
from __future__ import annotations

# include/Parameters.hpp:8-11
THERMAL_VOLTAGE = 0.02585       # [V]
ELECTRON_CHARGE = 1.62e-19      # [C]
VACUUM_PERMITTIVITY = 8.85e-14  # [A s V^-1 cm^-1]


def scale(ph: dict) -> dict:
    """ph: physical values keyed like pecs_physical_params.  Returns the scaled
    values keyed like the pecs_params fields they land in, plus the scale
    factors the reference keeps (rescale_current, rescaled_k_et/k_ht,
    mobility_scale, schottky_bias)."""
    L = ph["characteristic_length"]
    rho = ph["characteristic_density"]
    T = ph["characteristic_time"]
    out = {}
    # Parameters.hpp:181-191
    out["n_i"] = ph["intrinsic_density"] / rho
    out["tau_n"] = ph["electron_recombination_time"] / T
    out["tau_p"] = ph["hole_recombination_time"] / T
    out["s_n"] = ph["electron_recombination_velocity"] * (T / L)
    out["s_p"] = ph["hole_recombination_velocity"] * (T / L)
    # Parameters.hpp:193-196 and Generation.cpp:8-27 (dark: both zero)
    if ph["illuminated"]:
        out["gen_kind"] = 1
        out["G0"] = ph["photon_flux"] * (T / rho)
        out["alpha"] = ph["absorption_coeff"] * L
    else:
        out["gen_kind"] = 0
        out["G0"] = 0.0
        out["alpha"] = 0.0
    # Parameters.hpp:198-205 (the material permittivity is left out on purpose)
    out["lambda2"] = (THERMAL_VOLTAGE * VACUUM_PERMITTIVITY) / (ELECTRON_CHARGE * rho * L * L)
    # Parameters.hpp:207-215
    ms = (T * THERMAL_VOLTAGE) / (L * L)
    out["mobility_scale"] = ms
    out["mu"] = (ph["electron_mobility"] * ms, ph["hole_mobility"] * ms,
                 ph["reductant_mobility"] * ms, ph["oxidant_mobility"] * ms)
    # Parameters.hpp:217-233: rescaled rates from the unscaled constants first
    out["rescaled_k_et"] = ELECTRON_CHARGE * ph["electron_transfer_rate"] * rho * rho
    out["rescaled_k_ht"] = ELECTRON_CHARGE * ph["hole_transfer_rate"] * rho * rho
    out["k_et"] = ph["electron_transfer_rate"] * (T * rho / L)
    out["k_ht"] = ph["hole_transfer_rate"] * (T * rho / L)
    # Parameters.hpp:235-237
    out["phi_app"] = ph["applied_bias"] / THERMAL_VOLTAGE
    out["phi_bi"] = ph["built_in_bias"] / THERMAL_VOLTAGE
    out["schottky_bias"] = ph["schottky_bias"] / THERMAL_VOLTAGE
    # Parameters.hpp:239-242
    out["rescale_current"] = (ELECTRON_CHARGE * rho * L) / T
    # SolarCell.cpp:67-85: permittivities unscaled; Parameters.hpp:124,132:
    # time step and mesh height are read already scaled
    out["eps_semi"] = ph["semiconductor_permittivity"]
    out["eps_elec"] = ph["electrolyte_permittivity"]
    out["dt"] = ph["time_step"]
    out["height"] = ph["mesh_height"]
    return out
