// Physical parameters -> the scaled (nondimensional) parameters of a run.
//
// Restates ParameterSpace::Parameters::parse_and_scale_parameters
// (include/Parameters.hpp:117-287 of the reference): the values read from
// input_file.prm are divided by the characteristic density, length and time
// and the thermal voltage, with the physical constants of
// include/Parameters.hpp:8-11.  Every product is evaluated in the reference's
// order, so the scaled values are the same doubles the reference computes.
// The .prm reader itself (ParameterReader.cpp) is not restated: callers fill
// pecs_physical_params, or start from pecs_reference_physical_params.
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/pecs.h"

namespace pecs {
void set_error_external(const std::string& m);
}

namespace {
// include/Parameters.hpp:8-11
constexpr double kThermalVoltage = 0.02585;      // [V]
constexpr double kElectronCharge = 1.62e-19;     // [C]
constexpr double kVacuumPermittivity = 8.85e-14; // [A s V^-1 cm^-1]
}  // namespace

extern "C" {

void pecs_reference_physical_params(pecs_physical_params* ph) {
  if (!ph) return;
  std::memset(ph, 0, sizeof(*ph));
  // the reference's input_file.prm
  ph->time_step = 0.05;
  ph->mesh_height = 1.0;
  ph->illuminated = 1;
  ph->applied_bias = 0.0;
  ph->built_in_bias = 0.41;
  ph->schottky_bias = 0.0;
  ph->characteristic_length = 1.0e-4;
  ph->characteristic_density = 1.0e16;
  ph->characteristic_time = 1.0e-12;
  ph->intrinsic_density = 2.564e9;
  ph->photon_flux = 1.2e17;
  ph->absorption_coeff = 1.74974e5;
  ph->semiconductor_permittivity = 11.9;
  ph->electrolyte_permittivity = 1000.0;
  ph->electron_mobility = 1350.0;
  ph->hole_mobility = 480.0;
  ph->reductant_mobility = 1.0;
  ph->oxidant_mobility = 1.0;
  ph->electron_recombination_time = 5e-5;
  ph->hole_recombination_time = 5e-5;
  ph->electron_recombination_velocity = 3e5;
  ph->hole_recombination_velocity = 2.9e5;
  ph->electron_transfer_rate = 1e-19;
  ph->hole_transfer_rate = 1e-14;
}

int pecs_scale_params(const pecs_physical_params* ph, pecs_params* p, pecs_scales* scales) {
  if (!ph || !p) {
    pecs::set_error_external("pecs_scale_params: NULL argument");
    return PECS_E_ARG;
  }
  const double L = ph->characteristic_length, rho = ph->characteristic_density,
               T = ph->characteristic_time;
  if (!(L > 0.0) || !(rho > 0.0) || !(T > 0.0) || !std::isfinite(L) || !std::isfinite(rho) ||
      !std::isfinite(T)) {
    pecs::set_error_external(
        "pecs_scale_params: the characteristic length, density and time must be positive and finite");
    return PECS_E_ARG;
  }
  // Parameters.hpp:181-191
  p->n_i = ph->intrinsic_density / rho;
  p->tau_n = ph->electron_recombination_time / T;
  p->tau_p = ph->hole_recombination_time / T;
  p->s_n = ph->electron_recombination_velocity * (T / L);
  p->s_p = ph->hole_recombination_velocity * (T / L);
  // Parameters.hpp:193-196; Generation::set_illuminated_params / set_dark_params
  // (Generation.cpp:8-27) take the flux and coefficient only when illuminated
  if (ph->illuminated) {
    p->gen_kind = 1;
    p->G0 = ph->photon_flux * (T / rho);
    p->alpha = ph->absorption_coeff * L;
  } else {
    p->gen_kind = 0;
    p->G0 = 0.0;
    p->alpha = 0.0;
  }
  // Parameters.hpp:198-205: the Debye length squared, without the material
  // permittivity (the permittivities enter the Poisson matrix separately)
  p->lambda2 = (kThermalVoltage * kVacuumPermittivity) / (kElectronCharge * rho * L * L);
  // Parameters.hpp:207-215
  const double mobility_scale = (T * kThermalVoltage) / (L * L);
  p->mu[0] = ph->electron_mobility * mobility_scale;
  p->mu[1] = ph->hole_mobility * mobility_scale;
  p->mu[2] = ph->reductant_mobility * mobility_scale;
  p->mu[3] = ph->oxidant_mobility * mobility_scale;
  // Parameters.hpp:217-233: the rescaled rates use the unscaled rate constants
  const double rescaled_k_et = kElectronCharge * ph->electron_transfer_rate * rho * rho;
  const double rescaled_k_ht = kElectronCharge * ph->hole_transfer_rate * rho * rho;
  p->k_et = ph->electron_transfer_rate * (T * rho / L);
  p->k_ht = ph->hole_transfer_rate * (T * rho / L);
  // Parameters.hpp:235-237; SolarCell.cpp:47-48 hand them to the bias functions
  p->phi_app = ph->applied_bias / kThermalVoltage;
  p->phi_bi = ph->built_in_bias / kThermalVoltage;
  // SolarCell.cpp:67-85: the material permittivities pass through unscaled
  p->eps_semi = ph->semiconductor_permittivity;
  p->eps_elec = ph->electrolyte_permittivity;
  // already-scaled values of the .prm (Parameters.hpp:124, 132)
  p->dt = ph->time_step;
  p->height = ph->mesh_height;
  if (scales) {
    scales->mobility_scale = mobility_scale;
    scales->rescale_current = (kElectronCharge * rho * L) / T;  // Parameters.hpp:239-242
    scales->rescaled_k_et = rescaled_k_et;
    scales->rescaled_k_ht = rescaled_k_ht;
    scales->schottky_bias = ph->schottky_bias / kThermalVoltage;
  }
  return PECS_OK;
}

}  // extern "C"
