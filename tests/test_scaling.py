"""pecs_scale_params: the reference's nondimensional scaling
(Parameters::parse_and_scale_parameters, include/Parameters.hpp:117-287).

CPU only.  The library must give exactly the doubles of the oracle's
restatement (same operations in the same order), hand-computed decimal values
for the reference's input_file.prm, and leave every non-physical field alone.
"""
import dataclasses
import math

import numpy as np
import pytest

import pecs_gb300 as pg
from oracle import scaling as osc

# the values of the reference's input_file.prm, as a caller would write them
PRM = {
    "computational": {"end time": "5e1", "global refinements": "4", "time step size": "0.05"},
    "electrons": {"mobility": "1350.0", "recombination time": "5e-5",
                  "recombination velocity": "3e5", "transfer rate": "1e-19"},
    "holes": {"mobility": "480.0", "recombination time": "5e-5",
              "recombination velocity": "2.9e5", "transfer rate": "1e-14"},
    "mesh": {"boundary layer": "0.1", "mesh height": "1", "mesh length": "1.0"},
    "oxidants": {"mobility": "1.0"},
    "physical": {"absorption coefficient": "1.74974e5", "applied bias": "0.0",
                 "built in bias": "0.41", "characteristic density": "1.0e16",
                 "characteristic length": "1.0e-4", "characteristic time": "1.0e-12",
                 "electrolyte permittivity": "1000", "illumination status": "true",
                 "insulated": "true", "intrinsic density": "2.564e9", "photon flux": "1.2e17",
                 "schottky bias": "0.0", "schottky status": "true",
                 "semiconductor permittivity": "11.9"},
    "reductants": {"mobility": "1.0"},
}


def _prm_text(sections):
    lines = ["# written by the test"]
    for sec, kv in sections.items():
        lines.append(f"subsection {sec}")
        for k, v in kv.items():
            lines.append(f"  set {k:<24} = {v}   # {sec}")
        lines.append("end")
    return "\n".join(lines) + "\n"


def _as_dict(ph):
    return {f.name: getattr(ph, f.name) for f in dataclasses.fields(ph)}


def test_reference_values_read_from_prm_text(pecs_lib):
    ph = pg.read_prm(_prm_text(PRM), base=dataclasses.replace(pg.PhysicalParams(), **{
        f.name: 0.0 for f in dataclasses.fields(pg.PhysicalParams) if f.name != "illuminated"}))
    assert ph == pg.PhysicalParams.reference() == pg.PhysicalParams()


def test_prm_reader_rejects_malformed_text(pecs_lib):
    with pytest.raises(ValueError):
        pg.read_prm("subsection physical\n set built in bias 0.4\nend\n")
    with pytest.raises(ValueError):
        pg.read_prm("subsection physical\n set built in bias = 0.4\n")
    with pytest.raises(ValueError):
        pg.read_prm("subsection physical\n set illumination status = yes\nend\n")
    ph = pg.read_prm("subsection physical\n  set built in bias = 0.3 # V\nend\n")
    assert ph.built_in_bias == 0.3 and ph.photon_flux == 1.2e17


def _check_against_oracle(ph):
    p0 = pg.half_cell(3)
    p, sc = pg.scale_params(ph, p0)
    want = osc.scale(_as_dict(ph))
    for k, v in want.items():
        got = sc[k] if k in sc else getattr(p, k)
        if isinstance(v, tuple):
            assert tuple(got) == v, k
        else:
            assert got == v, (k, got, v)      # bit-identical: same operations, same order
    # nothing else changes
    touched = set(want) - set(sc)
    for f in dataclasses.fields(pg.Params):
        if f.name not in touched:
            assert getattr(p, f.name) == getattr(p0, f.name), f.name
    return p, sc


def test_scaling_matches_oracle_bitwise_on_reference_and_random_values(pecs_lib):
    _check_against_oracle(pg.PhysicalParams.reference())
    rng = np.random.default_rng(5)
    for trial in range(50):
        ph = pg.PhysicalParams(**{
            f.name: (bool(trial % 2) if f.name == "illuminated"
                     else float(10.0 ** rng.uniform(-20, 20)) * (1 if rng.random() < 0.8 else -1))
            for f in dataclasses.fields(pg.PhysicalParams)})
        ph.characteristic_length = abs(ph.characteristic_length)
        ph.characteristic_density = abs(ph.characteristic_density)
        ph.characteristic_time = abs(ph.characteristic_time)
        _check_against_oracle(ph)


def test_scaled_reference_values(pecs_lib):
    """Decimal values worked out by hand from the formulas of
    Parameters.hpp:181-243 and the reference's input_file.prm."""
    p, sc = pg.scale_params(pg.PhysicalParams.reference())
    expect = {
        "lambda2": 0.02585 * 8.85e-14 / 1.62e-11,     # V_t eps0 / (q rho L^2) = 1.41218e-4
        "n_i": 2.564e-7, "tau_n": 5e7, "tau_p": 5e7, "s_n": 3e-3, "s_p": 2.9e-3,
        "G0": 1.2e-11, "alpha": 17.4974, "k_et": 1e-11, "k_ht": 1e-6,
        "phi_bi": 0.41 / 0.02585, "phi_app": 0.0, "eps_semi": 11.9, "eps_elec": 1000.0,
        "dt": 0.05, "height": 1.0,
    }
    for k, v in expect.items():
        assert math.isclose(getattr(p, k), v, rel_tol=1e-14, abs_tol=0.0), (k, getattr(p, k), v)
    assert math.isclose(p.lambda2, 1.4121759259259258e-4, rel_tol=1e-14)
    assert p.gen_kind == 1
    for got, mob in zip(p.mu, (1350.0, 480.0, 1.0, 1.0)):
        assert math.isclose(got, mob * 2.585e-6, rel_tol=1e-14)
    assert math.isclose(sc["mobility_scale"], 2.585e-6, rel_tol=1e-14)
    assert math.isclose(sc["rescale_current"], 1.62e5, rel_tol=1e-14)
    assert math.isclose(sc["rescaled_k_et"], 1.62e-19 * 1e-19 * 1e32, rel_tol=1e-14)
    assert math.isclose(sc["rescaled_k_ht"], 1.62e-19 * 1e-14 * 1e32, rel_tol=1e-14)
    # dark: no generation at all (Generation::set_dark_params)
    dark, _ = pg.scale_params(dataclasses.replace(pg.PhysicalParams.reference(), illuminated=False))
    assert dark.gen_kind == 0 and dark.G0 == 0.0 and dark.alpha == 0.0


def test_scaling_rejects_bad_scales(pecs_lib):
    for field in ("characteristic_length", "characteristic_density", "characteristic_time"):
        for bad in (0.0, -1.0, float("nan"), float("inf")):
            ph = dataclasses.replace(pg.PhysicalParams(), **{field: bad})
            with pytest.raises(pg.PecsError) as e:
                pg.scale_params(ph)
            assert e.value.code == pg._ffi.PECS_E_ARG
            assert "characteristic" in str(e.value)


def test_scaled_parameters_give_the_oracles_matrices(pecs_lib):
    """The scaled reference values (Debye length squared 1.4e-4, permittivities
    11.9 / 1000, mobilities ~1e-3) set up on the host give the oracle's LDG and
    mixed matrices."""
    import oracle
    p, _ = pg.scale_params(pg.PhysicalParams.reference(), pg.half_cell(2))
    ctx = pg.Context(p, host_setup_only=True)
    pb = oracle.Problem(oracle.Params(**dataclasses.asdict(p)))
    for which, A in ((pg.MAT_POISSON, pb.A_P), (pg.MAT_N, pb.A_n), (pg.MAT_O, pb.A_o)):
        B = ctx.matrix(which)
        err = abs(B - A).max() / abs(A).max()
        assert err < 1e-14, (which, err)
