"""The committed golden fixtures (tests/golden/, written from the oracle by
tests/golden/make_golden.py): the oracle must still reproduce them, and the
library's host setup must give their initial densities (CPU).  The GPU path
is checked against them in test_zz_golden_gpu.py."""
import glob
import os

import numpy as np
import pytest

import pecs_gb300 as pg
from golden.make_golden import fixture, params_of
from helpers import FIELD_OF, max_rel, rel_err, to_lib

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
IDS = [os.path.basename(f)[:-4] for f in FILES]

INIT_TOL = 1e-11   # initial state: one direct Poisson solve (multifrontal vs SuperLU)
RHS_TOL = 1e-12    # carrier right-hand sides from that state (max-norm relative)
STEP_TOL = 1e-10   # trajectories, relative L2 per field, and I_Sigma


def _load(path):
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def check_against(fx, init=None, rhs0=None, final=None, current=None):
    """Compares whichever of the four parts are given with the fixture."""
    for part, got, tol, err in (("init", init, INIT_TOL, rel_err), ("rhs0", rhs0, RHS_TOL, max_rel),
                                ("final", final, STEP_TOL, rel_err)):
        if got is None:
            continue
        keys = [k for k in fx if k.startswith(part + "_")]
        assert keys and set(k[len(part) + 1:] for k in keys) == set(got), part
        for k in keys:
            e = err(got[k[len(part) + 1:]], fx[k])
            assert e < tol, (k, e)
    if current is not None and "current" in fx:
        ref = float(fx["current"])
        assert abs(current - ref) <= STEP_TOL * max(abs(ref), 1e-30), (current, ref)


def test_fixtures_present():
    assert len(FILES) >= 5


@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_oracle_reproduces_fixture(path):
    fx = _load(path)
    P = params_of(fx)
    new = fixture(P, int(fx["steps"]))
    strip = lambda d, p: {k[len(p) + 1:]: v for k, v in d.items() if k.startswith(p + "_")}  # noqa: E731
    # the oracle is deterministic; across machines and numpy builds allow rounding
    check_against(fx, init=strip(new, "init"), rhs0=strip(new, "rhs0"), final=strip(new, "final"),
                  current=float(new["current"]) if "current" in new else None)
    for k in fx:
        if k not in ("params", "steps"):
            assert np.abs(new[k] - fx[k]).max() <= 1e-11 * max(np.abs(fx[k]).max(), 1e-300), k


@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_library_setup_matches_fixture(pecs_lib, path):
    fx = _load(path)
    ctx = pg.Context(to_lib(params_of(fx)), host_setup_only=True)
    for f in ("n", "p", "r", "o"):
        if "init_" + f in fx:
            v = ctx.setup_vector(pg.SETUP_INITIAL, FIELD_OF[f])
            ref = fx["init_" + f]
            assert np.abs(v - ref).max() <= 1e-13 * np.abs(ref).max(), f
