"""The GPU path against the committed golden fixtures (tests/golden/): the
initial state, the first carrier right-hand sides, the trajectory and the
interface current of each fixture, with no oracle run in the loop."""
import pytest

import pecs_gb300 as pg
from helpers import FIELD_OF, to_lib
from golden.make_golden import params_of
from test_golden import FILES, IDS, _load, check_against

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", FILES, ids=IDS)
def test_gpu_matches_fixture(pecs_lib, path):
    fx = _load(path)
    P = to_lib(params_of(fx))
    names = [k[len("init_"):] for k in fx if k.startswith("init_")]
    ctx = pg.Context(P)
    ctx.initialize()
    init = {f: ctx.get_state(FIELD_OF[f]) for f in names}
    ctx.assemble_carrier_rhs()
    rhs0 = {f: ctx.get_rhs(FIELD_OF[f]) for f in names if f != "P"}
    check_against(fx, init=init, rhs0=rhs0)
    ctx.close()
    ctx = pg.Context(P)
    ctx.initialize()
    ctx.step(int(fx["steps"]))
    final = {f: ctx.get_state(FIELD_OF[f]) for f in names}
    current = float(ctx.interface_current()[0]) if "current" in fx else None
    check_against(fx, final=final, current=current)
