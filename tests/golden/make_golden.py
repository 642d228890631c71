"""Writes the golden fixtures in this directory from the oracle.

The reference is a deal.II program that cannot be built here, and its own
test programs record no numbers, so these vectors come from the oracle -- the
CPU FP64 restatement of the reference's numerics, pinned against the
reference's known-answer tests (tests/test_oracle_known_answers.py).  They
let the library be checked on the GPU without running the oracle there, and
they pin the oracle itself against drift.

Each <case>.npz holds:
  params       JSON of the parameter set (the oracle's / library's fields)
  steps        number of IMEX steps marched
  init_<f>     the initial state (projection + initial Poisson solve)
  rhs0_<f>     the carrier right-hand sides assembled from the initial state
  final_<f>    the state after `steps` steps
  current      the interface current I_Sigma of the final state (full system)
with <f> in n, p, r, o (carriers, [J_x | J_y | u]) and P ([D | Phi]).

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle  # noqa: E402

D, N, I, S = oracle.DIRICHLET, oracle.NEUMANN, oracle.INTERFACE, oracle.SCHOTTKY


def cases():
    """name -> (parameters, steps): small meshes the oracle marches in seconds."""
    return {
        "pn_junction_16x16_k1": (oracle.pn_junction_params(), 20),
        "halfcell_4x4_k1": (oracle.half_cell_params(n_refine=2, phi_bi=0.4, phi_app=0.1), 20),
        "halfcell_4x4_k2": (oracle.half_cell_params(n_refine=2, degree=2), 10),
        "reference_8x8_k1": (oracle.reference_params(3, 1, dt=1e-4), 10),
        # the reference input file's insulated + Schottky layout (Grid.cpp:112-131),
        # on a mesh graded 4:1 toward the interface
        "halfcell_4x8_insulated_schottky_graded": (
            oracle.half_cell_params(n_refine=2, ny=8, grading=4.0, s_n=0.5, s_p=0.25,
                                    bc_semi=(N, I, D, S), bc_elec=(I, D, N, N),
                                    bc_poisson=(N, D, D, S), bc_poisson_elec=(0, 0, N, S)),
            20),
    }


def fixture(P, steps):
    pb = oracle.Problem(P)
    st0 = pb.initial_state()
    rhs0 = pb.carrier_rhs(st0)
    st, _, _ = pb.run(steps)
    out = {"params": np.array(json.dumps(dataclasses.asdict(P))), "steps": np.array(steps)}
    for f, v in st0.items():
        out[f"init_{f}"] = v
    for f, v in rhs0.items():
        out[f"rhs0_{f}"] = v
    for f, v in st.items():
        out[f"final_{f}"] = v
    if P.full_system:
        out["current"] = np.array(pb.interface_current(st))
    return out


def params_of(fx) -> "oracle.Params":
    """The oracle parameter set stored in a fixture."""
    d = json.loads(str(fx["params"]))
    return oracle.Params(**{k: tuple(v) if isinstance(v, list) else v for k, v in d.items()})


def main():
    for name, (P, steps) in cases().items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **fixture(P, steps))
        print(name)


if __name__ == "__main__":
    main()
