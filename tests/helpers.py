"""Shared helpers for the tests: map between oracle and library parameter
sets and compare results."""
import dataclasses

import numpy as np

import oracle
import pecs_gb300 as pg

FIELD_OF = {"n": pg.FIELD_N, "p": pg.FIELD_P, "r": pg.FIELD_R, "o": pg.FIELD_O, "P": pg.FIELD_POISSON}


def to_lib(P: "oracle.Params") -> pg.Params:
    return pg.Params(**dataclasses.asdict(P))


def with_layout(P: "oracle.Params", insulated: bool, schottky: bool) -> "oracle.Params":
    """Oracle parameters carrying the library's boundary_layout of P."""
    lib = pg.boundary_layout(to_lib(P), insulated=insulated, schottky=schottky)
    return oracle.Params(**dataclasses.asdict(lib))


def rel_err(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def max_rel(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
