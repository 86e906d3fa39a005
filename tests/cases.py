"""Test inputs: golden fixtures and synthetic MCMainFunction argument tuples
(the builders live in mcsolver_gb300.lattice and are cross-checked against
tuples captured from the reference's own Python in tests/test_oracle.py)."""
from __future__ import annotations

import gzip
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "golden.json.gz")

_golden = None


def golden():
    global _golden
    if _golden is None:
        with gzip.open(GOLDEN, "rt") as f:
            _golden = json.load(f)
    return _golden


def as_args(lst):
    return tuple(tuple(a) if isinstance(a, list) else a for a in lst)


def golden_case(name):
    c = golden()["cases"][name]
    return c["model"], as_args(c["args"]), c


from mcsolver_gb300.lattice import (  # noqa: E402,F401
    HC_POS, J9, SQ_CIRCUITS, honeycomb_args, lattice_args, square_args, square_args_fast)


def flat(t):
    out = []
    for x in t:
        if isinstance(x, tuple):
            out += list(x)
        else:
            out.append(x)
    return out


def with_program(model, args, nthermal=None, nsweep=None, tau=None, algo=None):
    a = list(args)
    if model == "ising":
        idx = dict(algo=0, nthermal=2, nsweep=3, tau=4)
    else:
        idx = dict(algo=0, nthermal=3, nsweep=4, tau=5)
    for k, v in (("algo", algo), ("nthermal", nthermal), ("nsweep", nsweep), ("tau", tau)):
        if v is not None:
            a[idx[k]] = v
    return tuple(a)
