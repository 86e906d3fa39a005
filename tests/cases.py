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


GOLDEN_LARGE = os.path.join(HERE, "golden", "golden_large.json.gz")
_golden_large = None


def golden_large():
    """Reference results on the benchmark configurations' own lattices
    (tests/golden/make_golden_large.py); None when not generated."""
    global _golden_large
    if _golden_large is None and os.path.isfile(GOLDEN_LARGE):
        with gzip.open(GOLDEN_LARGE, "rt") as f:
            _golden_large = json.load(f)
    return _golden_large


def spec_args(spec, arrays=False, nthermal=None, nsweep=None, T=None, h=None, frames=None):
    """The MCMainFunction tuple of a fixture spec (the reference caller's
    inputs: lattice, bonds, S, D, T, h, program) built by this package's
    vectorised builder; tests check its fingerprint against the tuple the
    reference's own Python built."""
    from mcsolver_gb300.lattice import LatticeTemplate
    model = spec["model"]
    algo = 0 if spec["algo"].startswith("Metro") else 1
    ki = ((spec["ki"][0][0], spec["ki"][0][1]), tuple(spec["ki"][1]))
    tmpl = LatticeTemplate(model, tuple(spec["L"]), len(spec["pos"]),
                           [(b[0], b[1], tuple(b[2]), list(b[3])) for b in spec["bonds"]],
                           S=list(spec["S"]), D=[list(d) for d in spec["D"]],
                           nthermal=spec["nthermal"] if nthermal is None else nthermal,
                           nsweep=spec["nsweep"] if nsweep is None else nsweep, tau=spec["tau"], algo=algo, ki=ki,
                           groups=tuple(tuple(g) for g in spec["orbGroups"]),
                           circuits=[tuple((c[0], tuple(c[1])) for c in circ) for circ in spec["circuits"]],
                           frames=spec["spinFrame"] if frames is None else frames, group_in_sc=spec["groupInSC"])
    return tmpl.at(spec["T"] if T is None else T, h=spec["h"] if h is None else h, arrays=arrays)
