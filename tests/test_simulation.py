"""CPU tests of the parameter-file driver (mcsolver_gb300.simulation).

* ``load_param`` reads the version-3.0 files exactly as the reference's
  fileio.loadParam did (fixture: what the reference parsed from the same files);
* ``point_args`` builds, for a grid point, the same MCMainFunction tuple the
  reference's own model build passes (fixture: captured reference arguments);
* ``save_param`` writes files that ``load_param`` reads back unchanged;
* unsupported inputs are rejected with a message.
"""
import gzip
import json
import os

import numpy as np
import pytest

from mcsolver_gb300 import simulation as sim

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _fixture():
    with gzip.open(os.path.join(GOLD, "params_parsed.json.gz"), "rt") as f:
        return json.load(f)["cases"]


def _norm(x):
    if isinstance(x, (tuple, list)):
        return [_norm(y) for y in x]
    return x


@pytest.mark.parametrize("name", ["square_xy", "honeycomb_heisenberg", "square_ising_field"])
def test_load_param_matches_reference_parser(name):
    want = _fixture()[name]["parsed"]
    got = sim.load_param(os.path.join(GOLD, "params", name + ".txt"))
    for k, v in want.items():
        assert _norm(got[k]) == _norm(v), k


@pytest.mark.parametrize("name", ["square_xy", "honeycomb_heisenberg", "square_ising_field"])
def test_point_args_match_reference_marshalling(name):
    case = _fixture()[name]
    p = sim.load_param(os.path.join(GOLD, "params", name + ".txt"))
    T, H = case["point"]
    model, args = sim.point_args(p, T, H)
    want = case["args"]
    assert len(args) == len(want)
    for k, (a, b) in enumerate(zip(args, want)):
        np.testing.assert_allclose(np.asarray(a, float), np.asarray(b, float), rtol=1e-12, atol=1e-12,
                                   err_msg="argument %d" % k)


def test_save_param_round_trip(tmp_path):
    p = sim.load_param(os.path.join(GOLD, "params", "honeycomb_heisenberg.txt"))
    path = str(tmp_path / "again.txt")
    sim.save_param(p, path)
    q = sim.load_param(path)
    for k in p:
        assert _norm(q[k]) == _norm(p[k]), k


def test_unsupported_inputs_are_rejected(tmp_path):
    p = sim.load_param(os.path.join(GOLD, "params", "square_xy.txt"))
    with pytest.raises(ValueError, match="dipole"):
        sim.point_args(dict(p, dipoleAlpha=0.5), 1.0, 0.0)
    with pytest.raises(ValueError, match="algorithm"):
        sim.point_args(dict(p, algorithm="Swendsen-Wang"), 1.0, 0.0)
    bad = tmp_path / "v2.txt"
    bad.write_text("This is mcsolver's save file, version: 2.0\n")
    with pytest.raises(ValueError, match="version"):
        sim.load_param(str(bad))
    text = open(os.path.join(GOLD, "params", "square_xy.txt")).read().replace("Ncores:", "Cores:")
    bad.write_text(text)
    with pytest.raises(ValueError, match="Ncores"):
        sim.load_param(str(bad))
