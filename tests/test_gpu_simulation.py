"""GPU test of the parameter-file driver: a whole (T, H) grid as one batch.

``start_simulation`` on the committed parameter files writes the reference's
result files (``out``, ``spinDotSpin.txt``, spin frames, ``result.txt``) and
each result row equals the point solved alone through the C ABI with the same
Philox key (seed + point ID)."""
import os

import numpy as np
import pytest

from mcsolver_gb300 import simulation as sim

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "params")


@pytest.mark.parametrize("name", ["square_xy", "honeycomb_heisenberg", "square_ising_field"])
def test_grid_run_writes_reference_files_and_matches_solves(engine, tmp_path, name):
    path = os.path.join(GOLD, name + ".txt")
    p = sim.load_param(path)
    rows = sim.start_simulation(path, workdir=str(tmp_path), seed=11)
    npts = p["nT"] * p["nH"]
    assert len(rows) == npts
    res = open(tmp_path / "result.txt").read().splitlines()
    assert len(res) == npts + 1 and res[0].startswith("#Temp")
    out = open(tmp_path / "out").read().splitlines()
    assert len(out) == npts + 1 and out[0] == "#T #H"
    sds = open(tmp_path / "spinDotSpin.txt").read().splitlines()
    on = p["modelType"] != "Ising"
    assert len(sds) == (npts + 1 if on and p["orbGroupList"] else 1)
    frames = [f for f in os.listdir(tmp_path) if "SpinDistribution" in f]
    assert len(frames) == npts * p["spinFrame"]
    TList = np.linspace(p["T0"], p["T1"], p["nT"])
    HList = np.linspace(p["H0"], p["H1"], p["nH"])
    ID = 0
    for iH, H in enumerate(HList):
        for iT, T in enumerate(TList):
            model, args = sim.point_args(p, T, H)
            r, _ = engine.solve(model, args, seed=11 + ID)
            Tc = max(T, 0.1)
            E = (r[4] if model == "ising" else r[8]) * Tc
            U4 = r[8] if model == "ising" else r[10]
            row = rows[ID]
            assert row[0] == pytest.approx(T) and row[1] == pytest.approx(H)
            assert row[5] == pytest.approx(E, rel=1e-6, abs=1e-9)
            assert row[8] == pytest.approx(U4, rel=1e-6, abs=1e-9)
            ID += 1
