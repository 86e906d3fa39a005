"""Drift of the FP32-update engine against an FP64-everywhere run.

The oracle's engine-stream mode runs the same algorithm on the same random
words (colour order, Philox counters) with every quantity in FP64.  The table
printed here (run with `pytest -s`) is the largest relative difference, over 4
seeds, of all 27 O(n) observables, and separately of the energy <e>, <e^2>
and U4, after 10, 100 and 1000 sweeps.  Short runs must agree to FP32
resolution (the trajectories coincide); long runs may take one borderline
acceptance differently, after which the chains decorrelate and the
difference is a statistical one, bounded by the 3-sigma tests instead.
"""
import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu

CASES = [
    ("XY L=32, T=0.9", "xy", lambda n: C.square_args("xy", 32, 0.9, nthermal=0, nsweep=n)),
    ("Heisenberg L=16, DMI 0.4, h=0.2, T=0.5", "heisenberg",
     lambda n: C.square_args("heisenberg", 16, 0.5, h=0.2, dmi=0.4, nthermal=0, nsweep=n)),
    ("Heisenberg honeycomb 8x8 (1NN Kitaev-type + 2NN, Az), T=6", "heisenberg",
     lambda n: C.honeycomb_args("heisenberg", 8, 6.0, nthermal=0, nsweep=n)),
]
SWEEPS = (10, 100, 1000)
SHORT_RTOL = 2e-5   # energies and U4 after 10 and 100 sweeps (same trajectory, FP32 state)


def _tilt(args):
    a = list(args)
    a[15] = 0.6  # flunc: random initial tilt drawn from the engine stream
    return tuple(a)


def _rel(a, b, floor):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), floor)))


def test_fp32_drift_against_fp64(engine, oracle_lib, capsys):
    rows = []
    for name, model, mk in CASES:
        row = [name]
        for n in SWEEPS:
            d_all = d_e = 0.0
            for seed in range(4):
                args = _tilt(mk(n))
                res, _ = engine.solve(model, args, seed=100 + seed)
                ref, _ = oracle_lib.solve(model, args, seed=100 + seed, mode=1)
                obs, robs = np.array(res[:27]), np.array(ref[:27])
                keep = np.abs(robs) > 1e-6  # Q and other observables that vanish by symmetry
                d_all = max(d_all, _rel(obs[keep], robs[keep], 1e-6))
                d_e = max(d_e, _rel(obs[[8, 9, 10]], robs[[8, 9, 10]], 1e-6))
            row.append((d_all, d_e))
            if n <= 100:
                assert d_e < SHORT_RTOL, (name, n, d_e)
        rows.append(row)
    with capsys.disabled():
        print("\nlargest relative difference, FP32 engine vs FP64 oracle (4 seeds): all observables / e, e^2, U4")
        for r in rows:
            print("  %-58s" % r[0] + "".join("  %d sweeps: %.1e / %.1e" % (n, a, e) for n, (a, e) in zip(SWEEPS, r[1:])))
