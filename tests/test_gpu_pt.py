"""GPU tests of parallel tempering (no counterpart in the reference, which
runs every temperature independently; its oracle is therefore independent
runs at each temperature).

* the PT slot at T = 8 K of a honeycomb 1NN+2NN Heisenberg model agrees with
  the reference library's 24-seed statistics at T = 8 K (golden fixture);
* every slot agrees with independent engine runs at that temperature;
* neighbouring slots exchange (acceptance strictly between 0 and 1).
Means over independent chains within 4 standard errors (+ FP32 floor).
"""
import math

import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu

TEMPS = [4.0 * 2 ** (k / 3) for k in range(7)]   # 4 .. 16 K, contains 8 K
NCHAIN = 8


def _pt_runs(engine, nthermal, nsweep):
    phys = C.honeycomb_args("heisenberg", 6, 1.0, nthermal=nthermal, nsweep=nsweep)
    betas = [1.0 / T for T in TEMPS]
    out = []
    acc = []
    for c in range(NCHAIN):
        pt = engine.ParallelTempering("heisenberg", phys, betas, seed=77 + c)
        pt.run()
        out.append([pt.result(k)[0] for k in range(len(TEMPS))])
        acc.append(pt.stats()["swap_acceptance"])
        pt.close()
    return out, np.array(acc)


def _agree(a, b, floor=2e-6):
    a, b = np.asarray(a, float), np.asarray(b, float)
    se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    return abs(a.mean() - b.mean()) < 4 * se + floor * max(1.0, abs(a.mean())), (a.mean(), b.mean(), se)


def test_pt_matches_reference_at_8K(engine):
    _, _, c = C.golden_case("stat_heis_hc6_T8_metro")
    ref = np.array([c["ref"][str(s)][:27] for s in c["seeds"]], float)
    runs, acc = _pt_runs(engine, 300, 2000)
    k8 = TEMPS.index(8.0)
    pt = np.array([r[k8][:27] for r in runs], float)
    for k in (6, 10, 18):                           # <si.sj>, U4, e_r in units of 1/T... dimensionless
        ok, info = _agree(pt[:, k] if k != 18 else pt[:, k] / 8.0, ref[:, k])
        assert ok, (k, info)
    ok, info = _agree(pt[:, 8] / 8.0, ref[:, 8])    # PT energies are physical; the reference's are E/T
    assert ok, info
    assert (acc > 0).all() and (acc < 1).all(), acc


def test_pt_matches_independent_runs(engine):
    runs, _ = _pt_runs(engine, 200, 1000)
    from mcsolver_gb300.lattice import rescale_args
    phys = C.honeycomb_args("heisenberg", 6, 1.0, nthermal=200, nsweep=1000)
    for k, T in enumerate(TEMPS):
        b = engine.Batch()
        for s in range(NCHAIN):
            b.add("heisenberg", rescale_args("heisenberg", phys, T), seed=900 + s)
        b.run()
        ind = np.array([b.result(i)[0][8] * T for i in range(NCHAIN)])
        b.close()
        pt = np.array([r[k][8] for r in runs])
        ok, info = _agree(pt, ind)
        assert ok, (T, info)
