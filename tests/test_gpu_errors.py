"""Observables against the reference library within 3 sigma of binned,
autocorrelation-corrected error bars.

For every statistical golden case (the reference C library run with 24 seeds,
tests/golden), the engine runs 4 replicas of the same model, temperature and
field with ten times the reference's measurements per seed and
``record_series=True``.  Each replica's series gives means with binned errors
(blocking analysis) and, for U4 = <M^2>^2/<M^4>, jackknife errors over the same
blocks.  The engine's value and error are the mean over the replicas and the
combined error; the reference's are the 24-seed mean and its standard error.
They must agree within 3.5 combined sigma, plus the resolution of FP32 spin
state.  The printed table (pytest -s) gives the integrated autocorrelation
time of each series beside the comparison.

Compared entries of the result tuple: <s_i.s_j> (Ising 2, O(n) 6), the
renormalised energy (Ising 6, O(n) 18), U4 (Ising 8, O(n) 10) and, where the
reported energy is absolute, <e> and <e^2> (O(n) 8, 9; Ising Wolff 4, 5).  The
Ising Metropolis <e> is offset by the energy at the end of thermalisation
(isingLib.c:359), a single sample per run, so it is compared through the
Onsager test instead.
"""
import math

import numpy as np
import pytest

from mcsolver_gb300 import analysis as A
from tests import cases as C

pytestmark = pytest.mark.gpu

FP32_FLOOR = 2e-6
STAT = [n for n in C.golden()["cases"] if n.startswith("stat_")]


@pytest.mark.parametrize("name", STAT)
def test_observables_within_binned_error_bars(engine, name, capsys):
    model, args, c = C.golden_case(name)
    ising = model == "ising"
    nth = args[2] if ising else args[3]
    nsw = args[3] if ising else args[4]
    algo = args[0]
    long_args = C.with_program(model, args, nthermal=nth, nsweep=10 * nsw)
    N = len(args[1])
    b = engine.Batch()
    R = 4
    for k in range(R):
        b.add(model, long_args, seed=9000 + k, record_series=True)
    b.run()
    runs = [b.result(k)[1]["series"] for k in range(R)]
    b.close()
    summ = [A.summarize(s, N) for s in runs]
    nv = 10 if ising else 27  # the scalar entries (the O(n) tuple ends with the orbital-group tuple)
    ref = np.array([c["ref"][str(s)][:nv] for s in c["seeds"]], float)
    cmp = [("sij", 2 if ising else 6), ("e_r", 6 if ising else 18), ("U4", 8 if ising else 10)]
    if not ising:
        cmp += [("e", 8), ("e2", 9)]
    elif algo == 1:
        cmp += [("e", 4), ("e2", 5)]
    lines = []
    for key, idx in cmp:
        vals = np.array([s[key][0] for s in summ])
        errs = np.array([s[key][1] for s in summ])
        m_eng, e_eng = vals.mean(), math.sqrt((errs ** 2).sum()) / R
        x = ref[:, idx]
        m_ref, se_ref = x.mean(), x.std(ddof=1) / math.sqrt(len(x))
        sig = math.sqrt(e_eng ** 2 + se_ref ** 2)
        tau = summ[0][key][2]
        lines.append("  %-4s engine %.6g +- %.2g (tau_int %s)  reference %.6g +- %.2g  |z| %.2f"
                     % (key, m_eng, e_eng, "%.1f" % tau if tau is not None else "-", m_ref, se_ref,
                        abs(m_eng - m_ref) / sig if sig > 0 else 0.0))
        assert abs(m_eng - m_ref) <= 3.5 * sig + FP32_FLOOR * max(1.0, abs(m_ref)), (name, key, lines[-1])
    with capsys.disabled():
        print("\n" + name + "\n" + "\n".join(lines))
