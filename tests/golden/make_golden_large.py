"""Generate tests/golden/golden_large.json.gz from the reference itself, on
the lattices of the benchmark configurations.

Run where the reference sources and the reference libraries built by
``make -C oracle ref`` are present:

    python tests/golden/make_golden_large.py [case ...]

For every case below it
  1. builds the model with the reference's own Python (Lattice.py /
     mcMain.py, unchanged, GUI modules stubbed) and captures the positional
     argument tuple mcMain passes to MCMainFunction;
  2. stores a fingerprint of that tuple (per argument: length, sum, a
     position-weighted sum and the sum of squares), so that a test can check,
     without the reference, that mcsolver_gb300.lattice builds the same
     tuple at full size -- the tuples themselves (millions of couplings) are
     not stored;
  3. runs the reference C library (oracle/_ref) on the tuple after srand(seed)
     for every listed seed, one process per host core, and stores each
     returned result tuple (the orbital-group tuple dropped);
  4. runs the oracle's mode 2 on the same tuple and seeds: the reference's
     own algorithm and order of draws with a SplitMix64 generator in place of
     glibc rand() (stored as "alg").  glibc rand() is an additive
     lagged-Fibonacci generator and the XY library draws from a 15-bit rand();
     at low temperatures both shift the reference library's energies by more
     than the statistical error of these runs, so the engine's exact sampling
     is compared with "alg" as well as with the library.

The reference starts every run from its own initial state (all spins along
+x, mcMain passes flunc = 0: heisenbergLib.c:154-172, xyLib.c:120-131), so
the engine runs in the tests start from the same state.  Sweep counts are
reduced from the benchmark configurations (stated per case) and chosen, from
measured relaxation and autocorrelation times, so that every run reaches
equilibrium well inside its thermalisation sweeps.
"""
from __future__ import annotations

import gzip
import json
import multiprocessing as mp
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import make_golden as mg  # noqa: E402  (bond lists and the spec format)

SEEDS = list(range(1, 33))


def fingerprint(args):
    """Per positional argument: scalars as they are; sequences as [length,
    sum, sum of x_i * (1 + i % 1009), sum of squares] in FP64."""
    import numpy as np
    out = []
    for a in args:
        if np.ndim(a) == 0:  # Python or numpy scalar
            out.append(float(a))
        elif isinstance(a, (tuple, list)) or hasattr(a, "shape"):
            x = np.asarray(a, dtype=np.float64).reshape(-1)
            w = 1.0 + (np.arange(x.size) % 1009)
            out.append([int(x.size), float(x.sum()), float((x * w).sum()), float((x * x).sum())])
        else:
            out.append(float(a))
    return out


def _cases():
    c = {}
    # cfg2: square XY, Jxx = Jyy = -1 K, L = 128, Metropolis, tau = N
    for T in XY_TEMPS:
        c["xy_sq128_T%g_metro" % T] = mg.spec("xy", (128, 128, 1), T, mg.SQ_ON, nthermal=XY_PROG[0],
                                              nsweep=XY_PROG[1], groups=[[0]])
    # cfg4: square Heisenberg J = -1 K with DMI 0.4 and field, two circuits per cell, L = 64
    for T, h in DMI_POINTS:
        c["heis_sq64_dmi_T%g_h%g_metro" % (T, h)] = mg.spec("heisenberg", (64, 64, 1), T, mg.SQ_DMI, h=h,
                                                           nthermal=DMI_PROG[0], nsweep=DMI_PROG[1], groups=[[0]],
                                                           circuits=mg.SQ_CIRC)
    # cfg3: honeycomb Heisenberg, 1NN Kitaev-type + 2NN, Az = -0.5, 64 x 64 cells (temperatures of the
    # 64-rung geometric ladder 5..50 K)
    for k in HC_RUNGS:
        T = 5.0 * 10 ** (k / 63.0)
        c["heis_hc64_T%.4f_metro" % T] = mg.spec("heisenberg", (64, 64, 1), T, mg.HC_1NN + mg.HC_2NN, pos=mg.HC_POS,
                                                S=[1.0, 1.0], D=[[0, 0, -0.5], [0, 0, -0.5]], LM=mg.HEX,
                                                groups=[[0], [1]], nthermal=HC_PROG[0], nsweep=HC_PROG[1])
    return c


# (nthermal, nsweep) per family, reduced from the configurations' 5000 + 20000
# (XY) and 50,000 (honeycomb): from the ordered start the energies settle
# within 1000 sweeps at every point below; the integrated autocorrelation
# times of e are 6-19 measurements (XY), 7-19 (DMI), about 1 (honeycomb).
XY_TEMPS = (0.5, 0.9, 1.3)
XY_PROG = (3000, 6000)
DMI_POINTS = ((0.05, 0.6), (0.5, 0.3), (1.0, 0.1))   # 0.05 K runs at mcMain's clamp, 0.1 K
DMI_PROG = (2000, 6000)
HC_RUNGS = (0, 20)                                   # T = 5.0 and 10.4 K
HC_PROG = (1000, 5000)


def _run_one(job):
    from oracle import refharness as rh
    model, args, seed = job
    r = rh.run_reference(model, args, seed=seed)
    n = 10 if model == "ising" else 27
    return seed, [float(v) for v in r[:n]]


def _run_alg(job):
    from oracle import oracle as orc
    model, args, seed = job
    r, _ = orc.solve(model, args, seed=seed, mode=2)
    n = 10 if model == "ising" else 27
    return seed, [float(v) for v in r[:n]]


def refresh_fingerprints():
    """Recompute the stored fingerprints from the reference's marshalling
    (no library runs)."""
    from oracle import refharness as rh
    path = os.path.join(HERE, "golden_large.json.gz")
    with gzip.open(path, "rt") as f:
        out = json.load(f)
    cases = _cases()
    for name, c in out["cases"].items():
        c["fingerprint"] = fingerprint(rh.capture_args(cases[name]))
    with gzip.open(path, "wt") as f:
        json.dump(out, f)


def main(names=None):
    from oracle import refharness as rh
    path = os.path.join(HERE, "golden_large.json.gz")
    out = {"generator": "tests/golden/make_golden_large.py", "machine": platform.machine(), "cases": {}}
    if os.path.isfile(path):
        with gzip.open(path, "rt") as f:
            out = json.load(f)
    cases = _cases()
    todo = [n for n in cases if not names or n in names]
    for name in todo:
        sp = cases[name]
        t = time.time()
        args = rh.capture_args(sp)
        fp = fingerprint(args)
        with mp.get_context("fork").Pool(os.cpu_count() or 1) as pool:
            res = dict(pool.map(_run_one, [(sp["model"], args, s) for s in SEEDS]))
            alg = dict(pool.map(_run_alg, [(sp["model"], args, s) for s in SEEDS]))
        out["cases"][name] = {"model": sp["model"], "spec": mg.to_jsonable(sp), "fingerprint": fp,
                              "ref": {str(s): res[s] for s in SEEDS}, "alg": {str(s): alg[s] for s in SEEDS},
                              "seeds": SEEDS, "seconds": round(time.time() - t, 1)}
        print(name, "N=%d" % len(args[1]), "%.0f s" % (time.time() - t), flush=True)
        with gzip.open(path, "wt") as f:
            json.dump(out, f)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if sys.argv[1:] == ["--fingerprints"]:
        refresh_fingerprints()
    else:
        main(sys.argv[1:] or None)
