"""Generate tests/golden/golden.json.gz from the reference itself.

Run in a checkout that has the reference tree and the reference libraries
built by ``make -C oracle ref``:

    python tests/golden/make_golden.py

For every case below it
  1. builds the model with the reference's own Python (Lattice.py /
     mcMain.py, unchanged, GUI modules stubbed) and captures the exact
     positional argument tuple mcMain passes to MCMainFunction;
  2. runs the reference C library (oracle/_ref) on those arguments after
     srand(seed) for each listed seed and stores the returned tuple.

The fixture therefore holds real caller-produced inputs and real reference
outputs; tests on machines without the reference tree read only this file.
"""
from __future__ import annotations

import gzip
import json
import os
import platform
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import refharness as rh  # noqa: E402

I3 = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
HEX = [[1.0, 0.0, 0.0], [-0.5, 0.866025404, 0.0], [0.0, 0.0, 1.0]]


def J9(xx, yy=0, zz=0, xy=0, xz=0, yz=0, yx=0, zx=0, zy=0):
    return [xx, yy, zz, xy, xz, yz, yx, zx, zy]


SQ_IS = [(0, 0, (1, 0, 0), J9(-1)), (0, 0, (0, 1, 0), J9(-1))]
SQ_ON = [(0, 0, (1, 0, 0), J9(-1, -1, -1)), (0, 0, (0, 1, 0), J9(-1, -1, -1))]
# DMI on the square lattice, antisymmetric off-diagonal 0.4|J| (Jxz=+d, Jzx=-d on [1 0 0]; Jyz=+d, Jzy=-d on [0 1 0])
SQ_DMI = [(0, 0, (1, 0, 0), J9(-1, -1, -1, xz=0.4, zx=-0.4)),
          (0, 0, (0, 1, 0), J9(-1, -1, -1, yz=0.4, zy=-0.4))]
SQ_CIRC = [((0, (0, 0, 0)), (0, (1, 0, 0)), (0, (1, 1, 0))),
           ((0, (0, 0, 0)), (0, (1, 1, 0)), (0, (0, 1, 0)))]
# honeycomb, 1NN Kitaev-type (diag -1.5,-1.5,-1.8 with Jxy=Jyx=0.3) and 2NN isotropic -0.3
HC_POS = [[0.333333333, 0.666666667, 0.0], [0.666666667, 0.333333333, 0.0]]
HC_1NN = [(0, 1, o, J9(-1.5, -1.5, -1.8, xy=0.3, yx=0.3)) for o in ((0, 0, 0), (-1, 0, 0), (0, 1, 0))]
HC_2NN = [(a, a, o, J9(-0.3, -0.3, -0.3)) for a in (0, 1) for o in ((1, 0, 0), (1, 1, 0), (0, 1, 0))]


def spec(model, L, T, bonds, algo="Metropolis", tau=0, nthermal=20, nsweep=30, h=0.0,
         pos=None, S=None, D=None, LM=I3, ki=((0, 0), (0, 0, 0)), groups=None, circuits=None):
    pos = pos or [[0, 0, 0]]
    norb = len(pos)
    return dict(model=model, LMatrix=LM, pos=pos, S=S or [1.0] * norb, D=D or [[0, 0, 0]] * norb,
                bonds=bonds, L=L, T=T, h=h, nthermal=nthermal, nsweep=nsweep, tau=tau, algo=algo,
                ki=ki, orbGroups=groups if groups is not None else [], groupInSC=True,
                circuits=circuits or [], spinFrame=0)


# Lattices with an odd side or a side of 4 are left out: there the reference's
# renormalised-link table holds -1 entries and isingLib.c:158 /
# heisenbergLib.c:269 dereference lattice[-1] (it crashes).
PIN = [7]
STAT = list(range(1, 25))

CASES = {
    # ---- short runs that pin the restatement bit for bit
    "pin_ising_sq8_metro": (spec("ising", (8, 8, 1), 2.0, SQ_IS), PIN),
    "pin_ising_sq8_metro_h": (spec("ising", (8, 8, 1), 2.0, SQ_IS, h=0.3), PIN),
    "pin_ising_sq8_wolff": (spec("ising", (8, 8, 1), 2.5, SQ_IS, algo="Wolff", tau=1), PIN),
    "pin_ising_sq8_wolff_h": (spec("ising", (8, 8, 1), 2.5, SQ_IS, algo="Wolff", tau=2, h=0.2), PIN),
    "pin_ising_hc6_metro": (spec("ising", (6, 6, 1), 3.0, [(0, 1, o, J9(-1)) for o in ((0, 0, 0), (-1, 0, 0), (0, 1, 0))],
                                 pos=HC_POS, S=[1.5, 1.5], LM=HEX, ki=((0, 1), (0, 0, 0))), PIN),
    "pin_heis_sq8_metro": (spec("heisenberg", (8, 8, 1), 0.7, SQ_ON, groups=[[0]], circuits=SQ_CIRC), PIN),
    "pin_heis_sq8_dmi_metro": (spec("heisenberg", (8, 8, 1), 0.4, SQ_DMI, h=0.2, D=[[0, 0, -0.1]],
                                    groups=[[0]], circuits=SQ_CIRC), PIN),
    "pin_heis_sq8_dmi_wolff": (spec("heisenberg", (8, 8, 1), 0.6, SQ_DMI, algo="Wolff", tau=1, h=0.1,
                                    D=[[0, 0, -0.2]], groups=[[0]], circuits=SQ_CIRC), PIN),
    "pin_heis_hc6_metro": (spec("heisenberg", (6, 6, 1), 8.0, HC_1NN + HC_2NN, pos=HC_POS, S=[1.0, 1.0],
                                D=[[0, 0, -0.5], [0, 0, -0.5]], LM=HEX, groups=[[0], [1]]), PIN),
    "pin_xy_sq8_metro": (spec("xy", (8, 8, 1), 0.9, SQ_ON, groups=[[0]]), PIN),
    "pin_xy_sq8_wolff": (spec("xy", (8, 8, 1), 0.9, SQ_ON, algo="Wolff", tau=1, groups=[[0]]), PIN),
    # ---- statistical cases: many seeds give the reference's spread
    "stat_ising_sq16_T2.5_metro": (spec("ising", (16, 16, 1), 2.5, SQ_IS, nthermal=300, nsweep=2000), STAT),
    "stat_ising_sq16_T2.0_h0.1_metro": (spec("ising", (16, 16, 1), 2.0, SQ_IS, nthermal=300, nsweep=2000, h=0.1), STAT),
    "stat_ising_sq16_T2.4_wolff": (spec("ising", (16, 16, 1), 2.4, SQ_IS, algo="Wolff", tau=4, nthermal=200, nsweep=1500), STAT),
    "stat_xy_sq16_T0.9_metro": (spec("xy", (16, 16, 1), 0.9, SQ_ON, nthermal=300, nsweep=2000, groups=[[0]]), STAT),
    "stat_xy_sq16_T1.1_wolff": (spec("xy", (16, 16, 1), 1.1, SQ_ON, algo="Wolff", tau=2, nthermal=300, nsweep=2000, groups=[[0]]), STAT),
    "stat_heis_sq12_dmi_T0.5_h0.3_metro": (spec("heisenberg", (12, 12, 1), 0.5, SQ_DMI, h=0.3, nthermal=300, nsweep=2000,
                                                groups=[[0]], circuits=SQ_CIRC), STAT),
    "stat_heis_hc6_T8_metro": (spec("heisenberg", (6, 6, 1), 8.0, HC_1NN + HC_2NN, pos=HC_POS, S=[1.0, 1.0],
                                    D=[[0, 0, -0.5], [0, 0, -0.5]], LM=HEX, groups=[[0], [1]], nthermal=300, nsweep=2000), STAT),
    "stat_heis_sq12_T0.7_wolff": (spec("heisenberg", (12, 12, 1), 0.7, SQ_ON, algo="Wolff", tau=2, nthermal=300, nsweep=2000,
                                       groups=[[0]], circuits=SQ_CIRC), STAT),
}


def to_jsonable(x):
    if hasattr(x, "item") and not isinstance(x, (list, tuple)):
        return x.item()  # numpy scalar
    if isinstance(x, tuple):
        return [to_jsonable(v) for v in x]
    if isinstance(x, list):
        return [to_jsonable(v) for v in x]
    return x


def main():
    out = {"generator": "tests/golden/make_golden.py", "machine": platform.machine(), "cases": {}}
    for name, (sp, seeds) in CASES.items():
        args = rh.capture_args(sp)
        res = {}
        for s in seeds:
            r = rh.run_reference(sp["model"], args, seed=s)
            res[str(s)] = to_jsonable(r)
        out["cases"][name] = {"model": sp["model"], "spec": to_jsonable(sp), "args": to_jsonable(args),
                              "ref": res, "seeds": seeds}
        print(name, "N=%d" % len(args[1]), "seeds=%d" % len(seeds), flush=True)
    path = os.path.join(HERE, "golden.json.gz")
    with gzip.open(path, "wt") as f:
        json.dump(out, f)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
