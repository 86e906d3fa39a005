"""Generate parameter-file fixtures and what the reference's parser reads from them.

Writes three version-3.0 parameter files (square XY, honeycomb Heisenberg with
cell-only groups and circuits, square Ising with a field) with
``mcsolver_gb300.simulation.save_param`` into tests/golden/params/, then parses
each with the reference's own ``fileio.loadParam`` (fileio.py:169-313, GUI
modules stubbed), and for one (T, H) point of each captures the argument tuple
the reference's own model build passes to MCMainFunction (mcMain.MC +
mainLoopViaCLib[_On], through oracle/refharness.py).  Both go to
tests/golden/params_parsed.json.gz.  Run where the reference sources are
present (their directory is the oracle recipe's REF, or MCS_REFERENCE_SRC):

    python tests/golden/make_param_golden.py
"""
import gzip
import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from mcsolver_gb300.simulation import save_param  # noqa: E402
from oracle.refharness import REF_SRC as REF  # noqa: E402

J = lambda xx, yy=0, zz=0, xy=0, xz=0, yz=0, yx=0, zx=0, zy=0: [xx, yy, zz, xy, xz, yz, yx, zx, zy]  # noqa: E731

PARAMS = {
    "square_xy": dict(LMatrix=[[1, 0, 0], [0, 1, 0], [0, 0, 1]], LPack=[8, 8, 1], pos=[[0, 0, 0]], S=[1.0],
                      DList=[[0, 0, 0]], bondList=[(0, 0, (1, 0, 0), J(-1, -1, -1)), (0, 0, (0, 1, 0), J(-1, -1, -1))],
                      GcOrb=((0, 0), (0, 0, 0)), orbGroupList=[[0]], groupInSC=True, localCircuitList=[],
                      T0=0.9, T1=1.2, nT=4, H0=0.0, H1=0.1, nH=2, dipoleAlpha=0.0, spinFrame=2,
                      nthermal=20, nsweep=40, ninterval=0, xAxisType="T", modelType="XY", algorithm="Metropolis",
                      ncores=4),
    "honeycomb_heisenberg": dict(
        LMatrix=[[1, 0, 0], [-0.5, 0.866025404, 0], [0, 0, 1]], LPack=[6, 6, 1],
        pos=[[0.333333333, 0.666666667, 0], [0.666666667, 0.333333333, 0]], S=[1.5, 1.5],
        DList=[[0, 0, -0.5], [0, 0, -0.5]],
        bondList=[(0, 1, (0, 0, 0), J(-1.5, -1.5, -1.8, xy=0.3, yx=0.3)), (0, 1, (-1, 0, 0), J(-1.5, -1.5, -1.8, xy=0.3, yx=0.3)),
                  (0, 1, (0, 1, 0), J(-1.5, -1.5, -1.8, xy=0.3, yx=0.3)), (0, 0, (1, 0, 0), J(-0.3, -0.3, -0.3)),
                  (0, 0, (1, 1, 0), J(-0.3, -0.3, -0.3)), (0, 0, (0, 1, 0), J(-0.3, -0.3, -0.3)),
                  (1, 1, (1, 0, 0), J(-0.3, -0.3, -0.3)), (1, 1, (1, 1, 0), J(-0.3, -0.3, -0.3)),
                  (1, 1, (0, 1, 0), J(-0.3, -0.3, -0.3))],
        GcOrb=((0, 1), (0, 0, 0)), orbGroupList=[[0], [1]], groupInSC=False,
        localCircuitList=[((0, (0, 0, 0)), (1, (0, 0, 0)), (0, (1, 0, 0))), ((1, (0, 0, 0)), (0, (1, 1, 0)), (1, (1, 0, 0)))],
        T0=5.0, T1=20.0, nT=3, H0=0.0, H1=0.0, nH=1, dipoleAlpha=0.0, spinFrame=0,
        nthermal=10, nsweep=30, ninterval=72, xAxisType="T", modelType="Heisenberg", algorithm="Wolff", ncores=8),
    "square_ising_field": dict(
        LMatrix=[[1, 0, 0], [0, 1, 0], [0, 0, 1]], LPack=[10, 10, 1], pos=[[0, 0, 0]], S=[1.0], DList=[[0, 0, 0]],
        bondList=[(0, 0, (1, 0, 0), J(-1.0)), (0, 0, (0, -1, 0), J(-1.0))],
        GcOrb=((0, 0), (1, 0, 0)), orbGroupList=[[0]], groupInSC=True, localCircuitList=[],
        T0=1.5, T1=3.5, nT=5, H0=-0.2, H1=0.2, nH=3, dipoleAlpha=0.0, spinFrame=1,
        nthermal=30, nsweep=60, ninterval=0, xAxisType="H", modelType="Ising", algorithm="Metropolis", ncores=2),
}


def reference_parse(path):
    sys.path.insert(0, REF)
    tk = types.ModuleType("tkinter")
    tk.filedialog = types.ModuleType("tkinter.filedialog")
    sys.modules["tkinter"] = tk
    sys.modules["tkinter.filedialog"] = tk.filedialog
    gui = types.ModuleType("guiMain")
    sys.modules["guiMain"] = gui
    win = types.ModuleType("win")
    win.settingFileVersion = 3.0
    sys.modules["win"] = win
    import fileio
    assert fileio.loadParam(updateGUI=False, rpath=path)
    f = fileio
    return dict(LMatrix=f.LMatrix, LPack=f.LPack, pos=f.pos, S=f.S, DList=f.DList,
                bondList=[[b[0], b[1], list(b[2]), list(b[3:])] for b in f.bondList],
                GcOrb=[list(f.GcOrb[0]), list(f.GcOrb[1])], orbGroupList=f.orbGroupList, groupInSC=f.groupInSC,
                localCircuitList=[[[c[0], list(c[1])] for c in circ] for circ in f.localCircuitList],
                T0=f.T0, T1=f.T1, nT=f.nT, H0=f.H0, H1=f.H1, nH=f.nH, dipoleAlpha=f.dipoleAlpha, spinFrame=f.spinFrame,
                nthermal=f.nthermal, nsweep=f.nsweep, ninterval=f.ninterval, xAxisType=f.xAxisType,
                modelType=f.modelType, algorithm=f.algorithm, ncores=f.ncores)


def reference_args(p, T, H):
    from oracle import refharness as rh
    rh.install_stubs()
    model = {"Ising": "ising", "XY": "xy", "Heisenberg": "heisenberg"}[p["modelType"]]
    spec = dict(model=model, LMatrix=p["LMatrix"], pos=p["pos"], S=p["S"], D=p["DList"],
                bonds=[(b[0], b[1], b[2], b[3]) for b in p["bondList"]], L=tuple(p["LPack"]), T=T, h=H,
                nthermal=p["nthermal"], nsweep=p["nsweep"], tau=p["ninterval"], algo=p["algorithm"],
                ki=(tuple(p["GcOrb"][0]), tuple(p["GcOrb"][1])), orbGroups=p["orbGroupList"],
                groupInSC=p["groupInSC"], circuits=[tuple((c[0], tuple(c[1])) for c in circ) for circ in p["localCircuitList"]],
                spinFrame=p["spinFrame"])
    args = rh.capture_args(spec)

    def plain(x):
        if isinstance(x, (tuple, list)):
            return [plain(y) for y in x]
        if hasattr(x, "item"):
            return x.item()
        return x
    return [plain(a) for a in args if not callable(a)]


def main():
    out = {}
    for name, p in PARAMS.items():
        path = os.path.join(HERE, "params", name + ".txt")
        save_param(p, path)
        parsed = reference_parse(path)
        T, H = parsed["T1"], parsed["H1"]
        out[name] = {"parsed": parsed, "point": [T, H], "args": reference_args(parsed, T, H)}
    with gzip.open(os.path.join(HERE, "params_parsed.json.gz"), "wt") as f:
        json.dump({"generator": "tests/golden/make_param_golden.py", "parser": "reference fileio.loadParam",
                   "args": "reference mcMain.MC + mainLoopViaCLib[_On] (captured MCMainFunction arguments)",
                   "cases": out}, f)


if __name__ == "__main__":
    main()
