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


def _reference_ready():
    from oracle import refharness as rh
    return rh.reference_tree_present() and rh.reference_libs_present()


class _OracleBatch:
    """Stand-in for mcsolver_gb300.Batch on CPU: each replica is solved by the
    oracle's reference stream (mode 0, bit-identical to the reference
    libraries for the same seed)."""

    def __init__(self, device=0):
        self.items = []

    def add(self, model, args, seed=1, **opt):
        self.items.append((model, args, seed))
        return len(self.items) - 1

    def run(self):
        pass

    def result(self, i):
        from oracle import oracle as orc
        model, args, seed = self.items[i]
        r, ex = orc.solve(model, args, seed=seed, mode=0)
        N = len(args[1])
        nf = args[14] if model == "ising" else args[20]
        ex["frames"] = [np.zeros((N, 3))] * nf
        return r, ex

    def close(self):
        pass


@pytest.mark.skipif(not _reference_ready(), reason="reference tree or reference libraries absent")
@pytest.mark.parametrize("name", ["square_xy", "honeycomb_heisenberg", "square_ising_field"])
def test_grid_files_match_the_reference_caller(monkeypatch, tmp_path, name):
    """The grid driver writes what the reference writes for the same results.
    Our side: start_simulation with every point solved by the oracle's
    reference stream (seed + point ID).  Reference side: for every point,
    srand(seed + ID), then the reference's own caller (mcMain.MC +
    mainLoopViaCLib[_On]) on the reference library, which writes ``out`` and
    ``spinDotSpin.txt`` itself; the result.txt rows are formed as
    win.startSimulation forms them (win.py:92-102, :131-142, :169-172).
    The files must agree line for line."""
    import mcsolver_gb300
    from oracle import refharness as rh
    monkeypatch.setattr(mcsolver_gb300, "Batch", _OracleBatch)
    path = os.path.join(GOLD, "params", name + ".txt")
    p = sim.load_param(path)
    seed = 11
    ours = tmp_path / "ours"
    ref = tmp_path / "ref"
    ours.mkdir()
    ref.mkdir()
    sim.start_simulation(path, workdir=str(ours), seed=seed, threads=1)

    model = {"Ising": "ising", "XY": "xy", "Heisenberg": "heisenberg"}[p["modelType"]]
    lib = rh.load_reference_lib(rh.LIBNAME[model])
    for f in ("out", "spinDotSpin.txt"):
        (ref / f).write_text("#T #H\n")  # win.py:43-46
    Lx, Ly, Lz = p["LPack"]
    N = Lx * Ly * Lz * len(p["pos"])
    rows = []
    TList = np.linspace(p["T0"], p["T1"], p["nT"])
    HList = np.linspace(p["H0"], p["H1"], p["nH"])
    for iH, H in enumerate(HList):
        for iT, T in enumerate(TList):
            spec = dict(model=model, LMatrix=p["LMatrix"], pos=p["pos"], S=p["S"], D=p["DList"],
                        bonds=[(b[0], b[1], tuple(b[2]), list(b[3])) for b in p["bondList"]], L=p["LPack"],
                        T=float(T), h=float(H), nthermal=p["nthermal"], nsweep=p["nsweep"], tau=p["ninterval"],
                        algo=p["algorithm"], ki=p["GcOrb"], orbGroups=p["orbGroupList"], groupInSC=p["groupInSC"],
                        circuits=p["localCircuitList"], spinFrame=p["spinFrame"])
            rh.srand(seed + iH * len(TList) + iT)
            ret = rh.run_caller_with(spec, lib, str(ref))
            if model == "ising":
                si, sj, sij, ac, E, E2, U4 = ret
                rows.append((T, H, si, sj, (sij - si * sj) / T, E, (E2 - E * E) / T ** 2 * N, 0.0, U4, ac))
            else:
                si, sj, sij, ac, E, E2, U4, Q = ret
                rows.append((T, H, np.sqrt(sum(si * si)), np.sqrt(sum(sj * sj)), (sij - np.dot(si, sj)) / T, E,
                             (E2 - E * E) / T ** 2 * N, Q, U4, ac))
    for f in ("out", "spinDotSpin.txt"):
        assert (ours / f).read_text().splitlines() == (ref / f).read_text().splitlines(), f
    want = ["%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E" % r for r in rows]
    assert (ours / "result.txt").read_text().splitlines()[1:] == want


def _bits(x):
    a = np.asarray(x)
    return a.view(np.uint64) if a.dtype == np.float64 else a


TEMPLATE_LATTICES = [
    ("xy", (8, 8, 1), 1, [(0, 0, (1, 0, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0]), (0, 0, (0, 1, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0])],
     dict(D=[[0.1, -0.2, 0.0]], groups=[[0]], frames=2)),
    ("heisenberg", (6, 6, 1), 1, [(0, 0, (1, 0, 0), [-1, -1, -1, 0, 0.4, 0, 0, -0.4, 0]),
                                  (0, 0, (0, 1, 0), [-1, -1, -1, 0, 0, 0.4, 0, 0, -0.4])],
     dict(D=[[0, 0, -0.2]], circuits=[((0, (0, 0, 0)), (0, (1, 0, 0)), (0, (1, 1, 0)))])),     # DMI
    ("heisenberg", (4, 4, 1), 2, [(0, 1, (0, 0, 0), [-1.5, -1.5, -1.8, 0.3, 0, 0, 0.3, 0, 0]),
                                  (0, 1, (-1, 0, 0), [-1.5, -1.5, -1.8, 0.3, 0, 0, 0.3, 0, 0]),
                                  (0, 0, (1, 0, 0), [-0.3, -0.3, -0.3, 0, 0, 0, 0, 0, 0])],
     dict(S=[1.5, 1.0], D=[[0, 0, -0.5], [0, 0, 0.1]], groups=[[0], [1]], group_in_sc=False, ki=((0, 1), (0, 0, 0)))),
    ("ising", (6, 6, 1), 2, [(0, 1, o, [-1.0] + [0] * 8) for o in ((0, 0, 0), (-1, 0, 0), (0, 1, 0))],
     dict(S=[1.5, 1.5], ki=((0, 1), (0, 0, 0)))),
    ("xy", (2, 2, 1), 1, [(0, 0, (1, 0, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0]), (0, 0, (0, 1, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0])],
     dict()),                                                                                    # merged duplicates
    ("xy", (7, 5, 1), 1, [(0, 0, (1, 0, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0]), (0, 0, (0, 1, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0])],
     dict(groups=[[0]])),                                                                        # odd sides
    ("heisenberg", (5, 5, 3), 1, [(0, 0, ov, [-1, -1, -1, 0, 0, 0, 0, 0, 0]) for ov in ((1, 0, 0), (0, 1, 0), (0, 0, 1))],
     dict()),                                                                                    # 3D
    ("heisenberg", (5, 7, 1), 2, [(0, 1, (0, 0, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0]), (1, 0, (1, 0, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0]),
                                  (0, 0, (0, 1, 0), [-1, -1, -1, 0, 0, 0, 0, 0, 0])],
     dict(S=[1.0, 0.5], groups=[[0], [1], [0, 1]], ki=((1, 0), (1, 1, 0)))),                     # two orbitals, groups
    ("ising", (4, 4, 1), 1, [(0, 0, (0, 0, 0), [-1.0] + [0] * 8), (0, 0, (1, 0, 0), [-1.0] + [0] * 8)], dict()),  # self link
]


def test_lattice_template_vectorises_lattices_without_duplicate_links():
    """The structure is built with numpy unless a site holds two links (or two
    renormalised links) to one target, where the reference's order depends
    on values and the per-site builder is kept."""
    from mcsolver_gb300.lattice import LatticeTemplate
    want = [True, True, False, True, False, True, True, True, False]
    for (model, L, norb, bonds, kw), v in zip(TEMPLATE_LATTICES, want):
        assert LatticeTemplate(model, L, norb, bonds, **kw).vectorised == v, (model, L)


@pytest.mark.parametrize("k", range(len(TEMPLATE_LATTICES)))
def test_lattice_template_equals_lattice_args_bit_for_bit(k):
    """The grid driver builds a lattice once (LatticeTemplate) and rescales J,
    D and h per point; every point's tuple must be the one lattice_args (itself
    checked against the reference's marshalling) builds, bit for bit,
    including the clamp T -> 0.1 and the off-diagonal flag."""
    from mcsolver_gb300.lattice import LatticeTemplate, lattice_args
    model, L, norb, bonds, kw = TEMPLATE_LATTICES[k]
    t = LatticeTemplate(model, L, norb, bonds, **kw)
    assert bool(t.merged) == (L[0] <= 2)
    for T, H in ((0.05, 0.0), (0.7, 0.2), (2.5, -0.1), (1e7, 0.0)):
        want = lattice_args(model, L, norb, bonds, T, h=H, **kw)
        for arrays in (False, True):
            got = t.at(T, H, arrays=arrays)
            assert len(got) == len(want)
            for i, (a, b) in enumerate(zip(got, want)):
                assert np.array_equal(_bits(np.asarray(a, dtype=np.asarray(b).dtype)), _bits(b)), (T, H, arrays, i)


def test_grid_template_matches_the_per_site_builder():
    from mcsolver_gb300.lattice import lattice_args
    for name in ("square_xy", "honeycomb_heisenberg", "square_ising_field"):
        p = sim.load_param(os.path.join(GOLD, "params", name + ".txt"))
        model, (L, norb, bonds), kw = sim._lattice_inputs(p)
        for T, H in ((p["T0"], p["H0"]), (p["T1"], p["H1"])):
            m2, got = sim.point_args(p, T, H)
            assert m2 == model and got == lattice_args(model, L, norb, bonds, T, h=H, **kw)
