"""CPU tests of the drop-in modules' marshalling (no GPU).

The module source (mcsolver_gb300/csrc/mcs_pymod.c) is compiled here against
a stand-in engine library (under another name than libmcsgpu.so, which the
dynamic loader would otherwise share with the real modules loaded by other
tests) whose mcs_solve() records the problem it was given and
fills the result with known values.  The tests check what the reference's
callers see: the argument layout each module reads (isingLib.c:277-284,
heisenbergLib.c:504-512), the result tuple's shape (isingLib.c:436-447: 11
items; heisenbergLib.c:853-884: 29 items, spin frames as nested tuples, the
orbital-group tuple or 0.0) and the error mapping (engine status -> ValueError
or RuntimeError with the engine's message).
"""
import ctypes
import importlib.machinery
import importlib.util
import os
import subprocess
import sysconfig

import pytest

from tests import cases as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "mcsolver_gb300", "csrc", "mcs_pymod.c")

FAKE = r"""
#include <string.h>
#include "mcsgpu.h"
static mcs_problem g_last;
static int g_rc = 0;
static int g_frames_written = -1;
void fake_set(int rc, int frames_written) { g_rc = rc; g_frames_written = frames_written; }
const mcs_problem *fake_last(void) { return &g_last; }
const char *mcs_last_error(void) { return "stand-in failure"; }
int mcs_solve(const mcs_problem *p, const mcs_options *o, mcs_result *r)
{
    (void)o;
    g_last = *p;
    if (g_rc) return g_rc;
    for (int k = 0; k < MCS_RESULT_VALUES; ++k) r->values[k] = k + 0.5;
    for (int k = 0; k < r->group_capacity && r->group_values; ++k) r->group_values[k] = -k;
    int fw = g_frames_written < 0 ? p->spin_frames : g_frames_written;
    r->frames_written = fw;
    for (long long f = 0; f < fw && r->frames; ++f)
        for (int i = 0; i < p->n_sites; ++i)
            for (int c = 0; c < 3; ++c) r->frames[(f * p->n_sites + i) * 3 + c] = (float)(100 * f + i + 0.25 * c);
    return 0;
}
"""


class FakeProblem(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("algorithm", ctypes.c_int32), ("n_sites", ctypes.c_int32),
                ("max_links", ctypes.c_int32), ("nthermal", ctypes.c_int64), ("nsweep", ctypes.c_int64),
                ("ninterval", ctypes.c_int64)] + [(n, ctypes.c_void_p) for n in (
                    "init_spin", "init_d", "nlink", "link_strength", "linked_orb", "circuits", "corr_pair",
                    "group_list", "r_orb", "r_cluster", "r_link")] + [
                ("flunc", ctypes.c_double), ("h", ctypes.c_double)] + [(n, ctypes.c_int32) for n in (
                    "n_circuits", "n_lat", "n_group", "max_group", "n_rorb", "n_in_cluster", "ignore_offdiag",
                    "spin_frames")]


@pytest.fixture(scope="module")
def dropin(tmp_path_factory):
    d = tmp_path_factory.mktemp("dropin")
    cc = os.environ.get("CC", "gcc")
    (d / "fake.c").write_text(FAKE)
    inc = os.path.join(ROOT, "include")
    subprocess.run([cc, "-O1", "-fPIC", "-shared", "-I" + inc, str(d / "fake.c"), "-o", str(d / "libmcsfake.so")],
                   check=True)
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    mods = {}
    for k, name in ((1, "isinglib"), (2, "xylib"), (3, "heisenberglib")):
        out = d / (name + ext)
        subprocess.run([cc, "-O1", "-fPIC", "-shared", "-DMCS_PYMOD=%d" % k, "-I" + sysconfig.get_paths()["include"],
                        SRC, "-o", str(out), "-L" + str(d), "-lmcsfake", "-Wl,-rpath," + str(d)], check=True)
        loader = importlib.machinery.ExtensionFileLoader(name, str(out))
        spec = importlib.util.spec_from_file_location(name, str(out), loader=loader)
        m = importlib.util.module_from_spec(spec)
        loader.exec_module(m)
        mods[name] = m
    fake = ctypes.CDLL(str(d / "libmcsfake.so"))
    fake.fake_last.restype = ctypes.POINTER(FakeProblem)
    fake.fake_set.argtypes = [ctypes.c_int, ctypes.c_int]
    yield mods, fake
    fake.fake_set(0, -1)


def test_ising_tuple_layout_and_arguments(dropin):
    mods, fake = dropin
    fake.fake_set(0, -1)
    args = C.square_args("ising", 4, 2.0, h=0.3, nthermal=3, nsweep=5, frames=2)
    out = mods["isinglib"].MCMainFunction(*args, None)
    assert len(out) == 11
    assert out[:10] == tuple(k + 0.5 for k in range(10))
    frames = out[10]
    assert len(frames) == 2 and len(frames[0]) == 16
    assert frames[1][3] == pytest.approx(103.0) and isinstance(frames[0][0], float)
    p = fake.fake_last().contents
    assert (p.model, p.n_sites, p.max_links, p.nthermal, p.nsweep, p.spin_frames) == (1, 16, 4, 3, 5, 2)
    assert p.n_lat == len(args[9]) // 2 and p.h == pytest.approx(args[10])
    assert p.n_rorb == len(args[11]) and p.n_in_cluster == len(args[12]) // len(args[11])


@pytest.mark.parametrize("name,model", [("xylib", "xy"), ("heisenberglib", "heisenberg")])
def test_on_tuple_layout_frames_and_group_tuple(dropin, name, model):
    mods, fake = dropin
    fake.fake_set(0, -1)
    args = list(C.square_args(model, 4, 0.7, h=0.2, nthermal=1, nsweep=3, frames=3))
    args[12], args[13], args[14] = 2, 2, (0, 1, 2, 3)  # two orbital groups
    out = mods[name].MCMainFunction(*args, None)
    assert len(out) == 29
    assert out[:27] == tuple(k + 0.5 for k in range(27))
    frames = out[27]
    assert len(frames) == 3 and len(frames[2]) == 16
    assert frames[2][5] == pytest.approx((205.0, 205.25, 205.5))
    G = 2
    assert out[28] == tuple(float(-k) for k in range((G + 1) ** 2 + (G + 1)))
    p = fake.fake_last().contents
    assert p.model == (2 if model == "xy" else 3) and p.n_group == 2 and p.max_group == 2
    assert p.n_circuits == len(args[10]) // 3 and p.flunc == pytest.approx(args[15])


def test_no_frames_and_no_groups_give_floats(dropin):
    mods, fake = dropin
    fake.fake_set(0, -1)
    args = list(C.square_args("heisenberg", 4, 0.7, nthermal=1, nsweep=2))
    args[12], args[13], args[14] = 0, 0, ()  # no orbital groups
    out = mods["heisenberglib"].MCMainFunction(*args, None)
    assert out[27] == 0.0 and out[28] == 0.0


def test_frames_not_written_are_none(dropin):
    mods, fake = dropin
    fake.fake_set(0, 1)
    out = mods["isinglib"].MCMainFunction(*C.square_args("ising", 4, 2.0, nthermal=1, nsweep=3, frames=3), None)
    assert out[10][0] is not None and out[10][1] is None and out[10][2] is None
    fake.fake_set(0, -1)


@pytest.mark.parametrize("rc,exc", [(1, ValueError), (5, ValueError), (2, RuntimeError), (3, RuntimeError)])
def test_engine_status_maps_to_exceptions(dropin, rc, exc):
    mods, fake = dropin
    fake.fake_set(rc, -1)
    with pytest.raises(exc, match="stand-in failure"):
        mods["isinglib"].MCMainFunction(*C.square_args("ising", 4, 2.0, nthermal=1, nsweep=2), None)
    fake.fake_set(0, -1)


@pytest.mark.parametrize("k,bad,msg", [
    (7, (1.0,), "sizes do not match"),          # linkStrength too short
    (9, (0,), "pairs"),                          # corrOrbPair odd
    (13, (), "linkedOrb_rnorm"),                 # renormalised links missing
    (14, 99, "spinFrame"),                       # more frames than measurements
])
def test_ising_validation_before_the_engine(dropin, k, bad, msg):
    mods, fake = dropin
    args = list(C.square_args("ising", 4, 2.0, nthermal=1, nsweep=2))
    args[k] = bad
    with pytest.raises(ValueError, match=msg):
        mods["isinglib"].MCMainFunction(*args, None)


def _reference_present():
    from oracle import refharness as rh
    return rh.reference_tree_present()


@pytest.mark.skipif(not _reference_present(), reason="reference tree absent")
@pytest.mark.parametrize("model", ["ising", "xy", "heisenberg"])
def test_reference_caller_runs_unchanged_on_the_dropin(dropin, tmp_path, model):
    """mcsolver's own caller (mainLoopViaCLib, mcMain.py:51-135;
    mainLoopViaCLib_On, mcMain.py:137-272), unmodified, calls the drop-in
    module in place of its compiled library: it marshals its arguments,
    unpacks the result tuple, rescales the energies by T, writes ``out``,
    the spin-frame files and ``spinDotSpin.txt``."""
    from oracle import refharness as rh
    mods, fake = dropin
    fake.fake_set(0, -1)
    J = C.J9(-1.0, -1.0, -1.0) if model != "ising" else C.J9(-1.0)
    T = 0.8
    spec = dict(model=model, LMatrix=[[1, 0, 0], [0, 1, 0], [0, 0, 1]], pos=[[0, 0, 0]], S=[1.0], D=[[0, 0, 0]],
                bonds=[(0, 0, (1, 0, 0), J), (0, 0, (0, 1, 0), J)], L=(4, 4, 1), T=T, h=0.1,
                nthermal=2, nsweep=3, tau=0, algo="Metropolis", spinFrame=2, orbGroups=[[0]])
    if model != "ising":
        spec["circuits"] = [[[0, (0, 0, 0)], [0, (1, 0, 0)], [0, (0, 1, 0)]]]
    name = {"ising": "isinglib", "xy": "xylib", "heisenberg": "heisenberglib"}[model]
    ret = rh.run_caller_with(spec, mods[name], str(tmp_path))
    p = fake.fake_last().contents
    assert (p.n_sites, p.nthermal, p.nsweep, p.spin_frames) == (16, 2, 3, 2)
    out = (tmp_path / "out").read_text().split()
    if model == "ising":
        # T h <|s_i|> <|s_j|> spin_tot <s_i s_j> E E2 E_r E2_r U4 (mcMain.py:128-130)
        assert float(out[0]) == pytest.approx(T) and float(out[2]) == pytest.approx(0.5)
        assert float(out[6]) == pytest.approx(4.5 * T, abs=1e-3)
        assert ret[4] == pytest.approx(4.5 * T)
        frames = sorted(tmp_path.glob("IsingSpinDistribution.*.txt"))
    else:
        vals = dict(zip(out[0::2], out[1::2]))
        assert float(vals["<E>="]) == pytest.approx(8.5 * T) and float(vals["<Q>="]) == pytest.approx(26.5)
        frames = sorted(tmp_path.glob("OnSpinDistribution.*.txt"))
        assert (tmp_path / "spinDotSpin.txt").is_file()
    assert len(frames) == 2
    rows = frames[1].read_text().splitlines()[1:]
    assert len(rows) == 16 and float(rows[3].split()[3]) == pytest.approx(103.0)
