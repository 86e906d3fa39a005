"""Harness that runs the reference mcsolver libraries in this process.

Test infrastructure only: it is imported by the fixture generator under
``tests/golden/`` and by CPU tests that are skipped when the reference tree is
absent.  Nothing in the product imports it.

What it does
------------
* stubs the GUI-only modules the reference's Python imports
  (``win``, ``matplotlib``, ``matplotlib.figure``, ``matplotlib.pyplot``,
  ``tkinter``, ``tkinter.filedialog``), so that ``mcMain.py`` and
  ``Lattice.py`` run unchanged (mcMain.py:5-13, Lattice.py:2);
* loads the reference C libraries compiled by ``oracle/Makefile`` into
  ``oracle/_ref`` (xy through ``xy_shim.c``);
* drives the reference's own model build and marshalling
  (``mcMain.MC.__init__`` mcMain.py:16-49, ``mainLoopViaCLib`` mcMain.py:51-135,
  ``mainLoopViaCLib_On`` mcMain.py:137-272) with a capturing stand-in for
  ``MCMainFunction`` to obtain the exact positional argument tuples the
  reference caller passes to the compiled library;
* seeds glibc ``rand()`` with ``srand`` before a reference call, which is the
  only random source of the reference libraries.
"""
from __future__ import annotations

import contextlib
import ctypes
import importlib.machinery
import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, "_ref")
def _reference_source() -> str:
    """The reference's ``mcsolver`` source directory: ``MCS_REFERENCE_SRC``
    when set, else the REF variable of the oracle's build recipe
    (``make -C oracle print-ref``), the one place that names it."""
    env = os.environ.get("MCS_REFERENCE_SRC")
    if env:
        return env
    import subprocess
    try:
        out = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"], capture_output=True,
                             text=True, timeout=30)
        return out.stdout.strip()
    except Exception:
        return ""


REF_SRC = _reference_source()

_LIBC = ctypes.CDLL(None)


def reference_tree_present() -> bool:
    return os.path.isfile(os.path.join(REF_SRC, "mcMain.py"))


def reference_libs_present() -> bool:
    return all(os.path.isfile(os.path.join(REF_BUILD, n + ".so"))
               for n in ("isinglib", "xylib", "heisenberglib"))


def install_stubs() -> None:
    """Register stand-ins for the GUI modules the reference imports."""
    if "matplotlib" not in sys.modules or not hasattr(sys.modules["matplotlib"], "_mcs_stub"):
        mpl = types.ModuleType("matplotlib")
        mpl._mcs_stub = True
        fig = types.ModuleType("matplotlib.figure")

        class Figure:  # noqa: D401 - stand-in only
            def __init__(self, *a, **k):
                pass
        fig.Figure = Figure
        plt = types.ModuleType("matplotlib.pyplot")
        mpl.figure = fig
        mpl.pyplot = plt
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.figure"] = fig
        sys.modules["matplotlib.pyplot"] = plt
    if "win" not in sys.modules:
        sys.modules["win"] = types.ModuleType("win")
    if "tkinter" not in sys.modules:
        tk = types.ModuleType("tkinter")
        tk.Tk = object
        fd = types.ModuleType("tkinter.filedialog")
        tk.filedialog = fd
        sys.modules["tkinter"] = tk
        sys.modules["tkinter.filedialog"] = fd


_mcmain = None
_lattice = None


def reference_python():
    """Import the reference ``mcMain`` and ``Lattice`` modules unchanged."""
    global _mcmain, _lattice
    if _mcmain is None:
        if not reference_tree_present():
            raise RuntimeError("reference tree not found at %s" % REF_SRC)
        install_stubs()
        if REF_SRC not in sys.path:
            sys.path.insert(0, REF_SRC)
        import Lattice  # noqa: E402  (the reference's own module)
        import mcMain   # noqa: E402
        _mcmain, _lattice = mcMain, Lattice
    return _mcmain, _lattice


_ref_mods: dict = {}


def load_reference_lib(name: str):
    """Load oracle/_ref/<name>.so (isinglib / xylib / heisenberglib)."""
    if name not in _ref_mods:
        path = os.path.join(REF_BUILD, name + ".so")
        if not os.path.isfile(path):
            raise RuntimeError("reference library not built: %s (run make -C oracle ref)" % path)
        loader = importlib.machinery.ExtensionFileLoader(name, path)
        spec = importlib.util.spec_from_file_location(name, path, loader=loader)
        mod = importlib.util.module_from_spec(spec)
        loader.exec_module(mod)
        _ref_mods[name] = mod
    return _ref_mods[name]


def srand(seed: int) -> None:
    _LIBC.srand(ctypes.c_uint(seed & 0xFFFFFFFF))


LIBNAME = {"ising": "isinglib", "xy": "xylib", "heisenberg": "heisenberglib"}


@contextlib.contextmanager
def _in_tmpdir():
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            yield d
        finally:
            os.chdir(old)


@contextlib.contextmanager
def _quiet_stdout():
    """Silence the reference's printf/print chatter (fd-level)."""
    sys.stdout.flush()
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    try:
        yield
    finally:
        _LIBC.fflush(None)
        os.dup2(saved, 1)
        os.close(devnull)
        os.close(saved)


def _run_caller(spec: dict, mod) -> object:
    """Build the model of ``spec`` with the reference's own Python and run its
    caller (``mainLoopViaCLib`` mcMain.py:51-135 or ``mainLoopViaCLib_On``
    mcMain.py:137-272) with ``mod`` standing in for the compiled library (the
    caller imports it by name, mcMain.py:110-113 / :228-237).  Runs in the
    current directory, where the caller writes its files.  Returns what the
    caller returns."""
    mcMain, Lattice = reference_python()
    model = spec["model"]
    on = model != "ising"
    bonds = [Lattice.Bond(b[0], b[1], np.array([int(x) for x in b[2]]), *b[3], on) for b in spec["bonds"]]
    name = LIBNAME[model]
    saved = sys.modules.get(name)
    sys.modules[name] = mod
    try:
        ki = spec.get("ki", ((0, 0), (0, 0, 0)))
        kw = dict(pos=spec["pos"], S=spec["S"], D=spec["D"], bondList=bonds, T=spec["T"],
                  Lx=spec["L"][0], Ly=spec["L"][1], Lz=spec["L"][2],
                  ki_s=ki[0][0], ki_t=ki[0][1], ki_overLat=list(ki[1]),
                  orbGroupList=spec.get("orbGroups", []), groupInSC=spec.get("groupInSC", True),
                  h=spec.get("h", 0.0), dipoleAlpha=0, spinFrame=spec.get("spinFrame", 0))
        if on:
            kw["On"] = 2 if model == "xy" else 3
            kw["localCircuitList"] = spec.get("circuits", [])
        mc = mcMain.MC(0, spec["LMatrix"], **kw)
        if on:
            return mc.mainLoopViaCLib_On(nsweep=spec["nsweep"], nthermal=spec["nthermal"],
                                         ninterval=spec["tau"], algo=spec["algo"], On=kw["On"])
        return mc.mainLoopViaCLib(nsweep=spec["nsweep"], nthermal=spec["nthermal"],
                                  ninterval=spec["tau"], algo=spec["algo"])
    finally:
        if saved is None:
            sys.modules.pop(name, None)
        else:
            sys.modules[name] = saved


def capture_args(spec: dict) -> tuple:
    """Run the reference's model build + marshalling for ``spec`` and return
    the positional argument tuple it passes to MCMainFunction.

    ``spec`` keys: model ('ising'|'xy'|'heisenberg'), LMatrix, pos, S, D,
    bonds [(source, target, overLat, [Jxx,Jyy,Jzz,Jxy,Jxz,Jyz,Jyx,Jzx,Jzy])],
    L (Lx,Ly,Lz), T, h, nthermal, nsweep, tau, algo ('Metropolis'|'Wolff'),
    ki ((s,t),(ox,oy,oz)), orbGroups, groupInSC, circuits, spinFrame.
    """
    captured = {}

    def fake(*args):
        captured["args"] = args
        raise _Captured()

    fake_mod = types.ModuleType(LIBNAME[spec["model"]])
    fake_mod.MCMainFunction = fake
    with _in_tmpdir(), _quiet_stdout():
        try:
            _run_caller(spec, fake_mod)
        except _Captured:
            pass
    args = captured["args"]
    # drop the trailing callback (never called by the libraries)
    return tuple(args[:-1])


def run_caller_with(spec: dict, mod, workdir: str) -> object:
    """Run the reference's caller for ``spec`` in ``workdir`` with ``mod``
    (a module exposing MCMainFunction, e.g. a drop-in) in place of the
    compiled library; returns the caller's return value.  The caller's files
    (``out``, spin frames, ``spinDotSpin.txt``) are left in ``workdir``."""
    old = os.getcwd()
    os.chdir(workdir)
    try:
        with _quiet_stdout():
            return _run_caller(spec, mod)
    finally:
        os.chdir(old)


class _Captured(Exception):
    pass


def run_reference(model: str, args: tuple, seed: int | None = None, quiet: bool = True):
    """Call the reference MCMainFunction(*args, callback) after srand(seed)."""
    mod = load_reference_lib(LIBNAME[model])
    if seed is not None:
        srand(seed)
    cb = (lambda k: None)
    if quiet:
        with _quiet_stdout():
            return mod.MCMainFunction(*args, cb)
    return mod.MCMainFunction(*args, cb)
