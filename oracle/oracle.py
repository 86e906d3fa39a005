"""ctypes front end of the C oracle (``oracle/mcs_oracle.c``).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, never by the product.

``solve(model, args, seed, mode)`` takes exactly the positional argument tuple
of the reference ``MCMainFunction`` (without the trailing callback; layouts in
isingLib.c:277-284 and heisenbergLib.c:504-512) and returns the reference's
result tuple (isingLib.c:436-447: 11 items; heisenbergLib.c:853-884: 29 items).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmcsoracle.so")
NSER = 4

MODEL_ID = {"ising": 1, "xy": 2, "heisenberg": 3}

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)


class OrProblem(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int32), ("algorithm", ctypes.c_int32),
        ("N", ctypes.c_int32), ("z", ctypes.c_int32),
        ("nthermal", ctypes.c_int64), ("nsweep", ctypes.c_int64), ("ninterval", ctypes.c_int64),
        ("init_spin", _f64p), ("init_D", _f64p), ("nlink", _i32p),
        ("link_strength", _f64p), ("linked_orb", _i32p), ("circuits", _i32p),
        ("corr_pair", _i32p), ("group_list", _i32p), ("r_orb", _i32p),
        ("r_cluster", _i32p), ("r_link", _i32p),
        ("flunc", ctypes.c_double), ("h", ctypes.c_double),
        ("ncirc", ctypes.c_int32), ("nlat", ctypes.c_int32),
        ("n_group", ctypes.c_int32), ("max_group", ctypes.c_int32),
        ("n_rorb", ctypes.c_int32), ("n_in_cluster", ctypes.c_int32),
        ("ignore_offdiag", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


class OrRun(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int32), ("use_spins_in", ctypes.c_int32),
        ("seed", ctypes.c_uint64), ("sweep_offset", ctypes.c_int64), ("meas_offset", ctypes.c_int64),
        ("spins_io", _f64p), ("series", _f64p), ("result", _f64p),
        ("stats", ctypes.POINTER(ctypes.c_int64)),
        ("result_cap", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


_lib = None


def build() -> str:
    """Compile the C oracle with the recipe in oracle/Makefile."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.mcs_oracle_solve.argtypes = [ctypes.POINTER(OrProblem), ctypes.POINTER(OrRun)]
        _lib.mcs_oracle_solve.restype = ctypes.c_int
        _lib.mcs_oracle_colour.argtypes = [ctypes.POINTER(OrProblem), _i32p]
        _lib.mcs_oracle_colour.restype = ctypes.c_int
        _lib.mcs_oracle_philox.argtypes = [ctypes.POINTER(ctypes.c_uint32 * 4), ctypes.POINTER(ctypes.c_uint32 * 2),
                                           ctypes.POINTER(ctypes.c_uint32 * 4)]
        _lib.mcs_oracle_philox.restype = None
    return _lib


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().mcs_oracle_philox(ctypes.byref(c), ctypes.byref(k), ctypes.byref(o))
    return tuple(o)


class Problem:
    """Arrays of one MCMainFunction call, kept alive for ctypes."""

    def __init__(self, model: str, args: tuple):
        self.model = model
        a = list(args)
        if model == "ising":
            (alg, init, nth, nsw, tau, z, nlink, ls, lo, cp, h, rorb, rcl, rlink, frames) = a[:15]
            self.init_D = np.zeros(3 * len(init))
            circ, ngroup, maxg, glist, flunc, ign = (), 0, 1, (), 0.0, 0
        else:
            (alg, init, initD, nth, nsw, tau, z, nlink, ls, lo, circ, cp, ngroup, maxg, glist,
             flunc, h, rorb, rcl, rlink, frames, ign) = a[:22]
            self.init_D = np.ascontiguousarray(initD, dtype=np.float64)
        N = len(init)
        self.N, self.z = N, int(z)
        self.init = np.ascontiguousarray(init, dtype=np.float64)
        self.nlink = np.ascontiguousarray(nlink, dtype=np.int32)
        self.ls = np.ascontiguousarray(ls, dtype=np.float64)
        self.lo = np.ascontiguousarray(lo, dtype=np.int32)
        self.circ = np.ascontiguousarray(circ if len(circ) else [0, 0, 0], dtype=np.int32)
        self.ncirc = len(circ) // 3
        self.cp = np.ascontiguousarray(cp, dtype=np.int32)
        self.glist = np.ascontiguousarray(glist if len(glist) else [-1], dtype=np.int32)
        self.rorb = np.ascontiguousarray(rorb, dtype=np.int32)
        self.rcl = np.ascontiguousarray(rcl, dtype=np.int32)
        self.rlink = np.ascontiguousarray(rlink if len(rlink) else [-1], dtype=np.int32)
        self.frames = int(frames)
        self.n_group = int(ngroup)
        s = OrProblem()
        s.model = MODEL_ID[model]
        s.algorithm = int(alg)
        s.N = N
        s.z = int(z)
        s.nthermal, s.nsweep, s.ninterval = int(nth), int(nsw), int(tau)
        s.init_spin = self.init.ctypes.data_as(_f64p)
        s.init_D = self.init_D.ctypes.data_as(_f64p)
        s.nlink = self.nlink.ctypes.data_as(_i32p)
        s.link_strength = self.ls.ctypes.data_as(_f64p)
        s.linked_orb = self.lo.ctypes.data_as(_i32p)
        s.circuits = self.circ.ctypes.data_as(_i32p)
        s.corr_pair = self.cp.ctypes.data_as(_i32p)
        s.group_list = self.glist.ctypes.data_as(_i32p)
        s.r_orb = self.rorb.ctypes.data_as(_i32p)
        s.r_cluster = self.rcl.ctypes.data_as(_i32p)
        s.r_link = self.rlink.ctypes.data_as(_i32p)
        s.flunc, s.h = float(flunc), float(h)
        s.ncirc = self.ncirc
        s.nlat = len(cp) // 2
        s.n_group, s.max_group = int(ngroup), int(maxg)
        s.n_rorb = len(rorb)
        s.n_in_cluster = len(rcl) // max(1, len(rorb))
        s.ignore_offdiag = int(ign)
        self.s = s


def solve(model: str, args: tuple, seed: int = 1, mode: int = 0, spins_in=None,
          sweep_offset: int = 0, meas_offset: int = 0, want_series: bool = False):
    """Run the oracle; returns (result_tuple, extras dict).

    ``extras`` holds ``spins`` (N x 3 final state), ``stats`` (accepted moves or
    clusters, flipped sites, clusters built, Metropolis site visits) and
    ``series`` (nsweep x 4 per-measurement e, M, e_r, <s_i.s_j>) when asked.
    """
    P = Problem(model, args)
    N = P.N
    spins = np.zeros(3 * N)
    if spins_in is not None:
        spins[:] = np.asarray(spins_in, dtype=np.float64).reshape(-1)[:3 * N]
    nsw = P.s.nsweep
    series = np.zeros(max(1, nsw) * NSER) if want_series else None
    G = P.n_group
    cap = 29 + (G + 1) ** 2 + (G + 1)
    res = np.zeros(cap)
    stats = np.zeros(4, dtype=np.int64)
    r = OrRun()
    r.mode = mode
    r.use_spins_in = 1 if spins_in is not None else 0
    r.seed = seed & 0xFFFFFFFFFFFFFFFF
    r.sweep_offset = sweep_offset
    r.meas_offset = meas_offset
    r.spins_io = spins.ctypes.data_as(_f64p)
    r.series = series.ctypes.data_as(_f64p) if series is not None else None
    r.result = res.ctypes.data_as(_f64p)
    r.stats = stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    r.result_cap = cap
    rc = lib().mcs_oracle_solve(ctypes.byref(P.s), ctypes.byref(r))
    if rc != 0:
        raise RuntimeError("oracle failed: %d" % rc)
    extras = {"spins": spins.reshape(N, 3), "stats": stats,
              "series": series.reshape(-1, NSER)[:nsw] if series is not None else None}
    if model == "ising":
        out = tuple(float(x) for x in res[:10]) + (0.0,)
    else:
        base = tuple(float(x) for x in res[:27]) + (0.0,)
        if G > 0:
            grp = tuple(float(x) for x in res[29:cap])
        else:
            grp = 0.0
        out = base + (grp,)
    return out, extras


def colouring(model: str, args: tuple):
    P = Problem(model, args)
    out = np.zeros(P.N, dtype=np.int32)
    n = lib().mcs_oracle_colour(ctypes.byref(P.s), out.ctypes.data_as(_i32p))
    return n, out
