"""GB300 Monte Carlo spin-lattice engine -- drop-in for mcsolver's compiled libraries.

Layers
------
* ``libmcsgpu.so`` (``include/mcsgpu.h``): the CUDA engine behind a plain C ABI.
* ``isinglib`` / ``xylib`` / ``heisenberglib`` CPython modules (built into
  ``mcsolver_gb300/lib``): ``MCMainFunction`` with the reference's positional
  arguments and result tuple, for mcsolver's unchanged ``mcMain.py``.
* this module: ctypes access to the C ABI for Python callers (single solves,
  batches, parallel tempering, the request server).

There is no CPU fallback: every entry point raises if the engine library is
not built or the GPU is not available.
"""
from __future__ import annotations

import ctypes
import importlib.machinery
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")
ENGINE_PATH = os.path.join(LIBDIR, "libmcsgpu.so")

MODEL_ID = {"ising": 1, "xy": 2, "heisenberg": 3}
SCHEDULE_ID = {"auto": 0, "plain": 1, "resident": 2, "tiled": 3}
SCHEDULE_NAME = {v: k for k, v in SCHEDULE_ID.items()}
NSER = 4

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)


class McsProblem(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int32), ("algorithm", ctypes.c_int32),
        ("n_sites", ctypes.c_int32), ("max_links", ctypes.c_int32),
        ("nthermal", ctypes.c_int64), ("nsweep", ctypes.c_int64), ("ninterval", ctypes.c_int64),
        ("init_spin", _f64p), ("init_d", _f64p), ("nlink", _i32p), ("link_strength", _f64p),
        ("linked_orb", _i32p), ("circuits", _i32p), ("corr_pair", _i32p), ("group_list", _i32p),
        ("r_orb", _i32p), ("r_cluster", _i32p), ("r_link", _i32p),
        ("flunc", ctypes.c_double), ("h", ctypes.c_double),
        ("n_circuits", ctypes.c_int32), ("n_lat", ctypes.c_int32),
        ("n_group", ctypes.c_int32), ("max_group", ctypes.c_int32),
        ("n_rorb", ctypes.c_int32), ("n_in_cluster", ctypes.c_int32),
        ("ignore_offdiag", ctypes.c_int32), ("spin_frames", ctypes.c_int32),
    ]


class McsOptions(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64), ("schedule", ctypes.c_int32), ("absolute_energy", ctypes.c_int32),
        ("recheck_every", ctypes.c_int32), ("record_series", ctypes.c_int32),
        ("random_init", ctypes.c_int32), ("fp64_update", ctypes.c_int32),
        ("device", ctypes.c_int32), ("reserved_", ctypes.c_int32),
    ]


class McsResult(ctypes.Structure):
    _fields_ = [
        ("values", ctypes.c_double * 29), ("group_values", _f64p), ("group_capacity", ctypes.c_int32),
        ("frames_written", ctypes.c_int32), ("frames", _f32p), ("series", _f64p),
        ("site_updates", ctypes.c_int64), ("clusters", ctypes.c_int64), ("flipped", ctypes.c_int64),
        ("accepted", ctypes.c_int64), ("exact_mismatches", ctypes.c_int64),
        ("energy_drift", ctypes.c_double), ("device_ms", ctypes.c_double),
        ("schedule_used", ctypes.c_int32), ("n_colours", ctypes.c_int32),
    ]


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("mcsgpu error %d: %s" % (code, msg))
        self.code = code


_lib = None

# every function declared in include/mcsgpu.h
ABI_FUNCTIONS = [
    "mcs_solve", "mcs_last_error", "mcs_abi_version", "mcs_build_info",
    "mcs_batch_create", "mcs_batch_add", "mcs_batch_run", "mcs_batch_prepare", "mcs_batch_advance",
    "mcs_batch_result", "mcs_batch_stats", "mcs_batch_memory", "mcs_batch_schedule", "mcs_batch_destroy",
    "mcs_pt_create", "mcs_pt_run", "mcs_pt_result", "mcs_pt_stats", "mcs_pt_destroy",
    "mcs_server_create", "mcs_server_submit", "mcs_server_step", "mcs_server_poll", "mcs_server_stats",
    "mcs_server_cancel", "mcs_server_destroy", "mcs_ising_square_noalloc",
]

# status codes (include/mcsgpu.h)
MCS_ENOMEM, MCS_ECUDA, MCS_ENOTFOUND, MCS_ECANCELLED, MCS_EFAILED = 4, 2, 7, 8, 9


def lib():
    """Load libmcsgpu.so (built by ``mcsolver_gb300.build``); raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.isfile(ENGINE_PATH):
            raise RuntimeError("libmcsgpu.so is not built (python -c 'import __graft_entry__ as g; g.build()')")
        L = ctypes.CDLL(ENGINE_PATH)
        L.mcs_solve.argtypes = [ctypes.POINTER(McsProblem), ctypes.POINTER(McsOptions), ctypes.POINTER(McsResult)]
        L.mcs_solve.restype = ctypes.c_int
        L.mcs_last_error.restype = ctypes.c_char_p
        L.mcs_build_info.restype = ctypes.c_char_p
        L.mcs_batch_create.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
        L.mcs_batch_add.argtypes = [ctypes.c_void_p, ctypes.POINTER(McsProblem), ctypes.POINTER(McsOptions), _i32p]
        L.mcs_batch_run.argtypes = [ctypes.c_void_p]
        L.mcs_batch_prepare.argtypes = [ctypes.c_void_p]
        L.mcs_batch_advance.argtypes = [ctypes.c_void_p, ctypes.c_int64, _f64p]
        L.mcs_batch_result.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(McsResult)]
        L.mcs_batch_stats.argtypes = [ctypes.c_void_p, _f64p, ctypes.POINTER(ctypes.c_int64), _i32p]
        L.mcs_batch_memory.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        L.mcs_batch_schedule.argtypes = [ctypes.c_void_p, ctypes.c_int32, _i32p, _i32p, _i32p, _i32p]
        L.mcs_batch_destroy.argtypes = [ctypes.c_void_p]
        L.mcs_batch_destroy.restype = None
        L.mcs_pt_create.argtypes = [ctypes.POINTER(McsProblem), ctypes.POINTER(McsOptions), _f64p, ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_void_p)]
        L.mcs_pt_run.argtypes = [ctypes.c_void_p]
        L.mcs_pt_result.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(McsResult)]
        L.mcs_pt_stats.argtypes = [ctypes.c_void_p, _f64p, _f64p, ctypes.POINTER(ctypes.c_int64)]
        L.mcs_pt_destroy.argtypes = [ctypes.c_void_p]
        L.mcs_pt_destroy.restype = None
        L.mcs_server_create.argtypes = [ctypes.c_int32, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
        L.mcs_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(McsProblem), ctypes.POINTER(McsOptions),
                                        ctypes.POINTER(ctypes.c_uint64)]
        L.mcs_server_step.argtypes = [ctypes.c_void_p, _i32p]
        L.mcs_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(McsResult)]
        L.mcs_server_stats.argtypes = [ctypes.c_void_p, _i32p, _i32p, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_int64)]
        L.mcs_server_cancel.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.mcs_server_destroy.argtypes = [ctypes.c_void_p]
        L.mcs_server_destroy.restype = None
        L.mcs_ising_square_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int32,
                                               ctypes.c_void_p, ctypes.c_void_p]
        L.mcs_ising_square_noalloc.restype = ctypes.c_int
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        msg = lib().mcs_last_error()
        raise EngineError(rc, msg.decode() if msg else "")


def load_dropin(name: str):
    """Import the built drop-in module ``isinglib`` / ``xylib`` / ``heisenberglib``."""
    path = os.path.join(LIBDIR, name + ".so")
    if not os.path.isfile(path):
        raise RuntimeError("%s is not built" % path)
    loader = importlib.machinery.ExtensionFileLoader(name, path)
    spec = importlib.util.spec_from_file_location(name, path, loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


def install_dropin() -> None:
    """Make ``import isinglib`` / ``xylib`` / ``heisenberglib`` resolve to this engine
    (the imports of mcMain.py:110-113 and :228-237)."""
    if LIBDIR not in sys.path:
        sys.path.insert(0, LIBDIR)


class Problem:
    """The arrays of one MCMainFunction call (positional tuple without the
    callback), held as numpy buffers for the C ABI."""

    def __init__(self, model: str, args: tuple):
        self.model = model
        a = list(args)
        if model == "ising":
            (alg, init, nth, nsw, tau, z, nlink, ls, lo, cp, h, rorb, rcl, rlink, frames) = a[:15]
            initD, circ, ngroup, maxg, glist, flunc, ign = None, (), 0, 1, (), 0.0, 0
        else:
            (alg, init, initD, nth, nsw, tau, z, nlink, ls, lo, circ, cp, ngroup, maxg, glist,
             flunc, h, rorb, rcl, rlink, frames, ign) = a[:22]
        N = len(init)
        self.N = N
        self._keep = []

        def arr(x, dt):
            v = np.ascontiguousarray(np.asarray(x if len(x) else [0], dtype=dt))
            self._keep.append(v)
            return v

        init_a = arr(init, np.float64)
        p = McsProblem()
        p.model = MODEL_ID[model]
        p.algorithm = int(alg)
        p.n_sites = N
        p.max_links = int(z)
        p.nthermal, p.nsweep, p.ninterval = int(nth), int(nsw), int(tau)
        p.init_spin = init_a.ctypes.data_as(_f64p)
        if initD is not None:
            p.init_d = arr(initD, np.float64).ctypes.data_as(_f64p)
        p.nlink = arr(nlink, np.int32).ctypes.data_as(_i32p)
        p.link_strength = arr(ls, np.float64).ctypes.data_as(_f64p)
        p.linked_orb = arr(lo, np.int32).ctypes.data_as(_i32p)
        p.circuits = arr(circ, np.int32).ctypes.data_as(_i32p)
        p.n_circuits = len(circ) // 3
        p.corr_pair = arr(cp, np.int32).ctypes.data_as(_i32p)
        p.n_lat = len(cp) // 2
        p.group_list = arr(glist, np.int32).ctypes.data_as(_i32p)
        p.n_group, p.max_group = int(ngroup), int(maxg)
        p.r_orb = arr(rorb, np.int32).ctypes.data_as(_i32p)
        p.n_rorb = len(rorb)
        p.r_cluster = arr(rcl, np.int32).ctypes.data_as(_i32p)
        p.n_in_cluster = len(rcl) // max(1, len(rorb))
        p.r_link = arr(rlink, np.int32).ctypes.data_as(_i32p)
        p.flunc, p.h = float(flunc), float(h)
        p.ignore_offdiag = int(ign)
        p.spin_frames = int(frames)
        self.struct = p
        self.n_group = int(ngroup) if model != "ising" else 0
        self.nsweep = int(nsw)
        self.frames = int(frames)


def make_options(seed=1, schedule="auto", absolute_energy=False, recheck_every=0, record_series=False,
                 random_init=False, device=0) -> McsOptions:
    o = McsOptions()
    o.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    o.schedule = SCHEDULE_ID[schedule] if isinstance(schedule, str) else int(schedule)
    o.absolute_energy = int(bool(absolute_energy))
    o.recheck_every = int(recheck_every)
    o.record_series = int(bool(record_series))
    o.random_init = int(bool(random_init))
    o.device = int(device)
    return o


class _ResultBuf:
    def __init__(self, P: Problem, series: bool):
        G = P.n_group
        self.ng = (G + 1) ** 2 + (G + 1)
        self.groups = np.zeros(self.ng)
        # spin frames only when the problem asks for them (the buffer is N*3 floats per frame)
        self.frames = np.zeros(P.frames * P.N * 3, dtype=np.float32) if P.frames > 0 else None
        self.series = np.zeros(max(1, P.nsweep) * NSER) if series else None
        r = McsResult()
        r.group_values = self.groups.ctypes.data_as(_f64p)
        r.group_capacity = self.ng
        r.frames = self.frames.ctypes.data_as(_f32p) if P.frames > 0 else None
        r.series = self.series.ctypes.data_as(_f64p) if series else None
        self.r = r

    def unpack(self, P: Problem):
        r = self.r
        v = list(r.values)
        if P.model == "ising":
            out = tuple(v[:10]) + (0.0,)
        else:
            out = tuple(v[:27]) + (0.0, tuple(self.groups) if P.n_group > 0 else 0.0)
        extras = dict(site_updates=r.site_updates, clusters=r.clusters, flipped=r.flipped, accepted=r.accepted,
                      exact_mismatches=r.exact_mismatches, energy_drift=r.energy_drift, device_ms=r.device_ms,
                      schedule=SCHEDULE_NAME.get(r.schedule_used, str(r.schedule_used)), n_colours=r.n_colours,
                      frames_written=r.frames_written)
        if self.series is not None:
            extras["series"] = self.series.reshape(-1, NSER)[:P.nsweep].copy()
        if P.frames > 0:
            extras["frames"] = self.frames.reshape(P.frames, P.N, 3)[:r.frames_written].copy()
        return out, extras


def solve(model: str, args: tuple, seed: int = 1, schedule: str = "auto", record_series: bool = False,
          absolute_energy: bool = False, random_init: bool = False, recheck_every: int = 0, device: int = 0):
    """One solve through the C ABI; returns (reference result tuple, extras).
    ``args`` is the MCMainFunction tuple or a prebuilt Problem."""
    P = args if isinstance(args, Problem) else Problem(model, args)
    o = make_options(seed, schedule, absolute_energy, recheck_every, record_series, random_init, device)
    rb = _ResultBuf(P, record_series)
    _check(lib().mcs_solve(ctypes.byref(P.struct), ctypes.byref(o), ctypes.byref(rb.r)))
    return rb.unpack(P)


class Batch:
    """Many replicas (uneven sizes, models, temperatures) run together."""

    def __init__(self, device: int = 0):
        import threading
        self._h = ctypes.c_void_p()
        _check(lib().mcs_batch_create(device, ctypes.byref(self._h)))
        self._problems = []
        self._bufs = []
        self._lock = threading.Lock()

    def add(self, model: str, args, record_series: bool = False, **opt) -> int:
        """Add one replica from an MCMainFunction tuple or a prebuilt Problem.
        Safe to call from several threads (the engine compiles in parallel)."""
        P = args if isinstance(args, Problem) else Problem(model, args)
        o = make_options(record_series=record_series, **opt)
        idx = ctypes.c_int32()
        _check(lib().mcs_batch_add(self._h, ctypes.byref(P.struct), ctypes.byref(o), ctypes.byref(idx)))
        with self._lock:
            while len(self._problems) <= idx.value:
                self._problems.append(None)
                self._bufs.append(False)
            self._problems[idx.value] = P
            self._bufs[idx.value] = record_series
        return idx.value

    def run(self):
        _check(lib().mcs_batch_run(self._h))

    def prepare(self):
        _check(lib().mcs_batch_prepare(self._h))

    def advance(self, units: int) -> float:
        """Run every replica `units` more units; returns the device milliseconds."""
        ms = ctypes.c_double()
        _check(lib().mcs_batch_advance(self._h, int(units), ctypes.byref(ms)))
        return ms.value

    def result(self, i: int):
        P = self._problems[i]
        rb = _ResultBuf(P, self._bufs[i])
        _check(lib().mcs_batch_result(self._h, i, ctypes.byref(rb.r)))
        return rb.unpack(P)

    def stats(self):
        ms = ctypes.c_double()
        su = ctypes.c_int64()
        nl = ctypes.c_int32()
        _check(lib().mcs_batch_stats(self._h, ctypes.byref(ms), ctypes.byref(su), ctypes.byref(nl)))
        return {"device_ms": ms.value, "site_updates": su.value, "launches": nl.value}

    SCHEDULES = {1: "plain", 2: "resident", 3: "tiled", 4: "wolff_shared", 5: "wolff_global", 6: "cluster"}

    def schedules(self):
        """[(schedule name, CTAs per replica, threads per CTA, replicas)] per launch group
        (after prepare; a resident group's cluster size is the autotuner's
        choice once it has run)."""
        out = []
        g = 0
        while True:
            k, c, t, n = (ctypes.c_int32() for _ in range(4))
            if lib().mcs_batch_schedule(self._h, g, ctypes.byref(k), ctypes.byref(c), ctypes.byref(t),
                                        ctypes.byref(n)) != 0:
                return out
            name = self.SCHEDULES.get(k.value, str(k.value))
            if k.value == 2 and c.value >= 1:
                name = "cluster"  # a resident group the autotuner moved to the cluster kernel
            # c < 0: resident kernel with -c copies of each replica (one per CTA of a cluster)
            out.append((name, -c.value if c.value < 0 else max(1, c.value), t.value, n.value))
            g += 1

    def memory(self):
        dev = ctypes.c_uint64()
        rb = ctypes.c_uint64()
        _check(lib().mcs_batch_memory(self._h, ctypes.byref(dev), ctypes.byref(rb)))
        return {"device_bytes": dev.value, "readback_bytes": rb.value}

    def close(self):
        if self._h:
            lib().mcs_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ParallelTempering:
    """Replica exchange over a ladder of inverse temperatures.

    ``args`` is an MCMainFunction tuple whose couplings, anisotropy and field
    are PHYSICAL (build it at T = 1); ``betas[k]`` = 1/T_k.  Energies in the
    results are physical too."""

    def __init__(self, model: str, args, betas, seed: int = 1, device: int = 0, record_series: bool = False):
        self.P = args if isinstance(args, Problem) else Problem(model, args)
        self.nt = len(betas)
        self._betas = np.ascontiguousarray(betas, dtype=np.float64)
        self._series = record_series
        o = make_options(seed=seed, device=device, record_series=record_series)
        self._h = ctypes.c_void_p()
        _check(lib().mcs_pt_create(ctypes.byref(self.P.struct), ctypes.byref(o),
                                   self._betas.ctypes.data_as(_f64p), self.nt, ctypes.byref(self._h)))

    def run(self):
        _check(lib().mcs_pt_run(self._h))

    def result(self, k: int):
        rb = _ResultBuf(self.P, self._series)
        _check(lib().mcs_pt_result(self._h, k, ctypes.byref(rb.r)))
        return rb.unpack(self.P)

    def stats(self):
        acc = np.zeros(max(1, self.nt - 1))
        ms = ctypes.c_double()
        su = ctypes.c_int64()
        _check(lib().mcs_pt_stats(self._h, acc.ctypes.data_as(_f64p), ctypes.byref(ms), ctypes.byref(su)))
        return {"swap_acceptance": acc, "device_ms": ms.value, "site_updates": su.value}

    def close(self):
        if self._h:
            lib().mcs_pt_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop: submit solves as they arrive, call
    step() to let the device work, poll() for finished results."""

    def __init__(self, hbm_budget_bytes: int = 8 << 30, max_slots: int = 512, device: int = 0):
        self._h = ctypes.c_void_p()
        _check(lib().mcs_server_create(device, int(hbm_budget_bytes), int(max_slots), ctypes.byref(self._h)))
        self._problems = {}

    def submit(self, model: str, args, **opt) -> int:
        P = args if isinstance(args, Problem) else Problem(model, args)
        o = make_options(**opt)
        t = ctypes.c_uint64()
        _check(lib().mcs_server_submit(self._h, ctypes.byref(P.struct), ctypes.byref(o), ctypes.byref(t)))
        self._problems[t.value] = P
        return t.value

    def step(self) -> int:
        n = ctypes.c_int32()
        _check(lib().mcs_server_step(self._h, ctypes.byref(n)))
        return n.value

    def poll(self, ticket: int):
        """The result tuple and extras when done, else None.  A request that
        failed or was cancelled raises EngineError with its own status code
        (``code``: MCS_ECANCELLED, MCS_ENOMEM, MCS_ECUDA, ...) and is released."""
        P = self._problems.get(ticket)
        rb = _ResultBuf(P, False) if P is not None else None
        if rb is not None:
            rb.r.frames = None
        rc = lib().mcs_server_poll(self._h, ticket, ctypes.byref(rb.r) if rb is not None else None)
        if rc == 1:
            return None
        if rc != 0:
            self._problems.pop(ticket, None)
            _check(rc)
        del self._problems[ticket]
        P.frames = 0
        return rb.unpack(P)

    def cancel(self, ticket: int) -> None:
        """Cancel a queued or active request; its poll then raises with
        code MCS_ECANCELLED (a finished request keeps its result)."""
        _check(lib().mcs_server_cancel(self._h, ticket))

    def stats(self):
        a = ctypes.c_int32()
        q = ctypes.c_int32()
        b = ctypes.c_uint64()
        su = ctypes.c_int64()
        _check(lib().mcs_server_stats(self._h, ctypes.byref(a), ctypes.byref(q), ctypes.byref(b), ctypes.byref(su)))
        return {"active": a.value, "queued": q.value, "bytes_in_use": b.value, "site_updates": su.value}

    def close(self):
        if self._h:
            lib().mcs_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
