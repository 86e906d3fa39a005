#!/usr/bin/env python
"""Benchmark of the batched Monte Carlo engine on one GB300.

Workload (the headline configuration): 2D square-lattice isotropic XY model,
J = 1 K ferromagnetic (mcsolver sign convention Jxx = Jyy = -1), no
anisotropy, L = 128 periodic (16384 sites), FP32 unit vectors with angles
uniform in [0, 2pi) from the seed, Metropolis with one sweep per measurement
(tau = N), 32 temperatures linear in 0.5..1.5 K, FP64 moment accumulators.
All 32 replicas run in one batch.  A "step" is STEP_SWEEPS sweeps of every
replica, each sweep followed by the full measurement of the reference.

Metric: site updates per second (one Metropolis trial on one site = 1).
* value: device time of the steps with the lattices already on the device
  (L2 flushed between steps by writing a 256 MB buffer);
* e2e:   the same work through the C ABI from host buffers: batch creation,
  model compile and upload, the sweeps, and the read-back of every result;
* cpu_baseline / --impl reference: the oracle's restatement of the reference
  CPU library (bit-identical to it on the same random stream), one process
  per host core, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L = 128
NTEMP = 32
TEMPS = [0.5 + k * (1.5 - 0.5) / (NTEMP - 1) for k in range(NTEMP)]
STEP_SWEEPS = 50
WORKLOAD = "xy_square_L128_32T_metropolis"


def base_config(sweeps):
    """The workload both arms of the benchmark report."""
    return {"workload": WORKLOAD, "model": "XY", "L": L, "n_temperatures": NTEMP, "T_range_K": [0.5, 1.5],
            "algorithm": "Metropolis", "sweeps_per_step": sweeps, "measurement": "every sweep (tau=N)",
            "replicas": NTEMP}


def workload_args(nsweep, nthermal=0):
    from mcsolver_gb300.lattice import rescale_args, square_args
    base = square_args("xy", L, 1.0, nthermal=nthermal, nsweep=nsweep, tau=0, groups=((0,),))
    return [rescale_args("xy", base, T) for T in TEMPS]


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.p = None
        self.path = os.path.join(tempfile.gettempdir(), "mcsgpu_bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def l2_flush():
    import torch
    global _flushbuf
    try:
        _flushbuf
    except NameError:
        _flushbuf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    _flushbuf.zero_()
    torch.cuda.synchronize()


# ---------------------------------------------------------------- CPU baseline
def _cpu_one(job):
    model, args, seed = job
    from oracle import oracle as orc
    t = time.time()
    orc.solve(model, args, seed=seed, mode=0)
    return time.time() - t


def _cpu_warm(_):
    from oracle import oracle as orc
    orc.lib()
    return os.getpid()


class CpuPool:
    """The reference's fan-out (win.startSimulation: one process per host
    core, one (T, H) point per task) over the oracle's reference-stream
    restatement of the compiled library (bit-identical to it).  The pool is
    started and its workers load the library before any timing."""

    def __init__(self):
        from oracle import oracle as orc
        orc.build()
        self.cores = os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(processes=self.cores)
        self.pool.map(_cpu_warm, range(self.cores))
        cal = workload_args(nsweep=4)[0]
        orc.lib()
        t0 = time.time()
        orc.solve("xy", cal, seed=1, mode=0)
        self.per_sweep = max(1e-4, (time.time() - t0) / 4)

    def sweeps_for(self, seconds):
        return max(4, int(seconds * self.cores / (NTEMP * self.per_sweep)))

    def run(self, sweeps, seed0=1):
        jobs = [("xy", a, seed0 + k) for k, a in enumerate(workload_args(nsweep=sweeps))]
        t = time.time()
        self.pool.map(_cpu_one, jobs, chunksize=1)
        return time.time() - t

    def close(self):
        self.pool.close()
        self.pool.join()


def build_marshal_seconds(points=2):
    """Host time to build and marshal one (T, H) point of the workload the way
    the reference's caller does (Lattice.establishLattice / establishLinking
    site by site, then the flattened tuples of mcMain.mainLoopViaCLib_On), by
    this package's per-site restatement of that code (lattice.square_args)."""
    from mcsolver_gb300.lattice import square_args
    t = time.time()
    for k in range(points):
        square_args("xy", L, TEMPS[k], nthermal=0, nsweep=10, tau=0, groups=((0,),))
    return (time.time() - t) / points


def cpu_baseline(target_s=15.0):
    """Solve-only throughput of the reference's CPU path on every host core,
    and the same with the reference caller's model build and marshalling of
    each point added (done per point inside each pool worker)."""
    cp = CpuPool()
    try:
        sweeps = cp.sweeps_for(target_s)
        wall = cp.run(sweeps)
    finally:
        cp.close()
    updates = NTEMP * sweeps * L * L
    bm = build_marshal_seconds()
    wall_b = wall + bm * math.ceil(NTEMP / cp.cores)
    return {"value": updates / wall, "unit": "site_updates/s", "cores": cp.cores, "kind": "port",
            "sample": "%d temperatures x %d sweeps (tau=N, measurement every sweep) of XY L=%d on %d processes, "
                      "%s %s" % (NTEMP, sweeps, L, cp.cores, platform.machine(), platform.processor() or ""),
            "wall_s": wall,
            "with_build": {"value": updates / wall_b, "unit": "site_updates/s", "wall_s": wall_b,
                           "build_marshal_s_per_point": bm,
                           "note": "model build + tuple marshalling per (T, H) point as the reference caller does "
                                   "it (Lattice.py:155-284, mcMain.py:137-248), timed by this package's per-site "
                                   "restatement of that code; one point per worker process at a time"}}


# ---------------------------------------------------------------- our arm
def run_ours(args):
    import numpy as np

    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    b.build()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        peaks = {"hbm_gbs": 6800.0}
    hbm = peaks.get("hbm_gbs", 6800.0)
    K, W, S = args.steps, args.warmup, args.sweeps
    total_sweeps = (W + K) * S + 1
    prob_args = workload_args(nsweep=total_sweeps)
    batch = eng.Batch(device=0)
    for k, a in enumerate(prob_args):
        batch.add("xy", a, seed=1000 + k, random_init=True, schedule=args.schedule)
    batch.prepare()
    for _ in range(W):
        batch.advance(S)
    l0 = batch.stats()["launches"]
    times = []
    with ClockSampler() as clk:
        wall0 = time.time()
        for _ in range(K):
            l2_flush()
            times.append(batch.advance(S))
        wall = time.time() - wall0
    launches = batch.stats()["launches"] - l0
    sched = batch.schedules()
    batch.close()
    per_step_updates = NTEMP * L * L * S
    dev_s = sum(times) / 1000.0
    value = per_step_updates * K / dev_s
    ms_per_step = sum(times) / K
    # roofline of the Metropolis kernel the autotuner chose (one launch per step)
    kname = {"cluster": "k_cluster_metro<2,%d>" % sched[0][2], "tiled": "k_tiled_sweep<2,SQUARE>"}.get(
        sched[0][0], "k_resident_metro<2,SQUARE>")
    prof = kernel_profile(kname)
    # e2e through the C ABI from host buffers
    # the step's inputs are host arrays in the reference's flattened layout
    e2e_args = workload_args(nsweep=S)
    problems = [eng.Problem("xy", a) for a in e2e_args]
    e2e_t = []
    h2d = d2h = 0
    from concurrent.futures import ThreadPoolExecutor
    pool = ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
    for it in range(max(3, min(K, 6))):
        t = time.time()
        bb = eng.Batch(device=0)
        list(pool.map(lambda kp: bb.add("xy", kp[1], seed=2000 + kp[0], random_init=True), enumerate(problems)))
        bb.run()
        outs = [bb.result(i) for i in range(NTEMP)]
        e2e_t.append(time.time() - t)
        mem = bb.memory()
        h2d, d2h = mem["device_bytes"], mem["readback_bytes"]
        bb.close()
    pool.shutdown()
    del outs, problems
    e2e_s = statistics.median(e2e_t[1:]) if len(e2e_t) > 1 else e2e_t[0]
    e2e_value = per_step_updates / e2e_s
    # plain engine (one solve per launch sequence, host-driven sweeps) on a sample
    plain = None
    if not args.no_plain:
        t_plain = []
        for k, a in enumerate(e2e_args[:4]):
            r, ex = eng.solve("xy", a, seed=3000 + k, schedule="plain", random_init=True)
            t_plain.append(ex["device_ms"])
        plain_v = (L * L * S) / (statistics.mean(t_plain) / 1000.0)
        plain = {"value": plain_v, "unit": "site_updates/s", "sample": "4 of the 32 replicas, one solve per launch "
                 "sequence (one launch per colour, per measurement and per finalize, no graph)",
                 "batched_over_plain": value / plain_v}
    clocks = clk.summary()
    roof = roofline(per_step_updates, ms_per_step, hbm, prof, clocks, kname)
    cpu = cpu_baseline(args.cpu_seconds) if not args.no_cpu else None
    # the served half of the metric (after the timed region): continuous batching
    # of a Poisson request stream, p50/p99 latency and the gain over the plain engine
    served = served_stream(args) if not args.no_served else None
    # the other configurations, each run whole (after the timed region)
    configs = None
    if not args.no_configs:
        configs = {"ising_square_L32_16T_metropolis": run_whole_solves(args, "ising", plain_sample=4),
                   "xy_square_L128_32T_wolff": run_whole_solves(args, "xy_wolff", plain_sample=2),
                   "pt_honeycomb_heisenberg_64x64_64T": run_pt(args),
                   "batched_heisenberg_dmi_256_uneven": run_batched4(args)}
    line = {
        "metric": "site_updates_per_s", "value": value, "unit": "site_updates/s", "n_gpus": 1, "steps": K,
        "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 update / f64 accumulate", "data": "synthetic",
        "config": dict(base_config(S), l2="flushed between steps (256 MB write)",
                       schedule=[{"schedule": g[0], "ctas_per_replica": g[1], "threads": g[2], "replicas": g[3]}
                                 for g in sched]),
        "e2e": {"value": e2e_value, "unit": "site_updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "C ABI mcs_batch_* from host arrays: create, compile+upload 32 replicas (16 host threads, "
                        "pinned staging), run, read every result back"},
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cpu,
        "plain_engine": plain,
        "served": served,
        "configs": configs,
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    print(json.dumps(line))


KERNEL_SOURCES = ("mcs_cluster.cu", "mcs_device.cuh", "mcs_internal.h")


def kernel_sources_sha():
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "mcsolver_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def kernel_profile(kname):
    """The ncu figures of the headline kernel configuration the autotuner
    chose (profiles/traffic.json holds each configuration it picks for this
    workload): warp instructions per site update and DRAM bytes per site
    update of one captured launch, with the hash of the kernel sources they
    were taken on."""
    try:
        tj = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except Exception:
        return None
    prof = dict(tj.get("kernels", {}).get(kname) or {})
    if not prof:
        return None
    prof["stale"] = tj.get("sources_sha") != kernel_sources_sha()
    return prof


def roofline(updates, ms, hbm, prof, clocks, kname):
    """The bound of the headline kernel is SM instruction issue: its lattice
    stays in shared memory for a whole launch, so DRAM carries about 1 % of
    the algorithmic bytes.  frac = issue-slot utilisation of this run: the
    kernel's warp instructions (ncu count per site update, from the profile
    of the same sources) over the issue slots of the measured launch time
    (152 SMs x 4 schedulers x the SM clock sampled during the timed steps).
    The HBM reading (algorithmic bytes: 16 B per XY site update, the FP32
    (x, y) pair read and written once per sweep) is given beside it."""
    alg = 16.0 * updates
    achieved = alg / (ms / 1000.0) / 1e9
    hb = {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "algorithmic_bytes": alg,
          "traffic": (prof["dram_bytes_per_site_update"] * updates) if prof else None,
          "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)"}
    out = {"bound": "sm_issue", "kernel": kname, "hbm": hb, "traffic": hb["traffic"]}
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    if prof:
        slots = (ms / 1000.0) * 152 * 4 * mhz * 1e6
        used = prof["warp_instructions_per_site_update"] * updates
        out.update({"achieved": used / slots, "peak": 1.0, "unit": "issue slots (fraction)", "frac": used / slots,
                    "warp_instructions_per_site_update": prof["warp_instructions_per_site_update"],
                    "ncu_issue_active": prof.get("sm_issue_active"), "profile_stale": prof["stale"]})
    else:
        out.update({"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                    "note": "no profile of this kernel: HBM reading only"})
    return out


def run_reference(args):
    """The reference's CPU path (the oracle's restatement of the compiled
    library, bit-identical to it, fanned out over every host core as
    win.startSimulation does) on the headline workload.  The process pool is
    started once, before the timed steps; each step is one bounded sample:
    every temperature for the same number of sweeps."""
    K, W = args.steps, args.warmup
    cp = CpuPool()
    try:
        sweeps = cp.sweeps_for(max(1.0, args.cpu_step_seconds))
        vals = []
        for i in range(W + K):
            wall = cp.run(sweeps, seed0=1 + 100 * i)
            if i >= W:
                vals.append(NTEMP * sweeps * L * L / wall)
    finally:
        cp.close()
    v = statistics.median(vals)
    sample = "%d temperatures x %d sweeps per step (tau=N, measurement every sweep) of XY L=%d on %d processes, " \
             "%s %s" % (NTEMP, sweeps, L, cp.cores, platform.machine(), platform.processor() or "")
    line = {"impl": "reference", "metric": "site_updates_per_s", "value": v, "unit": "site_updates/s", "n_gpus": 1,
            "steps": K, "warmup": W, "ms_per_step": NTEMP * sweeps * L * L / v * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": base_config(args.sweeps),
            "cpu_baseline": {"value": v, "unit": "site_updates/s", "cores": cp.cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "site_updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- other configurations
def _plain_rate(eng, model, args, seed):
    r, ex = eng.solve(model, args, seed=seed, schedule="plain", random_init=True)
    return ex["site_updates"], ex["device_ms"] / 1000.0


def run_served(args):
    print(json.dumps(served_stream(args)))


def served_stream(args):
    """Served stream: Poisson arrivals (mean 200 req/s, seeded) of mixed
    Ising / XY / Heisenberg (DMI, field) square-lattice solves, L log-uniform in
    32..512 (even), random (T, H) in each model's range, nthermal / nsweep as
    given.  The client marshals each request's arrays before the run (as
    mcsolver builds its tuples); inside the timed run a dispatcher submits each
    request at its arrival time to a pool of submit threads (host compile runs
    there, beside the device work), and the main thread steps the server and
    polls.  Latency = completion - arrival."""
    import queue
    import threading
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np

    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    from mcsolver_gb300.lattice import square_args_fast
    b.build()
    rng = np.random.default_rng(5)
    n = args.requests
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=n))
    reqs = []
    for k in range(n):
        model = ["ising", "xy", "heisenberg"][rng.integers(3)]
        L = int(round(math.exp(rng.uniform(math.log(32), math.log(512)))))
        L += L % 2
        if model == "ising":
            T, H = rng.uniform(1.5, 3.5), 0.0
            a = square_args_fast("ising", L, T, nthermal=args.nthermal, nsweep=args.nsweep, arrays=True)
        elif model == "xy":
            T, H = rng.uniform(0.5, 1.5), 0.0
            a = square_args_fast("xy", L, T, nthermal=args.nthermal, nsweep=args.nsweep, arrays=True)
        else:
            T, H = rng.uniform(0.05, 1.0), rng.uniform(0.0, 0.6)
            a = square_args_fast("heisenberg", L, T, h=H, dmi=0.4, nthermal=args.nthermal, nsweep=args.nsweep,
                                 arrays=True)
        reqs.append((model, eng.Problem(model, a), L))
    srv = eng.Server(hbm_budget_bytes=64 << 30, max_slots=4096)
    submitted = queue.Queue()
    pool = ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1))

    def submit(k, t_arr):
        model, P, L = reqs[k]
        submitted.put((srv.submit(model, P, seed=7000 + k, random_init=True), t_arr, k))

    def dispatch(t0):
        for k in range(n):
            d = t0 + arrivals[k] - time.time()
            if d > 0:
                time.sleep(d)
            pool.submit(submit, k, t0 + arrivals[k])

    lat, upd, pending, lat_of = [], 0, {}, {}
    t0 = time.time()
    th = threading.Thread(target=dispatch, args=(t0,))
    th.start()
    finished = 0
    while finished < n:
        while True:
            try:
                t, ta, k = submitted.get_nowait()
            except queue.Empty:
                break
            pending[t] = (ta, k)
        if not pending:
            time.sleep(0.0005)
            continue
        srv.step()
        now = time.time()
        for t in list(pending):
            r = srv.poll(t)
            if r is not None:
                ta, k = pending.pop(t)
                lat.append(now - ta)
                lat_of[k] = now - ta
                upd += r[1]["site_updates"]
                finished += 1
    makespan = time.time() - t0
    th.join()
    pool.shutdown()
    srv.close()
    # the plain engine (one solve at a time, host-driven launches per sweep) on a seeded sample
    pick = rng.choice(n, size=min(args.plain_sample, n), replace=False)
    ps, pt = 0, 0.0
    for k in pick:
        model, P, L = reqs[k]
        u, s = _plain_rate(eng, model, P, 7000 + int(k))
        ps += u
        pt += s
    # the same requests alone: each through a server of its own, submit to result
    alone = {}
    if not args.no_alone:
        for k in range(n):
            model, P, Lk = reqs[k]
            s1 = eng.Server(hbm_budget_bytes=64 << 30, max_slots=4)
            t1 = time.time()
            tk = s1.submit(model, P, seed=7000 + k, random_init=True)
            while s1.poll(tk) is None:
                s1.step()
            alone[k] = time.time() - t1
            s1.close()
    lat = np.array(lat)
    Ls = np.array([r[2] for r in reqs])
    sizes = np.array([r[2] ** 2 * (1 if r[0] != "heisenberg" else 1) for r in reqs], float)
    order = np.argsort(sizes, kind="stable")
    terciles = []
    for j, part in enumerate(np.array_split(order, 3)):
        lm = np.array([lat_of[k] for k in part])
        row = {"tercile": ["small", "medium", "large"][j], "L_range": [int(Ls[part].min()), int(Ls[part].max())],
               "requests": int(len(part)), "latency_p50_s": float(np.percentile(lm, 50)),
               "latency_p99_s": float(np.percentile(lm, 99))}
        if alone:
            la = np.array([alone[k] for k in part])
            row.update({"alone_p50_s": float(np.percentile(la, 50)), "alone_p99_s": float(np.percentile(la, 99))})
        terciles.append(row)
    return {"workload": "served_stream", "requests": n, "rate_req_s": args.rate,
            "nthermal": args.nthermal, "nsweep": args.nsweep,
            "L_range": [int(Ls.min()), int(Ls.max())], "site_updates": int(upd),
            "makespan_s": makespan, "last_arrival_s": float(arrivals[-1]),
            "solves_per_s": n / makespan, "site_updates_per_s": upd / makespan,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "plain_site_updates_per_s": ps / pt if pt > 0 else None,
            "served_over_plain": (upd / makespan) / (ps / pt) if pt > 0 else None,
            "plain_sample": [int(Ls[k]) for k in pick],
            "by_size": terciles,
            "note": "latency = completion - arrival; by_size: requests split by lattice sites into terciles, with "
                    "the same requests' latency alone (each through a server of its own: compile, upload, run, "
                    "result)"}


def run_batched4(args):
    """Batched grid: square Heisenberg with DMI (0.4 |J|, J = -1) and field,
    16 temperatures 0.05..1.0 (clamped to 0.1 as mcMain does) x 16 fields
    0..0.6 = 256 replicas of uneven sizes L in {64, 96, 128, 192, 256}, two
    circuits per cell, all in one launch sequence."""
    import numpy as np

    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    from mcsolver_gb300.lattice import rescale_args, square_args_fast
    b.build()
    sizes = [64, 96, 128, 192, 256]
    base = {L: square_args_fast("heisenberg", L, 1.0, dmi=0.4, nthermal=args.nthermal, nsweep=args.nsweep, arrays=True)
            for L in sizes}
    Ts = np.linspace(0.05, 1.0, 16)
    Hs = np.linspace(0.0, 0.6, 16)
    bt = eng.Batch()
    k = 0
    total = 0
    jobs = []
    for iT, T in enumerate(Ts):
        for iH, H in enumerate(Hs):
            L = sizes[k % len(sizes)]
            jobs.append((L, rescale_args("heisenberg", base[L], T, h=H)))
            k += 1
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as pool:
        list(pool.map(lambda kj: bt.add("heisenberg", kj[1][1], seed=11 + kj[0], random_init=True), enumerate(jobs)))
    for L, a in jobs:
        total += L * L * (args.nthermal + args.nsweep)
    bt.prepare()
    t = time.time()
    bt.run()
    wall = time.time() - t
    st = bt.stats()
    bt.close()
    u, s = _plain_rate(eng, "heisenberg", jobs[2][1], 99)
    return {"workload": "batched_heisenberg_dmi_256_uneven", "replicas": len(jobs), "sizes": sizes,
                      "nthermal": args.nthermal, "nsweep": args.nsweep, "site_updates": st["site_updates"],
                      "device_ms": st["device_ms"], "wall_s": wall,
                      "site_updates_per_s": st["site_updates"] / (st["device_ms"] / 1000.0),
                      "plain_site_updates_per_s_L128": u / s,
                      "batched_over_plain": (st["site_updates"] / (st["device_ms"] / 1000.0)) / (u / s)}


def run_whole_solves(args, workload=None, plain_sample=None):
    """Whole solves of one (model, lattice) over a temperature grid, all
    temperatures in one batch, against the plain engine on a sample.
    * ising:    square Ising ferromagnet (Jxx = -1), L = 32, h = 0, 16
                temperatures 1.5..3.5, Metropolis, tau = N, nthermal 2000,
                nsweep 10000 (the reference's CPU-runnable case);
    * xy_wolff: square XY (Jxx = Jyy = -1), L = 128, 32 temperatures 0.5..1.5,
                Wolff single-cluster updates, one cluster per measurement,
                nthermal 5000, nsweep 20000.
    Site updates: one Metropolis trial = 1; Wolff counts the flipped sites
    (cluster sizes) and also reports clusters/s.  `wall_s` is end to end through
    the C ABI from host arrays (batch creation, compile, upload, run, results)."""
    from concurrent.futures import ThreadPoolExecutor

    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    from mcsolver_gb300.lattice import rescale_args, square_args_fast
    b.build()
    workload = workload or args.workload
    nplain = args.plain_sample if plain_sample is None else plain_sample
    if workload == "ising":
        model, Lw, Ts, algo, tau = "ising", 32, [1.5 + k * 2.0 / 15 for k in range(16)], 0, 0
        nth, nsw = (args.nthermal, args.nsweep) if args.override_sweeps else (2000, 10000)
    else:
        model, Lw, Ts, algo, tau = "xy", 128, [0.5 + k * 1.0 / 31 for k in range(32)], 1, 1
        nth, nsw = (args.nthermal, args.nsweep) if args.override_sweeps else (5000, 20000)
    base = square_args_fast(model, Lw, 1.0, nthermal=nth, nsweep=nsw, tau=tau, algo=algo, arrays=True)
    jobs = [rescale_args(model, base, T) for T in Ts]
    t0 = time.time()
    bt = eng.Batch()
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as pool:
        list(pool.map(lambda kj: bt.add(model, kj[1], seed=21 + kj[0], random_init=True), enumerate(jobs)))
    bt.run()
    res = [bt.result(i) for i in range(len(jobs))]
    wall = time.time() - t0
    st = bt.stats()
    sched = bt.schedules()
    bt.close()
    clusters = sum(r[1]["clusters"] for r in res)
    mism = sum(r[1]["exact_mismatches"] for r in res)
    ps, pt = 0, 0.0
    for k in range(nplain):
        u, s = _plain_rate(eng, model, jobs[(k * 7) % len(jobs)], 99 + k)
        ps += u
        pt += s
    rate = st["site_updates"] / (st["device_ms"] / 1000.0)
    return {"workload": "%s_square_L%d_%dT_%s" % (model, Lw, len(Ts), "wolff" if algo else "metropolis"),
                      "replicas": len(jobs), "nthermal": nth, "nsweep": nsw, "site_updates": st["site_updates"],
                      "clusters": clusters if algo else None, "device_ms": st["device_ms"], "wall_s_e2e": wall,
                      "site_updates_per_s": rate, "e2e_site_updates_per_s": st["site_updates"] / wall,
                      "clusters_per_s": clusters / (st["device_ms"] / 1000.0) if algo else None,
                      "exact_mismatches": mism if model == "ising" else None,
                      "schedule": [{"schedule": g[0], "ctas_per_replica": g[1], "threads": g[2], "replicas": g[3]}
                                   for g in sched],
                      "plain_site_updates_per_s": ps / pt if pt > 0 else None,
                      "batched_over_plain": rate / (ps / pt) if pt > 0 else None}


def run_many_small(args):
    """Many small replicas: 1024 square Ising ferromagnets, L = 32, h = 0,
    temperatures spread over 1.5..3.5 K, Metropolis, tau = N, 200 + 1000
    sweeps, in one batch.  Timed three ways: with the autotuner's choice among
    its candidates for the group (one 128-thread CTA per replica, one warp per
    replica, copies over a cluster), and pinned to one CTA of 128 threads and
    to one warp per replica.  Device time of the whole run."""
    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    from mcsolver_gb300.lattice import rescale_args, square_args_fast
    b.build()
    n, Lw, nth, nsw = 1024, 32, 200, 1000
    base = square_args_fast("ising", Lw, 1.0, nthermal=nth, nsweep=nsw, arrays=True)
    jobs = [rescale_args("ising", base, 1.5 + 2.0 * k / (n - 1)) for k in range(n)]
    out = {"workload": "ising_square_L32_1024_replicas", "replicas": n, "nthermal": nth, "nsweep": nsw}
    for label, force in (("autotuned", None), ("cta128_per_replica", "0:128"), ("warp_per_replica", "0:32")):
        if force:
            os.environ["MCSGPU_FORCE"] = force
        else:
            os.environ.pop("MCSGPU_FORCE", None)
        bt = eng.Batch()
        for k, a in enumerate(jobs):
            bt.add("ising", a, seed=40000 + k, random_init=True)
        bt.prepare()
        bt.run()
        st = bt.stats()
        sched = bt.schedules()
        bt.close()
        out[label] = {"site_updates_per_s": st["site_updates"] / (st["device_ms"] / 1000.0), "device_ms": st["device_ms"],
                      "schedule": [{"schedule": g[0], "ctas_per_replica": g[1], "threads": g[2], "replicas": g[3]}
                                   for g in sched]}
    os.environ.pop("MCSGPU_FORCE", None)
    return out


def run_noalloc(args):
    """The allocation-free entry point mcs_ising_square_noalloc on caller-held
    device buffers: square Ising ferromagnet (K = -1/T, T = 2.3), L x L int8
    spins from a seeded random start, `--sweeps` sweeps per step (two colour
    launches and one sums launch per sweep).  Device time with CUDA events on
    the stream the entry point is given.  Algorithmic bytes: the int8 spin read
    and written once per site update (2 B); at L = 2048 (4 MB) the lattice
    lives in L2."""
    import ctypes

    import torch

    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    b.build()
    Ln, S, K, W = args.noalloc_L, args.sweeps, args.steps, args.warmup
    g = torch.Generator(device="cuda").manual_seed(5)
    sigma = (torch.randint(0, 2, (Ln * Ln,), generator=g, device="cuda", dtype=torch.int8) * 2 - 1).contiguous()
    sums = torch.zeros(2 * S, dtype=torch.int64, device="cuda")
    fn = eng.lib().mcs_ising_square_noalloc
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    T = 2.3
    sweep = 0
    for _ in range(W):
        assert fn(ctypes.c_void_p(sigma.data_ptr()), Ln, Ln, -1.0 / T, 0.0, 7, sweep, S,
                  ctypes.c_void_p(sums.data_ptr()), sp) == 0, eng.lib().mcs_last_error()
        sweep += S
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(K):
        fn(ctypes.c_void_p(sigma.data_ptr()), Ln, Ln, -1.0 / T, 0.0, 7, sweep, S, ctypes.c_void_p(sums.data_ptr()), sp)
        sweep += S
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    upd = Ln * Ln * S
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    gbs = 2.0 * upd / (ms / 1000.0) / 1e9
    m = sums.cpu().numpy().reshape(-1, 2)[-1]
    print(json.dumps({"workload": "ising_square_noalloc_L%d" % Ln, "sweeps_per_step": S, "steps": K,
                      "ms_per_step": ms, "site_updates_per_s": upd / (ms / 1000.0),
                      "launches_per_step": 3 * S, "last_sums": [int(m[0]), int(m[1])],
                      "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                                   "note": "2 B per site update; the %d MB lattice stays in L2" % (Ln * Ln >> 20)}}))


def run_pt(args):
    """Parallel tempering: honeycomb Heisenberg (2 sites/cell), 1NN Kitaev-type
    J = diag(-1.5,-1.5,-1.8) with Jxy = Jyx = 0.3, 2NN -0.3, Az = -0.5, 64x64
    cells, 64 replicas at geometric temperatures 5..50 K, exchange every sweep."""
    import numpy as np

    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    from mcsolver_gb300.lattice import honeycomb_args
    b.build()
    nth = args.pt_sweeps // 5
    phys = honeycomb_args("heisenberg", 64, 1.0, nthermal=nth, nsweep=args.pt_sweeps - nth)
    betas = 1.0 / np.geomspace(5.0, 50.0, 64)
    pt = eng.ParallelTempering("heisenberg", phys, betas, seed=3)
    t = time.time()
    pt.run()
    wall = time.time() - t
    st = pt.stats()
    pt.close()
    rate = st["site_updates"] / (st["device_ms"] / 1000.0)
    # the plain engine: one temperature per solve (the reference runs every
    # temperature on its own, win.py:440-444), host-driven launches, on a sample
    plain = None
    if args.plain_sample > 0:
        ps, ptime = 0, 0.0
        for k, T in enumerate((5.0, 15.0)):
            u, sec = _plain_rate(eng, "heisenberg", honeycomb_args("heisenberg", 64, T, nthermal=100, nsweep=400), 50 + k)
            ps += u
            ptime += sec
        plain = ps / ptime
    return {"workload": "pt_honeycomb_heisenberg_64x64_64T", "replicas": 64,
                      "sweeps": args.pt_sweeps, "site_updates": st["site_updates"],
                      "device_ms": st["device_ms"], "wall_s": wall,
                      "site_updates_per_s": st["site_updates"] / (st["device_ms"] / 1000.0),
                      "swap_acceptance_min": float(np.min(st["swap_acceptance"])),
                      "swap_acceptance_max": float(np.max(st["swap_acceptance"])),
                      "plain_site_updates_per_s": plain, "batched_over_plain": rate / plain if plain else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sweeps", type=int, default=STEP_SWEEPS)
    ap.add_argument("--schedule", default="auto", choices=["auto", "resident", "tiled"],
                    help="headline workload: schedule of the replicas (auto = autotuner and load balancer)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="cpu_baseline sample (seconds of CPU work)")
    ap.add_argument("--cpu-step-seconds", type=float, default=4.0,
                    help="--impl reference: seconds of CPU work per timed step")
    ap.add_argument("--no-configs", action="store_true",
                    help="headline: skip the other configurations (Ising L=32, XY Wolff, PT, uneven DMI batch)")
    ap.add_argument("--no-alone", action="store_true", help="served: skip the requests' latency alone")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-served", action="store_true", help="headline: skip the served-stream part of the line")
    ap.add_argument("--workload", default="headline", choices=["headline", "served", "batched4", "pt", "ising", "xy_wolff",
                                                                  "noalloc", "many_small"])
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--nthermal", type=int, default=1000)
    ap.add_argument("--nsweep", type=int, default=5000)
    ap.add_argument("--override-sweeps", action="store_true",
                    help="ising / xy_wolff: use --nthermal / --nsweep instead of the workload's own counts")
    ap.add_argument("--plain-sample", type=int, default=6)
    ap.add_argument("--pt-sweeps", type=int, default=50000)
    ap.add_argument("--noalloc-L", type=int, default=2048, help="noalloc workload: lattice side")
    args = ap.parse_args()
    if args.workload == "served":
        return run_served(args)
    if args.workload == "batched4":
        return print(json.dumps(run_batched4(args)))
    if args.workload == "pt":
        return print(json.dumps(run_pt(args)))
    if args.workload in ("ising", "xy_wolff"):
        return print(json.dumps(run_whole_solves(args)))
    if args.workload == "noalloc":
        return run_noalloc(args)
    if args.workload == "many_small":
        return print(json.dumps(run_many_small(args)))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.gpus > 1 or int(os.environ.get("WORLD_SIZE", "1")) > 1:
        run_multi(args)
        return
    run_ours(args)


def replica_seeds(rank: int, n: int):
    """Philox keys of the n replicas of rank `rank`: disjoint across ranks."""
    return [1000 + 100000 * rank + k for k in range(n)]


def combine_ranks(t_local: float, work_local: float, dist, device):
    """Slowest rank's time and the summed work of all ranks (replicas only:
    nothing else crosses ranks)."""
    import torch
    tt = torch.tensor([t_local], dtype=torch.float64, device=device)
    ww = torch.tensor([work_local], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    dist.all_reduce(ww, op=dist.ReduceOp.SUM)
    return tt.item(), ww.item()


def multi_line(work_total: float, tmax: float, n: int, K: int, W: int, S: int, launches: int, clocks=None,
               e2e=None):
    return {"metric": "site_updates_per_s", "value": work_total / tmax, "unit": "site_updates/s",
            "n_gpus": n, "steps": K, "warmup": W, "ms_per_step": tmax * 1000 / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 update / f64 accumulate", "data": "synthetic", "gpu_launches": launches,
            "config": dict(base_config(S), parallelism="replicas only (%d independent copies)" % n,
                           l2="flushed between steps (256 MB write)"),
            "clocks": clocks, "e2e": e2e}


def run_multi(args):
    """Replicas only: every rank runs the full workload on its own GPU; value
    sums the ranks' work over the slowest rank's time."""
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    import mcsolver_gb300 as eng
    from mcsolver_gb300 import build as b
    if local == 0:
        b.build()
    dist.barrier()
    K, W, S = args.steps, args.warmup, args.sweeps
    batch = eng.Batch(device=local)
    seeds = replica_seeds(dist.get_rank(), NTEMP)
    for k, a in enumerate(workload_args(nsweep=(W + K) * S + 1)):
        batch.add("xy", a, seed=seeds[k], random_init=True)
    batch.prepare()
    for _ in range(W):
        batch.advance(S)
    l0 = batch.stats()["launches"]
    dist.barrier()
    torch.cuda.synchronize()
    t = 0.0
    with ClockSampler(local) as clk:
        for _ in range(K):
            l2_flush()
            t += batch.advance(S) / 1000.0
    torch.cuda.synchronize()
    launches = batch.stats()["launches"] - l0
    batch.close()
    tmax, work = combine_ranks(t, float(NTEMP * L * L * S * K), dist, "cuda")
    # end to end on every rank: create, compile + upload, run, read back, from host arrays
    problems = [eng.Problem("xy", a) for a in workload_args(nsweep=S)]
    dist.barrier()
    te = time.time()
    bb = eng.Batch(device=local)
    for k, P in enumerate(problems):
        bb.add("xy", P, seed=seeds[k] + 50000, random_init=True)
    bb.run()
    for i in range(NTEMP):
        bb.result(i)
    te = time.time() - te
    mem = bb.memory()
    bb.close()
    temax, _ = combine_ranks(te, 0.0, dist, "cuda")
    e2e = {"value": NTEMP * L * L * S * dist.get_world_size() / temax, "unit": "site_updates/s",
           "h2d_bytes_per_step": mem["device_bytes"] * dist.get_world_size(),
           "d2h_bytes_per_step": mem["readback_bytes"] * dist.get_world_size(),
           "path": "C ABI mcs_batch_* from host arrays on every rank (slowest rank)"}
    if dist.get_rank() == 0:
        print(json.dumps(multi_line(work, tmax, dist.get_world_size(), K, W, S, launches, clk.summary(), e2e)))
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
