"""GPU parity of the thread-block-cluster schedule.

A replica split by rows over 2, 4 or 8 CTAs (DSMEM ghost rows) runs the same
per-site update with the same Philox words as the one-CTA resident schedule,
so the spin trajectory agrees to FP32 rounding of the local fields (the
neighbour sums are formed in the same order) and the observables agree with
the resident schedule within 1e-6 relative.
"""
import os

import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu


def _run(engine, model, args, cluster, seed=3):
    old = os.environ.get("MCSGPU_CLUSTER")
    os.environ["MCSGPU_CLUSTER"] = str(cluster)
    try:
        return engine.solve(model, args, seed=seed, schedule="resident" if cluster == 1 else "auto", random_init=True)
    finally:
        if old is None:
            os.environ.pop("MCSGPU_CLUSTER", None)
        else:
            os.environ["MCSGPU_CLUSTER"] = old


CASES = [
    ("xy_L32", "xy", lambda: C.square_args("xy", 32, 0.9, nthermal=10, nsweep=20, frames=20)),
    ("heis_L32_dmi_h", "heisenberg", lambda: C.square_args("heisenberg", 32, 0.6, h=0.2, dmi=0.4, D=[0, 0, -0.1],
                                                           nthermal=10, nsweep=20, frames=20)),
    ("xy_L64_tau2", "xy", lambda: C.square_args("xy", 64, 1.2, nthermal=6, nsweep=8, tau=2 * 64 * 64, frames=8)),
]


@pytest.mark.parametrize("csize", [2, 4, 8])
@pytest.mark.parametrize("name,model,mk", CASES, ids=[c[0] for c in CASES])
def test_cluster_matches_resident(engine, name, model, mk, csize):
    args = mk()
    a, ea = _run(engine, model, args, 1)
    b, eb = _run(engine, model, args, csize)
    np.testing.assert_allclose(eb["frames"], ea["frames"], atol=2e-5)
    n = 27
    np.testing.assert_allclose(np.array(b[:n]), np.array(a[:n]), rtol=1e-5, atol=1e-6)
    assert eb["site_updates"] == ea["site_updates"]


UNEVEN = [
    ("xy_L36_C8", "xy", 8, lambda: C.square_args("xy", 36, 0.9, nthermal=6, nsweep=12, frames=12)),
    ("xy_L40_C16", "xy", 16, lambda: C.square_args("xy", 40, 1.1, nthermal=6, nsweep=12, frames=12)),
    ("heis_L44_C4_dmi_h", "heisenberg", 4, lambda: C.square_args("heisenberg", 44, 0.6, h=0.2, dmi=0.4,
                                                                  nthermal=6, nsweep=12, frames=12)),
    ("heis_L72_C16_dmi", "heisenberg", 16, lambda: C.square_args_fast("heisenberg", 72, 0.7, dmi=0.4,
                                                                      nthermal=4, nsweep=8, frames=8)),
    # Ly/2 odd: the first site of row 1 is swept with the boundary rows
    ("xy_L34_C4_odd_half", "xy", 4, lambda: C.square_args("xy", 34, 0.9, nthermal=6, nsweep=12, frames=12)),
    ("heis_L30_C2_odd_half", "heisenberg", 2, lambda: C.square_args("heisenberg", 30, 0.6, h=0.2, dmi=0.4,
                                                                     nthermal=6, nsweep=12, frames=12)),
    ("xy_L26_C8_odd_half", "xy", 8, lambda: C.square_args("xy", 26, 1.0, nthermal=6, nsweep=12, frames=12)),
]


@pytest.mark.parametrize("name,model,csize,mk", UNEVEN, ids=[c[0] for c in UNEVEN])
def test_uneven_row_split_matches_resident(engine, name, model, csize, mk):
    """Row pairs dealt out unevenly (slabs of different heights, up to 16 CTAs)
    give the resident schedule's trajectory and observables."""
    args = mk()
    a, ea = _run(engine, model, args, 1)
    old = os.environ.get("MCSGPU_CLUSTER")
    os.environ["MCSGPU_CLUSTER"] = str(csize)
    try:
        bt = engine.Batch()
        bt.add(model, args, seed=3, random_init=True)
        bt.prepare()
        bt.run()
        sched = bt.schedules()
        b, eb = bt.result(0)
        bt.close()
    finally:
        if old is None:
            os.environ.pop("MCSGPU_CLUSTER", None)
        else:
            os.environ["MCSGPU_CLUSTER"] = old
    assert sched[0][0] == "cluster" and sched[0][1] == csize, sched
    np.testing.assert_allclose(eb["frames"], ea["frames"], atol=2e-5)
    np.testing.assert_allclose(np.array(b[:27]), np.array(a[:27]), rtol=1e-5, atol=1e-6)
    assert eb["site_updates"] == ea["site_updates"]


def test_replica_too_large_for_any_cluster_runs_once_on_tiles(engine):
    """XY L=512: 2 MB of spins fit neither one CTA nor a cluster of 8; the
    cluster group falls back to the tiled schedule and the replica must join
    that one group only (two groups would sweep it twice, side by side)."""
    args = C.square_args_fast("xy", 512, 0.9, nthermal=2, nsweep=4, frames=4)
    a, ea = engine.solve("xy", args, seed=5, schedule="tiled", random_init=True)
    b, eb = engine.solve("xy", args, seed=5, random_init=True)
    assert eb["site_updates"] == ea["site_updates"] == 512 * 512 * 6
    np.testing.assert_allclose(eb["frames"], ea["frames"], atol=2e-5)
    np.testing.assert_allclose(np.array(b[:27]), np.array(a[:27]), rtol=1e-6, atol=1e-6)


def test_balanced_batch_equals_alone(engine):
    """A large Ising replica among small ones, placed by the load balancer and
    the autotuner (the resident group, the cluster schedule or the tiled one);
    Ising spin trajectories are bit-exact across schedules, so the integer
    counts are equal and the FP64 averages agree to their summation order
    (1e-12)."""
    probs = [C.square_args_fast("ising", 256, 2.3, nthermal=4, nsweep=8)]
    probs += [C.square_args("ising", 16 + 4 * k, 2.0 + 0.1 * k, nthermal=4, nsweep=8) for k in range(6)]
    b = engine.Batch()
    for k, a in enumerate(probs):
        b.add("ising", a, seed=40 + k, random_init=True)
    b.prepare()
    kinds = [g[0] for g in b.schedules()]
    assert set(kinds) <= {"resident", "cluster", "tiled"}, kinds
    b.run()
    got = [b.result(k) for k in range(len(probs))]
    b.close()
    for k, a in enumerate(probs):
        alone, ex = engine.solve("ising", a, seed=40 + k, schedule="resident", random_init=True)
        np.testing.assert_allclose(np.array(got[k][0][:10]), np.array(alone[:10]), rtol=1e-12, atol=1e-12)
        assert got[k][1]["accepted"] == ex["accepted"] and got[k][1]["site_updates"] == ex["site_updates"]


COPIES = [
    ("ising_L32", "ising", lambda: C.square_args("ising", 32, 2.3, nthermal=8, nsweep=16, frames=4)),
    ("ising_L24_h", "ising", lambda: C.square_args("ising", 24, 2.6, h=0.1, nthermal=8, nsweep=16)),
    ("xy_L32", "xy", lambda: C.square_args("xy", 32, 0.9, nthermal=8, nsweep=16, frames=4)),
    ("heis_honeycomb8", "heisenberg", lambda: C.honeycomb_args("heisenberg", 8, 6.0, nthermal=8, nsweep=16)),
    ("heis_L24_dmi_h", "heisenberg", lambda: C.square_args("heisenberg", 24, 0.6, h=0.2, dmi=0.4, nthermal=8, nsweep=16)),
]


@pytest.mark.parametrize("copies", [2, 4])
@pytest.mark.parametrize("name,model,mk", COPIES, ids=[c[0] for c in COPIES])
def test_resident_copies_match_one_cta(engine, name, model, mk, copies):
    """A replica held in 2 or 4 CTAs of a cluster (each a full copy, colour
    phases shared out) runs the one-CTA trajectory: Ising bit-exact, O(n)
    within FP32 summation order."""
    args = mk()
    a, ea = engine.solve(model, args, seed=9, schedule="resident", random_init=True)
    old = os.environ.get("MCSGPU_COPIES")
    os.environ["MCSGPU_COPIES"] = str(copies)
    try:
        bt = engine.Batch()
        bt.add(model, args, seed=9, random_init=True, schedule="resident")
        bt.prepare()
        bt.run()
        sched = bt.schedules()
        b, eb = bt.result(0)
        bt.close()
    finally:
        if old is None:
            os.environ.pop("MCSGPU_COPIES", None)
        else:
            os.environ["MCSGPU_COPIES"] = old
    assert sched[0][0] == "resident" and sched[0][1] == copies, sched
    assert eb["site_updates"] == ea["site_updates"] and eb["accepted"] == ea["accepted"]
    if model == "ising":
        np.testing.assert_allclose(np.array(b[:10]), np.array(a[:10]), rtol=1e-12, atol=1e-12)
        assert eb["exact_mismatches"] == 0
    else:
        np.testing.assert_allclose(np.array(b[:27]), np.array(a[:27]), rtol=1e-5, atol=1e-6)
    if "frames" in ea:
        np.testing.assert_allclose(eb["frames"], ea["frames"], atol=2e-5)


SERIES_CASES = [
    ("ising_L16", "ising", lambda: C.square_args("ising", 16, 2.4, nthermal=20, nsweep=200)),
    ("xy_L16", "xy", lambda: C.square_args("xy", 16, 0.9, nthermal=20, nsweep=200)),
    ("heis_L12_dmi_h_circ", "heisenberg", lambda: C.square_args("heisenberg", 12, 0.5, h=0.3, dmi=0.4,
                                                                nthermal=20, nsweep=200)),
]
CANDIDATES = [(-2, 0), (-4, 0)] + [(c, t) for c in (1, 2, 4) for t in (256, 512, 1024)]


@pytest.mark.parametrize("cand", CANDIDATES, ids=["%d:%d" % c for c in CANDIDATES])
@pytest.mark.parametrize("name,model,mk", SERIES_CASES, ids=[c[0] for c in SERIES_CASES])
def test_every_candidate_records_the_same_series(engine, name, model, mk, cand):
    """Each configuration the autotuner may pick for a group (resident copies,
    the cluster kernel with 1, 2 or 4 CTAs at 256/512/1024 threads) records
    the per-measurement series row by row where the one-CTA resident run
    does, and gives its observables.  (A measurement index summed over the
    CTAs of a cluster once put rows at C*m.)"""
    args = mk()
    ref = engine.Batch()
    ref.add(model, args, seed=21, record_series=True, schedule="resident", random_init=True)
    old = os.environ.get("MCSGPU_FORCE")
    os.environ["MCSGPU_CLUSTER"] = "1"  # the one-CTA resident kernel only
    try:
        ref.prepare()
        ref.run()
        assert ref.schedules()[0][:2] == ("resident", 1)
    finally:
        os.environ.pop("MCSGPU_CLUSTER", None)
    a, ea = ref.result(0)
    ref.close()
    C_, th = cand
    if th == 0:
        os.environ["MCSGPU_COPIES"] = str(-C_)
    else:
        os.environ["MCSGPU_FORCE"] = "%d:%d" % cand
    try:
        bt = engine.Batch()
        bt.add(model, args, seed=21, record_series=True, random_init=True)
        bt.prepare()
        bt.run()
        sched = bt.schedules()
        b, eb = bt.result(0)
        bt.close()
    finally:
        os.environ.pop("MCSGPU_FORCE", None)
        os.environ.pop("MCSGPU_COPIES", None)
        if old is not None:
            os.environ["MCSGPU_FORCE"] = old
    want_kind = "resident" if th == 0 else "cluster"
    assert sched[0][0] == want_kind and sched[0][1] == abs(C_), sched
    assert eb["series"].shape == ea["series"].shape
    np.testing.assert_allclose(eb["series"], ea["series"], rtol=1e-5, atol=2e-5)
    np.testing.assert_allclose(np.array(b[:27]), np.array(a[:27]), rtol=1e-5, atol=1e-6)


WAVE_CASES = [
    ("xy_L26", "xy", lambda: C.square_args("xy", 26, 0.9, nthermal=20, nsweep=200), (13, 256)),
    ("heis_L12_dmi_h_circ", "heisenberg", dict((c[0], c[2]) for c in SERIES_CASES)["heis_L12_dmi_h_circ"], (6, 512)),
]


@pytest.mark.parametrize("name,model,mk,cand", WAVE_CASES, ids=[c[0] for c in WAVE_CASES])
def test_wave_filling_cluster_size_records_the_same_series(engine, name, model, mk, cand):
    """The autotuner's wave-filling candidate, a cluster size that is not a
    power of two (for one replica the largest its row pairs allow: 13 CTAs,
    whose rank-0 gather reads in two batches of eight, and 6), records the
    series of the one-CTA resident run."""
    test_every_candidate_records_the_same_series(engine, name, model, mk, cand)


@pytest.mark.parametrize("model", ["ising", "xy"])
def test_warp_per_replica_matches_alone(engine, model):
    """A group of many small replicas on one warp each (the resident kernel
    with 32-thread CTAs, the autotuner's candidate for groups of 32 or more
    replicas) runs each replica's trajectory: Ising bit-exact against the
    replica solved alone, O(n) within FP32 summation order."""
    probs = []
    for k in range(40):
        L = (16, 24, 32)[k % 3]
        T = (2.0 + 0.03 * k) if model == "ising" else (0.6 + 0.02 * k)
        probs.append(C.square_args(model, L, T, h=0.05 * (k % 2), nthermal=5, nsweep=12))
    os.environ["MCSGPU_FORCE"] = "0:32"
    try:
        bt = engine.Batch()
        for k, a in enumerate(probs):
            bt.add(model, a, seed=600 + k, random_init=True)
        bt.prepare()
        bt.run()
        sched = bt.schedules()
        got = [bt.result(k) for k in range(len(probs))]
        bt.close()
    finally:
        os.environ.pop("MCSGPU_FORCE", None)
    assert sched == [("resident", 1, 32, len(probs))], sched
    n = 10 if model == "ising" else 27
    for k in (0, 1, 2, 17, 39):
        alone, ex = engine.solve(model, probs[k], seed=600 + k, schedule="resident", random_init=True)
        if model == "ising":
            np.testing.assert_allclose(np.array(got[k][0][:n]), np.array(alone[:n]), rtol=1e-12, atol=1e-12)
            assert got[k][1]["exact_mismatches"] == 0
            assert got[k][1]["accepted"] == ex["accepted"]
        else:
            np.testing.assert_allclose(np.array(got[k][0][:n]), np.array(alone[:n]), rtol=1e-6, atol=1e-6)


ISING_CLUSTER = [
    ("L96_T2.2", lambda: C.square_args("ising", 96, 2.2, nthermal=30, nsweep=300, frames=10), (16, 256)),
    ("L64_T3_h", lambda: C.square_args("ising", 64, 3.0, h=0.2, nthermal=30, nsweep=300, frames=10), (8, 512)),
    ("L40_T2.6_uneven", lambda: C.square_args("ising", 40, 2.6, nthermal=30, nsweep=300, frames=10), (16, 256)),
    # Ly/2 odd: a Philox block of four sites spans two rows, and at a slab
    # boundary two CTAs
    ("L34_T2.3_odd_half", lambda: C.square_args("ising", 34, 2.3, nthermal=30, nsweep=300, frames=10), (4, 256)),
    ("L26_T2.5_odd_half_C8", lambda: C.square_args("ising", 26, 2.5, h=0.1, nthermal=30, nsweep=300, frames=10), (8, 512)),
    ("L48_antiferro_h", lambda: C.square_args("ising", 48, 1.5, J=1.0, h=0.5, nthermal=30, nsweep=300, frames=10),
     (4, 256)),
]


@pytest.mark.parametrize("name,mk,cand", ISING_CLUSTER, ids=[c[0] for c in ISING_CLUSTER])
def test_ising_cluster_kernel_is_bit_exact(engine, name, mk, cand):
    """Ising on the row-split cluster schedule (int8 slabs, ghost rows over
    DSMEM, the integer frame split by slabs and added by rank 0) gives the
    one-CTA resident run's results, per-measurement series and spin frames
    bit for bit, with the exact bookkeeping intact (uneven slabs included)."""
    args = mk()
    ref = engine.Batch()
    ref.add("ising", args, seed=33, record_series=True, schedule="resident")
    os.environ["MCSGPU_CLUSTER"] = "1"
    try:
        ref.prepare()
        ref.run()
        assert ref.schedules()[0][:2] == ("resident", 1)
    finally:
        os.environ.pop("MCSGPU_CLUSTER", None)
    a, ea = ref.result(0)
    ref.close()
    os.environ["MCSGPU_FORCE"] = "%d:%d" % cand
    try:
        bt = engine.Batch()
        bt.add("ising", args, seed=33, record_series=True)
        bt.prepare()
        bt.run()
        sched = bt.schedules()
        b, eb = bt.result(0)
        bt.close()
    finally:
        os.environ.pop("MCSGPU_FORCE", None)
    assert sched[0][0] == "cluster" and sched[0][1] == cand[0], sched
    assert eb["exact_mismatches"] == 0 and ea["exact_mismatches"] == 0
    assert eb["accepted"] == ea["accepted"] and eb["site_updates"] == ea["site_updates"]
    np.testing.assert_array_equal(eb["series"], ea["series"])
    np.testing.assert_array_equal(np.array(b[:10]), np.array(a[:10]))
    np.testing.assert_array_equal(eb["frames"], ea["frames"])
