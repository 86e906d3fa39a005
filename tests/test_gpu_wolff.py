"""GPU parity of the Wolff cluster updates.

* Ising: the device grows, accepts and flips exactly the oracle's clusters
  (coins keyed by the directed bond, thresholds on integer words), so spins
  after every cluster are identical and the observables agree to 1e-9; the
  integer energy bookkeeping equals the full recompute at every measurement.
* XY / Heisenberg: FP32 on the device vs FP64 in the oracle; a bond coin that
  sits within rounding of its probability can differ, after which the two
  chains part.  From the same start, the first clusters agree site for site
  (spins to 1e-4), and the statistics agree with the reference library.
"""
import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu

WOLFF_ISING = [
    ("sq16", lambda: C.square_args("ising", 16, 2.4, nthermal=20, nsweep=30, tau=1, algo=1, frames=30)),
    ("sq16_h", lambda: C.square_args("ising", 16, 2.4, h=0.15, nthermal=20, nsweep=30, tau=2, algo=1, frames=30)),
    ("sq32_low", lambda: C.square_args("ising", 32, 1.8, nthermal=10, nsweep=20, tau=1, algo=1, frames=20)),
    ("sq7_odd", lambda: C.square_args("ising", 7, 2.6, nthermal=10, nsweep=20, tau=1, algo=1, frames=20)),
    ("hc6_ell", lambda: C.lattice_args("ising", (6, 6, 1), 2, [(0, 1, o, C.J9(-1)) for o in ((0, 0, 0), (-1, 0, 0), (0, 1, 0))],
                                       2.0, S=[1.5, 1.5], nthermal=5, nsweep=15, tau=1, algo=1, ki=((0, 1), (0, 0, 0)),
                                       frames=15)),
    ("sq128_big", lambda: C.square_args("ising", 128, 2.3, nthermal=5, nsweep=10, tau=1, algo=1, frames=10)),
]


@pytest.mark.parametrize("name,mk", WOLFF_ISING, ids=[c[0] for c in WOLFF_ISING])
def test_ising_wolff_bit_exact(engine, oracle_lib, name, mk):
    args = mk()
    res, ex = engine.solve("ising", args, seed=321)
    ref, rex = oracle_lib.solve("ising", args, seed=321, mode=1)
    assert ex["exact_mismatches"] == 0
    np.testing.assert_array_equal(ex["frames"][-1][:, 0], rex["spins"][:, 0].astype(np.float32))
    np.testing.assert_allclose(np.array(res[:10]), np.array(ref[:10]), rtol=1e-9, atol=1e-12)
    assert ex["clusters"] == rex["stats"][2]
    assert ex["flipped"] == rex["stats"][1]
    assert ex["accepted"] == rex["stats"][0]


WOLFF_ON = [
    ("xy_sq16", "xy", lambda: C.square_args("xy", 16, 0.9, nthermal=0, nsweep=6, tau=1, algo=1, frames=6)),
    ("heis_sq12", "heisenberg", lambda: C.square_args("heisenberg", 12, 0.7, nthermal=0, nsweep=6, tau=1, algo=1, frames=6)),
    ("heis_sq12_dmi_h", "heisenberg", lambda: C.square_args("heisenberg", 12, 0.6, h=0.1, dmi=0.4, D=[0, 0, -0.2],
                                                            nthermal=0, nsweep=6, tau=1, algo=1, frames=6)),
]


@pytest.mark.parametrize("name,model,mk", WOLFF_ON, ids=[c[0] for c in WOLFF_ON])
def test_on_wolff_first_clusters_match_oracle(engine, oracle_lib, name, model, mk):
    a = list(mk())
    a[15] = 0.6  # random initial tilt from the engine stream
    args = tuple(a)
    res, ex = engine.solve(model, args, seed=17)
    dim = 2 if model == "xy" else 3
    agree = 0
    for f in range(ex["frames"].shape[0]):
        sub = C.with_program(model, args, nthermal=0, nsweep=f + 1)
        sub = sub[:20] + (0,) + sub[21:]
        _, rex = oracle_lib.solve(model, sub, seed=17, mode=1)
        d = np.abs(ex["frames"][f][:, :dim].astype(np.float64) - rex["spins"][:, :dim]).max()
        if d < 1e-4:
            agree += 1
        else:
            break
    assert agree >= 4, agree


def test_wolff_counts_and_energy_consistency(engine):
    """O(n) Wolff: the engine's incremental energy stays within FP32 drift of
    the full recompute; clusters counted."""
    args = C.square_args("heisenberg", 24, 0.6, dmi=0.3, nthermal=50, nsweep=200, tau=1, algo=1)
    res, ex = engine.solve("heisenberg", args, seed=5, recheck_every=8)
    assert ex["clusters"] == 250
    assert ex["energy_drift"] < 1e-3 * 24 * 24


@pytest.mark.parametrize("model,L,T", [("xy", 32, 0.7), ("heisenberg", 24, 0.5)])
def test_wolff_isotropic_energy_and_acceptance(engine, model, L, T):
    """Isotropic exchange without single-ion term or field: every cluster is
    accepted, and the energy from the boundary bonds alone stays within FP32
    drift of the full recompute (re-checked every 8 measurements)."""
    args = C.square_args(model, L, T, nthermal=50, nsweep=300, tau=1, algo=1)
    res, ex = engine.solve(model, args, seed=9, recheck_every=8)
    assert ex["clusters"] == 350
    assert ex["accepted"] == 350
    assert ex["flipped"] > 350
    assert ex["energy_drift"] < 1e-3 * L * L


@pytest.mark.parametrize("model,L,T", [("ising", 256, 2.3), ("xy", 160, 0.9)])
def test_wolff_global_state_schedule(engine, oracle_lib, model, L, T):
    """Lattices whose Wolff state does not fit in shared memory run the
    global-state instantiation; Ising stays bit-exact with the oracle there,
    and the O(n) model's first clusters agree site for site."""
    args = C.square_args(model, L, T, nthermal=0, nsweep=4, tau=1, algo=1, frames=4)
    if model == "xy":
        a = list(args)
        a[15] = 0.6  # random initial tilt from the engine stream
        args = tuple(a)
    b = engine.Batch()
    b.add(model, args, seed=77)
    b.prepare()
    assert b.schedules()[0][0] == "wolff_global"
    b.run()
    res, ex = b.result(0)
    b.close()
    ref, rex = oracle_lib.solve(model, args, seed=77, mode=1)
    if model == "ising":
        assert ex["exact_mismatches"] == 0
        np.testing.assert_array_equal(ex["frames"][-1][:, 0], rex["spins"][:, 0].astype(np.float32))
        assert ex["flipped"] == rex["stats"][1]
    else:
        d = np.abs(ex["frames"][-1][:, :2].astype(np.float64) - rex["spins"][:, :2]).max()
        assert d < 1e-4, d
