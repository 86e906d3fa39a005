"""CPU tests of the oracle: pinned against the reference's own outputs."""
import os
import platform

import numpy as np
import pytest

from tests import cases as C


def _close(a, b, exact):
    a, b = np.asarray(C.flat(a), float), np.asarray(C.flat(b), float)
    assert a.shape == b.shape
    if exact:
        same = (a == b) | (np.isnan(a) & np.isnan(b))
        assert same.all(), [(i, x, y) for i, (x, y) in enumerate(zip(a, b)) if x != y][:5]
    else:
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12)


PIN = [n for n in C.golden()["cases"] if n.startswith("pin_")]


@pytest.mark.parametrize("name", PIN)
def test_oracle_reference_stream_matches_reference(oracle_lib, name):
    """mode 0 (glibc rand stream) reproduces the reference library's output;
    bit for bit on the machine type the fixtures were generated on."""
    model, args, c = C.golden_case(name)
    exact = platform.machine() == C.golden()["machine"]
    for s in c["seeds"]:
        mine, _ = oracle_lib.solve(model, args, seed=int(s), mode=0)
        _close(mine, C.as_args(c["ref"][str(s)]), exact)


def test_philox_known_answers(oracle_lib):
    # Random123 known-answer vectors for Philox4x32-10
    kat = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in kat:
        assert oracle_lib.philox(ctr, key) == want


def test_synthetic_tuples_match_reference_marshalling():
    """tests/cases.py builds the same tuples the reference's mcMain passes."""
    def same(a, b):
        assert len(a) == len(b)
        for x, y in zip(a, b):
            np.testing.assert_allclose(np.asarray(x, float), np.asarray(y, float), rtol=1e-12, atol=1e-12)
    _, a, _ = C.golden_case("pin_ising_sq8_metro")
    same(a, C.square_args("ising", 8, 2.0, nthermal=20, nsweep=30))
    _, a, _ = C.golden_case("pin_ising_sq8_wolff_h")
    same(a, C.square_args("ising", 8, 2.5, h=0.2, nthermal=20, nsweep=30, tau=2, algo=1))
    _, a, _ = C.golden_case("pin_heis_sq8_dmi_metro")
    same(a, C.square_args("heisenberg", 8, 0.4, h=0.2, dmi=0.4, D=[0, 0, -0.1], nthermal=20, nsweep=30))
    _, a, _ = C.golden_case("pin_xy_sq8_metro")
    same(a, C.square_args("xy", 8, 0.9, nthermal=20, nsweep=30))
    _, a, _ = C.golden_case("pin_heis_hc6_metro")
    same(a, C.honeycomb_args("heisenberg", 6, 8.0, nthermal=20, nsweep=30))


@pytest.mark.parametrize("model,L", [("ising", 8), ("ising", 7), ("heisenberg", 5)])
def test_colouring_is_proper(oracle_lib, model, L):
    args = C.square_args(model, L, 1.0)
    n, col = oracle_lib.colouring(model, args)
    z = args[5] if model == "ising" else args[6]
    nl = args[6] if model == "ising" else args[7]
    lo = args[8] if model == "ising" else args[9]
    for i in range(len(col)):
        for l in range(nl[i]):
            j = lo[i * z + l]
            if j != i:
                assert col[i] != col[j]
    assert (n == 2) if L % 2 == 0 else (3 <= n <= 5)


STAT = [n for n in C.golden()["cases"] if n.startswith("stat_")]


@pytest.mark.parametrize("name", STAT)
def test_oracle_engine_stream_agrees_with_reference(oracle_lib, name):
    """The engine stream (colour sweeps, Philox) samples the reference's
    distribution: means over 24 seeds within 3 sigma of the reference's."""
    model, args, c = C.golden_case(name)
    nv = 10 if model == "ising" else 27
    ref = np.array([c["ref"][str(s)][:nv] for s in c["seeds"]], float)
    mine = np.array([oracle_lib.solve(model, args, seed=1000 + int(s), mode=1)[0][:nv] for s in c["seeds"]], float)
    idx = [0, 4, 5, 6, 8] if model == "ising" else [0, 6, 8, 9, 10, 18, 22]
    for k in idx:
        a, b = ref[:, k], mine[:, k]
        se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
        if se == 0:
            assert a.mean() == pytest.approx(b.mean())
            continue
        z = abs(a.mean() - b.mean()) / se
        assert z < 3.5, (k, a.mean(), b.mean(), z)


def _reference_present():
    from oracle import refharness as rh
    return rh.reference_tree_present()


@pytest.mark.skipif(not _reference_present(), reason="reference tree absent")
def test_reference_crashes_are_documented_cases():
    """Odd lattice sides give -1 renormalised links (the reference would read
    lattice[-1]); the oracle skips them."""
    from oracle import refharness as rh
    spec = dict(model="ising", LMatrix=[[1, 0, 0], [0, 1, 0], [0, 0, 1]], pos=[[0, 0, 0]], S=[1.0], D=[[0, 0, 0]],
                bonds=[(0, 0, (1, 0, 0), C.J9(-1)), (0, 0, (0, 1, 0), C.J9(-1))], L=(5, 5, 1), T=2.0,
                nthermal=1, nsweep=1, tau=0, algo="Metropolis")
    args = rh.capture_args(spec)
    assert -1 in args[13]


@pytest.mark.parametrize("model", ["ising", "xy", "heisenberg"])
@pytest.mark.parametrize("L", [6, 8, 12])
def test_vectorised_builder_equals_reference_order(model, L):
    """mcsolver_gb300.lattice.square_args_fast reproduces the reference-order
    tuples of square_args (itself checked against the reference's own
    marshalling above) value for value, as tuples and as arrays."""
    from mcsolver_gb300.lattice import square_args_fast
    kw = dict(h=0.2, nthermal=3, nsweep=4)
    if model != "ising":
        kw.update(D=[0, 0, -0.1], dmi=0.4 if model == "heisenberg" else 0.0)
    a = C.square_args(model, L, 0.7, **kw)
    for arrays in (False, True):
        b = square_args_fast(model, L, 0.7, arrays=arrays, **kw)
        assert len(a) == len(b)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(np.asarray(x, float), np.asarray(y, float))


def _onsager_energy(T, J=1.0):
    """Exact internal energy per site of the infinite 2D square Ising model
    (Onsager 1944): u = -J coth(2K) [1 + (2/pi)(2 tanh^2(2K) - 1) K(k)],
    k = 2 sinh(2K)/cosh^2(2K), K = J/T."""
    import math

    from scipy.special import ellipk
    K = J / T
    k = 2 * math.sinh(2 * K) / math.cosh(2 * K) ** 2
    return -J / math.tanh(2 * K) * (1 + 2 / math.pi * (2 * math.tanh(2 * K) ** 2 - 1) * ellipk(k * k))


def _ising_energy(spins, args):
    """Energy per site in beta units of an Ising state, summed over the ELL
    links (each bond seen from both ends, isingLib.c:121-127) and the field."""
    s = spins[:, 0]
    N, z = len(s), args[5]
    nlink = np.asarray(args[6])
    J = np.asarray(args[7], float).reshape(N, z)
    nb = np.asarray(args[8]).reshape(N, z)
    live = np.arange(z)[None, :] < nlink[:, None]
    bonds = (J * s[:, None] * s[np.where(live, nb, 0)] * live).sum()
    return 0.5 * bonds / N - args[10] * s.sum() / N


@pytest.mark.parametrize("mode", [0, 1], ids=["reference_stream", "engine_stream"])
@pytest.mark.parametrize("T", [1.6, 3.2])
def test_oracle_metropolis_energy_matches_onsager(oracle_lib, mode, T):
    """Both oracle streams sample the 2D Ising energy Onsager gives, at L=32
    away from Tc (finite-size shifts below 1e-4 per site).  The reference's
    Metropolis <e> is offset by the energy at the start of the measurement
    (isingLib.c:359), so the run starts from a thermalised state whose energy
    is computed here and added back; the error bar is the binned one of the
    per-measurement series."""
    from mcsolver_gb300 import analysis as A
    L = 32
    _, th = oracle_lib.solve("ising", C.square_args("ising", L, T, nthermal=1000, nsweep=1), seed=7, mode=mode)
    args = C.square_args("ising", L, T, nthermal=0, nsweep=4000)
    e0 = _ising_energy(th["spins"], args)
    _, ex = oracle_lib.solve("ising", args, seed=8, mode=mode, spins_in=th["spins"], want_series=True)
    m, err, _ = A.mean_error((ex["series"][:, 0] + e0) * T)
    exact = _onsager_energy(T)
    assert abs(m - exact) < 3.5 * err + 1e-4, (m, exact, err)


@pytest.mark.parametrize("T", [1.6, 2.0])
def test_oracle_wolff_energy_matches_onsager(oracle_lib, T):
    """The reference's Wolff path recomputes the absolute energy after every
    accepted cluster (isingLib.c:230-233), so its <e> is compared directly."""
    from mcsolver_gb300 import analysis as A
    args = C.square_args("ising", 32, T, nthermal=500, nsweep=4000, tau=1, algo=1)
    res, ex = oracle_lib.solve("ising", args, seed=9, mode=0, want_series=True)
    m, err, _ = A.mean_error(ex["series"][:, 0] * T)
    assert m == pytest.approx(res[4] * T, rel=1e-12)
    exact = _onsager_energy(T)
    assert abs(m - exact) < 3.5 * err + 1e-4, (m, exact, err)
