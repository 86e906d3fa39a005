"""The allocation-free entry point against the engine's own solve.

mcs_ising_square_noalloc() is for callers that cannot call cudaMalloc (they own
every device buffer through their own allocator): it takes device pointers for
the spins and the per-sweep sums and keeps its only scratch in a fixed array
inside the library.  Called twice in a row (sweeps 0..n1-1, then n1..n1+n2-1)
on the same spin buffer, it must reproduce what mcs_solve() computes for the
same lattice, couplings and seed: identical spins after each call (bit for
bit, Ising is exact) and per-sweep magnetisation and energy equal to the
solve's per-measurement series within 1e-12 relative.

This file is collected last on purpose (tests/test_zz_*): a failure here
leaves every other GPU test already run.
"""
import ctypes

import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("L,T,h", [(32, 2.3, 0.0), (64, 1.9, 0.25)])
def test_noalloc_matches_solve_on_two_calls(engine, L, T, h):
    torch = pytest.importorskip("torch")
    n1, n2, seed = 7, 9, 4242
    args = C.square_args("ising", L, T, h=h, nthermal=0, nsweep=n1 + n2, frames=n1 + n2)
    ref, ex = engine.solve("ising", args, seed=seed, absolute_energy=True, record_series=True)
    K, hb = -1.0 / T, h / T
    N = L * L
    sigma = torch.ones(N, dtype=torch.int8, device="cuda")
    sums = torch.zeros(2 * (n1 + n2), dtype=torch.int64, device="cuda")
    fn = engine.lib().mcs_ising_square_noalloc
    torch.cuda.synchronize()
    rc = fn(_ptr(sigma), L, L, K, hb, seed, 0, n1, _ptr(sums), None)
    assert rc == 0, engine.lib().mcs_last_error()
    torch.cuda.synchronize()
    first = sigma.cpu().numpy().astype(np.float32)
    np.testing.assert_array_equal(first, ex["frames"][n1 - 1][:, 0])
    rc = fn(_ptr(sigma), L, L, K, hb, seed, n1, n2, ctypes.c_void_p(sums.data_ptr() + 8 * 2 * n1), None)
    assert rc == 0, engine.lib().mcs_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(sigma.cpu().numpy().astype(np.float32), ex["frames"][-1][:, 0])
    s = sums.cpu().numpy().reshape(-1, 2).astype(np.float64)
    M, B = s[:, 0], s[:, 1]
    series = ex["series"]
    np.testing.assert_allclose(M / N, series[:, 1], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose((K * B - hb * M) / N, series[:, 0], rtol=1e-12, atol=1e-15)


def test_noalloc_rejects_bad_sizes(engine):
    torch = pytest.importorskip("torch")
    sigma = torch.ones(16, dtype=torch.int8, device="cuda")
    sums = torch.zeros(2, dtype=torch.int64, device="cuda")
    fn = engine.lib().mcs_ising_square_noalloc
    assert fn(_ptr(sigma), 3, 4, -1.0, 0.0, 1, 0, 1, _ptr(sums), None) == 1
    assert fn(_ptr(sigma), 4096, 4096, -1.0, 0.0, 1, 0, 1, _ptr(sums), None) == 1
    assert b"scratch" in engine.lib().mcs_last_error()
