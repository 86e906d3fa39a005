"""GPU tests of the continuous-batching server and of batches of uneven sizes.

* requests of mixed models and sizes submitted while others are already on
  the device give the same results as each solved alone (Ising to 1e-9,
  O(n) to 1e-6 relative: same spin trajectory, FP64 sums in another order);
* submits from several threads while the main thread steps the server
  (host compile beside device work) lose nothing and change nothing;
* a small HBM budget queues requests without losing any;
* each request advances by its own quota per step, so small requests that
  arrive with a large one finish first;
* a request that fails (an upload or result failure injected on the host) or
  is cancelled is retired with its own status while the others complete with
  the results they give alone, and the budget returns to zero;
* a batch of replicas of uneven lattice sizes (square Heisenberg with DMI,
  field and circuits, L in {64, 96, 128, 192, 256}) matches solves alone.
"""
import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu


def _reqs():
    return [
        ("ising", C.square_args("ising", 32, 2.2, nthermal=20, nsweep=40), 11),
        ("xy", C.square_args("xy", 48, 0.9, nthermal=20, nsweep=30), 12),
        ("heisenberg", C.square_args("heisenberg", 40, 0.5, h=0.2, dmi=0.4, nthermal=10, nsweep=30), 13),
        ("ising", C.square_args("ising", 64, 2.6, h=0.1, nthermal=10, nsweep=60), 14),
        ("heisenberg", C.honeycomb_args("heisenberg", 8, 6.0, nthermal=10, nsweep=20), 15),
        ("xy", C.square_args("xy", 128, 1.1, nthermal=5, nsweep=25), 16),
        ("ising", C.square_args("ising", 24, 2.4, nthermal=5, nsweep=30, tau=2, algo=1), 17),
        ("xy", C.square_args("xy", 16, 1.0, nthermal=5, nsweep=30, tau=1, algo=1), 18),
    ]


def _close(model, a, b):
    # O(n): the same trajectory; FP32 per-thread partials summed in another
    # order leave ~1e-8 absolute noise on quantities near zero (e.g. Q)
    n = 10 if model == "ising" else 27
    np.testing.assert_allclose(np.array(a[:n]), np.array(b[:n]), rtol=1e-9 if model == "ising" else 1e-6,
                               atol=1e-9 if model == "ising" else 1e-6)


def test_server_results_equal_alone_with_overlapping_arrivals(engine, monkeypatch):
    monkeypatch.setenv("MCSGPU_SERVER_STEP_US", "20")   # short steps, so that arrivals overlap
    reqs = _reqs()
    srv = engine.Server(hbm_budget_bytes=1 << 30, max_slots=64)
    tickets = {}
    # the first half arrives, runs a few steps; the rest arrives while those are on the device
    for m, a, s in reqs[:4]:
        tickets[srv.submit(m, a, seed=s)] = (m, a, s)
    for _ in range(2):
        srv.step()
    assert srv.stats()["active"] > 0
    for m, a, s in reqs[4:]:
        tickets[srv.submit(m, a, seed=s)] = (m, a, s)
    got = {}
    for _ in range(1000):
        srv.step()
        for t in list(tickets):
            if t in got:
                continue
            r = srv.poll(t)
            if r is not None:
                got[t] = r
        if len(got) == len(tickets):
            break
    assert len(got) == len(tickets)
    for t, (m, a, s) in tickets.items():
        alone, _ = engine.solve(m, a, seed=s)
        _close(m, got[t][0], alone)
    st = srv.stats()
    assert st["active"] == 0 and st["queued"] == 0 and st["bytes_in_use"] == 0
    srv.close()


def test_server_threaded_submits_while_stepping(engine, monkeypatch):
    import threading
    from concurrent.futures import ThreadPoolExecutor

    monkeypatch.setenv("MCSGPU_SERVER_STEP_US", "200")
    reqs = _reqs()
    srv = engine.Server(hbm_budget_bytes=1 << 30, max_slots=64)
    tickets, lock = {}, threading.Lock()

    def sub(k):
        m, a, s = reqs[k]
        t = srv.submit(m, a, seed=s + 100, random_init=(k % 2 == 0))
        with lock:
            tickets[t] = k

    pool = ThreadPoolExecutor(max_workers=4)
    futs = [pool.submit(sub, k) for k in range(len(reqs))]
    got = {}
    for _ in range(5000):
        srv.step()
        with lock:
            live = list(tickets)
        for t in live:
            if t not in got:
                r = srv.poll(t)
                if r is not None:
                    got[t] = r
        if len(got) == len(reqs):
            break
    for f in futs:
        f.result()
    pool.shutdown()
    assert len(got) == len(reqs)
    for t, k in tickets.items():
        m, a, s = reqs[k]
        alone, _ = engine.solve(m, a, seed=s + 100, random_init=(k % 2 == 0))
        _close(m, got[t][0], alone)
    st = srv.stats()
    assert st["active"] == 0 and st["queued"] == 0 and st["bytes_in_use"] == 0
    srv.close()


def test_server_budget_queues_requests(engine, monkeypatch):
    monkeypatch.setenv("MCSGPU_SERVER_STEP_US", "300")
    reqs = _reqs()[:4]
    srv = engine.Server(hbm_budget_bytes=600_000, max_slots=2)
    ts = [srv.submit(m, a, seed=s) for m, a, s in reqs]
    srv.step()
    st = srv.stats()
    assert st["queued"] >= 2 and st["active"] <= 2
    done = {}
    for _ in range(2000):
        srv.step()
        for t in ts:
            if t not in done:
                r = srv.poll(t)
                if r is not None:
                    done[t] = r
        if len(done) == len(ts):
            break
    assert len(done) == len(ts)
    with pytest.raises(Exception):
        srv.poll(123456)
    srv.close()


def test_batch_uneven_sizes(engine):
    sizes = [64, 96, 128, 192, 256]
    probs = []
    for i in range(10):
        L = sizes[i % len(sizes)]
        T = 0.1 + 0.09 * i
        H = 0.06 * i
        probs.append(C.square_args("heisenberg", L, T, h=H, dmi=0.4, nthermal=3, nsweep=6))
    b = engine.Batch()
    for i, a in enumerate(probs):
        b.add("heisenberg", a, seed=300 + i, random_init=True)
    b.run()
    res = [b.result(i)[0] for i in range(len(probs))]
    b.close()
    for i in (0, 3, 4, 9):
        alone, _ = engine.solve("heisenberg", probs[i], seed=300 + i, random_init=True)
        _close("heisenberg", res[i], alone)
    assert all(np.isfinite(r[:27]).all() for r in res)


def _drain(srv, tickets, steps=5000):
    """Step until every ticket is done; returns {ticket: result or EngineError}
    and the step at which each finished."""
    import mcsolver_gb300 as eng
    got, when = {}, {}
    for k in range(steps):
        srv.step()
        for t in tickets:
            if t in got:
                continue
            try:
                r = srv.poll(t)
            except eng.EngineError as e:
                r = e
            if r is not None:
                got[t] = r
                when[t] = k
        if len(got) == len(tickets):
            break
    return got, when


def test_small_requests_finish_before_a_large_one(engine, monkeypatch):
    """Requests submitted together: a large XY lattice and small Ising ones.
    Each advances by its own quota per step (about the same device time per
    request), so the small ones finish in a few steps while the large one
    is still running, and every result equals the solve alone."""
    monkeypatch.setenv("MCSGPU_SERVER_STEP_US", "1000")
    big = ("xy", C.square_args_fast("xy", 256, 1.0, nthermal=200, nsweep=800), 31)
    small = [("ising", C.square_args("ising", 16, 2.0 + 0.2 * k, nthermal=100, nsweep=300), 40 + k) for k in range(4)]
    srv = engine.Server(hbm_budget_bytes=1 << 30, max_slots=16)
    tb = srv.submit(big[0], big[1], seed=big[2])
    ts = [srv.submit(m, a, seed=s) for m, a, s in small]
    got, when = _drain(srv, [tb] + ts)
    assert len(got) == 5
    assert max(when[t] for t in ts) < when[tb], when
    for t, (m, a, s) in zip([tb] + ts, [big] + small):
        alone, _ = engine.solve(m, a, seed=s)
        _close(m, got[t][0], alone)
    assert srv.stats()["bytes_in_use"] == 0
    srv.close()


@pytest.mark.parametrize("inject", ["upload:2", "results:3"])
def test_injected_failure_retires_one_request(engine, monkeypatch, inject):
    """A failure injected on the host (the second upload, or the third
    result read-back, reports an error without touching the device) retires
    that request with its own status; the others give their results alone."""
    monkeypatch.setenv("MCSGPU_SERVER_STEP_US", "300")
    monkeypatch.setenv("MCSGPU_SERVER_INJECT", inject)
    reqs = _reqs()[:5]
    srv = engine.Server(hbm_budget_bytes=1 << 30, max_slots=64)
    ts = [srv.submit(m, a, seed=s) for m, a, s in reqs]
    got, _ = _drain(srv, ts)
    assert len(got) == len(ts)
    failed = [t for t in ts if isinstance(got[t], engine.EngineError)]
    assert len(failed) == 1, got
    err = got[failed[0]]
    assert "injected" in str(err) and err.code in (engine.MCS_ENOMEM, engine.MCS_ECUDA)
    for t, (m, a, s) in zip(ts, reqs):
        if t in failed:
            continue
        alone, _ = engine.solve(m, a, seed=s)
        _close(m, got[t][0], alone)
    st = srv.stats()
    assert st["active"] == 0 and st["queued"] == 0 and st["bytes_in_use"] == 0
    srv.close()


def test_cancel_active_and_queued_requests(engine, monkeypatch):
    """One request is cancelled while on the device, one while queued (slots
    full); both poll as cancelled, the rest complete as alone, and every byte
    of the budget comes back."""
    monkeypatch.setenv("MCSGPU_SERVER_STEP_US", "5")   # a few sweeps per step
    reqs = [("xy", C.square_args("xy", 64, 0.9 + 0.1 * k, nthermal=50, nsweep=400), 60 + k) for k in range(4)]
    srv = engine.Server(hbm_budget_bytes=1 << 30, max_slots=3)
    ts = [srv.submit(m, a, seed=s) for m, a, s in reqs]
    srv.step()
    st = srv.stats()
    assert st["active"] == 3 and st["queued"] == 1, st
    srv.cancel(ts[1])   # on the device
    srv.cancel(ts[3])   # still queued
    got, _ = _drain(srv, ts)
    for t in (ts[1], ts[3]):
        assert isinstance(got[t], engine.EngineError) and got[t].code == engine.MCS_ECANCELLED
    for t, (m, a, s) in zip(ts, reqs):
        if t in (ts[1], ts[3]):
            continue
        alone, _ = engine.solve(m, a, seed=s)
        _close(m, got[t][0], alone)
    st = srv.stats()
    assert st["active"] == 0 and st["queued"] == 0 and st["bytes_in_use"] == 0
    srv.close()
