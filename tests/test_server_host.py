"""CPU tests of the request server's host side (no device call is made):
submission compiles on the host, so a malformed request is refused alone,
an oversized one is refused against the HBM budget, and a queued request can
be cancelled.  What happens to requests on the device (admission, quotas,
failures injected on the host during a run) is tested in
tests/test_gpu_server.py."""
import pytest

from tests import cases as C


def _server(engine, budget=1 << 30, slots=8):
    return engine.Server(hbm_budget_bytes=budget, max_slots=slots)


def test_malformed_request_among_good_ones_is_refused_alone(engine):
    srv = _server(engine)
    good = C.square_args("ising", 8, 2.0, nthermal=2, nsweep=4)
    bad = good[:8] + (tuple([10 ** 6] + list(good[8][1:])),) + good[9:]  # link target out of range
    t1 = srv.submit("ising", good, seed=1)
    with pytest.raises(engine.EngineError) as ei:
        srv.submit("ising", bad, seed=2)
    assert ei.value.code == 1 and "linkedOrb" in str(ei.value)
    t2 = srv.submit("xy", C.square_args("xy", 8, 1.0, nthermal=2, nsweep=4), seed=3)
    assert t2 == t1 + 1
    st = srv.stats()
    assert st["queued"] == 2 and st["active"] == 0 and st["bytes_in_use"] == 0
    assert srv.poll(t1) is None and srv.poll(t2) is None  # pending
    srv.close()


def test_request_larger_than_budget_is_refused_at_submit(engine):
    srv = _server(engine, budget=64 << 10)
    with pytest.raises(engine.EngineError) as ei:
        srv.submit("xy", C.square_args_fast("xy", 64, 1.0, nthermal=2, nsweep=4), seed=1)
    assert ei.value.code == engine.MCS_ENOMEM
    srv.close()


def test_cancel_queued_request(engine):
    srv = _server(engine)
    ts = [srv.submit("ising", C.square_args("ising", 8, 2.0 + 0.1 * k, nthermal=2, nsweep=4), seed=k)
          for k in range(3)]
    srv.cancel(ts[1])
    assert srv.stats()["queued"] == 2
    with pytest.raises(engine.EngineError) as ei:
        srv.poll(ts[1])
    assert ei.value.code == engine.MCS_ECANCELLED and "cancelled" in str(ei.value)
    # the ticket is released: a second poll or cancel does not know it
    with pytest.raises(engine.EngineError) as ei:
        srv.poll(ts[1])
    assert ei.value.code == engine.MCS_ENOTFOUND
    with pytest.raises(engine.EngineError) as ei:
        srv.cancel(ts[1])
    assert ei.value.code == engine.MCS_ENOTFOUND
    assert srv.poll(ts[0]) is None and srv.poll(ts[2]) is None
    srv.close()
