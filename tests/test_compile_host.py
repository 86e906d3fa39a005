"""CPU tests of the host-side model compiler (mcs_model.cpp) and of request
admission limits, with no GPU.

mcs_server_submit() compiles a request on the calling thread (validation,
coupling classes, colouring, measurement lists, the arena image) and only
queues it; the device is touched by mcs_server_step().  So the compiler's
success on every lattice family the reference builds, and its rejection of
malformed input -- which the reference reads unchecked (PyArg_ParseTuple into
malloc'd arrays, isingLib.c:277-337, heisenbergLib.c:504-586) -- are tested
here without a device.
"""
import pytest

from tests import cases as C

EINVAL, ENOMEM, EUNSUPPORTED = 1, 4, 5


@pytest.fixture()
def server(engine):
    s = engine.Server(hbm_budget_bytes=1 << 30, max_slots=4)
    yield s
    s.close()


VALID = [
    ("ising", lambda: C.square_args("ising", 8, 2.0, h=0.1, frames=3)),
    ("ising", lambda: C.square_args("ising", 7, 2.5)),                              # odd side: 3+ colours
    ("ising", lambda: C.square_args("ising", 16, 2.4, tau=2, algo=1)),              # Wolff
    ("ising", lambda: C.square_args("ising", 32, 1.5, J=1.0, h=0.5)),               # antiferromagnet in a field
    ("ising", lambda: C.lattice_args("ising", (6, 6, 1), 2, [(0, 1, o, C.J9(-1)) for o in ((0, 0, 0), (-1, 0, 0),
                                                                                           (0, 1, 0))],
                                     3.0, S=[1.5, 1.5], ki=((0, 1), (0, 0, 0)))),  # honeycomb, S=3/2
    ("xy", lambda: C.square_args("xy", 16, 0.9, D=[0.1, -0.2, 0], h=0.2, frames=2)),
    ("xy", lambda: C.square_args("xy", 12, 1.1, tau=1, algo=1)),
    ("heisenberg", lambda: C.square_args("heisenberg", 16, 0.5, h=0.3, dmi=0.4, D=[0, 0, -0.2])),
    ("heisenberg", lambda: C.square_args("heisenberg", 9, 0.7)),
    ("heisenberg", lambda: C.honeycomb_args("heisenberg", 8, 8.0)),
    ("heisenberg", lambda: C.square_args("heisenberg", 8, 0.6, dmi=0.4, tau=1, algo=1)),
]


def test_every_lattice_family_compiles_on_the_host(engine, server):
    tickets = [server.submit(m, mk(), seed=k) for k, (m, mk) in enumerate(VALID)]
    assert len(set(tickets)) == len(VALID)
    st = server.stats()
    assert st["queued"] == len(VALID) and st["active"] == 0 and st["bytes_in_use"] == 0


def _code(engine, fn):
    with pytest.raises(engine.EngineError) as ei:
        fn()
    return ei.value


def _ising(k, v, **kw):
    a = list(C.square_args("ising", 8, 2.0, **kw))
    a[k] = v
    return tuple(a)


def _on(model, k, v, **kw):
    a = list(C.square_args(model, 8, 0.7, **kw))
    a[k] = v
    return tuple(a)


N8 = 64
BAD = [
    ("algorithm", lambda: ("ising", _ising(0, 2)), EINVAL, "algorithm"),
    ("no sites", lambda: ("ising", _ising(1, ())), EINVAL, "empty lattice"),
    ("nsweep 0", lambda: ("ising", _ising(3, 0)), EINVAL, "nsweep"),
    ("nthermal < 0", lambda: ("ising", _ising(2, -1)), EINVAL, "nthermal"),
    ("ninterval 0", lambda: ("ising", _ising(4, 0)), EINVAL, "ninterval"),
    ("maxNLinking 33", lambda: ("ising", _ising(5, 33)), EINVAL, "maxNLinking"),
    ("nlink > z", lambda: ("ising", _ising(6, (5,) + (4,) * (N8 - 1))), EINVAL, "nlink out of range"),
    ("linkedOrb past N", lambda: ("ising", _ising(8, (N8,) + tuple(C.square_args("ising", 8, 2.0)[8][1:]))),
     EINVAL, "linkedOrb index"),
    ("corrOrbPair past N", lambda: ("ising", _ising(9, (0, N8))), EINVAL, "corrOrbPair index"),
    ("rOrb past N", lambda: ("ising", _ising(11, (N8,) * len(C.square_args("ising", 8, 2.0)[11]))),
     EINVAL, "rOrb index"),
    ("rOrbCluster negative", lambda: ("ising", _ising(12, (-3,) * len(C.square_args("ising", 8, 2.0)[12]))),
     EINVAL, "rOrbCluster index"),
    ("spinFrame > nsweep", lambda: ("ising", _ising(14, 10 ** 6)), EINVAL, "spinFrame"),
    ("circuit past N", lambda: ("heisenberg", _on("heisenberg", 10, (0, 1, N8))), EINVAL, "circuit index"),
    ("group past N", lambda: ("heisenberg", _on("heisenberg", 14, (N8,) + tuple(range(1, N8)))), EINVAL,
     "orbital-group index"),
    ("nine groups", lambda: ("heisenberg", tuple(list(C.square_args("heisenberg", 8, 0.7))[:12] + [9, 1, tuple(range(9))]
                                                 + list(C.square_args("heisenberg", 8, 0.7))[15:])),
     EUNSUPPORTED, "orbital groups"),
]


@pytest.mark.parametrize("name,mk,code,msg", BAD, ids=[b[0] for b in BAD])
def test_malformed_problems_are_rejected_with_a_code_and_message(engine, server, name, mk, code, msg):
    model, args = mk()
    e = _code(engine, lambda: server.submit(model, args))
    assert e.code == code and msg in str(e), (e.code, str(e))
    assert server.stats()["queued"] == 0


def test_ising_with_five_coupling_values_is_unsupported(engine, server):
    """The Ising kernels index an integer acceptance table by the counts of
    up-neighbours per coupling class; more than four distinct coupling values
    is refused, not approximated."""
    a = list(C.square_args("ising", 8, 2.0))
    a[7] = tuple(-(1.0 + 0.1 * (k % 5)) for k in range(len(a[7])))
    e = _code(engine, lambda: server.submit("ising", tuple(a)))
    assert e.code == EUNSUPPORTED and "coupling values" in str(e)


def test_request_larger_than_the_budget_is_refused(engine):
    s = engine.Server(hbm_budget_bytes=4096, max_slots=2)
    try:
        e = _code(engine, lambda: s.submit("heisenberg", C.square_args("heisenberg", 32, 0.7)))
        assert e.code == ENOMEM and "budget" in str(e)
    finally:
        s.close()


@pytest.mark.parametrize("budget,slots", [(0, 4), (1 << 20, 0)])
def test_server_needs_a_budget_and_a_slot(engine, budget, slots):
    e = _code(engine, lambda: engine.Server(hbm_budget_bytes=budget, max_slots=slots))
    assert e.code == EINVAL


def _digest(engine, problem, template=None, **opt):
    import ctypes
    L = engine.lib()
    fn = L.mcs_test_compile_digest
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                   ctypes.POINTER(ctypes.c_int32)]
    o = engine.make_options(**opt)
    d, r = ctypes.c_uint64(), ctypes.c_int32()
    tp = ctypes.addressof(template.struct) if template is not None else None
    rc = fn(tp, ctypes.addressof(problem.struct), ctypes.addressof(o), ctypes.byref(d), ctypes.byref(r))
    assert rc == 0, L.mcs_last_error()
    return d.value, r.value


def _xy(T, **kw):
    return C.square_args("xy", 24, T, nthermal=3, nsweep=5, **kw)


TEMPLATE_CASES = [
    # (model, template problem, problem, the template's structure is taken)
    ("xy", lambda: _xy(0.6), lambda: _xy(1.3, D=[0.1, -0.05, 0], h=0.2), True),
    ("xy", lambda: _xy(0.6), lambda: tuple(list(_xy(0.9))[:15] + [0.3] + list(_xy(0.9))[16:]), True),  # flunc
    ("heisenberg", lambda: C.square_args("heisenberg", 16, 0.4, dmi=0.4, nthermal=3, nsweep=5),
     lambda: C.square_args("heisenberg", 16, 0.8, h=0.2, dmi=0.4, nthermal=7, nsweep=9, frames=3), True),
    ("heisenberg", lambda: C.honeycomb_args("heisenberg", 6, 9.0, nthermal=3, nsweep=5),
     lambda: C.honeycomb_args("heisenberg", 6, 5.0, h=0.3, nthermal=3, nsweep=5), True),
    # a different partition of the links into coupling classes (DMI on one lattice only): full compile
    ("heisenberg", lambda: C.square_args("heisenberg", 16, 0.4, nthermal=3, nsweep=5),
     lambda: C.square_args("heisenberg", 16, 0.4, dmi=0.4, nthermal=3, nsweep=5), False),
    # another lattice size: full compile
    ("xy", lambda: _xy(0.6), lambda: C.square_args("xy", 26, 0.6, nthermal=3, nsweep=5), False),
]


@pytest.mark.parametrize("k", range(len(TEMPLATE_CASES)))
@pytest.mark.parametrize("random_init", [False, True])
def test_template_compile_gives_the_bytes_of_a_full_compile(engine, k, random_init):
    """A batch compiles later O(n) replicas of a lattice it already holds from
    that replica's template.  The arena image and descriptor it uploads must
    be the bytes a full compile of the same problem gives."""
    model, mk_t, mk_p, taken = TEMPLATE_CASES[k]
    tp, pp = engine.Problem(model, mk_t()), engine.Problem(model, mk_p())
    full, r0 = _digest(engine, pp, seed=5, random_init=random_init)
    via, r1 = _digest(engine, pp, template=tp, seed=5, random_init=random_init)
    assert r0 == 0 and r1 == int(taken)
    assert via == full


def test_compile_is_deterministic_and_sees_every_input(engine):
    """The same problem compiles to the same bytes; the seed, the field and a
    coupling each change them."""
    base = engine.Problem("heisenberg", C.square_args("heisenberg", 12, 0.5, dmi=0.4, nthermal=3, nsweep=5))
    d0, _ = _digest(engine, base, seed=3)
    assert _digest(engine, base, seed=3)[0] == d0
    assert _digest(engine, base, seed=4)[0] != d0
    other = engine.Problem("heisenberg", C.square_args("heisenberg", 12, 0.5, h=0.1, dmi=0.4, nthermal=3, nsweep=5))
    assert _digest(engine, other, seed=3)[0] != d0
    other = engine.Problem("heisenberg", C.square_args("heisenberg", 12, 0.5, dmi=0.41, nthermal=3, nsweep=5))
    assert _digest(engine, other, seed=3)[0] != d0


def _compile_info(engine, model, args):
    import ctypes
    L = engine.lib()
    fn = L.mcs_test_compile_info
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    P = engine.Problem(model, args)
    o = engine.make_options()
    info = (ctypes.c_int32 * 8)()
    rc = fn(ctypes.addressof(P.struct), ctypes.addressof(o), info)
    assert rc == 0, L.mcs_last_error()
    return dict(zip(("geom", "cluster_ok", "meas_regular", "N", "Lx", "Ly", "ncol", "pair_identity"), list(info)))


ISING_CLUSTER_ELIGIBLE = [
    # square, one site type, every site its own pair, 2x2 blocks: the cluster schedule's integer frame
    ("L16", lambda: C.square_args("ising", 16, 2.4), 1),
    ("L34_odd_half", lambda: C.square_args("ising", 34, 2.3), 1),
    ("L26_field", lambda: C.square_args("ising", 26, 2.5, h=0.1), 1),
    ("L24_antiferro", lambda: C.square_args("ising", 24, 1.5, J=1.0, h=0.5), 1),
    # odd side: three colours, no square geometry
    ("L7_odd", lambda: C.square_args("ising", 7, 2.5), 0),
    # honeycomb: general neighbour lists
    ("honeycomb", lambda: C.lattice_args("ising", (6, 6, 1), 2, [(0, 1, o, C.J9(-1)) for o in ((0, 0, 0), (-1, 0, 0),
                                                                                             (0, 1, 0))],
                                         3.0, S=[1.5, 1.5], ki=((0, 1), (0, 0, 0))), 0),
]


@pytest.mark.parametrize("name,mk,ok", ISING_CLUSTER_ELIGIBLE, ids=[c[0] for c in ISING_CLUSTER_ELIGIBLE])
def test_ising_cluster_eligibility(engine, name, mk, ok):
    """The compiler offers the Ising cluster schedule only to square lattices
    with the regular renormalisation (the reference's builder lists a boundary
    chosen site's renormalised links in another order; the compiler records
    the slot of each direction for each of the four kinds of chosen site)."""
    info = _compile_info(engine, "ising", mk())
    assert info["cluster_ok"] == ok, info
