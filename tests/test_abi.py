"""CPU tests of the C ABI boundary: the library loads, exports every
declared symbol, and rejects malformed input before touching a GPU."""
import ctypes
import os
import re

import pytest

from tests import cases as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mcsgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char \*)\s*(mcs_\w+)\s*\(", src, re.M)))


def test_header_lists_match_python_front_end():
    import mcsolver_gb300 as eng
    assert declared_functions() == sorted(eng.ABI_FUNCTIONS)


def test_library_exports_every_declared_symbol(engine):
    L = engine.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.mcs_abi_version() == 1
    assert b"sm_103a" in L.mcs_build_info()


def test_dropin_modules_import_and_export_mcmainfunction(engine):
    for name in ("isinglib", "xylib", "heisenberglib"):
        mod = engine.load_dropin(name)
        assert callable(mod.MCMainFunction)


@pytest.mark.parametrize("mutate,msg", [
    (lambda a: a[:1] + ((),) + a[2:], "empty lattice"),
    (lambda a: a[:8] + (tuple([10 ** 6] + list(a[8][1:])),) + a[9:], "linkedOrb index out of range"),
    (lambda a: a[:9] + ((),) + a[10:], "at least one pair"),
    (lambda a: a[:4] + (0,) + a[5:], "ninterval"),
])
def test_malformed_input_is_rejected_without_gpu(engine, mutate, msg):
    """mcs_solve validates the whole problem before any device call: the
    error is MCS_EINVAL with its message, not a CUDA error."""
    args = C.square_args("ising", 8, 2.0)
    bad = mutate(args)
    with pytest.raises(engine.EngineError) as ei:
        engine.solve("ising", bad)
    assert ei.value.code == 1 and msg in str(ei.value), str(ei.value)


def test_dropin_rejects_wrong_arity(engine):
    mod = engine.load_dropin("isinglib")
    with pytest.raises(TypeError):
        mod.MCMainFunction(1, 2, 3)


def test_fp64_update_is_rejected_not_ignored(engine):
    """The engine updates spins in FP32 only; asking for FP64 updates is an
    error (compiled on the host, before any device work)."""
    import ctypes as ct
    L = engine.lib()
    P = engine.Problem("xy", C.square_args("xy", 8, 1.0))
    o = engine.make_options()
    o.fp64_update = 1
    srv = ct.c_void_p()
    assert L.mcs_server_create(0, 1 << 20, 4, ct.byref(srv)) == 0
    t = ct.c_uint64()
    rc = L.mcs_server_submit(srv, ct.byref(P.struct), ct.byref(o), ct.byref(t))
    assert rc != 0 and b"fp64_update" in L.mcs_last_error()
    L.mcs_server_destroy(srv)
