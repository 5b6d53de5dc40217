"""The C-ABI library: it loads, exports every function include/muca.h
declares, and rejects bad arguments on the host (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "muca.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(muca_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def libmuca():
    from muca_gb300 import build as b
    b.build()
    import muca_gb300
    return muca_gb300.lib()


def test_header_declares_the_binding_surface():
    import muca_gb300
    decl = declared_functions()
    assert len(decl) >= 20
    assert sorted(muca_gb300.EXPORTS) == decl


def test_library_exports_every_declared_symbol(libmuca):
    for name in declared_functions():
        assert hasattr(libmuca, name), name


def test_bad_arguments_rejected_on_host(libmuca):
    import muca_gb300 as m
    for L, mode, rounds in ((1, 0, 7), (129, 0, 7), (16, 5, 7), (16, 0, 9)):
        p = m.Params(L=L, nchains=256, ndev=1, device=0, rounds=rounds, mode=mode)
        h = C.c_void_p()
        assert libmuca.muca_create(C.byref(p), C.byref(h)) == 1  # MUCA_ERR_BAD_ARG
        assert h.value is None
        assert libmuca.muca_last_error(None)


def test_null_arguments(libmuca):
    assert libmuca.muca_create(None, None) == 1
    assert libmuca.muca_destroy(None) == 0
    assert libmuca.muca_get_info(None, None) == 1
    # no context: every per-context call is a BAD_ARG, never a crash
    assert libmuca.muca_iterate_host(None, None, 0, 100, 1000, 16, 16, 0, None, None, None) == 1
    assert libmuca.muca_sweep(None, 0, 100, 1000, 16, 16) == 1
    assert libmuca.muca_update_weights(None, 0, None) == 1
    assert libmuca.muca_init_chains(None, 5, 0) == 1
    assert libmuca.muca_set_log_bracket(None, 1e30) == 1
    assert libmuca.muca_set_wait_limit(None, 1000) == 1
    assert libmuca.muca_set_test_hooks(None, 0) == 1
    # measurement calls check their arguments before any device work
    out = C.c_double()
    assert libmuca.muca_sweep_floor(0, 0, 4096, None) == 1
    assert libmuca.muca_sweep_floor(0, 7, 4096, C.byref(out)) == 1
    assert libmuca.muca_sweep_floor(0, 0, 4097, C.byref(out)) == 1
    assert libmuca.muca_sweep_floor(0, 0, 0, C.byref(out)) == 1


def test_no_gpu_fails_loudly(libmuca):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import muca_gb300 as m
    with pytest.raises(m.MucaError):
        m.Engine(16, nchains=256)
