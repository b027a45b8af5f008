"""CPU tests of the C-ABI boundary: the library loads, exports every symbol
include/pimc.h declares, and rejects bad parameters before touching a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "pimc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pimc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = header_functions()
    for must in ("pimc_create", "pimc_run", "pimc_attempt_staging", "pimc_attempt_swap",
                 "pimc_eval_action", "pimc_adjoint", "pimc_get_state", "pimc_batch_run",
                 "pimc_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(engine_lib):
    from pimc._native import SIGNATURES
    names = header_functions()
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, missing
    # the ctypes signature table covers the whole header
    assert sorted(SIGNATURES) == names


def test_abi_version_and_error_text(engine_lib):
    assert engine_lib.pimc_abi_version() == 5
    assert isinstance(engine_lib.pimc_last_error(), bytes)


@pytest.mark.parametrize("bad", [dict(dim=3), dict(N=0), dict(M=2), dict(L=0.0), dict(T=-1.0),
                                 dict(lam=0.0), dict(semantics=5), dict(interactions=True),
                                 dict(interactions=True, r_a=3.0, L=4.0)])
def test_create_rejects_bad_parameters_without_gpu(engine_lib, bad):
    from pimc._native import Params
    from pimc.engine import ChainParams
    kw = dict(dim=2, N=4, M=8, L=4.0, T=1.0, lam=0.5, pair_sigma=0.5)
    kw.update(bad)
    p = ChainParams(**kw).to_c()
    h = C.c_void_p()
    rc = engine_lib.pimc_create(C.byref(p), C.byref(h))
    assert rc == -1, rc
    assert engine_lib.pimc_last_error()
    assert not h.value


def test_null_handle_calls_fail_cleanly(engine_lib):
    out = (C.c_double * 4)()
    assert engine_lib.pimc_eval_action(None, out) == -1
    assert engine_lib.pimc_run(None, 1) == -1
    assert engine_lib.pimc_destroy(None) == 0
