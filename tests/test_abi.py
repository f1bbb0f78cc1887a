"""The C-ABI library loads and exports every entry point declared in include/tennet.h
(CPU only: no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "tennet.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tn_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_api():
    syms = declared_symbols()
    for s in ("tn_ctx_create", "tn_env_create", "tn_env_product", "tn_env_update_position",
              "tn_env_fullsweep", "tn_svd_truncate", "tn_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(tn):
    lib = ctypes.CDLL(tn._lib.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_the_header(tn):
    assert set(declared_symbols()) <= set(tn._lib.PROTOS)


def test_no_gpu_fails_loudly(tn):
    import ctypes as C
    lib = tn._lib.load()
    h = C.c_void_p()
    rc = lib.tn_ctx_create(0, C.byref(h))
    if rc == 0:
        lib.tn_ctx_destroy(h)
        pytest.skip("a GB300 is present")
    assert rc == tn._lib.TN_E_NOGPU
    assert b"device" in lib.tn_last_error()


def test_version_string(tn):
    assert b"sm_103a" in tn._lib.load().tn_version()
