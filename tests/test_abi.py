"""The C-ABI library loads and exports every symbol include/btgpu.h declares.

No compute calls: these run without a GPU.
"""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "btgpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_surface():
    syms = declared_symbols()
    for s in ("bt_ctx_create", "bt_state_alloc", "bt_apply_matrix", "bt_apply_kraus", "bt_measure_z",
              "bt_sample", "bt_expect_pauli", "bt_reduced_dm"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import bluetangle_gpu._lib as L
    lib = ctypes.CDLL(L.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes binding covers the same surface
    assert sorted(L.SIGNATURES) == declared_symbols()


def test_version_and_status_strings():
    import bluetangle_gpu._lib as L
    lib = L.lib()
    assert lib.bt_abi_version() == 1
    assert b"CPTP" in lib.bt_status_string(L.BT_ERR_NOT_CPTP)
    assert lib.bt_status_string(0) == b"ok"


def test_null_arguments_are_errors_not_crashes():
    import bluetangle_gpu._lib as L
    lib = L.lib()
    assert lib.bt_ctx_create(0, 0, None) == L.BT_ERR_BAD_ARG
    assert lib.bt_state_free(None) == 0
    assert lib.bt_apply_matrix(None, 1, None, None, 0, None, -1) == L.BT_ERR_BAD_ARG
    assert lib.bt_last_error(None)
