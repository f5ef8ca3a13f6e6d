"""The C ABI library builds for sm_103a, loads, and exports every function include/diaq_gb300.h
declares (no GPU needed: nothing here launches a kernel)."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "diaq_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(diaq_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from diaq_gb300 import build

    build.build_lib()
    from diaq_gb300 import capi

    return capi


def test_header_declares_the_hot_path():
    names = declared()
    for must in ("diaq_matrix_create", "diaq_spmv_z", "diaq_spgemm_symbolic", "diaq_spgemm_numeric",
                 "diaq_expm_negative", "diaq_ham_sim", "diaq_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (diaq_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header(lib):
    assert sorted(lib.SIGNATURES) == declared()
    L = lib.lib()
    for name in declared():
        assert getattr(L, name) is not None
    assert b"sm_103a" in L.diaq_version()


def test_invalid_arguments_fail_without_a_gpu(lib):
    """Argument checks happen before any CUDA call, so they work on a CPU-only host."""
    import ctypes

    L = lib.lib()
    out = ctypes.c_void_p()
    st = L.diaq_matrix_create(4, 4, 1, None, None, None, 0, 0, None, ctypes.byref(out))
    assert st == 1 and b"offsets" in L.diaq_last_error()
    assert L.diaq_spmv_z(None, None, None, None, None, None) == 1
    assert L.diaq_matrix_destroy(None) == 0
    import numpy as np

    off = np.zeros(1, dtype=np.int32)
    st = L.diaq_matrix_create(1 << 31, 1 << 31, 1, off.ctypes.data, None, None, 0, 0, None, ctypes.byref(out))
    assert st == 4 and b"below 2^31" in L.diaq_last_error()   # 32-bit row indices in the kernels
    assert L.diaq_batch_set_interleaved(None, 1) == 1


def test_every_entry_point_rejects_null_arguments(lib):
    """Every function of the header called with NULL handles and pointers and zero sizes returns
    a status (DIAQ_OK for the destroy functions and empty work, else DIAQ_ERR_INVALID with a
    message) without touching memory or the GPU."""
    import ctypes

    L = lib.lib()
    not_status = {"diaq_last_error", "diaq_version", "diaq_mlp_num_params", "diaq_evolve_launches_per_step"}
    for name, (_, args) in sorted(lib.SIGNATURES.items()):
        if name in not_status:
            continue
        vals = [0.0 if a in (ctypes.c_double, ctypes.c_float) else None if a is ctypes.c_void_p else 0 for a in args]
        st = getattr(L, name)(*vals)
        if name.endswith("_destroy") or name == "diaq_spmm_dia_device":   # NULL / empty: nothing to do
            assert st == 0, name
        else:
            assert st == 1, (name, st)
            assert L.diaq_last_error(), name
