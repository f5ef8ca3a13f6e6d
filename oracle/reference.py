"""ctypes access to the reference's own CPU code (oracle/_ref/libdiaq_ref.so).

TEST INFRASTRUCTURE ONLY.  The library is built from the reference sources by
``make -C oracle ref`` where the reference tree exists; it pins the C restatement and generates
the golden fixtures under tests/golden/.  It is absent on hosts without the reference sources.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .oracle import OMatrix, _p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libdiaq_ref.so")
# Where the reference tree lies on a host that has it: the environment variable DIAQ_REFERENCE,
# else the default below.  The one place that names it; the Makefile and the fixture script take
# it from here.
REFERENCE_ROOT = os.environ.get("DIAQ_REFERENCE", "/root/reference")


def reference_present() -> bool:
    """True where the reference's CPU sources can be compiled (its src/ directory exists)."""
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "src"))
_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        P, i64, i32, f64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_threads.restype = ctypes.c_int
        L.ref_set_threads.argtypes = [ctypes.c_int]
        L.ref_spmv.argtypes = [i64, i64, i32, P, P, P, P, P, P, P]
        L.ref_matrix_new.restype = P
        L.ref_matrix_new.argtypes = [i64, i64, i32, P, P, P]
        L.ref_matrix_free.argtypes = [P]
        L.ref_matrix_info.argtypes = [P, P, P, P, P]
        L.ref_matrix_export.argtypes = [P, P, P, P]
        L.ref_spmv_h.argtypes = [P, P, P, P, P]
        L.ref_product.restype = P
        L.ref_product.argtypes = [P, P]
        L.ref_pow.restype = P
        L.ref_pow.argtypes = [P, ctypes.c_int]
        L.ref_expm_negative.restype = P
        L.ref_expm_negative.argtypes = [P, f64, ctypes.c_int, f64, f64]
        L.ref_expm_negative_pade.restype = P
        L.ref_expm_negative_pade.argtypes = [P, f64, ctypes.c_int, f64, f64]
        L.ref_expm.restype = P
        L.ref_expm.argtypes = [P, ctypes.c_int, f64, f64]
        L.ref_norm1_est.restype = f64
        L.ref_norm1_est.argtypes = [P]
        L.ref_frobenius.restype = f64
        L.ref_frobenius.argtypes = [P]
        L.ref_ham_sim.argtypes = [P, P, P, f64, i64, ctypes.c_int, P, P]
        _lib = L
    return _lib


class RefMatrix:
    """A matrix held on the reference side (diaQMatrix built with setContiguousData)."""

    def __init__(self, handle):
        if not handle:
            raise RuntimeError(lib().ref_last_error().decode())
        self.h = handle

    @staticmethod
    def from_omatrix(A: OMatrix) -> "RefMatrix":
        return RefMatrix(lib().ref_matrix_new(A.rows, A.cols, A.nd, _p(A.off), _p(A.re), _p(A.im)))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ref_matrix_free(self.h)
            self.h = None

    def to_omatrix(self) -> OMatrix:
        rows, cols, nd, total = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64()
        lib().ref_matrix_info(self.h, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nd), ctypes.byref(total))
        off = np.empty(max(nd.value, 1), dtype=np.int32)
        re, im = np.empty(max(total.value, 1)), np.empty(max(total.value, 1))
        lib().ref_matrix_export(self.h, _p(off), _p(re), _p(im))
        return OMatrix(rows.value, cols.value, off[: nd.value], re[: total.value], im[: total.value])


def spmv(A: OMatrix, x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.complex128)
    xr, xi = np.ascontiguousarray(x.real), np.ascontiguousarray(x.imag)
    yr, yi = np.empty(A.rows), np.empty(A.rows)
    if lib().ref_spmv(A.rows, A.cols, A.nd, _p(A.off), _p(A.re), _p(A.im), _p(xr), _p(xi), _p(yr), _p(yi)):
        raise RuntimeError(lib().ref_last_error().decode())
    return yr + 1j * yi


def product(A: OMatrix, B: OMatrix) -> OMatrix:
    a, b = RefMatrix.from_omatrix(A), RefMatrix.from_omatrix(B)
    return RefMatrix(lib().ref_product(a.h, b.h)).to_omatrix()


def pow(A: OMatrix, n: int) -> OMatrix:
    a = RefMatrix.from_omatrix(A)
    return RefMatrix(lib().ref_pow(a.h, n)).to_omatrix()


def expm_negative(A: OMatrix, t, max_iterations=100, scale_cutoff=1.0, tolerance=1e-12) -> OMatrix:
    a = RefMatrix.from_omatrix(A)
    return RefMatrix(lib().ref_expm_negative(a.h, t, max_iterations, scale_cutoff, tolerance)).to_omatrix()


def expm_negative_pade(A: OMatrix, t, max_iterations=100, scale_cutoff=1.0, tolerance=1e-12) -> OMatrix:
    """src/spME.cpp:298-445; raises RuntimeError with the reference's message where it throws."""
    a = RefMatrix.from_omatrix(A)
    return RefMatrix(lib().ref_expm_negative_pade(a.h, t, max_iterations, scale_cutoff, tolerance)).to_omatrix()


def expm(A: OMatrix, max_iterations=100, scale_cutoff=1.0, tolerance=1e-12) -> OMatrix:
    a = RefMatrix.from_omatrix(A)
    return RefMatrix(lib().ref_expm(a.h, max_iterations, scale_cutoff, tolerance)).to_omatrix()


def norm1_est(A: OMatrix) -> float:
    a = RefMatrix.from_omatrix(A)   # held until the call returns
    return lib().ref_norm1_est(a.h)


def frobenius(A: OMatrix) -> float:
    a = RefMatrix.from_omatrix(A)
    return lib().ref_frobenius(a.h)


def ham_sim(H: OMatrix, psi, t, r, m=100) -> np.ndarray:
    h = RefMatrix.from_omatrix(H)
    psi = np.asarray(psi, dtype=np.complex128)
    pr, pi = np.ascontiguousarray(psi.real), np.ascontiguousarray(psi.imag)
    outr, outi = np.empty(H.rows), np.empty(H.rows)
    if lib().ref_ham_sim(h.h, _p(pr), _p(pi), float(t), int(r), int(m), _p(outr), _p(outi)):
        raise RuntimeError(lib().ref_last_error().decode())
    return outr + 1j * outi
