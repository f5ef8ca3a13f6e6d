"""ctypes access to the timing restatement of the reference's CPU scheme (oracle/diaq_timing.c,
built into oracle/_build/libtiming.so).

TEST INFRASTRUCTURE ONLY: bench.py's CPU legs time it where the reference's own CPU library cannot
be built.  It is not the parity oracle (oracle.py is).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .oracle import HERE, OMatrix, _p, build

LIB_PATH = os.path.join(HERE, "_build", "libtiming.so")
_lib = None


def _l1_bytes() -> int:
    """L1 data cache of this host in bytes (0 when unknown: the 32 KB fallback)."""
    try:
        txt = open("/sys/devices/system/cpu/cpu0/cache/index0/size").read().strip().upper()
        return int(txt[:-1]) * 1024 if txt.endswith("K") else int(txt)
    except (OSError, ValueError):
        return 0


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "diaq_timing.c")
        ):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P, i64, i32, f64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        L.diaq_timing_set_l1.argtypes = [i64, i32]
        L.diaq_timing_tile.restype = i64
        L.diaq_timing_spmv.argtypes = [i64, i32, P, P, P, P, P, P, P]
        L.diaq_timing_ham_sim.argtypes = [i64, i32, P, P, P, P, P, f64, i64, i32]
        # the SIMD width of the reference's build on this host: 8 doubles (AVX-512), 2 (NEON)
        import platform

        L.diaq_timing_set_l1(_l1_bytes(), 8 if platform.machine() == "x86_64" else 2)
        _lib = L
    return _lib


def tile() -> int:
    return int(lib().diaq_timing_tile())


def spmv(H: OMatrix, x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.complex128)
    xr, xi = np.ascontiguousarray(x.real), np.ascontiguousarray(x.imag)
    yr, yi = np.empty(H.rows), np.empty(H.rows)
    lib().diaq_timing_spmv(H.rows, H.nd, _p(H.off), _p(H.re), _p(H.im), _p(xr), _p(xi), _p(yr), _p(yi))
    return yr + 1j * yi


def ham_sim(H: OMatrix, psi: np.ndarray, dt: float, substeps: int, m: int) -> np.ndarray:
    """One time step dt of psi as `substeps` sub-steps of exactly m Taylor terms each."""
    psi = np.asarray(psi, dtype=np.complex128)
    pr, pi = np.ascontiguousarray(psi.real).copy(), np.ascontiguousarray(psi.imag).copy()
    lib().diaq_timing_ham_sim(H.rows, H.nd, _p(H.off), _p(H.re), _p(H.im), _p(pr), _p(pi), float(dt) / substeps,
                              int(substeps), int(m))
    return pr + 1j * pi
