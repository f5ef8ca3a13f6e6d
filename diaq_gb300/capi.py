"""ctypes bindings of the C ABI (include/diaq_gb300.h) of libdiaq_gb300.so.

This is how a non-pybind caller -- a test, another language's FFI -- reaches the library; the
``diaq_gpu`` module is the other way in.  Every wrapper raises ``DiaqError`` on a non-zero status
with the library's message.  The library must have been built (``python -m diaq_gb300.build``);
there is no fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libdiaq_gb300.so")

C128, C64, C128F2 = 0, 1, 2
EVOLVE_C128, EVOLVE_MIXED, EVOLVE_HORNER = 0, 1, 2
_lib = None

# name -> (restype, argtypes); mirrors include/diaq_gb300.h
P, I64, I32, F64, INT = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_int
SIGNATURES = {
    "diaq_last_error": (ctypes.c_char_p, []),
    "diaq_version": (ctypes.c_char_p, []),
    "diaq_matrix_create": (INT, [I64, I64, I32, P, P, P, INT, INT, P, P]),
    "diaq_matrix_destroy": (INT, [P]),
    "diaq_matrix_info": (INT, [P, P, P, P, P, P]),
    "diaq_matrix_offsets": (INT, [P, P]),
    "diaq_matrix_live_values": (INT, [P, P, P]),
    "diaq_matrix_download": (INT, [P, P, P, INT, P]),
    "diaq_matrix_copy": (INT, [P, P, P]),
    "diaq_matrix_convert": (INT, [P, INT, P, P]),
    "diaq_matrix_prune": (INT, [P, P, P]),
    "diaq_spmv_z": (INT, [P, P, P, P, P, P]),
    "diaq_spmv_c": (INT, [P, P, P, P, P, P]),
    "diaq_spmm": (INT, [P, INT, P, P, I64, P, P, I64, P]),
    "diaq_spmv_host": (INT, [P, P, P, P, P]),
    "diaq_spmv_ntimes_host": (INT, [P, P, P, INT, P, P]),
    "diaq_spmm_dia_device": (INT, [P, P, INT, I64, I64, P, I64, P, INT, P]),
    "diaq_matrix_from_dense": (INT, [I64, I64, P, INT, INT, P, P]),
    "diaq_matrix_to_dense": (INT, [P, P, INT, P]),
    "diaq_spgemm_symbolic": (INT, [P, P, P, P, P]),
    "diaq_spgemm_numeric": (INT, [P, P, P, P]),
    "diaq_spgemm": (INT, [P, P, INT, P, P]),
    "diaq_norm1_est": (INT, [P, P, P]),
    "diaq_frobenius": (INT, [P, P, P]),
    "diaq_pow": (INT, [P, INT, INT, P, P]),
    "diaq_expm_negative": (INT, [P, F64, INT, F64, F64, INT, P, P, P, P]),
    "diaq_expm": (INT, [P, INT, F64, F64, INT, P, P]),
    "diaq_expm_negative_pade": (INT, [P, F64, INT, F64, F64, P, P]),
    "diaq_ham_sim": (INT, [P, P, P, F64, I64, INT, P, P, P]),
    "diaq_ham_sim_host": (INT, [P, P, P, F64, I64, INT, P, P]),
    "diaq_select_sm": (INT, [F64, F64, F64, F64, INT, P, P]),
    "diaq_evolve_create": (INT, [P, INT, INT, P]),
    "diaq_evolve_destroy": (INT, [P]),
    "diaq_evolve_run": (INT, [P, P, P, I64, F64, I64, INT, INT, P]),
    "diaq_evolve_launches_per_step": (INT, [P]),
    "diaq_evolve_set_config": (INT, [P, INT, INT, INT]),
    "diaq_evolve_config": (INT, [P, P, P, P]),
    "diaq_evolve_set_renormalize": (INT, [P, INT]),
    "diaq_evolve_run_host": (INT, [P, P, P, F64, I64, INT, INT]),
    "diaq_evolve_check": (INT, [P]),
    "diaq_evolve_set_wait_limit": (INT, [P, I64]),
    "diaq_select_sm_min_cost": (INT, [F64, F64, F64, INT, INT, P, P]),
    "diaq_ham_sim_noalloc": (INT, [P, P, P, F64, I64, INT, P, P, P]),
    "diaq_matrix_from_pauli": (INT, [INT, I32, P, P, P, P, INT, P, P]),
    "diaq_batch_create": (INT, [INT, P, P, P, P, P]),
    "diaq_batch_destroy": (INT, [P]),
    "diaq_batch_run": (INT, [P, F64, P, P, I64, P]),
    "diaq_batch_set_config": (INT, [P, INT, INT]),
    "diaq_batch_config": (INT, [P, P, P, P]),
    "diaq_batch_set_horner": (INT, [P, INT]),
    "diaq_batch_set_interleaved": (INT, [P, INT]),
    "diaq_mlp_num_params": (INT, []),
    "diaq_mlp_create": (INT, [ctypes.c_uint64, P]),
    "diaq_mlp_destroy": (INT, [P]),
    "diaq_mlp_get_params": (INT, [P, P]),
    "diaq_mlp_set_params": (INT, [P, P]),
    "diaq_mlp_forward": (INT, [P, P, INT, P, P]),
    "diaq_mlp_gradient": (INT, [P, P, P, P, INT, P, P, P]),
    "diaq_mlp_train_step": (INT, [P, P, P, P, INT, ctypes.c_float, P, P]),
    "diaq_mlp_propose": (INT, [P, P, INT, P, P, P]),
}


class DiaqError(RuntimeError):
    pass


def lib():
    """Load libdiaq_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m diaq_gb300.build` (nvcc, sm_103a)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != 0:
        raise DiaqError(lib().diaq_last_error().decode())


def ptr(a) -> int:
    """Data pointer of a numpy array or a torch tensor (or an int)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def select_sm(norm1: float, tau: float, tol: float, scale_cutoff: float = 1.0, max_m: int = 100):
    """(substeps_log2, m) of the norm-bound rule (diaq_select_sm)."""
    s, m = ctypes.c_int(), ctypes.c_int()
    check(lib().diaq_select_sm(norm1, tau, tol, scale_cutoff, max_m, ctypes.byref(s), ctypes.byref(m)))
    return s.value, m.value


def select_sm_min_cost(norm1: float, tau: float, tol: float, max_s: int = 12, max_m: int = 60):
    """(substeps_log2, m) minimising 2^s * m under the same remainder bound (diaq_select_sm_min_cost)."""
    s, m = ctypes.c_int(), ctypes.c_int()
    check(lib().diaq_select_sm_min_cost(norm1, tau, tol, max_s, max_m, ctypes.byref(s), ctypes.byref(m)))
    return s.value, m.value


class Matrix:
    """Owning handle of a device matrix (diaq_matrix_t)."""

    def __init__(self, handle):
        self.h = ctypes.c_void_p(handle) if not isinstance(handle, ctypes.c_void_p) else handle

    @staticmethod
    def create(rows, cols, offsets, re=None, im=None, precision=C128, on_device=False, stream=None) -> "Matrix":
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        if re is not None and not on_device:
            re = np.ascontiguousarray(re, dtype=np.float64)
            im = np.ascontiguousarray(im, dtype=np.float64)
        out = ctypes.c_void_p()
        check(lib().diaq_matrix_create(rows, cols, len(off), off.ctypes.data, ptr(re), ptr(im),
                                       1 if on_device else 0, precision, stream, ctypes.byref(out)))
        return Matrix(out)

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.diaq_matrix_destroy(self.h)
            self.h = None

    def info(self):
        r, c, t = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        nd, p = ctypes.c_int32(), ctypes.c_int()
        check(lib().diaq_matrix_info(self.h, ctypes.byref(r), ctypes.byref(c), ctypes.byref(nd), ctypes.byref(t),
                                     ctypes.byref(p)))
        return r.value, c.value, nd.value, t.value, p.value

    def offsets(self) -> np.ndarray:
        nd = self.info()[2]
        off = np.empty(max(nd, 1), dtype=np.int32)
        check(lib().diaq_matrix_offsets(self.h, off.ctypes.data))
        return off[:nd]

    def live_values(self) -> int:
        """Stored values in 32-row tiles that hold a nonzero (what the SpMV kernels read)."""
        out = ctypes.c_int64()
        check(lib().diaq_matrix_live_values(self.h, ctypes.byref(out), None))
        return out.value

    def download(self):
        """(offsets, re, im) packed, float64, on the host."""
        rows, cols, nd, total, _ = self.info()
        re, im = np.empty(max(total, 1)), np.empty(max(total, 1))
        check(lib().diaq_matrix_download(self.h, re.ctypes.data, im.ctypes.data, 0, None))
        return self.offsets(), re[:total], im[:total]

    @staticmethod
    def from_pauli(n_qubits: int, coeffs, x_masks, z_masks, precision=C128, stream=None) -> "Matrix":
        """H = sum_k c_k P_k from Pauli strings (masks over the basis index, qubit 0 = top bit)."""
        c = np.asarray(coeffs, dtype=np.complex128)
        cr, ci = np.ascontiguousarray(c.real), np.ascontiguousarray(c.imag)
        xm = np.ascontiguousarray(x_masks, dtype=np.uint64)
        zm = np.ascontiguousarray(z_masks, dtype=np.uint64)
        out = ctypes.c_void_p()
        check(lib().diaq_matrix_from_pauli(n_qubits, len(c), cr.ctypes.data, ci.ctypes.data, xm.ctypes.data,
                                           zm.ctypes.data, precision, stream, ctypes.byref(out)))
        return Matrix(out)

    def _new(self, fn, *args) -> "Matrix":
        out = ctypes.c_void_p()
        check(fn(self.h, *args, ctypes.byref(out)))
        return Matrix(out)

    @staticmethod
    def from_dense(a, precision=C128, stream=None) -> "Matrix":
        """From a dense complex array: a numpy array (copied to the device) or a CUDA torch tensor."""
        out = ctypes.c_void_p()
        if hasattr(a, "data_ptr"):
            rows, cols = a.shape
            check(lib().diaq_matrix_from_dense(rows, cols, a.data_ptr(), 1, precision, stream, ctypes.byref(out)))
        else:
            a = np.ascontiguousarray(a, dtype=np.complex128)
            rows, cols = a.shape
            check(lib().diaq_matrix_from_dense(rows, cols, a.ctypes.data, 0, precision, stream, ctypes.byref(out)))
        return Matrix(out)

    def to_dense(self) -> np.ndarray:
        rows, cols = self.info()[:2]
        a = np.empty((rows, cols), dtype=np.complex128)
        check(lib().diaq_matrix_to_dense(self.h, a.ctypes.data, 0, None))
        return a

    def copy(self):
        return self._new(lib().diaq_matrix_copy, None)

    def convert(self, precision):
        return self._new(lib().diaq_matrix_convert, precision, None)

    def prune(self):
        return self._new(lib().diaq_matrix_prune, None)


class Evolve:
    """Owning handle of an evolution plan (diaq_evolve_t)."""

    def __init__(self, H: Matrix, nrhs: int, mode: int = EVOLVE_C128):
        self.H = H   # the plan refers to H: keep it alive
        out = ctypes.c_void_p()
        check(lib().diaq_evolve_create(H.h, nrhs, mode, ctypes.byref(out)))
        self.h = out

    def run(self, psi_re, psi_im, ld, dt, steps, substeps_log2, m, stream=None):
        check(lib().diaq_evolve_run(self.h, ptr(psi_re), ptr(psi_im), ld, dt, steps, substeps_log2, m, stream))

    def run_host(self, psi_re: np.ndarray, psi_im: np.ndarray, dt, steps, substeps_log2, m):
        """In place on host float64 arrays of nrhs*N values."""
        check(lib().diaq_evolve_run_host(self.h, psi_re.ctypes.data, psi_im.ctypes.data, dt, steps, substeps_log2, m))

    def set_config(self, states_per_block: int, rows_per_thread: int = 0, pipelined: int = 0):
        """Force a launch shape (0 states: automatic, autotuned on the next run).  pipelined: 0
        registers only, 1 cp.async pipeline, 2 / 3 / 4 shuffled state windows with an L2 prefetch of
        the matrix 4 / 8 / 0 diagonals ahead."""
        check(lib().diaq_evolve_set_config(self.h, states_per_block, rows_per_thread, int(pipelined)))

    def config(self):
        """(states per block, rows per thread) of the current shape."""
        k, v, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().diaq_evolve_config(self.h, ctypes.byref(k), ctypes.byref(v), ctypes.byref(p)))
        return k.value, v.value

    def pipelined(self) -> int:
        """The kernel variant of the current shape (0 registers, 1 cp.async, 2-4 shuffled windows)."""
        k, v, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().diaq_evolve_config(self.h, ctypes.byref(k), ctypes.byref(v), ctypes.byref(p)))
        return p.value

    def set_renormalize(self, on: bool = True):
        check(lib().diaq_evolve_set_renormalize(self.h, 1 if on else 0))

    def check(self):
        """Wait for the last run; raise if a bounded wait of a bulk-copy kernel gave up in it."""
        check(lib().diaq_evolve_check(self.h))

    def set_wait_limit(self, wait_ns: int):
        """Time bound of one device-side wait of the bulk-copy kernels, in ns (0: the default)."""
        check(lib().diaq_evolve_set_wait_limit(self.h, int(wait_ns)))

    def launches_per_step(self) -> int:
        return lib().diaq_evolve_launches_per_step(self.h)

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.diaq_evolve_destroy(self.h)
            self.h = None


class Mlp:
    """Owning handle of the (s, m) proposer network (diaq_mlp_t); tensors are torch CUDA tensors."""

    N_IN, N_S, N_M = 16, 21, 30

    def __init__(self, seed: int = 0):
        out = ctypes.c_void_p()
        check(lib().diaq_mlp_create(seed, ctypes.byref(out)))
        self.h = out
        self.n_params = lib().diaq_mlp_num_params()

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.diaq_mlp_destroy(self.h)
            self.h = None

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, dtype=np.float32)
        check(lib().diaq_mlp_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        check(lib().diaq_mlp_set_params(self.h, p.ctypes.data))

    def forward(self, X, logits, stream=None):
        check(lib().diaq_mlp_forward(self.h, ptr(X), X.shape[0], ptr(logits), stream))

    def gradient(self, X, ys, ym, grad, loss, stream=None):
        check(lib().diaq_mlp_gradient(self.h, ptr(X), ptr(ys), ptr(ym), X.shape[0], ptr(grad), ptr(loss), stream))

    def train_step(self, X, ys, ym, lr, loss=None, stream=None):
        check(lib().diaq_mlp_train_step(self.h, ptr(X), ptr(ys), ptr(ym), X.shape[0], lr, ptr(loss), stream))

    def propose(self, X, s_out, m_out, stream=None):
        check(lib().diaq_mlp_propose(self.h, ptr(X), X.shape[0], ptr(s_out), ptr(m_out), stream))


class Batch:
    """Owning handle of a batched evolution (diaq_batch_t).  Keeps the matrices and the state
    tensors (lists of torch CUDA float64 tensors, shape (nrhs_i, N_i)) alive."""

    def __init__(self, mats, psi_re, psi_im):
        self.mats, self.pr, self.pi = list(mats), list(psi_re), list(psi_im)
        n = len(self.mats)
        H = (ctypes.c_void_p * n)(*[m.h.value for m in self.mats])
        k = (ctypes.c_int * n)(*[int(t.shape[0]) for t in self.pr])
        R = (ctypes.c_void_p * n)(*[t.data_ptr() for t in self.pr])
        I = (ctypes.c_void_p * n)(*[t.data_ptr() for t in self.pi])
        out = ctypes.c_void_p()
        check(lib().diaq_batch_create(n, H, k, R, I, ctypes.byref(out)))
        self.h = out

    def run(self, dt, s, m, steps, stream=None):
        n = len(self.mats)
        sa = (ctypes.c_int * n)(*[int(x) for x in s])
        ma = (ctypes.c_int * n)(*[int(x) for x in m])
        check(lib().diaq_batch_run(self.h, dt, sa, ma, steps, stream))

    def set_config(self, states_per_launch: int, rows_per_thread: int = 0):
        check(lib().diaq_batch_set_config(self.h, states_per_launch, rows_per_thread))

    def set_horner(self, on: bool = True):
        check(lib().diaq_batch_set_horner(self.h, 1 if on else 0))

    def set_interleaved(self, on: bool = True):
        check(lib().diaq_batch_set_interleaved(self.h, 1 if on else 0))

    def config(self):
        k, v, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().diaq_batch_config(self.h, ctypes.byref(k), ctypes.byref(v), ctypes.byref(p)))
        return k.value, v.value, p.value

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value and _lib is not None:
            _lib.diaq_batch_destroy(self.h)
            self.h = None
