"""CPU oracle for DiaQ's diagonal-sparse hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s
cpu_baseline / reference leg, to check results.  The product (``diaq_gb300``) never imports it.

The numeric primitives are the C restatement in ``diaq_oracle.c`` (SpMV, the SpGEMM dry-run
and numeric pass, norms, the time-evolution action).  The host-side algorithms that string them
together -- the Taylor loop of the matrix exponential, scaling and squaring, ``pow``, the union
``add`` -- are restated here over those primitives, citing the reference lines they follow.

Matrices are ``OMatrix``: shape, int32 offsets in slot order and packed float64 real/imag
arrays (diagonal k at ``starts[k]``, no padding), the DiaQ device layout of
src/deviceMatrix_gpu.cu:30-55.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build() -> str:
    """Compile diaq_oracle.c (gcc, OpenMP) into oracle/_build/liboracle.so."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "diaq_oracle.c")
        ):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i64, i32, f64 = ctypes.c_int64, ctypes.c_int32, ctypes.c_double
        L.diaq_len.restype = i64
        L.diaq_len.argtypes = [i64, i64, i32]
        L.diaq_spmv.argtypes = [i64, i64, i32, P, P, P, P, P, P, P]
        L.diaq_spgemm_symbolic.restype = i32
        L.diaq_spgemm_symbolic.argtypes = [i64, i32, P, i64, i32, P, P]
        L.diaq_spgemm_numeric.argtypes = [i64, i64, i32, P, P, P, i64, i32, P, P, P, i32, P, P, P]
        L.diaq_nonzero_diags.argtypes = [i64, i64, i32, P, P, P, P]
        L.diaq_norm1_est.restype = f64
        L.diaq_norm1_est.argtypes = [i64, i64, i32, P, P, P]
        L.diaq_frobenius.restype = f64
        L.diaq_frobenius.argtypes = [i64, P, P]
        L.diaq_ham_sim.argtypes = [i64, i32, P, P, P, P, P, f64, i64, i32, i32, P, P]
        L.diaq_spmm_dia.argtypes = [P, i32, i64, i64, P, P, i64, P, i32]
        L.diaq_oracle_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def diag_len(rows: int, cols: int, d: int) -> int:
    """src/diaQMatrix.hpp:390-409 for in-range d (0 outside)."""
    if d < 0:
        n = rows + d
    elif d > 0:
        n = cols - d
    else:
        n = min(rows, cols)
    if n > rows:
        n = rows
    elif n > cols:
        n = cols
    return max(n, 0)


class OMatrix:
    """A DiaQ matrix, packed: offsets in slot order, values back to back."""

    def __init__(self, rows, cols, off, re, im):
        self.rows, self.cols = int(rows), int(cols)
        self.off = np.ascontiguousarray(off, dtype=np.int32)
        self.re = np.ascontiguousarray(re, dtype=np.float64)
        self.im = np.ascontiguousarray(im, dtype=np.float64)
        self.lens = np.array([diag_len(self.rows, self.cols, int(d)) for d in self.off], dtype=np.int64)
        self.starts = np.zeros(len(self.off), dtype=np.int64)
        if len(self.off):
            self.starts[1:] = np.cumsum(self.lens)[:-1]
        total = int(self.lens.sum())
        if self.re.size != total or self.im.size != total:
            raise ValueError(f"value arrays hold {self.re.size}/{self.im.size} values, diagonals need {total}")

    @property
    def nd(self) -> int:
        return len(self.off)

    @property
    def total(self) -> int:
        return int(self.lens.sum())

    def diag(self, k):
        s, n = int(self.starts[k]), int(self.lens[k])
        return self.re[s : s + n], self.im[s : s + n]

    def copy(self):
        return OMatrix(self.rows, self.cols, self.off.copy(), self.re.copy(), self.im.copy())

    @staticmethod
    def zeros(rows, cols, off):
        off = np.asarray(off, dtype=np.int32)
        total = sum(diag_len(rows, cols, int(d)) for d in off)
        return OMatrix(rows, cols, off, np.zeros(total), np.zeros(total))

    @staticmethod
    def from_dense(a: np.ndarray) -> "OMatrix":
        """Nonzero diagonals in ascending order (src/dense_to_diagonals.hpp:20-58)."""
        rows, cols = a.shape
        off, re, im = [], [], []
        for d in range(-(rows - 1), cols):
            v = np.diagonal(a, offset=d)
            if np.any(v != 0):
                off.append(d)
                re.append(v.real.astype(np.float64))
                im.append(v.imag.astype(np.float64))
        return OMatrix(
            rows, cols, off,
            np.concatenate(re) if re else np.zeros(0),
            np.concatenate(im) if im else np.zeros(0),
        )

    def to_dense(self) -> np.ndarray:
        a = np.zeros((self.rows, self.cols), dtype=np.complex128)
        for k, d in enumerate(self.off):
            d = int(d)
            r, i = self.diag(k)
            n = len(r)
            rr = np.arange(n) + (0 if d >= 0 else -d)
            a[rr, rr + d] = r + 1j * i
        return a


def spmv(A: OMatrix, x: np.ndarray) -> np.ndarray:
    """y = A x (src/spMV.cpp:27-322)."""
    x = np.asarray(x, dtype=np.complex128)
    xr, xi = np.ascontiguousarray(x.real), np.ascontiguousarray(x.imag)
    yr, yi = np.empty(A.rows), np.empty(A.rows)
    lib().diaq_spmv(A.rows, A.cols, A.nd, _p(A.off), _p(A.re), _p(A.im), _p(xr), _p(xi), _p(yr), _p(yi))
    return yr + 1j * yi


def spmm_dia(offsets, vals: np.ndarray, n_cols: int, B: np.ndarray) -> np.ndarray:
    """C = A B for A in the row-aligned DIA format (vals[k, r] = A[r, r + offsets[k]]), B dense
    (n_cols x R), float64 or complex128 (src/spMM_device_gpu.cu:44-127)."""
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    cplx = np.iscomplexobj(vals) or np.iscomplexobj(B)
    dt = np.complex128 if cplx else np.float64
    V = np.ascontiguousarray(vals, dtype=dt)
    Bm = np.ascontiguousarray(B, dtype=dt)
    nd, M = V.shape
    R = Bm.shape[1]
    assert Bm.shape[0] == n_cols and len(off) == nd
    C = np.empty((M, R), dtype=dt)
    lib().diaq_spmm_dia(_p(off), nd, M, n_cols, _p(V), _p(Bm), R, _p(C), 1 if cplx else 0)
    return C


def spgemm_symbolic(A: OMatrix, B: OMatrix) -> np.ndarray:
    """Ascending distinct dA+dB within range (src/spGEMM.cpp:346-369)."""
    out = np.empty(max(A.nd * B.nd, 1), dtype=np.int32)
    n = lib().diaq_spgemm_symbolic(A.rows, A.nd, _p(A.off), B.cols, B.nd, _p(B.off), _p(out))
    return out[:n].copy()


def nonzero_diags(A: OMatrix) -> np.ndarray:
    keep = np.zeros(max(A.nd, 1), dtype=np.int8)
    lib().diaq_nonzero_diags(A.rows, A.cols, A.nd, _p(A.off), _p(A.re), _p(A.im), _p(keep))
    return keep[: A.nd].astype(bool)


def prune(A: OMatrix) -> OMatrix:
    """Drop the diagonals whose values are all exactly zero (src/diaQMatrix.hpp:1543-1604)."""
    keep = nonzero_diags(A)
    if keep.all():
        return A
    idx = np.nonzero(keep)[0]
    re = [A.diag(int(k))[0] for k in idx]
    im = [A.diag(int(k))[1] for k in idx]
    return OMatrix(
        A.rows, A.cols, A.off[idx],
        np.concatenate(re) if re else np.zeros(0),
        np.concatenate(im) if im else np.zeros(0),
    )


def _check_distinct(A: OMatrix, name: str):
    if len(np.unique(A.off)) != A.nd:
        raise ValueError(f"{name}: diagonal offsets must be distinct")


def product(A: OMatrix, B: OMatrix, prune_result: bool = True) -> OMatrix:
    """C = A B.  The host entry point prunes exact-zero diagonals (src/spGEMM.cpp:516-534);
    the device-resident one does not (src/spGEMM_gpu.cu:84-151)."""
    if A.cols != B.rows:
        raise RuntimeError("diaQMatrix product_cuda: dimension mismatch.")
    _check_distinct(A, "product")
    _check_distinct(B, "product")
    offC = spgemm_symbolic(A, B)
    C = OMatrix.zeros(A.rows, B.cols, offC)
    lib().diaq_spgemm_numeric(
        A.rows, A.cols, A.nd, _p(A.off), _p(A.re), _p(A.im),
        B.cols, B.nd, _p(B.off), _p(B.re), _p(B.im),
        C.nd, _p(C.off), _p(C.re), _p(C.im),
    )
    return prune(C) if prune_result else C


def norm1_est(A: OMatrix) -> float:
    """src/diaQMatrix.hpp:1287-1358."""
    return lib().diaq_norm1_est(A.rows, A.cols, A.nd, _p(A.off), _p(A.re), _p(A.im))


def frobenius(A: OMatrix) -> float:
    """src/diaQMatrix.hpp:1255-1284."""
    return lib().diaq_frobenius(A.total, _p(A.re), _p(A.im))


def identity(n: int) -> OMatrix:
    """src/specialMatrices.hpp:9-24."""
    return OMatrix(n, n, [0], np.ones(n), np.zeros(n))


def add(A: OMatrix, B: OMatrix, sign: float = 1.0) -> OMatrix:
    """Union of the offsets, ascending; A + sign*B (src/diaQMatrix.hpp:867-916)."""
    if A.rows != B.rows or A.cols != B.cols:
        raise RuntimeError("diaQMatrix::add: shape mismatch")
    union = np.unique(np.concatenate([A.off, B.off]))
    C = OMatrix.zeros(A.rows, A.cols, union)
    sa = {int(d): k for k, d in enumerate(A.off)}
    sb = {int(d): k for k, d in enumerate(B.off)}
    for k, d in enumerate(union):
        d = int(d)
        s, n = int(C.starts[k]), int(C.lens[k])
        if d in sa and d in sb:
            ar, ai = A.diag(sa[d])
            br, bi = B.diag(sb[d])
            C.re[s : s + n] = ar + sign * br
            C.im[s : s + n] = ai + sign * bi
        elif d in sa:
            ar, ai = A.diag(sa[d])
            C.re[s : s + n] = ar
            C.im[s : s + n] = ai
        else:
            br, bi = B.diag(sb[d])
            C.re[s : s + n] = sign * br
            C.im[s : s + n] = sign * bi
    return C


def pow(A: OMatrix, n: int, prune_result: bool = True) -> OMatrix:
    """src/spPow.cpp:19-56: s squarings for n = 2^s, else binary exponentiation."""
    if n < 0:
        raise RuntimeError("pow: negative exponent not supported")
    if n == 0:
        return identity(A.rows)
    if n == 1:
        return A.copy()
    base = A.copy()
    if n & (n - 1) == 0:
        for _ in range(n.bit_length() - 1):
            base = product(base, base, prune_result)
        return base
    result = identity(A.rows)
    e = n
    while e > 0:
        if e & 1:
            result = product(result, base, prune_result)
        e >>= 1
        if e:
            base = product(base, base, prune_result)
    return result


def scaling_exponent(norm_est: float, t_abs: float, cutoff: float) -> int:
    """s = ceil(log2((|t| ||A||_1 + 1e-12) / cutoff)) when positive (src/spME.cpp:256-262)."""
    scaled = t_abs * norm_est + 1e-12
    return int(math.ceil(math.log2(scaled / cutoff))) if scaled > cutoff else 0


def expm_negative_taylor(A: OMatrix, t: float, max_it: int, tol: float, prune_result=True):
    """exp(-i t A) by its Taylor series (src/spME.cpp:158-223)."""
    result = identity(A.rows)
    if A.nd == 1:
        r, i = A.diag(0)
        tr, ti = t * r, t * i
        eb = np.exp(ti)
        res = result.copy()
        n = len(r)
        res.re[:n] = eb * np.cos(tr)
        res.im[:n] = -eb * np.sin(tr)
        return res, 0
    X = OMatrix(A.rows, A.cols, A.off, A.im * t, A.re * -t)   # copy_and_scale_by_imag(-t)
    term = identity(A.rows)
    k = 0
    for k in range(1, max_it + 1):
        term = product(term, X, prune_result)
        term = OMatrix(term.rows, term.cols, term.off, term.re / k, term.im / k)
        result = add(result, term)
        if frobenius(term) < tol:
            break
    return result, k


def expm_negative(A: OMatrix, t: float, max_iterations=100, scale_cutoff=1.0, tolerance=1e-12,
                  prune_result=True, info=None):
    """exp(-i t A) by Taylor + scaling and squaring (src/spME.cpp:230-295)."""
    if A.nd == 1:
        U, _ = expm_negative_taylor(A, t, max_iterations, tolerance, prune_result)
        return U
    s = scaling_exponent(norm1_est(A), abs(t), scale_cutoff)
    ts = math.ldexp(t, -s)
    tol_s = max(1e-15, tolerance * math.ldexp(1.0, -s))
    U, terms = expm_negative_taylor(A, ts, max_iterations, tol_s, prune_result)
    if info is not None:
        info.update(s=s, terms=terms)
    return pow(U, 1 << s, prune_result)


def expm_negative_pade(A: OMatrix, t: float, max_iterations=100, scale_cutoff=1.0, tolerance=1e-12):
    """exp(-i t A) as the reference's Pade routine computes it (src/spME.cpp:298-445).

    One diagonal: the single-diagonal exponential of :309-336 (the same rule as the Taylor path's).
    Every other input fails there, and the messages are the reference's: a rectangular matrix in
    addMatrixScaled's shape check (src/diaQMatrix.hpp:1061-1072); a square one with two or more
    diagonals when the inverse of V - U (:433, :521-589) stores its solution with set(row, col)
    into a matrix built by diaQMatrix(s, numDiags), which holds about N of the 2N - 1 diagonals
    (src/diaQMatrix.hpp:68-81, :676-688); a square one with none at the inverse of the zero
    diagonal ("Matrix is singular", thrown inside an OpenMP loop: the reference's process ends
    there).  max_iterations, scale_cutoff and tolerance only steer the series built before the
    inverse."""
    if A.nd == 1:
        U, _ = expm_negative_taylor(A, t, max_iterations, tolerance)
        return U
    if A.rows != A.cols:
        raise RuntimeError("addMatrixScaled: matrix shapes do not match")
    if A.nd == 0:
        raise RuntimeError("Matrix is singular, cannot compute inverse.")
    raise RuntimeError("set: diagonal index not present in dIndices.")


def expm(A: OMatrix, max_iterations=100, scale_cutoff=1.0, tolerance=1e-12, prune_result=True):
    """exp(A) by Taylor + scaling and squaring (src/spME.cpp:13-150)."""
    if A.nd == 1:
        r, i = A.diag(0)
        res = identity(A.rows)
        n = len(r)
        ea = np.exp(r)
        res.re[:n] = ea * np.cos(i)
        res.im[:n] = ea * np.sin(i)
        return res
    s = scaling_exponent(norm1_est(A), 1.0, scale_cutoff)
    inv = math.ldexp(1.0, -s)
    X = OMatrix(A.rows, A.cols, A.off, A.re * inv, A.im * inv)
    tol_s = max(1e-15, tolerance * inv)
    result = identity(A.rows)
    term = identity(A.rows)
    for k in range(1, max_iterations + 1):
        term = product(term, X, prune_result)
        term = OMatrix(term.rows, term.cols, term.off, term.re / k, term.im / k)
        result = add(result, term)
        if frobenius(term) < tol_s:
            break
    return pow(result, 1 << s, prune_result)


def ham_sim(H: OMatrix, psi: np.ndarray, t: float, r: int, m: int = 100, substeps: int = 1) -> np.ndarray:
    """The time-evolution action (src/spHamSim_gpu_all_fused.cu:235-277, :347): t is the total
    time, r steps of exactly m Taylor terms; ``substeps`` > 1 splits each step."""
    if H.rows != H.cols:
        raise RuntimeError("hamiltonian_simulation_cuda: H must be square")
    psi = np.asarray(psi, dtype=np.complex128)
    if psi.size != H.cols:
        raise RuntimeError("hamiltonian_simulation_cuda: psi0 dimension mismatch")
    pr, pi = np.ascontiguousarray(psi.real), np.ascontiguousarray(psi.imag)
    outr, outi = np.empty(H.rows), np.empty(H.rows)
    lib().diaq_ham_sim(H.rows, H.nd, _p(H.off), _p(H.re), _p(H.im), _p(pr), _p(pi), float(t), int(r),
                       int(m), int(substeps), _p(outr), _p(outi))
    return outr + 1j * outi


def threads() -> int:
    return lib().diaq_oracle_threads()
