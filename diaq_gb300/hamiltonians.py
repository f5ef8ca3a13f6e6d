"""Spin-chain Hamiltonians in the DiaQ format, built directly from (offsets, values).

The reference builds test Hamiltonians with its Kronecker helpers (src/spKron.cpp:189-1271),
whose 32-bit flat indices overflow at 2^16 rows and more (src/diaQMatrix.hpp:455-509).  Here
every diagonal is computed from the bit pattern of its position instead, in 64-bit indices.

Qubit 0 is the most significant bit of the basis index (kron order).  A bit flip of the qubit
pair with masks m_hi > m_lo connects basis states whose index differs by +-(m_hi - m_lo); on
both diagonals +-delta the stored position j is the state with bit(m_hi) = 0 and bit(m_lo) = 1.
A single-qubit X on mask m gives diagonals +-m with the value at positions j with bit(m) = 0.

Each builder returns ``(n_rows, offsets:int32[ndiag] ascending, re:float64[], im:float64[])``
with the diagonals packed back to back, ready for ``diaq_gpu.from_diagonals`` / the C-ABI.
"""
from __future__ import annotations

import numpy as np


def _bits(n: int):
    idx = np.arange(1 << n, dtype=np.int64)
    return idx


def _bit(idx: np.ndarray, n: int, q: int) -> np.ndarray:
    return (idx >> (n - 1 - q)) & 1


def _assemble(n: int, diags: dict) -> tuple:
    N = 1 << n
    offs = sorted(diags)
    re, im = [], []
    for d in offs:
        v = diags[d]
        L = N - abs(d)
        assert v.shape == (L,), (d, v.shape, L)
        re.append(np.ascontiguousarray(v.real, dtype=np.float64))
        im.append(np.ascontiguousarray(v.imag, dtype=np.float64))
    return N, np.array(offs, dtype=np.int32), np.concatenate(re), np.concatenate(im)


def _add(diags: dict, d: int, v: np.ndarray):
    if d in diags:
        diags[d] = diags[d] + v
    else:
        diags[d] = v.astype(np.complex128)


def _x_flip(n: int, q: int, coeff: float, diags: dict):
    """coeff * X_q: diagonals +-m, value at positions with bit q = 0."""
    N = 1 << n
    m = 1 << (n - 1 - q)
    j = np.arange(N - m, dtype=np.int64)
    v = np.where(((j >> (n - 1 - q)) & 1) == 0, coeff, 0.0).astype(np.complex128)
    _add(diags, m, v)
    _add(diags, -m, v.copy())


def _pair_flip(n: int, qa: int, qb: int, coeff: float, diags: dict):
    """coeff * (sigma+ sigma- + sigma- sigma+) on qubits qa, qb (both orders)."""
    N = 1 << n
    ma, mb = 1 << (n - 1 - qa), 1 << (n - 1 - qb)
    m_hi, m_lo = max(ma, mb), min(ma, mb)
    delta = m_hi - m_lo
    j = np.arange(N - delta, dtype=np.int64)
    sel = ((j & m_hi) == 0) & ((j & m_lo) != 0)
    v = np.where(sel, coeff, 0.0).astype(np.complex128)
    _add(diags, delta, v)
    _add(diags, -delta, v.copy())


def tfim(n: int, J=1.0, h=0.7, periodic: bool = False):
    """H = -sum_i J_i Z_i Z_{i+1} - sum_i h_i X_i (open chain unless periodic).

    With scalar J = 1, h = 0.7 this is the 12-qubit transverse-field Ising chain with 25
    diagonals (0 and +-2^k)."""
    N = 1 << n
    Js = np.broadcast_to(np.asarray(J, dtype=np.float64), (n,))
    hs = np.broadcast_to(np.asarray(h, dtype=np.float64), (n,))
    idx = _bits(n)
    z = [1 - 2 * _bit(idx, n, q) for q in range(n)]
    bonds = n if periodic else n - 1
    diag = np.zeros(N, dtype=np.float64)
    for i in range(bonds):
        diag += -Js[i] * (z[i] * z[(i + 1) % n])
    diags = {0: diag.astype(np.complex128)}
    for q in range(n):
        _x_flip(n, q, -float(hs[q]), diags)
    return _assemble(n, diags)


def xxz_params(n: int, seed: int = 1):
    """J_i ~ U[0.5, 1.5] then h_i ~ U[-1, 1], both from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    J = rng.uniform(0.5, 1.5, n)
    h = rng.uniform(-1.0, 1.0, n)
    return J, h


def xxz(n: int, seed: int = 1, delta: float = 0.8, periodic: bool = True, J=None, h=None):
    """H = sum_i J_i (X_i X_{i+1} + Y_i Y_{i+1} + delta Z_i Z_{i+1}) + sum_i h_i Z_i.

    XX + YY = 2 (sigma+ sigma- + sigma- sigma+), so each bond flips an anti-aligned pair with
    amplitude 2 J_i.  Periodic n = 20 gives 41 diagonals: 0, +-2^k (k = 0..18), +-(2^19 - 1)."""
    if J is None or h is None:
        J, h = xxz_params(n, seed)
    N = 1 << n
    idx = _bits(n)
    z = [1 - 2 * _bit(idx, n, q) for q in range(n)]
    bonds = n if periodic else n - 1
    diag = np.zeros(N, dtype=np.float64)
    for i in range(bonds):
        diag += (delta * J[i]) * (z[i] * z[(i + 1) % n])
    for i in range(n):
        diag += h[i] * z[i]
    diags = {0: diag.astype(np.complex128)}
    for i in range(bonds):
        _pair_flip(n, i, (i + 1) % n, 2.0 * float(J[i]), diags)
    return _assemble(n, diags)


def random_state(N: int, seed: int = 0, k: int = 1) -> np.ndarray:
    """iid complex Gaussian entries (real parts drawn first, then imaginary), normalised.

    k > 1 draws k states one after another from the same generator: shape (k, N)."""
    rng = np.random.default_rng(seed)
    out = np.empty((k, N), dtype=np.complex128)
    for s in range(k):
        re = rng.standard_normal(N)
        im = rng.standard_normal(N)
        v = re + 1j * im
        out[s] = v / np.linalg.norm(v)
    return out[0] if k == 1 else out


def pauli_sum(n: int, terms):
    """sum_k c_k P_k for Pauli strings P_k given as (coeff, {qubit: 'X'|'Y'|'Z'}).

    Each string contributes one diagonal offset: the basis index changes by the XOR mask of its
    X/Y qubits, so the offset of position j is j ^ mask - j, which varies with j; the string is
    split into the diagonals it touches (at most 2^(#X/Y qubits) of them)."""
    N = 1 << n
    idx = np.arange(N, dtype=np.int64)
    diags = {}
    for coeff, ops in terms:
        mask = 0
        phase = np.ones(N, dtype=np.complex128)
        for q, p in ops.items():
            b = _bit(idx, n, q)
            m = 1 << (n - 1 - q)
            if p in ("X", "Y"):
                mask |= m
            if p == "Z":
                phase *= 1 - 2 * b
            elif p == "Y":
                # Y|0> = i|1>, Y|1> = -i|0>: the factor depends on the column's bit
                phase *= np.where(b == 0, 1j, -1j)
        cols = idx
        rows = idx ^ mask
        vals = coeff * phase
        d = cols - rows
        for dv in np.unique(d):
            dv = int(dv)
            sel = d == dv
            L = N - abs(dv)
            v = np.zeros(L, dtype=np.complex128)
            pos = np.where(dv >= 0, rows[sel], cols[sel])
            v[pos] = vals[sel]
            _add(diags, dv, v)
    # drop diagonals that cancelled exactly
    diags = {d: v for d, v in diags.items() if np.any(v != 0)}
    if not diags:
        diags = {0: np.zeros(N, dtype=np.complex128)}
    return _assemble(n, diags)


def pauli_masks(n: int, terms):
    """(coeffs, x_masks, z_masks) for diaq_matrix_from_pauli from (coeff, {qubit: 'X'|'Y'|'Z'})
    terms; bit p of a mask belongs to qubit n-1-p."""
    cs, xs, zs = [], [], []
    for coeff, ops in terms:
        x = z = 0
        for q, p in ops.items():
            b = 1 << (n - 1 - q)
            if p in ("X", "Y"):
                x |= b
            if p in ("Z", "Y"):
                z |= b
        cs.append(complex(coeff))
        xs.append(x)
        zs.append(z)
    return np.array(cs, dtype=np.complex128), np.array(xs, dtype=np.uint64), np.array(zs, dtype=np.uint64)


def random_pauli_terms(n: int, rng, n_strings: int, max_weight: int = 3):
    """n_strings random Pauli strings of weight 1..max_weight on distinct qubits with N(0,1)
    coefficients -- the training distribution of the learned (s, m) selector."""
    terms = []
    for _ in range(n_strings):
        w = int(rng.integers(1, max_weight + 1))
        qs = rng.choice(n, size=w, replace=False)
        ops = {int(q): "XYZ"[int(rng.integers(0, 3))] for q in qs}
        terms.append((float(rng.standard_normal()), ops))
    return terms
