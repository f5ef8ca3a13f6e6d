"""The learned selector's a-posteriori check, no GPU needed: every (s, m) the check accepts meets
the tolerance on the probe state when the truncated evolution is computed exactly (dense numpy
and scipy on a 6-qubit Hamiltonian), and the check refuses what lies outside its conditions."""
import math

import numpy as np
import pytest


def _hamiltonian(seed, n=6):
    """A random Hermitian sum of Pauli strings (X, Y, Z; weight <= 3) on n qubits, dense."""
    rng = np.random.default_rng(seed)
    P = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]),
         "Z": np.diag([1.0, -1.0])}
    H = np.zeros((2 ** n, 2 ** n), complex)
    for _ in range(4 * n):
        ops = ["I"] * n
        for q in rng.choice(n, size=rng.integers(1, 4), replace=False):
            ops[q] = "XYZ"[rng.integers(3)]
        M = np.array([[1.0]])
        for o in ops:
            M = np.kron(M, P[o])
        H += rng.standard_normal() * M
    return H


def _chain_norms(H, psi, M=40):
    """||u_k||, u_k = (-i H)^k psi / k!, k = 0..M."""
    u, out = psi.copy(), [np.linalg.norm(psi)]
    for k in range(1, M + 1):
        u = (-1j / k) * (H @ u)
        out.append(np.linalg.norm(u))
    return np.array(out)


def _taylor_powers(H, t, s, m_max):
    """For m = 1..m_max: (sum_{k<=m} (-i tau H)^k / k!)^(2^s), tau = t / 2^s, by s squarings."""
    tau = t / 2 ** s
    A = -1j * tau * H
    T = np.eye(H.shape[0], dtype=complex)
    term = T.copy()
    out = []
    for k in range(1, m_max + 1):
        term = term @ A / k
        T = T + term
        P = T
        for _ in range(s):
            P = P @ P
        out.append(P)
    return out


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("t", [0.01, 0.3, 2.0])
@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_accepted_proposals_meet_the_tolerance(seed, t, tol):
    from diaq_gb300 import learn

    H = _hamiltonian(seed)
    rng = np.random.default_rng(100 + seed)
    psi = rng.standard_normal(H.shape[0]) + 1j * rng.standard_normal(H.shape[0])
    psi /= np.linalg.norm(psi)
    unorm = _chain_norms(H, psi)
    norm1 = float(np.abs(H).sum(axis=0).max())
    from scipy.linalg import expm

    exact = expm(-1j * t * H) @ psi
    accepted = 0
    for s in range(0, 8):
        ok = [m for m in range(1, 25) if learn.check(unorm, t, tol, norm1, s, m)]
        if not ok:
            continue
        powers = _taylor_powers(H, t, s, max(ok))
        for m in ok:
            accepted += 1
            # the tolerance, plus the rounding of s dense squarings in float64
            err = np.linalg.norm(powers[m - 1] @ psi - exact)
            assert err <= tol + 2 ** s * 1e-14, (s, m, err)
    assert accepted > 0


def test_check_refuses_outside_its_conditions():
    from diaq_gb300 import learn

    unorm = np.array([1.0 / math.factorial(k) for k in range(61)])   # ||H|| = 1 for every k
    assert learn.check(unorm, 0.1, 1e-6, 1.0, 0, 8)
    assert not learn.check(unorm, 0.1, 1e-6, 1.0, -1, 8)               # s out of range
    assert not learn.check(unorm, 0.1, 1e-6, 1.0, learn.S_MAX + 1, 8)
    assert not learn.check(unorm, 0.1, 1e-6, 1.0, 0, 0)                # m out of range
    assert not learn.check(unorm, 0.1, 1e-6, 1.0, 0, learn.M_MAX + 1)
    assert not learn.check(unorm, 10.0, 1.0, 1.0, 0, 3)                # tau ||H|| / (m + 2) > 1/2
    assert not learn.check(unorm, 0.1, 1e-30, 1.0, 0, 8)               # next term above tol
