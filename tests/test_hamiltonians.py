"""The Hamiltonian builders against dense Kronecker-product constructions (CPU)."""
import numpy as np

from diaq_gb300 import hamiltonians as ham
from oracle.oracle import OMatrix

I2 = np.eye(2)
X = np.array([[0, 1], [1, 0]], complex)
Y = np.array([[0, -1j], [1j, 0]], complex)
Z = np.diag([1.0, -1.0]).astype(complex)


def op(n, ops):
    m = np.ones((1, 1), complex)
    for q in range(n):
        m = np.kron(m, ops.get(q, I2))
    return m


def dense(t):
    N, off, re, im = t
    return OMatrix(N, N, off, re, im).to_dense()


def test_tfim12_shape():
    N, off, re, im = ham.tfim(12)
    assert N == 4096 and len(off) == 25 and re.size == 94210
    assert list(off) == sorted(off)
    assert set(off) == {0} | {s * (1 << k) for k in range(12) for s in (1, -1)}


def test_tfim_matches_kron():
    n, J, h = 6, 1.0, 0.7
    want = sum(-J * op(n, {i: Z, i + 1: Z}) for i in range(n - 1)) + sum(-h * op(n, {i: X}) for i in range(n))
    assert np.abs(dense(ham.tfim(n, J, h)) - want).max() < 1e-14


def test_xxz_matches_kron():
    n = 6
    J, h = ham.xxz_params(n, 1)
    want = np.zeros((1 << n, 1 << n), complex)
    for i in range(n):
        j = (i + 1) % n
        want += J[i] * (op(n, {i: X, j: X}) + op(n, {i: Y, j: Y}) + 0.8 * op(n, {i: Z, j: Z}))
        want += h[i] * op(n, {i: Z})
    assert np.abs(dense(ham.xxz(n)) - want).max() < 1e-13


def test_xxz20_offsets():
    N, off, re, im = ham.xxz(20)
    assert N == 1 << 20 and len(off) == 41
    expect = {0, (1 << 19) - 1, -((1 << 19) - 1)} | {s * (1 << k) for k in range(19) for s in (1, -1)}
    assert set(off) == expect
    assert re.size == sum(N - abs(int(d)) for d in off)


def test_pauli_sum_matches_kron():
    n = 5
    terms = [(0.7, {0: "X", 2: "Y"}), (-1.3, {1: "Z", 3: "X", 4: "Y"}), (0.4, {2: "Y"}), (2.0, {4: "Z"})]
    want = np.zeros((1 << n, 1 << n), complex)
    conv = {"X": X, "Y": Y, "Z": Z}
    for c, ops in terms:
        want += c * op(n, {q: conv[p] for q, p in ops.items()})
    assert np.abs(dense(ham.pauli_sum(n, terms)) - want).max() < 1e-14


def test_random_state_is_normalised_and_seeded():
    a = ham.random_state(64, 0)
    b = ham.random_state(64, 0)
    assert np.array_equal(a, b) and abs(np.linalg.norm(a) - 1) < 1e-14
    rng = np.random.default_rng(0)
    v = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    assert np.allclose(a, v / np.linalg.norm(v))
