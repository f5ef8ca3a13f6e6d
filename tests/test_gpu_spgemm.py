"""SpGEMM on the GPU: the structural dry-run bit-exact, values within 1e-12 of the oracle."""
import ctypes

import numpy as np
import pytest

from conftest import golden, maxrel
from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _dev(capi, A: orc.OMatrix, precision=0):
    return capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im, precision=precision)


def _product(capi, A, B, prune=True, precision=0) -> orc.OMatrix:
    dA, dB = _dev(capi, A, precision), _dev(capi, B, precision)
    out = ctypes.c_void_p()
    capi.check(capi.lib().diaq_spgemm(dA.h, dB.h, 1 if prune else 0, None, ctypes.byref(out)))
    C = capi.Matrix(out)
    off, re, im = C.download()
    return orc.OMatrix(A.rows, B.cols, off, re, im)


def _symbolic(capi, A, B):
    dA, dB = _dev(capi, A), _dev(capi, B)
    out = np.empty(max(A.nd * B.nd, 1), dtype=np.int32)
    n = ctypes.c_int32()
    capi.check(capi.lib().diaq_spgemm_symbolic(dA.h, dB.h, out.ctypes.data, ctypes.byref(n), None))
    return out[: n.value]


def test_reference_cases(native):
    """The 51 hand-written cases of cpp_tests/test_main.cpp."""
    capi, _ = native
    g = golden("ref_spgemm_cases.npz")
    for i in g["case_ids"]:
        A, B = orc.OMatrix.from_dense(g[f"A{i}"]), orc.OMatrix.from_dense(g[f"B{i}"])
        C = _product(capi, A, B)
        assert np.array_equal(C.off, g[f"Coff{i}"]), i
        assert maxrel(C.to_dense(), g[f"C{i}"]) < 1e-12, i


def test_api_random(native):
    capi, _ = native
    g = golden("api_random.npz")
    for t in range(25):
        A, B = orc.OMatrix.from_dense(g[f"A{t}"]), orc.OMatrix.from_dense(g[f"B{t}"])
        C = _product(capi, A, B)
        assert np.array_equal(C.off, g[f"Coff{t}"]), t
        assert maxrel(C.to_dense(), g[f"C{t}"]) < 1e-12, t


def test_tfim12_square(native):
    capi, _ = native
    g = golden("tfim12.npz")
    H = orc.OMatrix(4096, 4096, *ham.tfim(12)[1:])
    C = _product(capi, H, H)
    assert np.array_equal(C.off, g["HH_off"]) and C.nd == 247
    assert maxrel(orc.spmv(C, g["psi"]), g["HHpsi"]) < 1e-12
    Cu = _product(capi, H, H, prune=False)
    assert np.array_equal(Cu.off, orc.spgemm_symbolic(H, H))   # device product keeps zero diagonals
    assert np.array_equal(orc.prune(Cu).off, g["HH_off"])


def test_xxz16_square_against_oracle(native):
    capi, _ = native
    N, off, re, im = ham.xxz(16)
    H = orc.OMatrix(N, N, off, re, im)
    C = _product(capi, H, H)
    W = orc.product(H, H)
    assert np.array_equal(C.off, W.off)
    assert maxrel(C.re, W.re) < 1e-12 and maxrel(C.im, W.im) < 1e-12


@pytest.mark.parametrize("seed", range(6))
def test_symbolic_bit_exact(native, seed):
    """Dry-run on the device against the oracle's sort/unique, including offsets that fall out."""
    capi, _ = native
    rng = np.random.default_rng(100 + seed)
    r, c, k = (int(x) for x in rng.integers(1, 3000, size=3))
    A = orc.OMatrix.zeros(r, c, rng.choice(np.arange(-(r - 1), c), size=min(60, r + c - 1), replace=False))
    B = orc.OMatrix.zeros(c, k, rng.choice(np.arange(-(c - 1), k), size=min(45, c + k - 1), replace=False))
    assert np.array_equal(_symbolic(capi, A, B), orc.spgemm_symbolic(A, B))


def test_rectangular_random_values(native):
    capi, _ = native
    rng = np.random.default_rng(21)
    for _ in range(10):
        r, c, k = (int(x) for x in rng.integers(1, 200, size=3))
        A = _randm(rng, r, c, int(rng.integers(1, 12)))
        B = _randm(rng, c, k, int(rng.integers(1, 12)))
        C, W = _product(capi, A, B), orc.product(A, B)
        assert np.array_equal(C.off, W.off)
        assert maxrel(C.to_dense(), W.to_dense()) < 1e-12


def test_c64_product(native):
    capi, _ = native
    N, off, re, im = ham.xxz(12)
    H = orc.OMatrix(N, N, off, re, im)
    C, W = _product(capi, H, H, precision=1), orc.product(H, H)
    assert np.array_equal(C.off, W.off)
    assert maxrel(C.re, W.re) < 1e-5


def test_dimension_mismatch(native):
    capi, _ = native
    A, B = orc.OMatrix.zeros(4, 5, [0]), orc.OMatrix.zeros(4, 5, [0])
    with pytest.raises(capi.DiaqError, match="dimension mismatch"):
        _product(capi, A, B)


def test_empty_operands(native):
    capi, _ = native
    A = orc.OMatrix.zeros(6, 6, [])
    B = orc.OMatrix(6, 6, [1], np.ones(5), np.zeros(5))
    C = _product(capi, A, B, prune=False)
    assert C.nd == 0


def _randm(rng, r, c, nd):
    offs = rng.choice(np.arange(-(r - 1), c), size=min(nd, r + c - 1), replace=False)
    tot = sum(orc.diag_len(r, c, int(d)) for d in offs)
    return orc.OMatrix(r, c, offs, rng.standard_normal(tot), rng.standard_normal(tot))


def test_full_size_xxz20_square_structure_and_norm(native):
    """Config 2's H H at full size (20 qubits: 731 result diagonals, 689 M stored values): the
    pruned offsets bit-exact and the Frobenius norm within 1e-12 of the oracle's product's -- the
    size-independent checks (the values themselves are checked at smaller sizes above)."""
    import ctypes

    capi, _ = native
    N, off, re, im = ham.xxz(20)
    H = orc.OMatrix(N, N, off, re, im)
    dH = _dev(capi, H)
    out = ctypes.c_void_p()
    capi.check(capi.lib().diaq_spgemm(dH.h, dH.h, 1, None, ctypes.byref(out)))
    C = capi.Matrix(out)
    fro = ctypes.c_double()
    capi.check(capi.lib().diaq_frobenius(C.h, ctypes.byref(fro), None))
    got_off = C.offsets()
    del C
    W = orc.product(H, H)
    assert np.array_equal(got_off, W.off)
    # numpy's pairwise sums (a sequential float64 sum of 689 M squares drifts by ~1e-11)
    want = float(np.sqrt(np.sum(W.re ** 2) + np.sum(W.im ** 2)))
    assert abs(fro.value - want) / want < 1e-12
