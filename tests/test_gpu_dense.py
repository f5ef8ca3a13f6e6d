"""Dense <-> DiaQ on the device (diaq_matrix_from_dense / diaq_matrix_to_dense) against the
oracle's restatement of from_numpy (src/dense_to_diagonals.hpp:20-58): offsets bit-exact, values
exact (c128), round trips exact."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _sparse_dense(rng, r, c, nd):
    a = np.zeros((r, c), dtype=np.complex128)
    for o in rng.choice(np.arange(-(r - 1), c), size=min(nd, r + c - 1), replace=False):
        idx = np.arange(max(0, -o), min(r, c - o))
        a[idx, idx + o] = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
        a[idx[:: 3], idx[:: 3] + o] = 0   # zeros inside a diagonal stay stored
    return a


@pytest.mark.parametrize("seed", range(5))
def test_from_dense_matches_oracle(native, seed):
    capi, _ = native
    rng = np.random.default_rng(seed)
    r, c = (int(v) for v in rng.integers(1, 300, size=2))
    a = _sparse_dense(rng, r, c, int(rng.integers(1, 25)))
    M = capi.Matrix.from_dense(a)
    want = orc.OMatrix.from_dense(a)
    off, re, im = M.download()
    assert np.array_equal(off, want.off)
    assert np.array_equal(re, want.re) and np.array_equal(im, want.im)
    assert np.array_equal(M.to_dense(), a)


def test_device_input_and_precisions(native):
    import torch

    capi, _ = native
    rng = np.random.default_rng(7)
    a = _sparse_dense(rng, 257, 129, 17)
    t = torch.from_numpy(a).cuda()
    M = capi.Matrix.from_dense(t)
    assert np.array_equal(M.to_dense(), a)
    want = orc.OMatrix.from_dense(a)
    for prec, tol in ((capi.C64, 1e-7), (capi.C128F2, 1e-14)):
        P = capi.Matrix.from_dense(t, precision=prec)
        assert P.info()[4] == prec
        assert np.array_equal(P.offsets(), want.off)
        d = P.to_dense()
        assert np.abs(d - a).max() <= tol * np.abs(a).max()


def test_reference_cases_structure(native):
    """The dense operands of the reference's SpGEMM cases (cpp_tests/test_main.cpp:35-1546)."""
    capi, _ = native
    g = golden("ref_spgemm_cases.npz")
    for i in g["case_ids"]:
        for key in (f"A{i}", f"B{i}"):
            a = g[key]
            M = capi.Matrix.from_dense(a)
            assert np.array_equal(M.offsets(), orc.OMatrix.from_dense(a).off), key
            assert np.array_equal(M.to_dense(), a), key


def test_empty_and_zero(native):
    capi, _ = native
    Z = capi.Matrix.from_dense(np.zeros((6, 4), dtype=np.complex128))
    assert Z.info()[2] == 0
    assert np.array_equal(Z.to_dense(), np.zeros((6, 4)))


def test_module_functions(native):
    """from_numpy_device / to_numpy(DeviceMatrix) in the drop-in module agree with the host path."""
    _, mod = native
    rng = np.random.default_rng(3)
    a = _sparse_dense(rng, 64, 64, 9)
    dM = mod.from_numpy_device(a)
    assert list(dM.diagonals) == list(mod.from_numpy(a).dIndices)
    assert np.array_equal(mod.to_numpy(dM), a)
    x = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    y = mod.to_numpy_vector(mod.spMV(dM, mod.from_numpy_vector(x)))
    assert np.abs(y - a @ x).max() <= 1e-13 * np.abs(a @ x).max()
