"""SpMV on the GPU through the C ABI, against the oracle (1e-12 relative for c128)."""
import ctypes

import numpy as np
import pytest

from conftest import golden, maxrel
from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _rand(rng, r, c, nd, fill=1.0):
    offs = rng.choice(np.arange(-(r - 1), c), size=min(nd, r + c - 1), replace=False).astype(np.int32)
    tot = sum(orc.diag_len(r, c, int(d)) for d in offs)
    re = rng.standard_normal(tot) * (rng.random(tot) < fill)
    im = rng.standard_normal(tot) * (rng.random(tot) < fill)
    return orc.OMatrix(r, c, offs, re, im)


def _spmv_capi(capi, A: orc.OMatrix, x: np.ndarray, precision=0, nrhs=1, shift=0):
    """Device SpMV through diaq_spmv_z / diaq_spmv_c / diaq_spmm with torch device buffers.
    shift > 0 offsets x and y by that many elements from an aligned allocation."""
    import torch

    M = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im, precision=precision)
    f64 = precision != 1   # c128 and c128f2 take float64 vectors, c64 float32
    dt = torch.float64 if f64 else torch.float32
    X = np.atleast_2d(x)
    k = X.shape[0]
    xr = torch.zeros(k * A.cols + shift, dtype=dt, device="cuda")
    xi = torch.zeros_like(xr)
    xr[shift:] = torch.from_numpy(X.real.ravel().copy()).to(dt)
    xi[shift:] = torch.from_numpy(X.imag.ravel().copy()).to(dt)
    yr = torch.full((k * A.rows + shift,), float("nan"), dtype=dt, device="cuda")
    yi = torch.full_like(yr, float("nan"))
    L = capi.lib()
    s = torch.cuda.current_stream().cuda_stream
    esz = xr.element_size()
    px, pxi = xr.data_ptr() + shift * esz, xi.data_ptr() + shift * esz
    py, pyi = yr.data_ptr() + shift * esz, yi.data_ptr() + shift * esz
    if nrhs == 1 and k == 1:
        fn = L.diaq_spmv_z if f64 else L.diaq_spmv_c
        capi.check(fn(M.h, px, pxi, py, pyi, s))
    else:
        capi.check(L.diaq_spmm(M.h, k, px, pxi, A.cols, py, pyi, A.rows, s))
    torch.cuda.synchronize()
    y = (yr[shift:] + 1j * yi[shift:]).cpu().numpy().astype(np.complex128).reshape(k, A.rows)
    return y[0] if x.ndim == 1 else y


def test_tfim12_golden(native):
    capi, _ = native
    g = golden("tfim12.npz")
    H = orc.OMatrix(4096, 4096, *ham.tfim(12)[1:])
    assert maxrel(_spmv_capi(capi, H, g["psi"]), g["Hpsi"]) < 1e-12


def test_xxz20_against_oracle(native):
    capi, _ = native
    N, off, re, im = ham.xxz(20)
    H = orc.OMatrix(N, N, off, re, im)
    psi = ham.random_state(N, 0)
    assert maxrel(_spmv_capi(capi, H, psi), orc.spmv(H, psi)) < 1e-12


@pytest.mark.parametrize("shape", [(1, 1), (7, 7), (33, 17), (17, 33), (1000, 1000), (4097, 4095)])
def test_random_shapes(native, shape):
    capi, _ = native
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    for nd in (1, 3, 9):
        A = _rand(rng, *shape, nd)
        x = rng.standard_normal(shape[1]) + 1j * rng.standard_normal(shape[1])
        assert maxrel(_spmv_capi(capi, A, x), orc.spmv(A, x)) < 1e-12


def test_reference_cases(native):
    capi, _ = native
    g = golden("ref_spgemm_cases.npz")
    rng = np.random.default_rng(5)
    for i in g["case_ids"]:
        A = g[f"A{i}"]
        x = rng.standard_normal(A.shape[1]) + 1j * rng.standard_normal(A.shape[1])
        y = _spmv_capi(capi, orc.OMatrix.from_dense(A), x)
        assert maxrel(y, A @ x) < 1e-12, i


def test_unaligned_vectors(native):
    """x and y pointers off the 16-byte grid take the element-wise path."""
    capi, _ = native
    rng = np.random.default_rng(3)
    A = _rand(rng, 777, 777, 11)
    x = rng.standard_normal(777) + 1j * rng.standard_normal(777)
    want = orc.spmv(A, x)
    for shift in (1, 3):
        assert maxrel(_spmv_capi(capi, A, x, shift=shift), want) < 1e-12


def test_multi_rhs(native):
    capi, _ = native
    rng = np.random.default_rng(9)
    A = _rand(rng, 2048, 2048, 13)
    for k in (2, 3, 5, 8, 13):
        X = rng.standard_normal((k, 2048)) + 1j * rng.standard_normal((k, 2048))
        Y = _spmv_capi(capi, A, X, nrhs=k)
        for q in range(k):
            assert maxrel(Y[q], orc.spmv(A, X[q])) < 1e-12


def test_c64(native):
    """Complex-float storage and arithmetic: float32 rounding, relative 1e-5."""
    capi, _ = native
    N, off, re, im = ham.xxz(14)
    H = orc.OMatrix(N, N, off, re, im)
    psi = ham.random_state(N, 0)
    assert maxrel(_spmv_capi(capi, H, psi, precision=1), orc.spmv(H, psi)) < 1e-5
    X = np.stack([ham.random_state(N, s) for s in range(4)])
    Y = _spmv_capi(capi, H, X, precision=1, nrhs=4)
    assert maxrel(Y[3], orc.spmv(H, X[3])) < 1e-5


def test_empty_and_zero(native):
    capi, _ = native
    A = orc.OMatrix(5, 4, np.zeros(0, np.int32), np.zeros(0), np.zeros(0))
    y = _spmv_capi(capi, A, np.ones(4, complex))
    assert np.array_equal(y, np.zeros(5))
    B = orc.OMatrix.zeros(0, 0, [])
    M = capi.Matrix.create(0, 0, [], None, None)
    capi.check(capi.lib().diaq_spmv_z(M.h, None, None, None, None, None))


def test_invalid_structures_raise(native):
    capi, _ = native
    with pytest.raises(capi.DiaqError, match="outside"):
        capi.Matrix.create(4, 4, [4], np.zeros(0), np.zeros(0))
    with pytest.raises(capi.DiaqError, match="twice"):
        capi.Matrix.create(4, 4, [1, 1], np.zeros(6), np.zeros(6))
    M = capi.Matrix.create(4, 4, [0], np.ones(4), np.zeros(4), precision=1)
    with pytest.raises(capi.DiaqError, match="c128"):
        capi.check(capi.lib().diaq_spmv_z(M.h, 1, 1, 1, 1, None))


def test_roundtrip_upload_download(native):
    capi, _ = native
    rng = np.random.default_rng(1)
    A = _rand(rng, 300, 500, 17)
    M = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im)
    off, re, im = M.download()
    assert np.array_equal(off, A.off) and np.array_equal(re, A.re) and np.array_equal(im, A.im)
    C = M.copy()
    assert np.array_equal(C.download()[1], A.re)
    F = M.convert(1)
    assert np.array_equal(F.download()[1], A.re.astype(np.float32).astype(np.float64))


def test_pauli_builder_matches_host_builder(native):
    """diaq_matrix_from_pauli against the numpy builder on random strings (structure bit-exact)."""
    capi, _ = native
    rng = np.random.default_rng(17)
    for n in (3, 6, 9):
        terms = ham.random_pauli_terms(n, rng, 4 * n)
        N, off, re, im = ham.pauli_sum(n, terms)
        c, x, z = ham.pauli_masks(n, terms)
        M = capi.Matrix.from_pauli(n, c, x, z)
        goff, gre, gim = M.download()
        assert np.array_equal(goff, off)
        assert maxrel(gre + 1j * gim, re + 1j * im) < 1e-14


def test_pauli_builder_xxz(native):
    """The XXZ chain as a Pauli sum equals the direct builder."""
    capi, _ = native
    n = 10
    J, h = ham.xxz_params(n, 1)
    terms = []
    for i in range(n):
        j = (i + 1) % n
        terms += [(J[i], {i: "X", j: "X"}), (J[i], {i: "Y", j: "Y"}), (0.8 * J[i], {i: "Z", j: "Z"})]
    terms += [(h[i], {i: "Z"}) for i in range(n)]
    M = capi.Matrix.from_pauli(n, *ham.pauli_masks(n, terms))
    goff, gre, gim = M.download()
    N, off, re, im = ham.xxz(n)
    assert np.array_equal(goff, off)
    assert maxrel(gre + 1j * gim, re + 1j * im) < 1e-14
