"""DIAQ_C128F2 matrices (float64 values held as float pairs, SpMV on the FP32 pipes) against the
oracle: the same 1e-12 relative bar as the float64 path, structure unchanged."""
import numpy as np
import pytest

from conftest import golden, maxrel
from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc
from test_gpu_spmv import _rand, _spmv_capi

pytestmark = pytest.mark.gpu

F2 = 2


def test_tfim12_golden(native):
    capi, _ = native
    g = golden("tfim12.npz")
    H = orc.OMatrix(4096, 4096, *ham.tfim(12)[1:])
    assert maxrel(_spmv_capi(capi, H, g["psi"], precision=F2), g["Hpsi"]) < 1e-12


def test_xxz20_against_oracle(native):
    capi, _ = native
    N, off, re, im = ham.xxz(20)
    A = orc.OMatrix(N, N, off, re, im)
    x = ham.random_state(N, 3)
    assert maxrel(_spmv_capi(capi, A, x, precision=F2), orc.spmv(A, x)) < 1e-12


@pytest.mark.parametrize("seed", range(6))
def test_random_shapes(native, seed):
    """Rectangular, sparse and dense diagonal sets, values spread over 12 decades."""
    capi, _ = native
    rng = np.random.default_rng(100 + seed)
    r, c = (int(v) for v in rng.integers(1, 700, size=2))
    A = _rand(rng, r, c, int(rng.integers(1, 40)), fill=0.8)
    scale = 10.0 ** rng.uniform(-6, 6, size=len(A.re))
    A = orc.OMatrix(r, c, A.off, A.re * scale, A.im * scale)
    x = rng.standard_normal(c) + 1j * rng.standard_normal(c)
    assert maxrel(_spmv_capi(capi, A, x, precision=F2), orc.spmv(A, x)) < 1e-12


@pytest.mark.parametrize("shift", [1, 3])
def test_unaligned_vectors(native, shift):
    """x and y start off the 16-byte boundary: the split copies of x are aligned anyway."""
    capi, _ = native
    rng = np.random.default_rng(5)
    A = _rand(rng, 333, 333, 17)
    x = rng.standard_normal(333) + 1j * rng.standard_normal(333)
    assert maxrel(_spmv_capi(capi, A, x, precision=F2, shift=shift), orc.spmv(A, x)) < 1e-12


def test_several_states(native):
    capi, _ = native
    rng = np.random.default_rng(9)
    A = _rand(rng, 257, 190, 23)
    X = rng.standard_normal((3, 190)) + 1j * rng.standard_normal((3, 190))
    got = _spmv_capi(capi, A, X, precision=F2, nrhs=3)
    for q in range(3):
        assert maxrel(got[q], orc.spmv(A, X[q])) < 1e-12


def test_download_and_convert_round_trip(native):
    """Values survive the float-pair split to ~2^-48 relative; c128 -> f2 -> c128 keeps offsets."""
    capi, _ = native
    rng = np.random.default_rng(2)
    A = _rand(rng, 120, 150, 30)
    M = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im, precision=F2)
    assert M.info()[4] == F2
    off, re, im = M.download()
    assert np.array_equal(off, A.off)
    assert np.abs(re - A.re).max() <= 2.0 ** -46 * np.abs(A.re).max()
    assert np.abs(im - A.im).max() <= 2.0 ** -46 * np.abs(A.im).max()
    D = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im)
    back = D.convert(F2).convert(capi.C128)
    off2, re2, im2 = back.download()
    assert np.array_equal(off2, A.off) and np.array_equal(re2, re) and np.array_equal(im2, im)
    c = M.copy()
    assert np.array_equal(c.download()[1], re)


def test_from_pauli(native):
    """The Pauli builder makes the float64 matrix and splits it."""
    import torch

    capi, _ = native
    n = 10
    terms = ham.random_pauli_terms(n, np.random.default_rng(8), 30)
    M = capi.Matrix.from_pauli(n, *ham.pauli_masks(n, terms), precision=F2)
    N, off, re, im = ham.pauli_sum(n, terms)
    A = orc.OMatrix(N, N, off, re, im)
    assert np.array_equal(M.offsets(), A.off)
    x = ham.random_state(N, 1)
    xr = torch.from_numpy(x.real.copy()).cuda()
    xi = torch.from_numpy(x.imag.copy()).cuda()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    s = torch.cuda.current_stream().cuda_stream
    capi.check(capi.lib().diaq_spmv_z(M.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), s))
    torch.cuda.synchronize()
    assert maxrel((yr + 1j * yi).cpu().numpy(), orc.spmv(A, x)) < 1e-12


def test_host_entry(native):
    capi, _ = native
    rng = np.random.default_rng(4)
    A = _rand(rng, 64, 64, 9)
    M = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im, precision=F2)
    x = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    xr, xi = np.ascontiguousarray(x.real), np.ascontiguousarray(x.imag)
    yr, yi = np.empty(64), np.empty(64)
    capi.check(capi.lib().diaq_spmv_host(M.h, xr.ctypes.data, xi.ctypes.data, yr.ctypes.data, yi.ctypes.data))
    assert maxrel(yr + 1j * yi, orc.spmv(A, x)) < 1e-12


def test_other_operations_refuse(native):
    capi, _ = native
    M = capi.Matrix.create(8, 8, [0, 1], np.ones(15), np.zeros(15), precision=F2)
    with pytest.raises(capi.DiaqError, match="c128"):
        M.prune()
    with pytest.raises(capi.DiaqError):
        capi.Evolve(M, 1)


@pytest.mark.parametrize("lo_exp,hi_exp", [(-6, 6), (-28, -20), (20, 36), (-28, 36)])
def test_x_over_the_split_ranges(native, lo_exp, hi_exp):
    """x spread over decades that the split of x into float pairs handles with bit operations
    (|x| in about 1e-22 .. 3e38) and with the IEEE fallback below that, zeros included: every
    element of the float-pair SpMV within 1e-12 of the float64 oracle, relative to |A| |x| of its
    row (the products' own scale: x spans many decades within one vector)."""
    capi, _ = native
    rng = np.random.default_rng(lo_exp + 100)
    N = 2048
    off = [0, 1, -3]
    lens = [N, N - 1, N - 3]
    re = np.concatenate([rng.uniform(0.5, 1.5, n) for n in lens])
    im = np.concatenate([rng.uniform(-0.5, 0.5, n) for n in lens])
    A = orc.OMatrix(N, N, off, re, im)
    A_abs = orc.OMatrix(N, N, off, np.hypot(re, im), np.zeros_like(im))
    mag = 10.0 ** rng.uniform(lo_exp, hi_exp, N)
    x = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) * mag
    x[::97] = 0
    got = _spmv_capi(capi, A, x, precision=F2)
    want = orc.spmv(A, x)
    scale = orc.spmv(A_abs, np.abs(x)).real
    ok = scale > 0
    assert np.all(np.abs(got - want)[ok] <= 1e-12 * scale[ok])
    assert np.all(got[~ok] == 0)
