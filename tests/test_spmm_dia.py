"""spmm_dia_device (row-aligned DIA x dense, every array on the device): the oracle against dense
products on CPU, the CUDA kernel against the oracle on the GPU.  The cases are the reference's
(python_tests/test_spmm_dia_device.py:10-11), its bound 1e-13 (max |C - ref| / max |ref|)."""

import numpy as np
import pytest

from oracle import oracle as orc

CASES = [(4096, 4096, 64, [-3, -1, 0, 2, 5]), (1000, 1200, 1, [0, 7, -9]), (300, 200, 17, list(range(-40, 41, 3))),
         (64, 64, 3, list(range(-63, 64)))]


def _case(M, K, R, offs, cplx, seed=0):
    rng = np.random.default_rng(seed)
    r = np.arange(M)
    if cplx:
        V = rng.standard_normal((len(offs), M)) + 1j * rng.standard_normal((len(offs), M))
        B = rng.standard_normal((K, R)) + 1j * rng.standard_normal((K, R))
    else:
        V = rng.standard_normal((len(offs), M))
        B = rng.standard_normal((K, R))
    A = np.zeros((M, K), dtype=V.dtype)
    for k, o in enumerate(offs):
        ok = (r + o >= 0) & (r + o < K)
        V[k][~ok] = 0
        A[r[ok], r[ok] + o] += V[k][ok]
    return np.array(offs, dtype=np.int64), V, B, A


def _rel(C, ref):
    return float(np.abs(C - ref).max() / max(np.abs(ref).max(), 1e-300))


@pytest.mark.parametrize("cplx", [True, False])
@pytest.mark.parametrize("case", range(4))
def test_oracle_against_dense(case, cplx):
    M, K, R, offs = CASES[case]
    off, V, B, A = _case(M, K, R, offs, cplx)
    assert _rel(orc.spmm_dia(off, V, K, B), A @ B) < 1e-13


def test_oracle_ignores_out_of_range_entries():
    """Values stored where the column leaves [0, n_cols) do not count (src/spMM_device_gpu.cu:69-71)."""
    off = np.array([2, -1, 9], dtype=np.int64)
    V = np.arange(15, dtype=float).reshape(3, 5) + 1
    B = np.arange(8, dtype=float).reshape(4, 2)
    A = np.zeros((5, 4))
    for k, o in enumerate(off):
        for r in range(5):
            if 0 <= r + o < 4:
                A[r, r + o] += V[k, r]
    assert np.array_equal(orc.spmm_dia(off, V, 4, B), A @ B)


def _device_spmm(capi, off, V, K, B, stream_ptr=None):
    import torch

    cplx = np.iscomplexobj(V)
    dt = torch.complex128 if cplx else torch.float64
    toff = torch.from_numpy(off).cuda()
    tV = torch.from_numpy(np.ascontiguousarray(V)).to("cuda", dt)
    tB = torch.from_numpy(np.ascontiguousarray(B)).to("cuda", dt)
    M, R = V.shape[1], B.shape[1]
    tC = torch.full((M, R), float("nan"), dtype=dt, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    capi.check(capi.lib().diaq_spmm_dia_device(toff.data_ptr(), tV.data_ptr(), len(off), M, K, tB.data_ptr(), R,
                                               tC.data_ptr(), 1 if cplx else 0, s))
    torch.cuda.synchronize()
    return tC.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("cplx", [True, False])
@pytest.mark.parametrize("case", range(4))
def test_device_against_oracle(native, case, cplx):
    capi, _ = native
    M, K, R, offs = CASES[case]
    off, V, B, A = _case(M, K, R, offs, cplx, seed=case)
    assert _rel(_device_spmm(capi, off, V, K, B), orc.spmm_dia(off, V, K, B)) < 1e-13


@pytest.mark.gpu
def test_device_edges(native):
    capi, _ = native
    rng = np.random.default_rng(3)
    # unsorted offsets with a duplicate and one entirely outside the matrix; 33 right-hand columns
    off = np.array([5, -2, 0, 5, 40, -7], dtype=np.int64)
    V = rng.standard_normal((6, 31)) + 1j * rng.standard_normal((6, 31))
    B = rng.standard_normal((29, 33)) + 1j * rng.standard_normal((29, 33))
    assert _rel(_device_spmm(capi, off, V, 29, B), orc.spmm_dia(off, V, 29, B)) < 1e-13
    # no diagonals: C is zero
    C = _device_spmm(capi, np.zeros(0, dtype=np.int64), np.zeros((0, 7)), 5, rng.standard_normal((5, 3)))
    assert np.array_equal(C, np.zeros((7, 3)))
    with pytest.raises(capi.DiaqError, match="non-negative"):
        capi.check(capi.lib().diaq_spmm_dia_device(None, None, 0, -1, 4, None, 1, None, 0, None))


@pytest.mark.gpu
def test_module_binding(native):
    """The drop-in module's spmm_dia_device, called as the reference's test calls it."""
    import torch

    _, mod = native
    M, K, R, offs = CASES[2]
    off, V, B, A = _case(M, K, R, offs, True, seed=5)
    toff = torch.from_numpy(off).cuda()
    tV, tB = torch.from_numpy(V).cuda(), torch.from_numpy(B).cuda()
    tC = torch.empty(M, R, dtype=torch.complex128, device="cuda")
    mod.spmm_dia_device(toff.data_ptr(), tV.data_ptr(), len(offs), M, K, tB.data_ptr(), R, tC.data_ptr(), True,
                        torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert _rel(tC.cpu().numpy(), A @ B) < 1e-13
