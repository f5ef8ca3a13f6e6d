"""The diaq_gpu drop-in module, exercised the way the reference's own GPU test uses its module
(python_tests/test_device_matrix.py:20-49): banded matrices against numpy at max-rel 1e-12."""
import numpy as np
import pytest

from conftest import maxrel

pytestmark = pytest.mark.gpu


def banded(n, offsets, rng):
    A = np.zeros((n, n), complex)
    for off in offsets:
        k = np.arange(max(0, -off), min(n, n - off))
        A[k, k + off] = rng.standard_normal(len(k)) + 1j * rng.standard_normal(len(k))
    return A


def test_device_matrix_like_reference(native):
    _, d = native
    rng = np.random.default_rng(0)
    n = 2048
    A = banded(n, (-3, -1, 0, 2, 5), rng)
    B = banded(n, (-7, -2, 0, 3, 11), rng)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    dA, dB = d.to_device(d.from_numpy(A)), d.DeviceMatrix(d.from_numpy(B))
    worst = 0.0
    worst = max(worst, maxrel(d.to_numpy(dA.to_host()), A))
    worst = max(worst, maxrel(d.to_numpy_vector(d.spMV(dA, d.from_numpy_vector(x))), A @ x))
    worst = max(worst, maxrel(d.to_numpy(d.product(dA, dB).to_host()), A @ B))
    worst = max(worst, maxrel(d.to_numpy(d.product(d.product(dA, dB), dA).to_host()), A @ B @ A))
    worst = max(worst, maxrel(d.to_numpy(d.product(d.from_numpy(A), d.from_numpy(B))), A @ B))
    single = banded(n, (4,), rng)
    worst = max(worst, maxrel(d.to_numpy_vector(d.spMV(d.to_device(d.from_numpy(single)), d.from_numpy_vector(x))),
                              single @ x))
    small = banded(64, (-1, 0, 1), rng) / 4
    worst = max(worst, maxrel(d.to_numpy(d.pow(d.from_numpy(small), 7)), np.linalg.matrix_power(small, 7)))
    worst = max(worst, maxrel(d.to_numpy(d.pow(d.from_numpy(small), 8)), np.linalg.matrix_power(small, 8)))
    assert worst < 1e-12, worst
    assert dA.shape == [n, n] and dA.num_diags == 5 and dA.diagonals == [-3, -1, 0, 2, 5]


def test_spmv_device_torch_pointers(native):
    import torch

    _, d = native
    rng = np.random.default_rng(0)
    A = banded(2048, (-3, -1, 0, 2, 5), rng)
    x = rng.standard_normal(2048) + 1j * rng.standard_normal(2048)
    dA = d.to_device(d.from_numpy(A))
    xr = torch.as_tensor(x.real, device="cuda").contiguous()
    xi = torch.as_tensor(x.imag, device="cuda").contiguous()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    d.spmv_device(dA, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert maxrel((yr + 1j * yi).cpu().numpy(), A @ x) < 1e-12


def test_spmv_host_overloads_and_ntimes(native):
    _, d = native
    rng = np.random.default_rng(4)
    A = banded(300, (-2, 0, 1, 7), rng) / 3
    x = rng.standard_normal(300) + 1j * rng.standard_normal(300)
    qA, vx = d.from_numpy(A), d.from_numpy_vector(x)
    assert maxrel(d.to_numpy_vector(d.spMV(qA, vx)), A @ x) < 1e-12
    y = d.vector(300)
    d.spMV(qA, vx, y)
    assert maxrel(d.to_numpy_vector(y), A @ x) < 1e-12
    for n in (0, 1, 2, 5):
        want = np.linalg.matrix_power(A, n) @ x
        assert maxrel(d.to_numpy_vector(d.spMV_ntimes(qA, vx, n)), want) < 1e-12
    R = d.from_numpy(banded(300, (0,), rng)[:200])
    with pytest.raises(RuntimeError, match="square"):
        d.spMV_ntimes(R, vx, 2)
    with pytest.raises(RuntimeError, match="dimension mismatch"):
        d.spMV(qA, d.from_numpy_vector(x[:10]))


def test_host_matrix_api(native):
    _, d = native
    A = d.diaQMatrix([4, 6], [-1, 0, 2])
    assert A.matrix_shape == [4, 6] and A.num_diags() == 3 and A.totalLength == 3 + 4 + 4
    A.set_at_diag(2, 1, 1.5, -0.5)
    D = d.to_numpy(A)
    assert D[1, 3] == 1.5 - 0.5j
    A.pruneMatrix()
    assert A.dIndices == [2]
    S = d.diaQMatrix(8, 3)
    assert S.dIndices == [0, -1, 1]
    info = d.install_info()
    assert info["CUDA_ENABLED"] and info["GPU_ARCH"] == "sm_103a"
