"""Out-of-memory reporting: with DIAQ_DEVICE_ALLOC_LIMIT capping a single device allocation, the
entry points that allocate return DIAQ_ERR_OOM with a CUDA error message (the reference raises
RuntimeError("CUDA error: ...") for a failed cudaMalloc, src/cuda_check.hpp:11-18), leave nothing
half-built, and work again once the cap is lifted.  The failure is made on the host, before the
driver is asked; no GPU fault is involved."""
import ctypes

import numpy as np
import pytest

from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

OOM = 3
CAP = "DIAQ_DEVICE_ALLOC_LIMIT"


@pytest.fixture
def cap(monkeypatch):
    """Set the cap (bytes) for the test; lifted again afterwards."""

    def set_cap(nbytes):
        if nbytes is None:
            monkeypatch.delenv(CAP, raising=False)
        else:
            monkeypatch.setenv(CAP, str(int(nbytes)))

    yield set_cap
    monkeypatch.delenv(CAP, raising=False)


def _create(L, N, off, re, im):
    out = ctypes.c_void_p()
    off32 = np.ascontiguousarray(off, dtype=np.int32)
    st = L.diaq_matrix_create(N, N, len(off32), off32.ctypes.data, re.ctypes.data, im.ctypes.data, 0, 0, None,
                              ctypes.byref(out))
    return st, out


def test_matrix_create_oom_then_ok(native, cap):
    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.xxz(14)   # 29 diagonals x 16384 rows x 16 B: about 7.6 MB per plane
    cap(1 << 20)
    st, out = _create(L, N, off, re, im)
    assert st == OOM
    assert "CUDA error" in L.diaq_last_error().decode()
    cap(None)
    st, out = _create(L, N, off, re, im)
    assert st == 0
    M = capi.Matrix(out)
    o, r2, i2 = M.download()
    assert np.array_equal(o, off) and np.array_equal(r2, re) and np.array_equal(i2, im)


def test_spgemm_oom_then_ok(native, cap):
    """A and B fit under the cap, their product does not: the product reports OOM; lifted, the
    same call gives the oracle's product."""
    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.xxz(12)
    H = capi.Matrix.create(N, N, off, re, im)   # 25 diagonals: about 0.8 MB per plane
    cap(2 << 20)
    C = ctypes.c_void_p()
    assert L.diaq_spgemm(H.h, H.h, 1, None, ctypes.byref(C)) == OOM
    cap(None)
    capi.check(L.diaq_spgemm(H.h, H.h, 1, None, ctypes.byref(C)))
    C = capi.Matrix(C)
    Ho = orc.OMatrix(N, N, off, re, im)
    W = orc.product(Ho, Ho)
    o, r2, i2 = C.download()
    assert np.array_equal(o, np.asarray(W.off))
    d = max(np.abs(r2 - W.re).max(), np.abs(i2 - W.im).max())
    assert d / max(np.abs(W.re).max(), np.abs(W.im).max()) < 1e-12


def test_evolve_create_oom_then_ok(native, cap):
    """The plan's work vectors exceed the cap: OOM, no plan; lifted, a plan that evolves like the
    oracle."""
    import torch

    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.xxz(14)
    H = capi.Matrix.create(N, N, off, re, im)
    cap(1 << 20)
    E = ctypes.c_void_p()
    assert L.diaq_evolve_create(H.h, 8, capi.EVOLVE_HORNER, ctypes.byref(E)) == OOM
    assert not E.value
    cap(None)
    P = ham.random_state(N, 0, k=8)
    plan = capi.Evolve(H, 8, capi.EVOLVE_HORNER)
    pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
    pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
    plan.run(pr, pi, N, 0.05, 2, 0, 12)
    torch.cuda.synchronize()
    got = (pr + 1j * pi).cpu().numpy()
    want = orc.ham_sim(orc.OMatrix(N, N, off, re, im), P[5], 0.1, 2, 12)
    assert np.linalg.norm(got[5] - want) / np.linalg.norm(want) < 1e-6


def test_cap_ignores_bad_values(native, cap):
    """An unparsable cap is no cap."""
    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.xxz(10)
    for v in ("", "12abc"):
        import os

        os.environ[CAP] = v
        st, out = _create(L, N, off, re, im)
        assert st == 0
        L.diaq_matrix_destroy(out)
