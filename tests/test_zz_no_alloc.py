"""diaq_ham_sim_noalloc, the allocation-free variant of the time evolution for callers that
cannot allocate device memory (plugins inside a framework that owns the GPU's memory pool,
latency-critical loops that cannot afford cudaMalloc).  Checked through the C ABI against the
existing entry point diaq_ham_sim, on two calls in a row (the scratch keeps the previous call's
contents, so the second call must not depend on them).  Collected last on purpose."""
import numpy as np
import pytest

from conftest import maxrel
from diaq_gb300 import hamiltonians as ham

pytestmark = pytest.mark.gpu


def _evolve(capi, fn, H, p, t, r, m):
    import torch

    pr = torch.from_numpy(p.real.copy()).cuda()
    pi = torch.from_numpy(p.imag.copy()).cuda()
    outr, outi = torch.empty_like(pr), torch.empty_like(pi)
    s = torch.cuda.current_stream().cuda_stream
    capi.check(fn(H.h, pr.data_ptr(), pi.data_ptr(), t, r, m, outr.data_ptr(), outi.data_ptr(), s))
    torch.cuda.synchronize()
    return (outr + 1j * outi).cpu().numpy()


def test_noalloc_matches_ham_sim_twice(native):
    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.xxz(12)
    H = capi.Matrix.create(N, N, off, re, im)
    cases = [(ham.random_state(N, 0), 0.3, 4, 15), (ham.random_state(N, 1), 0.7, 6, 20)]
    for p, t, r, m in cases:  # two calls in a row
        want = _evolve(capi, L.diaq_ham_sim, H, p, t, r, m)
        got = _evolve(capi, L.diaq_ham_sim_noalloc, H, p, t, r, m)
        assert maxrel(got, want) < 1e-12


def test_noalloc_allocates_nothing(native):
    import torch

    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.tfim(16)   # 65536 rows: the largest size the scratch holds
    H = capi.Matrix.create(N, N, off, re, im)
    p = ham.random_state(N, 3)
    pr = torch.from_numpy(p.real.copy()).cuda()
    pi = torch.from_numpy(p.imag.copy()).cuda()
    outr, outi = torch.empty_like(pr), torch.empty_like(pi)
    s = torch.cuda.current_stream().cuda_stream
    capi.check(L.diaq_ham_sim_noalloc(H.h, pr.data_ptr(), pi.data_ptr(), 0.1, 2, 10, outr.data_ptr(),
                                      outi.data_ptr(), s))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    capi.check(L.diaq_ham_sim_noalloc(H.h, pr.data_ptr(), pi.data_ptr(), 0.1, 2, 10, outr.data_ptr(),
                                      outi.data_ptr(), s))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    want = _evolve(capi, L.diaq_ham_sim, H, p, 0.1, 2, 10)
    assert maxrel((outr + 1j * outi).cpu().numpy(), want) < 1e-12


def test_noalloc_rejects_large_matrices(native):
    capi, _ = native
    L = capi.lib()
    N, off, re, im = ham.tfim(17)
    H = capi.Matrix.create(N, N, off, re, im)
    st = L.diaq_ham_sim_noalloc(H.h, 1, 1, 0.1, 1, 5, 1, 1, None)
    assert st == 1 and b"65536" in L.diaq_last_error()
