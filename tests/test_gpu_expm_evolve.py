"""Matrix exponential, pow and the reference-semantics time evolution on the GPU, against the
golden fixtures from the reference and the oracle."""
import ctypes

import numpy as np
import pytest

from conftest import golden, maxrel
from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def omat(t):
    N, off, re, im = t
    return orc.OMatrix(N, N, off, re, im)


def _expm_negative(capi, A, t, prune=True, max_it=100, cutoff=1.0, tol=1e-12):
    dA = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im)
    out = ctypes.c_void_p()
    s, terms = ctypes.c_int(), ctypes.c_int()
    capi.check(capi.lib().diaq_expm_negative(dA.h, t, max_it, cutoff, tol, 1 if prune else 0, None, ctypes.byref(out),
                                             ctypes.byref(s), ctypes.byref(terms)))
    off, re, im = capi.Matrix(out).download()
    return orc.OMatrix(A.rows, A.cols, off, re, im), s.value, terms.value


@pytest.mark.parametrize("name", ["xxz6", "xxz8", "tfim8"])
def test_expm_negative_golden(native, name):
    capi, _ = native
    g = golden("expm_small.npz")
    A = {"xxz6": omat(ham.xxz(6)), "xxz8": omat(ham.xxz(8)), "tfim8": omat(ham.tfim(8))}[name]
    p = ham.random_state(A.rows, 0)
    for t in (0.3, 1.7):
        U, s, terms = _expm_negative(capi, A, t)
        assert np.array_equal(U.off, g[f"{name}_t{t}_off"])
        assert maxrel(orc.spmv(U, p), g[f"{name}_t{t}_Upsi"]) < 1e-12
        info = {}
        orc.expm_negative(A, t, info=info)
        assert (s, terms) == (info["s"], info["terms"])


def test_expm_negative_unpruned_matches_after_prune(native):
    capi, _ = native
    A = omat(ham.tfim(7))
    U, _, _ = _expm_negative(capi, A, 0.9, prune=False)
    W = orc.expm_negative(A, 0.9)
    assert np.array_equal(orc.prune(U).off, W.off)
    assert maxrel(U.to_dense(), W.to_dense()) < 1e-12


def test_tfim12_expm_golden(native):
    """The 12-qubit TFIM exponential of config 1 (the reference's CPU path takes minutes)."""
    capi, _ = native
    g = golden("tfim12.npz")
    H = omat(ham.tfim(12))
    U, s, _ = _expm_negative(capi, H, 0.1)
    assert s == 1
    assert np.array_equal(U.off, g["U_off"])
    assert maxrel(orc.spmv(U, g["psi"]), g["Upsi"]) < 1e-12


def test_hermitian_random_golden(native):
    _, d = native
    g = golden("expm_small.npz")
    for t in range(5):
        A = d.from_numpy(g[f"herm{t}"])
        assert maxrel(d.to_numpy(d.expm(A, 100, 1.0, 1e-14)), g[f"herm{t}_expm"]) < 1e-12
        assert maxrel(d.to_numpy(d.expm_negative(A, 0.3, 100, 1.0, 1e-14)), g[f"herm{t}_expmneg"]) < 1e-12


def test_pow_golden(native):
    _, d = native
    g = golden("expm_small.npz")
    for name, t in (("xxz6", ham.xxz(6)), ("tfim8", ham.tfim(8))):
        N, off, re, im = t
        A = d.from_diagonals(N, N, list(off), re * 0.25, im * 0.25)
        p = ham.random_state(N, 0)
        for n in (3, 8):
            P = d.pow(A, n)
            assert list(P.dIndices) == list(g[f"{name}_pow{n}_off"])
            PO = orc.OMatrix(N, N, P.dIndices, *P.diagonal_data()[1:])
            assert maxrel(orc.spmv(PO, p), g[f"{name}_pow{n}_Ppsi"]) < 1e-12
    A = d.from_numpy(np.diag(np.arange(1.0, 5.0)) + np.diag(np.ones(3), 1))
    assert np.allclose(d.to_numpy(d.pow(A, 0)), np.eye(4))
    with pytest.raises(RuntimeError):
        d.pow(A, -1)


def test_single_diagonal_fast_path(native):
    _, d = native
    v = np.array([0.3, -1.2, 2.0, 0.1])
    A = d.from_numpy(np.diag(v + 0.2j))
    U = d.to_numpy(d.expm_negative(A, 0.7))
    want = np.diag(np.exp(0.7 * 0.2) * (np.cos(0.7 * v) - 1j * np.sin(0.7 * v)))
    assert maxrel(U, want) < 1e-14


@pytest.mark.parametrize("name", ["tfim10", "xxz10"])
def test_ham_sim_golden(native, name):
    capi, d = native
    g = golden("ham_sim.npz")
    N, off, re, im = ham.tfim(10) if name == "tfim10" else ham.xxz(10)
    H = d.from_diagonals(N, N, list(off), re, im)
    psi0 = d.from_numpy_vector(g[f"{name}_psi0"])
    out = d.to_numpy_vector(d.hamiltonian_simulation_cuda(H, psi0, 0.5, 5, max_iterations=20))
    assert maxrel(out, g[f"{name}_t0.5_r5_m20"]) < 1e-12
    out = d.to_numpy_vector(d.hamiltonian_simulation_cuda(H, psi0, 0.2, 3))   # default 100 terms
    assert maxrel(out, g[f"{name}_t0.2_r3_m100"]) < 1e-12


def test_ham_sim_xxz20_against_oracle(native):
    """Config 2's Hamiltonian, 2 steps of dt = 0.05 with 12 terms, against the oracle."""
    _, d = native
    N, off, re, im = ham.xxz(20)
    H = orc.OMatrix(N, N, off, re, im)
    psi = ham.random_state(N, 0)
    got = d.to_numpy_vector(d.hamiltonian_simulation_cuda(d.from_diagonals(N, N, list(off), re, im),
                                                          d.from_numpy_vector(psi), 0.1, 2, 12))
    assert maxrel(got, orc.ham_sim(H, psi, 0.1, 2, 12)) < 1e-12


def test_ham_sim_edges(native):
    _, d = native
    N, off, re, im = ham.tfim(6)
    H = d.from_diagonals(N, N, list(off), re, im)
    p = ham.random_state(N, 2)
    assert np.array_equal(d.to_numpy_vector(d.hamiltonian_simulation_cuda(H, d.from_numpy_vector(p), 1.0, 0)), p)
    assert np.array_equal(d.to_numpy_vector(d.hamiltonian_simulation_cuda(H, d.from_numpy_vector(p), 1.0, 3, 0)), p)
    with pytest.raises(RuntimeError, match="psi0 dimension"):
        d.hamiltonian_simulation_cuda(H, d.from_numpy_vector(p[:5]), 1.0, 1)
    R = d.from_numpy(np.ones((3, 4), complex))
    with pytest.raises(RuntimeError, match="square"):
        d.hamiltonian_simulation_cuda(R, d.from_numpy_vector(np.ones(4, complex)), 1.0, 1)


def test_ham_sim_device_pointers(native):
    """diaq_ham_sim on device arrays, in place (psi_out == psi0), on a torch stream."""
    import torch

    capi, _ = native
    N, off, re, im = ham.xxz(12)
    H = capi.Matrix.create(N, N, off, re, im)
    p = ham.random_state(N, 4)
    pr = torch.from_numpy(p.real.copy()).cuda()
    pi = torch.from_numpy(p.imag.copy()).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        capi.check(capi.lib().diaq_ham_sim(H.h, pr.data_ptr(), pi.data_ptr(), 0.3, 4, 15, pr.data_ptr(),
                                           pi.data_ptr(), s.cuda_stream))
    s.synchronize()
    got = (pr + 1j * pi).cpu().numpy()
    assert maxrel(got, orc.ham_sim(orc.OMatrix(N, N, off, re, im), p, 0.3, 4, 15)) < 1e-12
