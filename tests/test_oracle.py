"""The CPU oracle pinned against the reference: golden fixtures generated from the reference's own
CPU library (tests/golden/make_golden.py) and the reference's hand-written SpGEMM cases.
CPU only."""
import numpy as np
import pytest

from conftest import golden, maxrel
from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc
from oracle import reference as ref


def omat(t):
    N, off, re, im = t
    return orc.OMatrix(N, N, off, re, im)


def test_reference_spgemm_cases():
    """cpp_tests/test_main.cpp:35-1546: product vs the dense product, structure as the reference."""
    g = golden("ref_spgemm_cases.npz")
    ids = list(g["case_ids"])
    assert len(ids) == 51
    for i in ids:
        A, B = g[f"A{i}"], g[f"B{i}"]
        C = orc.product(orc.OMatrix.from_dense(A), orc.OMatrix.from_dense(B))
        assert np.array_equal(C.off, g[f"Coff{i}"]), i
        assert maxrel(C.to_dense(), g[f"C{i}"]) < 1e-12, i   # eps 2e-5 in the reference's checkResult
        assert maxrel(C.to_dense(), g[f"Cref{i}"]) < 1e-14, i


def test_reference_spgemm_cases_as_spmv():
    g = golden("ref_spgemm_cases.npz")
    rng = np.random.default_rng(7)
    for i in g["case_ids"]:
        A = g[f"A{i}"]
        x = rng.standard_normal(A.shape[1]) + 1j * rng.standard_normal(A.shape[1])
        y = orc.spmv(orc.OMatrix.from_dense(A), x)
        assert maxrel(y, A @ x) < 1e-14


def test_api_random():
    g = golden("api_random.npz")
    for t in range(25):
        A, B, x = g[f"A{t}"], g[f"B{t}"], g[f"x{t}"]
        oa, ob = orc.OMatrix.from_dense(A), orc.OMatrix.from_dense(B)
        C = orc.product(oa, ob)
        assert np.array_equal(C.off, g[f"Coff{t}"])
        assert maxrel(C.to_dense(), g[f"C{t}"]) < 1e-14
        assert maxrel(orc.spmv(oa, x), g[f"y{t}"]) < 1e-14
        assert maxrel(C.to_dense(), A @ B) < 1e-13


def test_tfim12_spmv_and_product():
    g = golden("tfim12.npz")
    H = omat(ham.tfim(12))
    assert np.array_equal(H.off, g["off"])
    psi = g["psi"]
    assert np.array_equal(psi, ham.random_state(4096, 0))
    assert maxrel(orc.spmv(H, psi), g["Hpsi"]) < 1e-14
    HH = orc.product(H, H)
    assert np.array_equal(HH.off, g["HH_off"]) and HH.nd == 247
    assert maxrel(orc.spmv(HH, psi), g["HHpsi"]) < 1e-14


def test_tfim12_expm_structure():
    """expm_negative(H, 0.1) at 12 qubits fills to every diagonal; the oracle agrees on s."""
    g = golden("tfim12.npz")
    assert len(g["U_off"]) == 2 * 4096 - 1
    H = omat(ham.tfim(12))
    assert orc.norm1_est(H) == pytest.approx(19.4)
    assert orc.scaling_exponent(orc.norm1_est(H), 0.1, 1.0) == 1


@pytest.mark.parametrize("name", ["xxz6", "xxz8", "tfim8"])
def test_expm_small(name):
    g = golden("expm_small.npz")
    A = {"xxz6": omat(ham.xxz(6)), "xxz8": omat(ham.xxz(8)), "tfim8": omat(ham.tfim(8))}[name]
    p = ham.random_state(A.rows, 0)
    for t in (0.3, 1.7):
        U = orc.expm_negative(A, t)
        assert np.array_equal(U.off, g[f"{name}_t{t}_off"])
        assert maxrel(orc.spmv(U, p), g[f"{name}_t{t}_Upsi"]) < 1e-12
    for n in (3, 8):
        P = orc.pow(orc.OMatrix(A.rows, A.cols, A.off, A.re * 0.25, A.im * 0.25), n)
        assert np.array_equal(P.off, g[f"{name}_pow{n}_off"])
        assert maxrel(orc.spmv(P, p), g[f"{name}_pow{n}_Ppsi"]) < 1e-12


def test_expm_hermitian_random():
    g = golden("expm_small.npz")
    for t in range(5):
        A = orc.OMatrix.from_dense(g[f"herm{t}"])
        assert maxrel(orc.expm(A, 100, 1.0, 1e-14).to_dense(), g[f"herm{t}_expm"]) < 1e-13
        assert maxrel(orc.expm_negative(A, 0.3, 100, 1.0, 1e-14).to_dense(), g[f"herm{t}_expmneg"]) < 1e-13


@pytest.mark.parametrize("name", ["tfim10", "xxz10"])
def test_ham_sim(name):
    g = golden("ham_sim.npz")
    A = omat(ham.tfim(10) if name == "tfim10" else ham.xxz(10))
    p = g[f"{name}_psi0"]
    assert maxrel(orc.ham_sim(A, p, 0.5, 5, 20), g[f"{name}_t0.5_r5_m20"]) < 1e-13
    assert maxrel(orc.ham_sim(A, p, 0.2, 3, 100), g[f"{name}_t0.2_r3_m100"]) < 1e-13


@pytest.mark.parametrize("name", ["tfim10", "xxz10"])
def test_timing_restatement_against_fixtures(name):
    """The timing restatement of the reference's CPU scheme (bench.py's CPU baseline) computes the
    same evolution as the reference's own CPU build (the fixtures) and the parity oracle, and its
    SpMV equals the oracle's to rounding, with tiles shorter than the diagonals."""
    from oracle import timing as tim

    g = golden("ham_sim.npz")
    A = omat(ham.tfim(10) if name == "tfim10" else ham.xxz(10))
    p = g[f"{name}_psi0"]
    q = p
    for _ in range(5):   # 5 steps of dt = 0.1, 20 terms each: the fixture's t = 0.5, r = 5
        q = tim.ham_sim(A, q, 0.1, 1, 20)
    assert maxrel(q, g[f"{name}_t0.5_r5_m20"]) < 1e-13
    assert maxrel(tim.ham_sim(A, p, 0.1, 4, 12), orc.ham_sim(A, p, 0.1, 1, 12, substeps=4)) < 1e-13
    assert tim.tile() < A.rows
    x = ham.random_state(A.rows, 3)
    assert maxrel(tim.spmv(A, x), orc.spmv(A, x)) < 1e-14


def test_ham_sim_edges():
    A = omat(ham.tfim(6))
    p = ham.random_state(64, 1)
    assert np.array_equal(orc.ham_sim(A, p, 1.0, 0, 10), p)   # r = 0 returns psi0
    assert np.array_equal(orc.ham_sim(A, p, 1.0, 4, 0), p)    # no terms: identity
    with pytest.raises(RuntimeError):
        orc.ham_sim(A, p[:10], 1.0, 1, 10)


def test_ham_sim_converges_to_exact():
    """Enough Taylor terms reproduce exp(-i H t) psi (scipy as an independent method)."""
    import scipy.linalg as sl

    A = omat(ham.xxz(8))
    p = ham.random_state(A.rows, 0)
    exact = sl.expm(-1j * 0.7 * A.to_dense()) @ p
    assert maxrel(orc.ham_sim(A, p, 0.7, 10, 30), exact) < 1e-12


def test_symbolic_edges():
    A = orc.OMatrix.zeros(5, 7, [-4, 0, 6])
    B = orc.OMatrix.zeros(7, 3, [-6, 2])
    out = orc.spgemm_symbolic(A, B)
    want = sorted({a + b for a in (-4, 0, 6) for b in (-6, 2) if -4 <= a + b <= 2})
    assert list(out) == want
    assert list(orc.spgemm_symbolic(orc.OMatrix.zeros(5, 7, []), B)) == []


@pytest.mark.skipif(not ref.available(), reason="reference CPU library not built here")
def test_oracle_against_reference_random():
    """Directly against the reference library, on random structures (where it was built)."""
    rng = np.random.default_rng(11)
    for _ in range(20):
        r, c, k = (int(x) for x in rng.integers(2, 40, size=3))
        A = orc.OMatrix.from_dense(_rand(rng, r, c))
        B = orc.OMatrix.from_dense(_rand(rng, c, k))
        x = rng.standard_normal(c) + 1j * rng.standard_normal(c)
        assert maxrel(orc.spmv(A, x), ref.spmv(A, x)) < 1e-14
        C1, C2 = orc.product(A, B), ref.product(A, B)
        assert np.array_equal(C1.off, C2.off)
        assert maxrel(C1.to_dense(), C2.to_dense()) < 1e-14
        assert orc.norm1_est(A) == pytest.approx(ref.norm1_est(A), rel=1e-14)


def _rand(rng, r, c):
    A = np.zeros((r, c), complex)
    for o in rng.choice(np.arange(-(r - 1), c), size=min(int(rng.integers(1, 8)), r + c - 1), replace=False):
        idx = np.arange(max(0, -o), min(r, c - o))
        A[idx, idx + o] = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    return A


def test_mlp_oracle_gradient_finite_differences():
    from oracle import mlp as omlp

    rng = np.random.default_rng(0)
    p = (rng.standard_normal(omlp.N_PARAMS) * 0.2).astype(np.float32)
    X = rng.standard_normal((9, 16))
    ys = rng.integers(0, 21, 9)
    ym = rng.integers(1, 31, 9)
    loss, g = omlp.loss_and_grad(p, X, ys, ym)
    assert loss.shape == (9,) and g.shape == (omlp.N_PARAMS,)
    pd = p.astype(np.float64)
    for idx in rng.choice(omlp.N_PARAMS, 12, replace=False):
        h = 1e-6
        pp, pm = pd.copy(), pd.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (omlp.loss_and_grad(pp, X, ys, ym)[0].mean() - omlp.loss_and_grad(pm, X, ys, ym)[0].mean()) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-7 + 1e-5 * abs(g[idx])


def _pade_inputs(g):
    names = sorted({k[: -len("_shape")] for k in g.files if k.endswith("_shape")})
    for name in names:
        rows, cols = (int(v) for v in g[f"{name}_shape"])
        A = orc.OMatrix(rows, cols, g[f"{name}_off"], g[f"{name}_re"], g[f"{name}_im"])
        yield name, A, float(g[f"{name}_t"])


def test_pade_against_reference():
    """src/spME.cpp:298-445 run on the reference's own build (tests/golden/pade.npz): one-diagonal
    results to the last bit of the fixture's libm, and the same exception messages elsewhere."""
    g = golden("pade.npz")
    seen_error = seen_value = 0
    for name, A, t in _pade_inputs(g):
        if f"{name}_error" in g.files:
            with pytest.raises(RuntimeError) as ei:
                orc.expm_negative_pade(A, t)
            assert str(ei.value) == str(g[f"{name}_error"]), name
            seen_error += 1
        else:
            U = orc.expm_negative_pade(A, t)
            assert np.array_equal(U.off, g[f"{name}_U_off"]), name
            assert maxrel(U.re + 1j * U.im, g[f"{name}_U_re"] + 1j * g[f"{name}_U_im"]) < 1e-15, name
            seen_value += 1
    assert seen_error >= 4 and seen_value >= 5
