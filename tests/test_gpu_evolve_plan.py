"""Evolution plans (graph-captured steps, several states per launch): plain c128 against the
oracle at 1e-12, the mixed-precision form against the FP64 oracle at the 1e-6 bar."""
import numpy as np
import pytest

from conftest import maxrel
from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _setup(capi, n, k, mode, model="xxz"):
    import torch

    N, off, re, im = ham.xxz(n) if model == "xxz" else ham.tfim(n)
    H = capi.Matrix.create(N, N, off, re, im)
    E = capi.Evolve(H, k, mode)
    P = ham.random_state(N, 0, k=k) if k > 1 else ham.random_state(N, 0)[None, :]
    pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
    pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
    return orc.OMatrix(N, N, off, re, im), E, P, pr, pi


def _result(pr, pi):
    import torch

    torch.cuda.synchronize()
    return (pr + 1j * pi).cpu().numpy()


@pytest.mark.parametrize("sl,m", [(0, 14), (1, 9), (2, 6), (0, 1), (1, 1)])
def test_plain_matches_oracle(native, sl, m):
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 12, 3, capi.EVOLVE_C128)
    E.run(pr, pi, A.rows, 0.05, 4, sl, m)
    got = _result(pr, pi)
    for q in range(3):
        want = orc.ham_sim(A, P[q], 0.05 * 4, 4, m, substeps=1 << sl)
        assert maxrel(got[q], want) < 1e-12, q
    assert E.launches_per_step() == (1 << sl) * m   # one launch per term covers every state


def test_plain_single_state_equals_reference_rule(native):
    """nrhs = 1, no sub-steps, m = max_iterations: the reference's hamiltonian_simulation_cuda."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 1, capi.EVOLVE_C128, "tfim")
    E.run(pr, pi, A.rows, 0.1, 5, 0, 20)
    assert maxrel(_result(pr, pi)[0], orc.ham_sim(A, P[0], 0.5, 5, 20)) < 1e-12


def test_plain_many_states_chunks(native):
    """More than 8 states: launches run in chunks of 8 right-hand sides."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 11, capi.EVOLVE_C128)
    E.run(pr, pi, A.rows, 0.05, 3, 1, 8)
    got = _result(pr, pi)
    for q in (0, 7, 8, 10):
        assert maxrel(got[q], orc.ham_sim(A, P[q], 0.15, 3, 8, substeps=2)) < 1e-12


@pytest.mark.parametrize("k", [1, 4, 8])
def test_mixed_accuracy(native, k):
    """complex64 terms, compensated float sums, float64 state: within 1e-6 of the FP64 oracle
    after 20 steps of dt = 0.05 (the same (s, m))."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 12, k, capi.EVOLVE_MIXED)
    E.run(pr, pi, A.rows, 0.05, 20, 1, 12)
    got = _result(pr, pi)
    for q in range(k):
        want = orc.ham_sim(A, P[q], 1.0, 20, 12, substeps=2)
        err = np.linalg.norm(got[q] - want) / np.linalg.norm(want)
        assert err < 1e-6, (q, err)


def test_mixed_odd_launch_count(native):
    """s = 0 and odd m: the step ends with one copy so the next replay finds fp32(psi)."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 2, capi.EVOLVE_MIXED)
    E.run(pr, pi, A.rows, 0.02, 6, 0, 11)
    got = _result(pr, pi)
    want = orc.ham_sim(A, P[1], 0.12, 6, 11)
    assert np.linalg.norm(got[1] - want) / np.linalg.norm(want) < 1e-6


def test_repeated_runs_reuse_graph(native):
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 2, capi.EVOLVE_C128)
    for _ in range(3):
        E.run(pr, pi, A.rows, 0.05, 2, 0, 10)
    got = _result(pr, pi)
    assert maxrel(got[0], orc.ham_sim(A, P[0], 0.3, 6, 10)) < 1e-12


def test_graph_cache_is_bounded(native):
    """A new time step per call records a new step each time; past the plan's limit of 16 the
    recorded steps are dropped and recorded again, and every result still follows the oracle."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 2, capi.EVOLVE_C128)
    want = [P[0], P[1]]
    for i in range(20):
        dt = 0.01 + 0.001 * i
        E.run(pr, pi, A.rows, dt, 1, 0, 10)
        want = [orc.ham_sim(A, w, dt, 1, 10) for w in want]
    got = _result(pr, pi)
    for q in range(2):
        assert maxrel(got[q], want[q]) < 1e-12, q


@pytest.mark.parametrize("mode", ["c128", "horner"])
def test_run_host_calls_in_a_row(native, mode):
    """diaq_evolve_run_host keeps its device copy of the states between calls: two calls in a row
    (2 then 3 steps) equal 5 steps of the oracle (c128: 1e-12; the float32 Horner form: the 1e-6
    bar)."""
    capi, _ = native
    N, off, re, im = ham.xxz(10)
    A = orc.OMatrix(N, N, off, re, im)
    H = capi.Matrix.create(N, N, off, re, im)
    E = capi.Evolve(H, 3, capi.EVOLVE_C128 if mode == "c128" else capi.EVOLVE_HORNER)
    P = ham.random_state(N, 0, k=3)
    hr = np.ascontiguousarray(P.real).ravel().copy()
    hi = np.ascontiguousarray(P.imag).ravel().copy()
    E.run_host(hr, hi, 0.05, 2, 1, 9)
    E.run_host(hr, hi, 0.05, 3, 1, 9)
    got = (hr + 1j * hi).reshape(3, N)
    for q in range(3):
        want = orc.ham_sim(A, P[q], 0.25, 5, 9, substeps=2)
        tol = 1e-12 if mode == "c128" else 1e-6
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < tol, q


@pytest.mark.parametrize("mode,k,renorm", [("horner", 8, False), ("mixed", 8, True), ("horner", 10, True),
                                           ("horner", 16, False)])
def test_run_host_single_steps_split_same_bits(native, mode, k, renorm):
    """One step per diaq_evolve_run_host call of 8 or more float32-term states runs as two half
    plans overlapping the copies with the run: the same bits as the same steps on device buffers
    through diaq_evolve_run (one step per call), and within the 1e-6 bar of the oracle."""
    import torch

    capi, _ = native
    N, off, re, im = ham.xxz(12)
    A = orc.OMatrix(N, N, off, re, im)
    H = capi.Matrix.create(N, N, off, re, im)
    md = capi.EVOLVE_HORNER if mode == "horner" else capi.EVOLVE_MIXED
    P = ham.random_state(N, 1, k=k)
    Eh, Ed = capi.Evolve(H, k, md), capi.Evolve(H, k, md)
    for E in (Eh, Ed):
        E.set_config(4, 1, 12)
        E.set_renormalize(renorm)
    hr = np.ascontiguousarray(P.real).ravel().copy()
    hi = np.ascontiguousarray(P.imag).ravel().copy()
    pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
    pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
    for i in range(3):
        dt = 0.04 + 0.01 * i
        Eh.run_host(hr, hi, dt, 1, 0, 11)
        Ed.run(pr, pi, N, dt, 1, 0, 11)
    got = (hr + 1j * hi).reshape(k, N)
    assert np.array_equal(got, _result(pr, pi))
    for q in (0, k // 2, k - 1):
        want = P[q]
        for i in range(3):
            want = orc.ham_sim(A, want, 0.04 + 0.01 * i, 1, 11)
            if renorm:
                want = want / np.linalg.norm(want)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6, q


def test_plan_rejects_bad_input(native):
    capi, _ = native
    M = capi.Matrix.create(4, 6, [0], np.ones(4), np.zeros(4))
    with pytest.raises(capi.DiaqError, match="square"):
        capi.Evolve(M, 1)
    S = capi.Matrix.create(4, 4, [0], np.ones(4), np.zeros(4), precision=capi.C64)
    with pytest.raises(capi.DiaqError, match="c128"):
        capi.Evolve(S, 1)
    A, E, P, pr, pi = _setup(capi, 6, 1, capi.EVOLVE_C128)
    E.run(pr, pi, A.rows, 0.05, 1, 0, 8)
    with pytest.raises(capi.DiaqError, match="finite"):   # never a replay of the 0.05 step
        E.run(pr, pi, A.rows, float("nan"), 1, 0, 8)


@pytest.mark.parametrize("cfg", [(8, 1, 0), (8, 2, 0), (8, 4, 0), (4, 2, 0), (4, 4, 0), (2, 4, 0), (1, 4, 0),
                                 (1, 1, 0), (8, 4, 1), (4, 4, 1), (2, 4, 1), (1, 4, 1),
                                 (8, 4, 2), (4, 4, 2), (2, 4, 2), (1, 4, 2), (8, 4, 3), (4, 4, 3), (8, 4, 4),
                                 (2, 4, 4), (4, 1, 6), (4, 1, 7), (4, 1, 8), (4, 1, 9)])
def test_mixed_every_launch_shape(native, cfg):
    """Each (states per launch, rows per thread, pipelined) shape the autotuner may pick gives
    the same answer (3 states: the last launch of a chunked shape runs with masked slots)."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 11, 3, capi.EVOLVE_MIXED)
    E.set_config(*cfg)
    assert E.config() == cfg[:2] and E.pipelined() == cfg[2]
    E.run(pr, pi, A.rows, 0.05, 5, 0, 13)
    got = _result(pr, pi)
    for q in range(3):
        want = orc.ham_sim(A, P[q], 0.25, 5, 13)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6


@pytest.mark.parametrize("cfg", [(8, 1, 0), (8, 2, 0), (4, 2, 0), (2, 2, 0), (1, 2, 0), (1, 1, 0)])
def test_plain_every_launch_shape(native, cfg):
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 5, capi.EVOLVE_C128)
    E.set_config(*cfg)
    E.run(pr, pi, A.rows, 0.05, 3, 1, 9)
    got = _result(pr, pi)
    for q in (0, 4):
        assert maxrel(got[q], orc.ham_sim(A, P[q], 0.15, 3, 9, substeps=2)) < 1e-12


@pytest.mark.parametrize("n", [3, 7, 16])
@pytest.mark.parametrize("variant", [2, 3, 4])
def test_prefetch_kernel_edges(native, n, variant):
    """The L2-prefetch kernel: 8-row matrices (every strip partial), 7 qubits (one warp strip of
    128 rows, offsets +-1, +-2 with shuffled windows), 16 qubits (many blocks, all offsets)."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, n, 3, capi.EVOLVE_MIXED)
    E.set_config(4, 4, variant)
    E.run(pr, pi, A.rows, 0.05, 3, 0, 11)
    got = _result(pr, pi)
    for q in range(3):
        want = orc.ham_sim(A, P[q], 0.15, 3, 11)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6


@pytest.mark.parametrize("variant", [6, 7, 9, 10, 11, 12])
@pytest.mark.parametrize("k,sl,m,renorm", [(5, 0, 11, False), (5, 1, 7, True), (8, 0, 12, False), (3, 2, 5, True),
                                            (12, 0, 9, False), (20, 1, 6, True)])
def test_interleaved_states(native, k, sl, m, renorm, variant):
    """The interleaved kernels (states in tiles of 32 rows x 4, padded to a power of two): odd and
    even launch counts, sub-steps, renormalisation, padding states, 1 to 8 warps per row block."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 11, k, capi.EVOLVE_MIXED)
    E.set_config(4, 1, variant)
    E.set_renormalize(renorm)
    E.run(pr, pi, A.rows, 0.05, 4, sl, m)
    got = _result(pr, pi)
    for q in range(k):
        want = orc.ham_sim(A, P[q], 0.2, 4, m, substeps=1 << sl)
        if renorm:
            want = orc.ham_sim(A, P[q], 0.05, 1, m, substeps=1 << sl)
            for _ in range(3):
                want = want / np.linalg.norm(want)
                want = orc.ham_sim(A, want, 0.05, 1, m, substeps=1 << sl)
            want = want / np.linalg.norm(want)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6, q


@pytest.mark.parametrize("cfg", [(8, 4, 0), (2, 4, 0), (4, 2, 0), (8, 1, 0), (4, 1, 6), (4, 1, 8), (4, 1, 9), (4, 1, 10),
                                 (4, 1, 11), (4, 1, 12)])
@pytest.mark.parametrize("sl,m", [(0, 12), (1, 7), (0, 1)])
def test_horner_accuracy(native, cfg, sl, m):
    """Horner-form float32 evaluation: within 1e-6 of the FP64 oracle after 20 steps, every
    launch shape, with sub-steps and the one-term case (whose launch reads and refreshes fp32(psi))."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 12, 5, capi.EVOLVE_HORNER)
    E.set_config(*cfg)
    dt = 0.05 if m > 1 else 0.002
    E.run(pr, pi, A.rows, dt, 20, sl, m)
    got = _result(pr, pi)
    for q in range(5):
        want = orc.ham_sim(A, P[q], dt * 20, 20, m, substeps=1 << sl)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6, q


@pytest.mark.parametrize("layout", [0, 6])
def test_horner_renormalize(native, layout):
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 4, capi.EVOLVE_HORNER)
    E.set_config(4, 4 if layout == 0 else 1, layout)
    E.set_renormalize(True)
    E.run(pr, pi, A.rows, 0.1, 3, 0, 8)
    got = _result(pr, pi)
    assert np.abs(np.linalg.norm(got, axis=1) - 1).max() < 1e-12
    want = P[2]
    for _ in range(3):
        want = orc.ham_sim(A, want, 0.1, 1, 8)
        want = want / np.linalg.norm(want)
    assert np.linalg.norm(got[2] - want) < 1e-6


def test_autotuner_caches_its_choice(native, tmp_path, monkeypatch):
    capi, _ = native
    cache = tmp_path / "autotune.json"
    monkeypatch.setenv("DIAQ_AUTOTUNE_CACHE", str(cache))
    A, E, P, pr, pi = _setup(capi, 12, 4, capi.EVOLVE_MIXED)
    E.run(pr, pi, A.rows, 0.05, 2, 0, 12)
    k, v = E.config()
    assert k in (1, 2, 4) and v in (1, 2, 4)
    import json

    saved = json.load(open(cache))
    assert any(val[:2] == [k, v] for val in saved.values())
    # the tuning ran on scratch copies: the states advanced exactly 2 steps
    got = _result(pr, pi)
    want = orc.ham_sim(A, P[2], 0.1, 2, 12)
    assert np.linalg.norm(got[2] - want) / np.linalg.norm(want) < 1e-6
    # a new plan for the same problem takes the cached shape without timing
    E2 = capi.Evolve(capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im), 4, capi.EVOLVE_MIXED)
    E2.run(pr, pi, A.rows, 0.05, 1, 0, 12)
    assert E2.config() == (k, v)


@pytest.mark.parametrize("mode", [0, 1])
def test_renormalize(native, mode):
    """With renormalisation every state leaves each step with norm 1 (float64), and the states
    stay within the form's tolerance of the oracle."""
    import torch

    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 10, 2, mode)
    E.set_renormalize(True)
    E.run(pr, pi, A.rows, 0.1, 6, 0, 8)    # few terms: the series alone would lose norm
    got = _result(pr, pi)
    norms = np.linalg.norm(got, axis=1)
    assert np.abs(norms - 1).max() < 1e-12
    want = orc.ham_sim(A, P[1], 0.6, 6, 8)
    want = want / np.linalg.norm(want)
    assert np.linalg.norm(got[1] - want) < (1e-12 if mode == 0 else 1e-6)


def test_pipelined_large_unaligned_offsets(native):
    """The pipelined kernel on the 16-qubit XXZ chain: offsets +-1, +-2 and +-(2^15 - 1) take the
    element-wise copies, the rest the 16-byte ones; 5 states = one full and one masked chunk."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 16, 5, capi.EVOLVE_MIXED)
    E.set_config(4, 4, True)
    E.run(pr, pi, A.rows, 0.05, 2, 0, 10)
    got = _result(pr, pi)
    for q in (0, 4):
        want = orc.ham_sim(A, P[q], 0.1, 2, 10)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6


@pytest.mark.parametrize("model", ["xxz", "tfim"])
@pytest.mark.parametrize("mode", ["horner", "mixed"])
def test_full_size_chosen_form_against_c128(native, mode, model):
    """The bench line's workload size: a 20-qubit chain (XXZ, periodic; transverse-field Ising,
    open), 8 states, 5 steps of dt = 0.05 in the float32 forms on the bench line's kernel
    (variant 12, zero tiles skipped), against the complex128 plan at a tight step tolerance --
    within the 1e-6 bar."""
    import ctypes

    capi, _ = native
    N, off, re, im = ham.xxz(20) if model == "xxz" else ham.tfim(20)
    H = capi.Matrix.create(N, N, off, re, im)
    nrm = ctypes.c_double()
    capi.check(capi.lib().diaq_norm1_est(H.h, ctypes.byref(nrm), None))
    s_c, m_c = capi.select_sm(nrm.value, 0.05, 1e-8, 1.0, 100)
    s_r, m_r = capi.select_sm(nrm.value, 0.05, 1e-14, 1.0, 100)
    P = ham.random_state(N, 0, k=8)
    out = {}
    for name, md, sl, m, cfg in (("c128", capi.EVOLVE_C128, s_r, m_r, None),
                                 (mode, capi.EVOLVE_HORNER if mode == "horner" else capi.EVOLVE_MIXED, s_c, m_c,
                                  (4, 1, 12))):
        import torch

        E = capi.Evolve(H, 8, md)
        if cfg:
            E.set_config(*cfg)
        pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
        pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
        E.run(pr, pi, N, 0.05, 5, sl, m)
        out[name] = _result(pr, pi)
        del E
    for q in range(8):
        want = out["c128"][q]
        assert np.linalg.norm(out[mode][q] - want) / np.linalg.norm(want) < 1e-6, q


@pytest.mark.parametrize("variant", [10, 11])
def test_bulk_copy_wait_limit_reports_timeout(native, variant):
    """The bulk-copy kernels' bounded waits: with a 1 ns bound the consumers give up their first
    wait for a filled stage (a copy takes microseconds).  The run's error comes back as
    DIAQ_ERR_TIMEOUT from diaq_evolve_check and is cleared; the producer drained its copies, so
    the same plan with the default bound runs again and matches the oracle."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 14, 8, capi.EVOLVE_HORNER)
    E.set_config(4, 1, variant)
    E.set_wait_limit(1)
    E.run(pr, pi, A.rows, 0.05, 1, 0, 10)
    with pytest.raises(capi.DiaqError, match="gave up"):
        E.check()
    E.check()   # reported once, then cleared
    E.set_wait_limit(0)
    import torch

    pr.copy_(torch.from_numpy(np.ascontiguousarray(P.real)))
    pi.copy_(torch.from_numpy(np.ascontiguousarray(P.imag)))
    E.run(pr, pi, A.rows, 0.05, 2, 0, 10)
    E.check()
    got = _result(pr, pi)
    for q in (0, 7):
        want = orc.ham_sim(A, P[q], 0.1, 2, 10)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6, q


def test_wait_limit_and_check_on_the_register_kernel(native):
    """The register kernels have no waits: a 1 ns bound changes nothing and check() stays OK; a
    negative bound is rejected."""
    capi, _ = native
    A, E, P, pr, pi = _setup(capi, 12, 4, capi.EVOLVE_HORNER)
    E.set_config(4, 1, 12)
    with pytest.raises(capi.DiaqError):
        E.set_wait_limit(-1)
    E.set_wait_limit(1)
    E.run(pr, pi, A.rows, 0.05, 2, 0, 12)
    E.check()
    got = _result(pr, pi)
    want = orc.ham_sim(A, P[3], 0.1, 2, 12)
    assert np.linalg.norm(got[3] - want) / np.linalg.norm(want) < 1e-6


@pytest.mark.parametrize("N,k", [(1500, 8), (2048 + 96, 8), (3000, 5), (777, 16)])
def test_horner_il32_ragged_sizes(native, N, k):
    """The bench line's kernel (variant 12) on row counts that are not powers of two: the last
    32-row tile padded, grids that the block swizzle maps (a multiple of 4 blocks) and that it
    leaves in order (not), and the fp32(psi) tile of rows past the end skipped -- against the
    oracle, on a random Hermitian matrix with near, far and unaligned offsets."""
    import torch

    capi, _ = native
    rng = np.random.default_rng(N)
    offs = sorted({0, 1, 3, 32, 100, N // 3, N - 5})
    off, re, im = [], [], []
    for d in offs:
        L = N - d
        a = rng.standard_normal(L) + 1j * rng.standard_normal(L)
        if d == 0:
            a = a.real + 0j
        a[rng.random(L) < 0.4] = 0          # zero runs: some 32-row tiles hold only zeros
        for dd, v in ((d, a), (-d, np.conj(a))) if d else ((0, a),):
            off.append(dd)
            re.append(v.real * 0.3)
            im.append(v.imag * 0.3)
    order = np.argsort(off)
    off = np.asarray(off, dtype=np.int32)[order]
    re = np.concatenate([re[i] for i in order])
    im = np.concatenate([im[i] for i in order])
    H = capi.Matrix.create(N, N, off, re, im)
    E = capi.Evolve(H, k, capi.EVOLVE_HORNER)
    E.set_config(4, 1, 12)
    P = ham.random_state(N, 3, k=k)
    pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
    pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
    E.run(pr, pi, N, 0.02, 3, 0, 12)
    got = _result(pr, pi)
    A = orc.OMatrix(N, N, off, re, im)
    for q in (0, k - 1):
        want = orc.ham_sim(A, P[q], 0.06, 3, 12)
        assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6, q


@pytest.mark.parametrize("mode", ["horner", "mixed"])
@pytest.mark.parametrize("N,k", [(1500, 8), (2048 + 96, 8), (777, 16), (3000, 4)])
def test_il32_same_bits_as_variant_9(native, mode, N, k):
    """Variant 12 (32-bit loop, L2 prefetches, block swizzle, fp32(psi) tile, packed two-lane
    FMAs, middle and last terms as separate instantiations) does the sums of variant 9 in the same
    order with the same roundings: the evolved states agree bit for bit."""
    import torch

    capi, _ = native
    rng = np.random.default_rng(N + k)
    offs = sorted({0, 1, 2, 33, 64, 100, N // 3, N - 7})
    off, re, im = [], [], []
    for d in offs:
        L = N - d
        a = rng.standard_normal(L) + 1j * rng.standard_normal(L)
        if d == 0:
            a = a.real + 0j
        a[rng.random(L) < 0.5] = 0
        for dd, v in ((d, a), (-d, np.conj(a))) if d else ((0, a),):
            off.append(dd)
            re.append(v.real * 0.3)
            im.append(v.imag * 0.3)
    order = np.argsort(off)
    off = np.asarray(off, dtype=np.int32)[order]
    re = np.concatenate([re[i] for i in order])
    im = np.concatenate([im[i] for i in order])
    H = capi.Matrix.create(N, N, off, re, im)
    P = ham.random_state(N, 5, k=k)
    out = []
    for variant in (9, 12):
        E = capi.Evolve(H, k, capi.EVOLVE_HORNER if mode == "horner" else capi.EVOLVE_MIXED)
        E.set_config(4, 1, variant)
        pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
        pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
        E.run(pr, pi, N, 0.03, 4, 0, 11)
        out.append(_result(pr, pi))
    assert np.array_equal(out[0], out[1])
