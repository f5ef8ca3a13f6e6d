"""The learned (s, m) selection end to end on a small scale: labels meet the tolerance, the
network trained by the project's kernels proposes, every proposal is checked, and the checked
choice is never less accurate and never dearer than the norm-bound selection -- and cheaper
on average, which is the gain the network brings."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_labels_meet_tolerance(native):
    from diaq_gb300 import learn

    rng = np.random.default_rng(5)
    for _ in range(12):
        n, terms, t, tol = learn.random_instance(rng, 8, 10)
        r = learn.instance_record(n, terms, t, tol, seed=int(rng.integers(1 << 30)))
        s, m, cost = r["label"]
        assert learn._error(r, t, s, m) <= tol
        s_ref, m_ref = r["ref"]
        assert cost <= 2 ** s_ref * m_ref
        assert r["f"].shape == (16,) and np.all(np.isfinite(r["f"]))


def test_chain_tail_matches_evolution(native):
    """The chain's truncation error equals the error of an actual Taylor step on the GPU."""
    import torch

    from diaq_gb300 import capi, learn
    from diaq_gb300 import hamiltonians as ham
    from oracle import oracle as orc

    rng = np.random.default_rng(8)
    n, terms, _, _ = learn.random_instance(rng, 9, 9)
    H = learn.build(n, terms)
    psi = ham.random_state(1 << n, 3)
    U = learn.chain(H, torch.from_numpy(psi).cuda())
    off, re, im = H.download()
    A = orc.OMatrix(1 << n, 1 << n, off, re, im)
    exact = orc.ham_sim(A, psi, 0.05, 1, 60)
    tail, _ = learn.tails(U, 0.05)
    for m in (3, 6, 10):
        approx = orc.ham_sim(A, psi, 0.05, 1, m)
        assert abs(np.linalg.norm(approx - exact) - tail[m - 1]) <= 1e-12 + 1e-6 * tail[m - 1]


def test_trained_selector_gains_over_norm_bound(native):
    from diaq_gb300 import learn

    X, ys, ym, cost_lab, cost_ref = learn.generate(600, seed=2, n_lo=8, n_hi=10, log_every=0)
    assert np.all(cost_lab <= cost_ref)
    net, hist = learn.train(X, ys, ym, epochs=60, batch=128, lr=3e-3, log=False)
    assert hist[-1] < hist[0]
    rows = learn.evaluate(net, 25, seed=99, n_lo=10, n_hi=11)
    for r in rows:
        assert r["cost"] <= r["cost_ref"]
        assert r["err"] <= r["tol"], r   # every row: the chain's tail, or direct evolution beyond its reach
    gain = np.mean([r["cost_ref"] / r["cost"] for r in rows])
    assert gain > 1.0, gain


def test_selection_streams_the_chain(native):
    """At selection time the chain is not stored: its norms and <u0, u1> are streamed, and the
    features and the checked choice equal those computed from the stored chain."""
    from diaq_gb300 import learn

    rng = np.random.default_rng(21)
    for _ in range(4):
        n, terms, t, tol = learn.random_instance(rng, 9, 11)
        H = learn.build(n, terms)
        full = learn.record_for(H, n, t, tol, seed=77, with_label=True)
        lean = learn.record_for(H, n, t, tol, seed=77, with_label=False)
        assert "U" not in lean
        assert np.allclose(lean["unorm"], full["unorm"], rtol=1e-12, atol=0)
        assert np.allclose(lean["f"], full["f"], rtol=1e-6, atol=1e-7)
        net = learn.load()
        if net is not None:
            assert learn.choose(net, lean, t, tol) == learn.choose(net, full, t, tol)


def test_evolve_error_beyond_the_chain(native):
    """Where tau ||H||_1 > 8 the chain cannot give the truncation error; the direct evolution does,
    and inside the chain's reach the two agree."""
    from diaq_gb300 import learn

    rng = np.random.default_rng(5)
    n, terms, _, _ = learn.random_instance(rng, 9, 9)
    H = learn.build(n, terms)
    rec = learn.record_for(H, n, 0.05, 1e-10, seed=3, with_label=True)
    t = 2.0 / rec["norm1"]    # tau ||H||_1 = 2: inside the chain's reach
    for s, m in ((0, 8), (1, 6), (0, 14)):
        e_chain = learn._error(rec, t, s, m)
        e_direct = learn.evolve_error(H, rec["U"][0], t, s, m, rec["norm1"])
        assert abs(e_chain - e_direct) <= 1e-12 + 1e-6 * e_chain, (s, m, e_chain, e_direct)
    # tau ||H||_1 = 12 at s = 0: beyond the chain's reach, the direct evolution takes over; check
    # it against the degree-m Taylor step of the oracle and a dense exp(-i t H) (scipy)
    import scipy.linalg as sl

    from oracle import oracle as orc

    t = 12.0 / rec["norm1"]
    off, re, im = H.download()
    A = orc.OMatrix(1 << n, 1 << n, off, re, im)
    psi = rec["U"][0].cpu().numpy()
    exact = sl.expm(-1j * t * A.to_dense()) @ psi
    for s, m in ((0, 14), (0, 30), (0, 22)):   # all beyond the chain: direct evolution
        e = learn._error(rec, t, s, m)
        want = np.linalg.norm(orc.ham_sim(A, psi, t, 1, m, substeps=1 << s) - exact)
        assert abs(e - want) <= 1e-13 + 1e-6 * want, (s, m, e, want)
