"""Batched evolution of Hamiltonians of uneven size, several states each, against the oracle."""
import numpy as np
import pytest

from diaq_gb300 import hamiltonians as ham
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _make(capi, specs, precision):
    import torch

    mats, oms, prs, pis, P0 = [], [], [], [], []
    for (model, n, k, seed) in specs:
        N, off, re, im = ham.xxz(n, seed=seed) if model == "xxz" else ham.tfim(n, J=0.9, h=0.6 + 0.1 * seed)
        oms.append(orc.OMatrix(N, N, off, re, im))
        mats.append(capi.Matrix.create(N, N, off, re, im, precision=precision))
        P = ham.random_state(N, seed, k=k) if k > 1 else ham.random_state(N, seed)[None, :]
        P0.append(P)
        prs.append(torch.from_numpy(np.ascontiguousarray(P.real)).cuda())
        pis.append(torch.from_numpy(np.ascontiguousarray(P.imag)).cuda())
    return mats, oms, prs, pis, P0


SPECS = [("xxz", 10, 3, 1), ("tfim", 9, 1, 2), ("xxz", 12, 5, 3), ("tfim", 11, 2, 4), ("xxz", 8, 1, 5)]


@pytest.mark.parametrize("precision,tol", [(1, 1e-6), (0, 1e-12)])
def test_batched_matches_oracle(native, precision, tol):
    import torch

    capi, _ = native
    mats, oms, prs, pis, P0 = _make(capi, SPECS, precision)
    B = capi.Batch(mats, prs, pis)
    s = [0, 1, 0, 2, 0]
    m = [11, 8, 13, 6, 9]   # instance 0: 11 launches per step (odd: the copy phase runs)
    B.run(0.02, s, m, 4)
    torch.cuda.synchronize()
    for i, A in enumerate(oms):
        got = (prs[i] + 1j * pis[i]).cpu().numpy()
        for q in range(P0[i].shape[0]):
            want = orc.ham_sim(A, P0[i][q], 0.08, 4, m[i], substeps=1 << s[i])
            err = np.linalg.norm(got[q] - want) / np.linalg.norm(want)
            assert err < tol, (i, q, err)
    k, v, phases = B.config()
    assert phases == max((1 << si) * mi + ((1 << si) * mi) % 2 for si, mi in zip(s, m))


@pytest.mark.parametrize("precision,tol", [(1, 1e-6), (0, 1e-12)])
def test_batched_horner_matches_oracle(native, precision, tol):
    """The Horner form in the batch: instances with m >= 2 evaluate from the inside out, the
    m = 1 instance keeps the compensated path; no copy phase for the Horner instances."""
    import torch

    capi, _ = native
    mats, oms, prs, pis, P0 = _make(capi, SPECS, precision)
    B = capi.Batch(mats, prs, pis)
    B.set_horner(True)
    s = [0, 1, 0, 2, 0]
    m = [11, 8, 13, 6, 1]
    dts = [0.02, 0.02, 0.02, 0.02, 0.02]
    B.run(0.02, s, m, 4)
    torch.cuda.synchronize()
    for i, A in enumerate(oms):
        got = (prs[i] + 1j * pis[i]).cpu().numpy()
        for q in range(P0[i].shape[0]):
            want = orc.ham_sim(A, P0[i][q], 4 * dts[i], 4, m[i], substeps=1 << s[i])
            err = np.linalg.norm(got[q] - want) / np.linalg.norm(want)
            assert err < (tol if m[i] > 1 else max(tol, 1e-6)), (i, q, err)
    _, _, phases = B.config()
    assert phases == max((1 << si) * mi + (((1 << si) * mi) % 2 if mi == 1 else 0) for si, mi in zip(s, m))


@pytest.mark.parametrize("cfg", [(8, 1), (8, 2), (4, 4), (2, 4), (1, 4), (1, 1)])
def test_batched_every_launch_shape(native, cfg):
    import torch

    capi, _ = native
    mats, oms, prs, pis, P0 = _make(capi, SPECS[:3], 1)
    B = capi.Batch(mats, prs, pis)
    B.set_config(*cfg)
    B.run(0.02, [0, 0, 1], [10, 12, 7], 3)
    torch.cuda.synchronize()
    for i, (sl, mm) in enumerate(zip([0, 0, 1], [10, 12, 7])):
        got = (prs[i] + 1j * pis[i]).cpu().numpy()
        want = orc.ham_sim(oms[i], P0[i][-1], 0.06, 3, mm, substeps=1 << sl)
        assert np.linalg.norm(got[-1] - want) / np.linalg.norm(want) < 1e-6


def test_batched_autotune_keeps_states(native, tmp_path, monkeypatch):
    import torch

    capi, _ = native
    monkeypatch.setenv("DIAQ_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    mats, oms, prs, pis, P0 = _make(capi, SPECS[:2], 1)
    B = capi.Batch(mats, prs, pis)
    B.run(0.02, [0, 0], [10, 10], 2)   # autotunes on scratch, then 2 steps
    torch.cuda.synchronize()
    got = (prs[0] + 1j * pis[0]).cpu().numpy()
    want = orc.ham_sim(oms[0], P0[0][0], 0.04, 2, 10)
    assert np.linalg.norm(got[0] - want) / np.linalg.norm(want) < 1e-6
    assert (tmp_path / "tune.json").exists()


IL_SPECS = [("xxz", 11, 4, 1), ("tfim", 10, 5, 2), ("xxz", 9, 8, 3), ("tfim", 8, 16, 4), ("xxz", 7, 32, 5),
            ("tfim", 3, 6, 6), ("xxz", 6, 33, 7), ("tfim", 9, 1, 8), ("xxz", 5, 3, 9)]


@pytest.mark.parametrize("horner", [False, True])
def test_batched_interleaved_matches_planar_and_oracle(native, horner):
    """complex64 instances with 4-32 states run interleaved (8 or 4 states per thread, rows
    padded to 32: the 3-qubit instance has 8 rows), the rest planar; the same arithmetic in the
    same order, so both layouts give the same bits, and both match the oracle."""
    import torch

    capi, _ = native
    s = [0, 1, 0, 0, 1, 0, 0, 2, 0]
    m = [9, 7, 12, 6, 5, 11, 8, 3, 10]
    out = {}
    for il in (True, False):
        mats, oms, prs, pis, P0 = _make(capi, IL_SPECS, 1)
        B = capi.Batch(mats, prs, pis)
        B.set_horner(horner)
        B.set_interleaved(il)
        B.set_config(4, 2)
        B.run(0.02, s, m, 3)
        torch.cuda.synchronize()
        out[il] = [(p + 1j * q).cpu().numpy() for p, q in zip(prs, pis)]
    for i, A in enumerate(oms):
        assert np.array_equal(out[True][i], out[False][i]), i
        for q in range(P0[i].shape[0]):
            want = orc.ham_sim(A, P0[i][q], 0.06, 3, m[i], substeps=1 << s[i])
            err = np.linalg.norm(out[True][i][q] - want) / np.linalg.norm(want)
            assert err < 1e-6, (i, q, err)


def test_batched_layout_toggle_on_one_batch(native):
    """set_interleaved between runs of the same batch re-records the step with the other item
    lists; the results agree with a batch that never switched."""
    import torch

    capi, _ = native
    s, m = [0, 1, 0, 0, 1, 0, 0, 2, 0], [9, 7, 12, 6, 5, 11, 8, 3, 10]
    mats, oms, prs, pis, P0 = _make(capi, IL_SPECS, 1)
    B = capi.Batch(mats, prs, pis)
    B.set_horner(True)
    B.run(0.02, s, m, 2)
    B.set_interleaved(False)
    B.run(0.02, s, m, 1)
    B.set_interleaved(True)
    B.run(0.02, s, m, 1)
    torch.cuda.synchronize()
    for i, A in enumerate(oms):
        got = (prs[i] + 1j * pis[i]).cpu().numpy()
        for q in range(P0[i].shape[0]):
            want = orc.ham_sim(A, P0[i][q], 0.08, 4, m[i], substeps=1 << s[i])
            assert np.linalg.norm(got[q] - want) / np.linalg.norm(want) < 1e-6, (i, q)
