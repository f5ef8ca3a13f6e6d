"""The (s, m) proposer's hand-written FP32 kernels against the CPU restatement: forward pass,
per-row loss and the full gradient, then that Adam steps reduce the loss."""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu


def _batch(B, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((B, 16)).astype(np.float32)
    ys = rng.integers(0, 21, B).astype(np.int32)
    ym = rng.integers(1, 31, B).astype(np.int32)
    return X, ys, ym


def test_param_count(native):
    capi, _ = native
    assert capi.lib().diaq_mlp_num_params() == omlp.N_PARAMS


def test_forward_matches_oracle(native):
    import torch

    capi, _ = native
    M = capi.Mlp(seed=3)
    X, _, _ = _batch(300, 1)
    Xd = torch.from_numpy(X).cuda()
    logits = torch.empty(300, 51, dtype=torch.float32, device="cuda")
    M.forward(Xd, logits)
    torch.cuda.synchronize()
    want, _ = omlp.forward(M.params(), X)
    got = logits.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-4 * max(1.0, np.abs(want).max())


@pytest.mark.parametrize("B", [1, 7, 256, 1000])
def test_gradient_matches_oracle(native, B):
    import torch

    capi, _ = native
    M = capi.Mlp(seed=B)
    X, ys, ym = _batch(B, 10 + B)
    ys[0] = 40   # an out-of-range label contributes neither loss nor gradient for its head
    grad = torch.empty(omlp.N_PARAMS, dtype=torch.float32, device="cuda")
    loss = torch.empty(B, dtype=torch.float32, device="cuda")
    M.gradient(torch.from_numpy(X).cuda(), torch.from_numpy(ys).cuda(), torch.from_numpy(ym).cuda(), grad, loss)
    torch.cuda.synchronize()
    wl, wg = omlp.loss_and_grad(M.params(), X, ys, ym)
    g = grad.cpu().numpy()
    assert np.abs(loss.cpu().numpy() - wl).max() <= 1e-4 * max(1.0, np.abs(wl).max())
    assert np.abs(g - wg).max() <= 1e-4 * max(1e-3, np.abs(wg).max()), np.abs(g - wg).max()
    # a finite-difference spot check of the oracle itself on two parameters
    p = M.params().astype(np.float64)
    for idx in (5, omlp.N_PARAMS - 3):
        h = 1e-4
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (omlp.loss_and_grad(pp, X, ys, ym)[0].mean() - omlp.loss_and_grad(pm, X, ys, ym)[0].mean()) / (2 * h)
        assert abs(fd - wg[idx]) <= 1e-5 + 1e-3 * abs(wg[idx])


def test_training_reduces_loss(native):
    import torch

    capi, _ = native
    M = capi.Mlp(seed=0)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((512, 16)).astype(np.float32)
    ys = (np.abs(X[:, 0]) * 5).astype(np.int32).clip(0, 20)   # learnable labels
    ym = (np.abs(X[:, 1]) * 8 + 1).astype(np.int32).clip(1, 30)
    Xd, ysd, ymd = torch.from_numpy(X).cuda(), torch.from_numpy(ys).cuda(), torch.from_numpy(ym).cuda()
    loss = torch.empty(512, dtype=torch.float32, device="cuda")
    M.gradient(Xd, ysd, ymd, None, loss)
    l0 = float(loss.mean())
    for _ in range(300):
        M.train_step(Xd, ysd, ymd, 3e-3, loss)
    M.gradient(Xd, ysd, ymd, None, loss)
    assert float(loss.mean()) < 0.5 * l0
    s = torch.empty(512, dtype=torch.int32, device="cuda")
    m = torch.empty_like(s)
    M.propose(Xd, s, m)
    acc = (s.cpu().numpy() == ys).mean()
    assert acc > 0.5 and (m.cpu().numpy() >= 1).all() and (m.cpu().numpy() <= 30).all()
