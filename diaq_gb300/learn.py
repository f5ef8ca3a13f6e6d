"""Learned choice of the sub-step count 2^s and Taylor degree m for exp(-i t H) psi.

The network (FP32 MLP 16 -> 64 -> 64 -> 21 + 30, kernels in csrc/mlp.cu) maps 16 cheap features
of (H, t, tol) to logits over s in 0..20 and m in 1..30.  Every proposal is checked a posteriori
before use; the plain norm-bound selection (diaq_select_sm: the reference's scaling rule
s = ceil(log2(t ||H||_1)) with the Taylor remainder bound for m) is both the fallback and the
yardstick of the gain.

Chain.  For a probe state psi (unit, seeded) one device run of M = 60 products gives
u_k = (-i H)^k psi / k!, k = 0..M.  For a sub-step tau the k-th Taylor term of exp(-i tau H) psi
is tau^k u_k, so the truncation error of degree m is the tail ||sum_{k>m} tau^k u_k|| -- for
every m and every tau from the same chain, against the M-term expansion (tau ||H||_1 <= 8 keeps
the neglected rest below 1e-28).  Over 2^s sub-steps the errors add up (unitary propagation
keeps their size): E(s, m) = 2^s ||tail_m(t / 2^s)||.

Label.  The cheapest (2^s * m) pair with E(s, m) <= tol, s in 0..20, m in 1..30.

Check.  A proposal (s, m) is accepted when the next term bounds the rest:
2^s * 2 * ||tau^(m+1) u_(m+1)|| <= tol with tau ||H||_1 / (m + 2) <= 1/2 (then the tail is at
most twice its first term), and when it costs no more than the norm-bound choice.  Otherwise
the norm-bound choice is used.

Features (all O(1)):
  0 log10(theta), theta = t ||H||_1          1 log10 t            2 log10 ||H||_1
  3 -log10(tol) / 10                         4 n / 20             5 log10(#diagonals) / 3
  6 log2(max |offset| + 1) / n               7-10 log10(t (k! ||u_k||)^(1/k)), k = 1..4
  11 log10(||H||_F / sqrt(N))                12 |<psi, H psi>| / ||H psi|| (probe Rayleigh ratio)
  13 norm-bound s / 20                       14 norm-bound m / 30 (capped)
  15 log10(2 ||u_2|| / ||u_1||^2)

Training set: n uniform on 8..16, 2n..8n Pauli strings of weight 1..3 with N(0,1) coefficients,
t log-uniform on [1e-3, 10], tol in {1e-6, 1e-10}.  Held-out evaluation: n = 18..20.

    python -m diaq_gb300.learn --count 50000 --epochs 30 --out <dir>
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import time

import numpy as np

from . import capi
from . import hamiltonians as ham

M_CHAIN = 60
S_MAX, M_MAX = 20, 30
PARAMS_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "sm_mlp_params.npy")


# ---- instances ------------------------------------------------------------------------------------
def random_instance(rng, n_lo=8, n_hi=16):
    n = int(rng.integers(n_lo, n_hi + 1))
    k = int(rng.integers(2 * n, 8 * n + 1))
    terms = ham.random_pauli_terms(n, rng, k, 3)
    t = float(10 ** rng.uniform(-3, 1))
    tol = float(rng.choice([1e-6, 1e-10]))
    return n, terms, t, tol


def build(n, terms) -> capi.Matrix:
    return capi.Matrix.from_pauli(n, *ham.pauli_masks(n, terms))


# ---- chain and features -----------------------------------------------------------------------------
def chain(H: capi.Matrix, psi, M: int = M_CHAIN):
    """U[k] = (-i H)^k psi / k!, k = 0..M, as a complex128 CUDA tensor (M+1, N)."""
    import torch

    L = capi.lib()
    N = H.info()[0]
    U = torch.empty((M + 1, N), dtype=torch.complex128, device="cuda")
    U[0] = psi
    xr = U[0].real.contiguous()
    xi = U[0].imag.contiguous()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    s = torch.cuda.current_stream().cuda_stream
    for k in range(1, M + 1):
        capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), s))
        # u_k = (-i / k) (H u_{k-1}) = (y_im / k, -y_re / k)
        xr = yi / k
        xi = -yr / k
        U[k] = torch.complex(xr, xi)
    return U


def chain_stats(H: capi.Matrix, psi, M: int = M_CHAIN):
    """The norms ||u_k||, k = 0..M, of the chain of `chain` and |<u_0, u_1>|, without storing the
    chain: what the features and the a-posteriori check need at selection time."""
    import torch

    L = capi.lib()
    xr = psi.real.contiguous()
    xi = psi.imag.contiguous()
    x0r, x0i = xr.clone(), xi.clone()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    s = torch.cuda.current_stream().cuda_stream
    norms = [torch.sqrt(torch.dot(xr, xr) + torch.dot(xi, xi))]
    v01 = None
    for k in range(1, M + 1):
        capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), s))
        xr = yi / k
        xi = -yr / k
        norms.append(torch.sqrt(torch.dot(xr, xr) + torch.dot(xi, xi)))
        if k == 1:   # <u_0, u_1> = conj(u_0) . u_1
            v01 = torch.complex(torch.dot(x0r, xr) + torch.dot(x0i, xi), torch.dot(x0r, xi) - torch.dot(x0i, xr))
    unorm = torch.stack(norms).cpu().numpy()
    return unorm, float(torch.abs(v01).item())


def tails(U, tau: float, m_max: int = M_MAX):
    """||sum_{k>m} tau^k u_k|| for m = 1..m_max (float64 numpy), and ||tau^k u_k|| for k = 0..M."""
    import torch

    M = U.shape[0] - 1
    k = torch.arange(M + 1, device=U.device, dtype=torch.float64)
    logc = k * math.log(tau) if tau > 0 else torch.where(k == 0, 0.0, -math.inf)
    c = torch.exp(logc)
    W = torch.zeros((m_max, M + 1), dtype=torch.float64, device=U.device)
    for m in range(1, m_max + 1):
        W[m - 1, m + 1:] = c[m + 1:]
    T = W.to(torch.complex128) @ U
    tail = torch.linalg.vector_norm(T, dim=1).cpu().numpy()
    term = (c * torch.linalg.vector_norm(U, dim=1)).cpu().numpy()
    return tail, term


def norm_bound(norm1: float, t: float, tol: float):
    return capi.select_sm(norm1, t, tol, 1.0, 100)


def features(n, H: capi.Matrix, unorm, v01, t, tol, norm1, fro):
    """16 features from the matrix, the chain norms unorm = ||u_k|| and v01 = |<u_0, u_1>|."""
    N, _, nd, _, _ = H.info()
    off = H.offsets()
    un = unorm[:5]
    s_ref, m_ref = norm_bound(norm1, t, tol)
    theta = t * norm1
    f = np.zeros(16, dtype=np.float32)
    f[0] = math.log10(max(theta, 1e-30))
    f[1] = math.log10(t)
    f[2] = math.log10(max(norm1, 1e-30))
    f[3] = -math.log10(tol) / 10
    f[4] = n / 20
    f[5] = math.log10(max(nd, 1)) / 3
    f[6] = math.log2(float(np.abs(off).max()) + 1) / n if nd else 0.0
    for k in range(1, 5):
        hk = math.factorial(k) * un[k]
        f[6 + k] = math.log10(max(t * hk ** (1.0 / k), 1e-30))
    f[11] = math.log10(max(fro / math.sqrt(N), 1e-30))
    # u_1 = -i H psi, so <psi, H psi> = i <u_0, u_1>
    f[12] = v01 / max(un[1], 1e-300)
    f[13] = s_ref / 20
    f[14] = min(m_ref, 100) / 30
    f[15] = math.log10(max(2 * un[2] / max(un[1] ** 2, 1e-300), 1e-30))
    return f


def label(U, t, tol, norm1):
    """Cheapest (s, m) with 2^s * tail_m(t / 2^s) <= tol; None when no candidate qualifies."""
    theta = t * norm1
    best = None
    for s in range(0, S_MAX + 1):
        if theta / 2 ** s > 8.0:
            continue
        tail, _ = tails(U, t / 2 ** s)
        ok = np.nonzero(2 ** s * tail <= tol)[0]
        if ok.size == 0:
            continue
        m = int(ok[0]) + 1
        cost = 2 ** s * m
        if best is None or cost < best[2]:
            best = (s, m, cost)
        if 2 ** s > best[2]:   # more sub-steps cannot be cheaper
            break
    return best


def check(unorm, t, tol, norm1, s, m):
    """The a-posteriori next-term test of a proposal (see the module docstring); unorm[k] = ||u_k||."""
    if not (0 <= s <= S_MAX and 1 <= m <= M_MAX):
        return False
    tau = t / 2 ** s
    if tau * norm1 / (m + 2) > 0.5:
        return False
    term = math.exp((m + 1) * math.log(tau)) * float(unorm[m + 1]) if tau > 0 else 0.0
    return 2 ** s * 2 * term <= tol


def instance_record(n, terms, t, tol, seed):
    """Everything the selector needs about one instance: features, label, norm-bound choice."""
    return record_for(build(n, terms), n, t, tol, seed)


def record_for(H: capi.Matrix, n, t, tol, seed, with_label=True):
    """Features, chain, norm-bound choice (and label) for a device matrix H of 2^n rows."""
    import torch

    norm1 = ctypes.c_double()
    fro = ctypes.c_double()
    capi.check(capi.lib().diaq_norm1_est(H.h, ctypes.byref(norm1), None))
    capi.check(capi.lib().diaq_frobenius(H.h, ctypes.byref(fro), None))
    N = 1 << n
    psi = torch.from_numpy(ham.random_state(N, seed)).cuda()
    rec = {"norm1": norm1.value, "H": H, "ref": norm_bound(norm1.value, t, tol), "label": None}
    if with_label:   # the whole chain: labels need the exact tails
        U = chain(H, psi)
        unorm = torch.linalg.vector_norm(U, dim=1).cpu().numpy()
        v01 = float(torch.abs(torch.vdot(U[0], U[1])).item())
        rec["U"] = U
        rec["label"] = label(U, t, tol, norm1.value)
    else:            # selection only: norms, streamed
        unorm, v01 = chain_stats(H, psi)
    rec["unorm"] = unorm
    rec["f"] = features(n, H, unorm, v01, t, tol, norm1.value, fro.value)
    return rec


def generate(count, seed, n_lo=8, n_hi=16, log_every=1000):
    rng = np.random.default_rng(seed)
    X = np.zeros((count, 16), dtype=np.float32)
    ys = np.zeros(count, dtype=np.int32)
    ym = np.zeros(count, dtype=np.int32)
    cost_ref = np.zeros(count)
    cost_lab = np.zeros(count)
    t0 = time.time()
    i = 0
    while i < count:
        n, terms, t, tol = random_instance(rng, n_lo, n_hi)
        r = instance_record(n, terms, t, tol, seed=int(rng.integers(1 << 30)))
        if r["label"] is None:
            continue
        X[i] = r["f"]
        ys[i], ym[i] = r["label"][0], r["label"][1]
        cost_lab[i] = r["label"][2]
        cost_ref[i] = 2 ** r["ref"][0] * r["ref"][1]
        i += 1
        if log_every and i % log_every == 0:
            print(f"  {i}/{count} instances, {time.time() - t0:.0f} s", flush=True)
    return X, ys, ym, cost_lab, cost_ref


# ---- training ----------------------------------------------------------------------------------------
def train(X, ys, ym, epochs=30, batch=1024, lr=2e-3, seed=0, log=True):
    import torch

    net = capi.Mlp(seed)
    n = X.shape[0]
    Xd = torch.from_numpy(X).cuda()
    ysd = torch.from_numpy(ys).cuda()
    ymd = torch.from_numpy(ym).cuda()
    g = torch.Generator(device="cpu").manual_seed(seed)
    loss = torch.empty(batch, dtype=torch.float32, device="cuda")
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).cuda()
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            xb, sb, mb = Xd[idx].contiguous(), ysd[idx].contiguous(), ymd[idx].contiguous()
            net.train_step(xb, sb, mb, lr * (0.5 * (1 + math.cos(math.pi * ep / epochs))), loss)
            tot += float(loss.sum())
            cnt += batch
        hist.append(tot / max(cnt, 1))
        if log:
            print(f"  epoch {ep + 1}/{epochs}: loss {hist[-1]:.4f}", flush=True)
    return net, hist


def propose(net, X):
    import torch

    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
    s = torch.empty(X.shape[0], dtype=torch.int32, device="cuda")
    m = torch.empty_like(s)
    net.propose(Xd, s, m)
    torch.cuda.synchronize()
    return s.cpu().numpy(), m.cpu().numpy()


def load(path: str = PARAMS_PATH):
    """The trained proposer shipped with the package (None if absent)."""
    if not os.path.exists(path):
        return None
    net = capi.Mlp(0)
    net.set_params(np.load(path))
    return net


def choose(net, record, t, tol):
    """(s, m, source) for one instance.  The network proposes (s, m); the next-term check then
    settles the degree near it -- the smallest m' in [m-3, m+4] that passes -- and the result
    is used when it costs no more than the norm-bound choice, which is taken otherwise."""
    s, m = propose(net, record["f"][None, :])
    s, m = int(s[0]), int(m[0])
    s_ref, m_ref = record["ref"]
    for mm in range(max(1, m - 3), min(M_MAX, m + 4) + 1):
        if 2 ** s * mm > 2 ** s_ref * m_ref:
            break
        if check(record["unorm"], t, tol, record["norm1"], s, mm):
            return s, mm, "learned"
    return s_ref, m_ref, "norm-bound"


def learned_sm(H: capi.Matrix, t: float, tol: float, net=None, seed: int = 12345):
    """(s, m, source, record) for evolving states under the device matrix H over time t to
    tolerance tol: the shipped network's checked proposal, or the norm-bound choice."""
    n = int(H.info()[0]).bit_length() - 1
    rec = record_for(H, n, t, tol, seed, with_label=False)
    net = net if net is not None else load()
    if net is None:
        s, m = rec["ref"]
        return s, m, "norm-bound (no trained network)", rec
    s, m, src = choose(net, rec, t, tol)
    return s, m, src, rec


def evaluate(net, count, seed, n_lo=18, n_hi=20):
    """Held-out instances: cost of the checked proposals against the norm-bound choice, and the
    error each actually reaches (E(s, m) from the chain) against tol."""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(count):
        n, terms, t, tol = random_instance(rng, n_lo, n_hi)
        r = instance_record(n, terms, t, tol, seed=int(rng.integers(1 << 30)))
        s, m, src = choose(net, r, t, tol)
        s_ref, m_ref = r["ref"]
        err = _error(r, t, s, m)
        err_ref = _error(r, t, s_ref, m_ref)
        rows.append({"n": n, "t": t, "tol": tol, "theta": t * r["norm1"], "s": s, "m": m, "source": src,
                     "cost": 2 ** s * m, "s_ref": s_ref, "m_ref": m_ref, "cost_ref": 2 ** s_ref * m_ref,
                     "err": err, "err_ref": err_ref, "label": r["label"]})
        del r
    return rows


def _error(r, t, s, m):
    """The error (s, m) reaches on the instance's probe state: E(s, m) from the chain where the
    chain covers the sub-step (tau ||H||_1 <= 8, m <= M_MAX), else by direct evolution."""
    if t / 2 ** s * r["norm1"] > 8.0 or m > M_MAX:
        return evolve_error(r["H"], r["U"][0], t, s, m, r["norm1"])
    tail, _ = tails(r["U"], t / 2 ** s)
    return float(2 ** s * tail[m - 1])


def evolve_error(H: capi.Matrix, psi, t, s, m, norm1):
    """|| T_m(t / 2^s)^(2^s) psi - exp(-i t H) psi ||: the probe state evolved over t in 2^s
    sub-steps of the degree-m Taylor polynomial, against the same state evolved at a 1e-15
    remainder bound per step (complex128 plans on the device, both pinned to the FP64 oracle)."""
    import torch

    N = H.info()[0]

    def run(s_, m_):
        E = capi.Evolve(H, 1, capi.EVOLVE_C128)
        pr, pi = psi.real.contiguous().clone(), psi.imag.contiguous().clone()
        E.run(pr, pi, N, t, 1, s_, m_)
        torch.cuda.synchronize()
        return torch.complex(pr, pi)

    s_r, m_r = capi.select_sm(norm1, t, 1e-15, 1.0, 100)
    return float(torch.linalg.vector_norm(run(s, m) - run(s_r, m_r)).item())


def heldout_summary(rows):
    cost = np.array([r["cost"] for r in rows], dtype=float)
    cref = np.array([r["cost_ref"] for r in rows], dtype=float)
    errs = np.array([r["err"] / r["tol"] for r in rows])
    return {"instances": len(rows), "n": [18, 20],
            "accepted_learned": int(sum(r["source"] == "learned" for r in rows)),
            "mean_cost_learned_checked": float(cost.mean()), "mean_cost_norm_bound": float(cref.mean()),
            "speedup_geomean": float(np.exp(np.mean(np.log(cref / cost)))),
            "max_err_over_tol": float(errs.max()) if errs.size else None,
            "all_within_tol": bool(np.all(errs <= 1.0))}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--count", type=int, default=50000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--eval", type=int, default=30)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=".")
    ap.add_argument("--evaluate-only", action="store_true",
                    help="evaluate the shipped network on the held-out instances (no training)")
    args = ap.parse_args()
    from . import build as b

    b.build()
    os.makedirs(args.out, exist_ok=True)
    if args.evaluate_only:
        net = load()
        if net is None:
            raise SystemExit(f"no trained network at {PARAMS_PATH}")
        rows = evaluate(net, args.eval, args.seed + 1000)
        report = {"heldout": heldout_summary(rows), "rows": rows}
        for r in report["rows"]:
            r["label"] = list(r["label"]) if r["label"] else None
        json.dump(report, open(os.path.join(args.out, "sm_eval.json"), "w"), indent=1, default=float)
        print(json.dumps(report["heldout"], default=float), flush=True)
        return
    t0 = time.time()
    X, ys, ym, cost_lab, cost_ref = generate(args.count, args.seed)
    t_gen = time.time() - t0
    np.savez_compressed(os.path.join(args.out, "sm_dataset.npz"), X=X, ys=ys, ym=ym, cost_lab=cost_lab,
                        cost_ref=cost_ref)
    ntr = int(0.9 * args.count)
    net, hist = train(X[:ntr], ys[:ntr], ym[:ntr], epochs=args.epochs)
    s_hat, m_hat = propose(net, X[ntr:])
    val = {"s_acc": float((s_hat == ys[ntr:]).mean()), "m_acc": float((m_hat == ym[ntr:]).mean()),
           "m_within1": float((np.abs(m_hat - ym[ntr:]) <= 1).mean())}
    np.save(os.path.join(args.out, "sm_mlp_params.npy"), net.params())
    rows = evaluate(net, args.eval, args.seed + 1000)
    report = {
        "train_instances": ntr, "val_instances": args.count - ntr, "generate_s": t_gen,
        "train_loss": hist, "validation": val,
        "label_cost_over_norm_bound_train": float(np.mean(cost_lab / cost_ref)),
        "heldout": heldout_summary(rows),
        "rows": rows,
    }
    for r in report["rows"]:
        r["label"] = list(r["label"]) if r["label"] else None
    json.dump(report, open(os.path.join(args.out, "sm_report.json"), "w"), indent=1, default=float)
    print(json.dumps({k: v for k, v in report.items() if k != "rows"}, default=float), flush=True)


if __name__ == "__main__":
    main()
