"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout that has the reference tree and its CPU library built (``make -C oracle ref``):

    python tests/golden/make_golden.py [--ref /path/to/reference] [--skip-slow]

What it writes (all small .npz files):
  ref_spgemm_cases.npz  the 51 hand-written SpGEMM cases of the reference's C++ tests
                        (cpp_tests/test_main.cpp:35-1546, read as text): dense A, B, the dense
                        product the reference checks against (denseProduct) and the offsets of the
                        reference library's pruned DIA product.
  tfim12.npz            12-qubit TFIM: H.psi, (H.H) structure and (H.H).psi, expm_negative(H, 0.1).psi
                        from the reference library (the last takes minutes: --skip-slow keeps the
                        previous value).
  expm_small.npz        expm_negative / expm / pow of small Hamiltonians through the reference.
  ham_sim.npz           the reference's time-evolution rule (dt = t/r, exactly m Taylor terms per
                        step) run on the reference's own CPU spMV.
  api_random.npz        random rectangular products and SpMVs (the kind test_api_vs_numpy.py draws),
                        reference results.
"""
from __future__ import annotations

import argparse
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from oracle import reference as ref  # noqa: E402
from diaq_gb300 import hamiltonians as ham  # noqa: E402


# ---- the reference's hand-written SpGEMM cases ---------------------------------------------------
_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$")


def _value(tok: str, env: dict) -> float:
    t = tok.strip().replace(" ", "")
    if not t:
        raise ValueError("empty")
    if _NUM.match(t):
        return float(t)
    if t in env:
        return env[t]
    m = re.match(r"^(-?)1\*(\w+)$", t) or re.match(r"^(-)(\w+)$", t)
    if m and m.group(2) in env:
        return -env[m.group(2)] if m.group(1) == "-" else env[m.group(2)]
    raise ValueError(f"cannot evaluate {tok!r}")


def parse_spgemm_cases(path: str):
    src = open(path).read()
    env = {"h_val": 1.0 / np.sqrt(2.0)}
    arrays = {}
    decl = r"valType\s+([ab]\d+(?:_real|_imag)?)\s*\[\s*(\d+(?:\s*\*\s*\d+)?)\s*\]\s*=\s*\{(.*?)\};"
    for m in re.finditer(decl, src, re.S):
        name, body = m.group(1), m.group(3)
        n = int(np.prod([int(x) for x in m.group(2).split("*")]))
        body = re.sub(r"//[^\n]*", "", body)
        toks = [t for t in body.replace("\n", " ").split(",") if t.strip()]
        try:
            vals = [_value(t, env) for t in toks]
        except ValueError:
            continue
        if len(vals) <= n:  # aggregate initialisation zero-fills the rest
            arrays[name] = np.array(vals + [0.0] * (n - len(vals)))
    shapes = {}
    for m in re.finditer(r"std::array<unsigned int,\s*2>\s+shape([AB]\d+)\s*=\s*\{\s*(\d+)\s*,\s*(\d+)\s*\}", src):
        shapes[m.group(1)] = (int(m.group(2)), int(m.group(3)))
    mats = {}
    ctor = (r"([AB]\d+)\s*=\s*std::make_shared<diaq::denseMatrix>\(\s*(\w+)\s*,\s*heap\((\w+)\)"
            r"(?:\s*,\s*heap\((\w+)\))?\s*\)")
    for m in re.finditer(ctor, src, re.S):
        mat, dim, re_name, im_name = m.group(1), m.group(2), m.group(3), m.group(4)
        shape = (int(dim), int(dim)) if dim.isdigit() else shapes.get(dim[5:]) if dim.startswith("shape") else None
        if shape is None or re_name not in arrays or (im_name and im_name not in arrays):
            continue
        k = shape[0] * shape[1]
        # the dense constructor reads rows*cols values from the array it is given
        if arrays[re_name].size < k or (im_name and arrays[im_name].size < k):
            continue
        v = arrays[re_name][:k].astype(complex)
        if im_name:
            v = v + 1j * arrays[im_name][:k]
        mats[mat] = v.reshape(shape)
    cases = []
    for i in range(64):
        A, B = mats.get(f"A{i}"), mats.get(f"B{i}")
        if A is not None and B is not None and A.shape[1] == B.shape[0]:
            cases.append((i, A, B))
    return cases


def omat(n_off_re_im) -> orc.OMatrix:
    N, off, re_, im_ = n_off_re_im
    return orc.OMatrix(N, N, off, re_, im_)


def rand_dia(rng, r, c, n_diags=None, fill=0.7):
    """A random rectangular diagonal-sparse complex matrix (dense form)."""
    A = np.zeros((r, c), complex)
    k = min(n_diags or int(rng.integers(1, 6)), r + c - 1)
    for o in rng.choice(np.arange(-(r - 1), c), size=k, replace=False):
        idx = np.arange(max(0, -o), min(r, c - o))
        keep = rng.random(len(idx)) < fill
        A[idx[keep], idx[keep] + o] = rng.standard_normal(keep.sum()) + 1j * rng.standard_normal(keep.sum())
    return A


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=ref.REFERENCE_ROOT, help="the reference tree (default: $DIAQ_REFERENCE)")
    ap.add_argument("--skip-slow", action="store_true")
    ap.add_argument("--only", choices=["pade"], help="write only this fixture file")
    args = ap.parse_args()
    if not ref.available():
        sys.exit("build the reference CPU library first: make -C oracle ref")
    if args.only == "pade":
        write_pade()
        return

    # 1. hand-written SpGEMM cases
    cases = parse_spgemm_cases(os.path.join(args.ref, "cpp_tests", "test_main.cpp"))
    out = {"case_ids": np.array([c[0] for c in cases])}
    for i, A, B in cases:
        oa, ob = orc.OMatrix.from_dense(A), orc.OMatrix.from_dense(B)
        C = ref.product(oa, ob)
        out[f"A{i}"], out[f"B{i}"], out[f"C{i}"] = A, B, A @ B
        out[f"Coff{i}"] = C.off
        out[f"Cref{i}"] = C.to_dense()
    np.savez_compressed(os.path.join(HERE, "ref_spgemm_cases.npz"), **out)
    print("spgemm cases:", len(cases))

    # 2. TFIM n = 12
    H = omat(ham.tfim(12))
    psi = ham.random_state(H.rows, 0)
    HH = ref.product(H, H)
    t12 = {"off": H.off, "psi": psi, "Hpsi": ref.spmv(H, psi), "HH_off": HH.off, "HHpsi": orc.spmv(HH, psi)}
    prev = os.path.join(HERE, "tfim12.npz")
    if args.skip_slow and os.path.exists(prev):
        old = np.load(prev)
        for k in ("U_off", "Upsi"):
            t12[k] = old[k]
    else:
        U = ref.expm_negative(H, 0.1)
        t12["U_off"], t12["Upsi"] = U.off, orc.spmv(U, psi)
    np.savez_compressed(prev, **t12)
    print("tfim12: HH diags", HH.nd, "U diags", len(t12["U_off"]))

    # 3. small exponentials / powers
    ex = {}
    small = {"xxz6": omat(ham.xxz(6)), "xxz8": omat(ham.xxz(8)), "tfim8": omat(ham.tfim(8))}
    for name, A in small.items():
        p = ham.random_state(A.rows, 0)
        for t in (0.3, 1.7):
            U = ref.expm_negative(A, t)
            ex[f"{name}_t{t}_off"], ex[f"{name}_t{t}_Upsi"] = U.off, orc.spmv(U, p)
        for n in (3, 8):
            P = ref.pow(OScaled(A, 0.25), n)
            ex[f"{name}_pow{n}_off"], ex[f"{name}_pow{n}_Ppsi"] = P.off, orc.spmv(P, p)
    rng = np.random.default_rng(3)
    for trial in range(5):
        n = int(rng.integers(2, 10))
        Hd = rand_dia(rng, n, n, 3)
        Hd = (Hd + Hd.conj().T) / 8
        A = orc.OMatrix.from_dense(Hd)
        ex[f"herm{trial}"] = Hd
        ex[f"herm{trial}_expm"] = ref.expm(A, 100, 1.0, 1e-14).to_dense()
        ex[f"herm{trial}_expmneg"] = ref.expm_negative(A, 0.3, 100, 1.0, 1e-14).to_dense()
    np.savez_compressed(os.path.join(HERE, "expm_small.npz"), **ex)
    print("expm_small:", len(ex))

    # 4. time evolution on the reference's spMV
    hs = {}
    for name, A in {"tfim10": omat(ham.tfim(10)), "xxz10": omat(ham.xxz(10))}.items():
        p = ham.random_state(A.rows, 0)
        hs[f"{name}_psi0"] = p
        hs[f"{name}_t0.5_r5_m20"] = ref.ham_sim(A, p, 0.5, 5, 20)
        hs[f"{name}_t0.2_r3_m100"] = ref.ham_sim(A, p, 0.2, 3, 100)
    np.savez_compressed(os.path.join(HERE, "ham_sim.npz"), **hs)
    print("ham_sim:", len(hs))

    # 5. random rectangular products / SpMVs
    rng = np.random.default_rng(3)
    api = {}
    for trial in range(25):
        r, c, k = (int(x) for x in rng.integers(2, 12, size=3))
        A, B = rand_dia(rng, r, c), rand_dia(rng, c, k)
        x = rng.standard_normal(c) + 1j * rng.standard_normal(c)
        oa, ob = orc.OMatrix.from_dense(A), orc.OMatrix.from_dense(B)
        C = ref.product(oa, ob)
        api[f"A{trial}"], api[f"B{trial}"], api[f"x{trial}"] = A, B, x
        api[f"C{trial}"], api[f"Coff{trial}"], api[f"y{trial}"] = C.to_dense(), C.off, ref.spmv(oa, x)
    np.savez_compressed(os.path.join(HERE, "api_random.npz"), **api)
    print("api_random: 25")

    write_pade()


def pade_cases():
    """Inputs of the Pade fixtures: (name, matrix, t).  One-diagonal matrices (main, upper, lower,
    rectangular, all-zero) and matrices the reference's routine rejects."""
    rng = np.random.default_rng(11)
    cases = []
    for name, n, off in (("main6", 6, 0), ("upper6", 6, 2), ("lower6", 6, -1), ("main64", 64, 0)):
        L = n - abs(off)
        cases.append((name, orc.OMatrix(n, n, [off], rng.uniform(-2, 2, L), rng.uniform(-0.5, 0.5, L)), 0.7))
    cases.append(("rect3x5", orc.OMatrix(3, 5, [1], np.array([1.0, 2.0, 3.0]), np.zeros(3)), 0.5))
    cases.append(("zero3", orc.OMatrix(3, 3, [0], np.zeros(3), np.zeros(3)), 0.5))
    cases.append(("tfim3", omat(ham.tfim(3)), 0.1))
    cases.append(("xxz4", omat(ham.xxz(4)), 2.0))
    cases.append(("two2x2", orc.OMatrix(2, 2, [0, -1], np.array([1.0, 2.0, 0.5]), np.zeros(3)), 0.3))
    cases.append(("rect3x5two", orc.OMatrix(3, 5, [0, 1], np.arange(1.0, 7.0), np.zeros(6)), 0.5))
    return cases


def write_pade():
    """6. The reference's Pade exponential (src/spME.cpp:298-445) on pade_cases(): the result
    (offsets, packed values) or the message of the exception it raises."""
    pd = {}
    for name, A, t in pade_cases():
        pd[f"{name}_shape"] = np.array([A.rows, A.cols])
        pd[f"{name}_off"], pd[f"{name}_re"], pd[f"{name}_im"], pd[f"{name}_t"] = A.off, A.re, A.im, np.array(t)
        try:
            U = ref.expm_negative_pade(A, t)
            pd[f"{name}_U_off"], pd[f"{name}_U_re"], pd[f"{name}_U_im"] = U.off, U.re, U.im
        except RuntimeError as e:
            pd[f"{name}_error"] = np.array(str(e))
    np.savez_compressed(os.path.join(HERE, "pade.npz"), **pd)
    print("pade:", len(pade_cases()))


def OScaled(A: orc.OMatrix, s: float) -> orc.OMatrix:
    return orc.OMatrix(A.rows, A.cols, A.off, A.re * s, A.im * s)


if __name__ == "__main__":
    main()
