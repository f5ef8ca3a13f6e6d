"""The byte and multiply-add counts behind the bench line's rooflines, against brute force on
small matrices (no GPU): values in live 32-row tiles, and the complex multiply-adds of A A whose
two factors lie in live tiles."""
import numpy as np

import bench
from diaq_gb300 import hamiltonians as ham


def _zero_tiled(N, offs, seed):
    rng = np.random.default_rng(seed)
    re, im = [], []
    for d in offs:
        lo, L = max(0, -d), N - abs(d)
        rows = lo + np.arange(L)
        a = rng.standard_normal(L) + 1j * rng.standard_normal(L)
        a[(rng.random((N + 31) // 32) < 0.5)[rows // 32]] = 0
        re.append(a.real)
        im.append(a.imag)
    return np.array(offs), np.concatenate(re), np.concatenate(im)


def _row_live(N, offs, re, im):
    """Per diagonal: rows whose 32-row tile holds a nonzero of that diagonal (brute force)."""
    out, pos = {}, 0
    for d in offs:
        d = int(d)
        lo, L = max(0, -d), N - abs(d)
        v = np.zeros(N, dtype=bool)
        v[lo:lo + L] = (re[pos:pos + L] != 0) | (im[pos:pos + L] != 0)
        live = np.zeros(N, dtype=bool)
        for t in range((N + 31) // 32):
            live[32 * t:32 * t + 32] = v[32 * t:32 * t + 32].any()
        inside = np.zeros(N, dtype=bool)
        inside[lo:lo + L] = True
        out[d] = live & inside
        pos += L
    return out


def test_tile_live_values_against_brute_force():
    for N, offs, seed in [(200, [0, 1, -1, 5, -7, 33, -40, 64], 0), (1000, [0, 3, -3, 31, -32, 500], 1)]:
        off, re, im = _zero_tiled(N, offs, seed)
        want = sum(int(v.sum()) for v in _row_live(N, off, re, im).values())
        assert bench.tile_live_values(N, off, re, im) == want


def test_tile_live_values_of_the_xxz_chain():
    N, off, re, im = ham.xxz(12)
    live = bench.tile_live_values(N, off, re, im)
    assert 0 < live < re.size          # the hops leave whole tiles zero from the 5th qubit on
    N, off, re, im = ham.xxz(4)        # 16 rows: one tile, every stored value live
    assert bench.tile_live_values(N, off, re, im) == re.size


def test_live_macs_against_brute_force():
    N, offs = 200, [0, 1, -1, 5, -7, 33, -40, 64]
    off, re, im = _zero_tiled(N, offs, 2)
    rl = _row_live(N, off, re, im)
    want = 0
    for da in rl:
        for db in rl:
            if not -N < da + db < N:
                continue
            for r in range(N):
                if 0 <= r + da < N and rl[da][r] and rl[db][r + da]:
                    want += 1
    assert bench._live_macs(N, off, re, im) == want


def test_cpu_baseline_sample_returns_the_evolved_state():
    """The CPU baseline sample evolves psi0 (seed 0) for the steps it reports and returns that
    state: the reference the bench line's state-0 accuracy is measured against."""
    from oracle import oracle as orc

    N, off, re, im = ham.xxz(8)
    base, psi, done = bench.cpu_baseline_sample(N, off, re, im, 1, 6, steps=3)
    assert done == 3 and base["unit"] == "states·steps/s" and base["value"] > 0 and base["kind"] == "port"
    want = orc.ham_sim(orc.OMatrix(N, N, off, re, im), ham.random_state(N, 0), 3 * bench.DT, 3, 6, substeps=2)
    assert np.linalg.norm(psi - want) / np.linalg.norm(want) < 1e-12
