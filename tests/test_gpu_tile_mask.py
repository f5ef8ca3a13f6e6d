"""Zero-tile skipping in the term kernels: matrices whose diagonals hold runs of exact zeros
(whole 32-row tiles, tiles zero but for one row, diagonals entirely zero), at sizes that are not
multiples of 32 or 1024, evolved by every plan kernel and checked against the oracle."""
import numpy as np
import pytest

from conftest import maxrel
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _zero_tiled(N, offsets, seed):
    """Packed values with random 32-row tiles (by row index) zeroed, one lone nonzero row kept in
    some zeroed tiles, and the last diagonal all zero."""
    rng = np.random.default_rng(seed)
    re, im = [], []
    for j, d in enumerate(offsets):
        lo = max(0, -d)
        L = N - abs(d)
        rows = lo + np.arange(L)
        a = rng.standard_normal(L) + 1j * rng.standard_normal(L)
        dead = rng.random((N + 31) // 32) < 0.6
        keep_one = rng.random((N + 31) // 32) < 0.2
        z = dead[rows // 32] & ~(keep_one[rows // 32] & (rows % 32 == 7))
        a[z] = 0
        if j == len(offsets) - 1:
            a[:] = 0
        a *= 0.3
        re.append(a.real)
        im.append(a.imag)
    return np.array(offsets, dtype=np.int32), np.concatenate(re), np.concatenate(im)


def _hermitian_ish(N, seed):
    offs = [0, 1, -1, 37, -37, 700, -700, 1500, -1500, 64, 5]
    return _zero_tiled(N, offs, seed)


def _run(capi, N, off, re, im, k, mode, cfg, sl, m, steps, dt=0.05):
    import torch

    H = capi.Matrix.create(N, N, off, re, im)
    E = capi.Evolve(H, k, mode)
    if cfg is not None:
        E.set_config(*cfg)
    rng = np.random.default_rng(11)
    P = rng.standard_normal((k, N)) + 1j * rng.standard_normal((k, N))
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    pr = torch.from_numpy(np.ascontiguousarray(P.real)).cuda()
    pi = torch.from_numpy(np.ascontiguousarray(P.imag)).cuda()
    E.run(pr, pi, N, dt, steps, sl, m)
    torch.cuda.synchronize()
    A = orc.OMatrix(N, N, off, re, im)
    return A, P, (pr + 1j * pi).cpu().numpy()


@pytest.mark.parametrize("N", [3000, 2048 + 17])
@pytest.mark.parametrize("cfg", [(8, 1, 0), (8, 2, 0), (4, 2, 0), (1, 2, 0)])
def test_plain_skips_zero_tiles(native, N, cfg):
    capi, _ = native
    off, re, im = _hermitian_ish(N, 1)
    A, P, got = _run(capi, N, off, re, im, 3, capi.EVOLVE_C128, cfg, 1, 8, 3)
    for q in range(3):
        assert maxrel(got[q], orc.ham_sim(A, P[q], 0.15, 3, 8, substeps=2)) < 1e-12, q


@pytest.mark.parametrize("k", [3, 5, 16, 32])
@pytest.mark.parametrize("cfg", [(8, 4, 0), (8, 2, 0), (4, 1, 6), (4, 1, 7), (4, 1, 8), (4, 1, 9), (4, 1, 10),
                                 (4, 1, 11), (4, 1, 12)])
@pytest.mark.parametrize("mode", ["mixed", "horner"])
def test_float_forms_skip_zero_tiles(native, k, cfg, mode):
    capi, _ = native
    N = 3000
    off, re, im = _hermitian_ish(N, 2)
    md = capi.EVOLVE_MIXED if mode == "mixed" else capi.EVOLVE_HORNER
    A, P, got = _run(capi, N, off, re, im, k, md, cfg, 0, 10, 3)
    for q in sorted({0, k // 2, k - 1}):
        assert maxrel(got[q], orc.ham_sim(A, P[q], 0.15, 3, 10)) < 1e-6, q


def test_plain_plan_sees_values_written_after_creation(native):
    """The c128 plan reads the caller's matrix; its zero-tile mask is rebuilt at every run, so
    values written into the matrix after the plan was made (here by the numeric SpGEMM into a
    matrix created as zeros) are not skipped."""
    import ctypes

    import torch

    capi, _ = native
    N = 1500
    offA, reA, imA = _zero_tiled(N, [0, 3, -40], 5)
    A = capi.Matrix.create(N, N, offA, reA, imA)
    B = capi.Matrix.create(N, N, offA, reA, imA)
    L = capi.lib()
    cnt = ctypes.c_int32()
    offC = np.zeros(len(offA) ** 2, dtype=np.int32)
    capi.check(L.diaq_spgemm_symbolic(A.h, B.h, offC.ctypes.data, ctypes.byref(cnt), None))
    C = capi.Matrix.create(N, N, offC[:cnt.value])          # all zeros
    E = capi.Evolve(C, 1, capi.EVOLVE_C128)
    rng = np.random.default_rng(2)
    p = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    p /= np.linalg.norm(p)
    pr = torch.from_numpy(p.real.copy()[None, :]).cuda()
    pi = torch.from_numpy(p.imag.copy()[None, :]).cuda()
    E.run(pr, pi, N, 0.05, 1, 0, 6)                         # C = 0: psi unchanged
    torch.cuda.synchronize()
    assert np.array_equal((pr + 1j * pi).cpu().numpy()[0], p)
    capi.check(L.diaq_spgemm_numeric(A.h, B.h, C.h, None))  # C = A A
    torch.cuda.synchronize()
    E.run(pr, pi, N, 0.05, 2, 0, 6)
    torch.cuda.synchronize()
    Ao = orc.OMatrix(N, N, offA, reA, imA)
    Co = orc.product(Ao, Ao)
    assert maxrel((pr + 1j * pi).cpu().numpy()[0], orc.ham_sim(Co, p, 0.1, 2, 6)) < 1e-12


def _spmv(capi, M, x, fn="diaq_spmv_z"):
    import torch

    dt = torch.float64 if fn == "diaq_spmv_z" else torch.float32
    xr = torch.from_numpy(x.real.copy()).to("cuda", dt)
    xi = torch.from_numpy(x.imag.copy()).to("cuda", dt)
    yr, yi = torch.full_like(xr, float("nan")), torch.full_like(xi, float("nan"))
    capi.check(getattr(capi.lib(), fn)(M.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), None))
    torch.cuda.synchronize()
    return (yr.double() + 1j * yi.double()).cpu().numpy()


@pytest.mark.parametrize("N", [3000, 4096, 33])
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (2, 1e-13), (1, 1e-5)])
def test_spmv_skips_zero_tiles(native, N, prec, tol):
    capi, _ = native
    offs = [d for d in [0, 1, -1, 37, -37, 700, -700, 1500, -1500, 64, 5] if abs(d) < N]
    off, re, im = _zero_tiled(N, offs, 3)
    M = capi.Matrix.create(N, N, off, re, im, precision=prec)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    want = orc.spmv(orc.OMatrix(N, N, off, re, im), x)
    fn = "diaq_spmv_c" if prec == 1 else "diaq_spmv_z"
    for _ in range(2):  # the first call takes the mask, the second uses it
        assert maxrel(_spmv(capi, M, x, fn), want) < tol


def test_spmv_mask_follows_written_values(native):
    """SpMV of a matrix created as zeros (mask: nothing live), then filled by the numeric SpGEMM:
    the next SpMV sees the new values."""
    import ctypes

    capi, _ = native
    N = 2000
    offA, reA, imA = _zero_tiled(N, [0, 2, -33, 100], 6)
    A = capi.Matrix.create(N, N, offA, reA, imA)
    L = capi.lib()
    cnt = ctypes.c_int32()
    offC = np.zeros(len(offA) ** 2, dtype=np.int32)
    capi.check(L.diaq_spgemm_symbolic(A.h, A.h, offC.ctypes.data, ctypes.byref(cnt), None))
    C = capi.Matrix.create(N, N, offC[:cnt.value])
    x = np.random.default_rng(1).standard_normal(N) + 0j
    assert np.array_equal(_spmv(capi, C, x), np.zeros(N, dtype=complex))
    capi.check(L.diaq_spgemm_numeric(A.h, A.h, C.h, None))
    Ao = orc.OMatrix(N, N, offA, reA, imA)
    assert maxrel(_spmv(capi, C, x), orc.spmv(orc.product(Ao, Ao), x)) < 1e-12


def test_many_diagonals_cross_the_metadata_chunks(native):
    """300 diagonals: the kernels stage metadata and mask words in chunks of 256."""
    capi, _ = native
    N = 1200
    offs = sorted(set(range(-150, 150)))
    off, re, im = _zero_tiled(N, offs, 8)
    A = orc.OMatrix(N, N, off, re, im)
    x = np.random.default_rng(5).standard_normal(N) + 1j * np.random.default_rng(6).standard_normal(N)
    want = orc.spmv(A, x)
    # float pairs carry ~48 bits: a 300-term row sum ends near 1e-13
    for prec, fn, tol in ((0, "diaq_spmv_z", 1e-13), (2, "diaq_spmv_z", 1e-12), (1, "diaq_spmv_c", 1e-5)):
        M = capi.Matrix.create(N, N, off, re, im, precision=prec)
        assert maxrel(_spmv(capi, M, x, fn), want) < tol, prec
    re, im = re * 0.05, im * 0.05   # a short step for the evolution
    for mode, cfg, tol in ((capi.EVOLVE_C128, (4, 2, 0), 1e-12), (capi.EVOLVE_HORNER, (4, 1, 9), 1e-6),
                           (capi.EVOLVE_MIXED, (4, 1, 6), 1e-6), (capi.EVOLVE_HORNER, (4, 1, 10), 1e-6),
                           (capi.EVOLVE_HORNER, (4, 1, 12), 1e-6)):
        Ao, P, got = _run(capi, N, off, re, im, 5, mode, cfg, 0, 8, 2)
        for q in (0, 4):
            assert maxrel(got[q], orc.ham_sim(Ao, P[q], 0.1, 2, 8)) < tol, (mode, q)


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_spgemm_skips_zero_tiles(native, prec, tol):
    """A B with zero tiles in both factors and odd offsets (a thread's B rows straddle two tiles):
    the same offsets as the oracle, values within tol; rectangular shapes."""
    import ctypes

    capi, _ = native

    def rand(rows, cols, offs, seed):
        r = np.random.default_rng(seed)
        re, im = [], []
        for d in offs:
            lo, hi = max(0, -d), min(rows, cols - d)
            L = hi - lo
            rr = lo + np.arange(L)
            a = r.standard_normal(L) + 1j * r.standard_normal(L)
            dead = r.random((rows + 31) // 32) < 0.5
            a[dead[rr // 32]] = 0
            re.append(a.real)
            im.append(a.imag)
        return orc.OMatrix(rows, cols, np.array(offs, dtype=np.int32), np.concatenate(re), np.concatenate(im))

    A = rand(1500, 1300, [0, 1, -3, 33, -65, 7, 200], 1)
    B = rand(1300, 1700, [0, -1, 5, 31, -40, 129, 3], 2)
    dA = capi.Matrix.create(A.rows, A.cols, A.off, A.re, A.im, precision=prec)
    dB = capi.Matrix.create(B.rows, B.cols, B.off, B.re, B.im, precision=prec)
    out = ctypes.c_void_p()
    capi.check(capi.lib().diaq_spgemm(dA.h, dB.h, 0, None, ctypes.byref(out)))
    C = capi.Matrix(out)
    off, re, im = C.download()
    want = orc.product(A, B, prune_result=False)
    assert np.array_equal(np.sort(off), np.sort(want.off))
    got = orc.OMatrix(A.rows, B.cols, off, re, im)
    assert maxrel(got.to_dense(), want.to_dense()) < tol
