#!/usr/bin/env python3
"""expm(-iHt)·psi throughput (states·steps/s) on the 20-qubit periodic XXZ chain.

Workload: H = sum_i J_i (XX + YY + 0.8 ZZ)_{i,i+1} + sum_i h_i Z_i, J ~ U[0.5,1.5], h ~ U[-1,1]
(seed 1), 2^20 rows, 41 diagonals, complex128; random normalised states (seed 0); time steps of
dt = 0.05.  A bench "step" is one time step of every state in the batch.  Synthetic inputs, built
in-process.

  python bench.py [--steps K] [--warmup W] [--form plain|chosen] [--n 20]
  python bench.py --impl reference      # the CPU restatement of the same evolution (oracle port)
  torchrun ... bench.py --gpus N        # N independent replicas (the path does not shard)

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DT = 0.05
TOL_STEP = 1e-8     # per time step: 100 steps stay within 1e-6 of the exact evolution
METRIC = "expm(-iHt)·ψ states·steps/s"
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the chosen form's term kernel, from
# ncu captures (profiles/), keyed by (qubits, states, form, states per block, rows per thread,
# variant): for variant 12 the mean over the 12 launches of one time step (first, middle and last
# terms, as roofline.achieved averages them); for variant 9 one middle term.  The kernels skip
# all-zero 32-row tiles.
TRAFFIC_PER_LAUNCH = {(20, 8, "horner", 4, 1, 9): 390.6e6, (20, 8, "horner", 4, 1, 12): 378.3e6}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---- clocks ---------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = self.gpu_id(device_index)
        self.proc = None
        self.lines = []

    @staticmethod
    def gpu_id(device_index: int) -> str:
        """nvidia-smi's name for CUDA device `device_index`: its UUID.  nvidia-smi ignores
        CUDA_VISIBLE_DEVICES and may number the GPUs differently, so an index could name another
        GPU of the machine."""
        try:
            import torch

            u = str(torch.cuda.get_device_properties(device_index).uuid)
            return u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            return str(device_index)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: let its first sample land before the timed
            # region begins, so that the samples fall inside it
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = len(self.lines)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the samples taken inside the timed region (else the last one before it)
        for ln in self.lines[getattr(self, "skip", 0):] or self.lines[-1:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- workload -------------------------------------------------------------------------------------
def workload(n: int):
    from diaq_gb300 import hamiltonians as ham

    N, off, re, im = ham.xxz(n)
    return N, off, re, im


def plain_schedule(capi, norm1: float):
    s, m = capi.select_sm(norm1, DT, TOL_STEP, 1.0, 100)
    return s, m


# ---- reference arm: the CPU restatement -------------------------------------------------------------
def run_reference(args, rank):
    """The reference's own CPU code where it was built on this host (oracle/_ref, x86 builds of
    the reference sources), else the C restatement of the same algorithm (the GPU hosts, which
    do not have the reference sources)."""
    if rank != 0:
        return
    from oracle import oracle as orc
    from oracle import reference as ref
    from oracle import timing as tim
    from diaq_gb300 import hamiltonians as ham

    N, off, re, im = workload(args.n)
    H = orc.OMatrix(N, N, off, re, im)
    norm1 = orc.norm1_est(H)
    s, m = _select_sm_py(norm1)
    psi = ham.random_state(N, 0)
    steps = max(1, min(args.steps, args.ref_steps))
    warm = max(0, min(args.warmup, args.ref_steps))   # W untimed steps, bounded like the timed ones
    kind, cores = "port", orc.threads()
    step = lambda p: tim.ham_sim(H, p, DT, 1 << s, m)
    try:
        if ref.available():
            ref.lib()
            kind, cores = "reference", ref.lib().ref_threads()
            step = lambda p: ref.ham_sim(H, p, DT, 1 << s, m)
    except OSError:
        pass
    for _ in range(warm):
        psi = step(psi)
    t0 = time.perf_counter()
    for _ in range(steps):
        psi = step(psi)
    wall = time.perf_counter() - t0
    value = steps / wall
    what = ("the reference's CPU spMV (src/spMV.cpp) driving the time-evolution rule"
            if kind == "reference" else
            "C/OpenMP restatement of the reference's CPU scheme (oracle/diaq_timing.c: (diagonal, tile) "
            "tasks, thread-local y, -O3), within 2 % of the reference's own library where both were timed")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "states·steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * wall / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"xxz{args.n}_periodic_evolve", "n_qubits": args.n, "rows": N, "ndiag": len(off),
                   "dt": DT, "substeps": 1 << s, "taylor_terms": m, "states": 1},
        "cpu_baseline": {"value": value, "unit": "states·steps/s", "cores": cores, "kind": kind,
                         "sample": f"{steps} time step(s) of one state, {1 << s}x{m} SpMVs each, {what}"},
        "e2e": {"value": value, "unit": "states·steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if kind == "port":
        line["note"] = ("the reference's CPU sources are not on this host, so its CPU library cannot be built "
                        "here; the C restatement of its CPU scheme is timed")
    print(json.dumps(line), flush=True)


def _select_sm_py(norm1):
    """The same rule as diaq_select_sm, for hosts where only the oracle is built."""
    import math

    theta0 = DT * norm1
    s = math.ceil(math.log2((theta0 + 1e-12) / 1.0)) if theta0 + 1e-12 > 1.0 else 0
    theta = math.ldexp(theta0, -s)
    budget = math.ldexp(TOL_STEP, -s)
    term, k = theta * math.exp(theta), 0
    while k < 100:
        k += 1
        term *= theta / (k + 1)
        if term <= budget:
            break
    return s, k


# ---- our arm -----------------------------------------------------------------------------------------
def cpu_baseline_sample(N, off, re, im, s, m, steps=None):
    """The reference's time-evolution rule for psi0 (seed 0) on the host cores in FP64, timed: the
    restatement of the reference's CPU scheme (oracle/diaq_timing.c, pinned to the parity oracle by
    tests/test_oracle.py).  `steps` time steps when given, else whole steps until ~10 s have passed
    (at most 20).  Returns (baseline, final state, steps done): the state is the reference for the
    accuracy of a GPU run of the same steps from the same psi0."""
    from oracle import oracle as orc
    from oracle import timing as tim
    from diaq_gb300 import hamiltonians as ham

    H = orc.OMatrix(N, N, off, re, im)
    psi = ham.random_state(N, 0)
    # one time step = 2^s * m SpMVs, in the timing restatement of the reference's CPU scheme
    t0 = time.perf_counter()
    done = 0
    while True:
        psi = tim.ham_sim(H, psi, DT, 1 << s, m)
        done += 1
        if steps is not None and done >= steps:
            break
        if steps is None and (time.perf_counter() - t0 > 10.0 or done >= 20):
            break
    wall = time.perf_counter() - t0
    base = {"value": done / wall, "unit": "states·steps/s", "cores": orc.threads(), "kind": "port",
            "sample": f"{done} time step(s) of one state ({1 << s}x{m} SpMVs each) on the host: the C/OpenMP "
                      f"restatement of the reference's CPU scheme (oracle/diaq_timing.c)"}
    return base, psi, done


def _timed(stream, fn):
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def _max_over_ranks(ms, world, dev):
    import torch

    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def _sum_over_ranks(v, world, dev):
    import torch

    if world > 1:
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
        v = float(t.item())
    return v


def _barrier(world, cuda=True):
    import torch

    if cuda:
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    if cuda:
        torch.cuda.synchronize()


def partition_instances(costs, world):
    """Independent instances to ranks: largest first, each to the least-loaded rank (ties to the
    lower rank), so every rank gets about the same work; returns one index list per rank."""
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda j: (-costs[j], j)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def run_spmv_only(args):
    """Repeated SpMV on the workload (c128 and c64), for profiling the kernel on its own."""
    import torch

    from diaq_gb300 import build, capi
    from diaq_gb300 import hamiltonians as ham

    build.build()
    L = capi.lib()
    N, off, re, im = workload(args.n)
    H = capi.Matrix.create(N, N, off, re, im)
    Hc = H.convert(capi.C64)
    Hf = H.convert(capi.C128F2)
    psi = ham.random_state(N, 0)
    sp = torch.cuda.current_stream().cuda_stream
    live = tile_live_values(N, off, re, im)
    out = {"stored_values": int(re.size), "live_tile_values": live}
    for name, M, dt, fn in (("c128", H, torch.float64, L.diaq_spmv_z), ("c64", Hc, torch.float32, L.diaq_spmv_c),
                            ("c128f2", Hf, torch.float64, L.diaq_spmv_z)):
        xr = torch.from_numpy(psi.real.copy()).to("cuda", dt)
        xi = torch.from_numpy(psi.imag.copy()).to("cuda", dt)
        yr, yi = torch.empty_like(xr), torch.empty_like(xi)
        for _ in range(args.warmup):
            capi.check(fn(M.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))

        def loop():   # y = A x from the same x each time (float pairs overflow above ~1e38)
            for _ in range(args.spmv_reps):
                capi.check(fn(M.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))

        torch.cuda.synchronize()
        us = 1e3 * _timed(torch.cuda.current_stream(), loop) / args.spmv_reps
        # algorithmic bytes: the values of the live tiles (the kernels skip the all-zero ones), x, y
        w = 8 if name == "c64" else 16
        by = w * live + 2 * w * N
        peak, _ = peaks()
        out[name] = {"us": us, "gbs": by / us / 1e3, "frac": by / us / 1e3 / peak, "bytes": by,
                     "effective_gbs": (w * int(re.size) + 2 * w * N) / us / 1e3}
        if name == "c128":
            out[name]["dfma_per_s"] = 4 * live / (us * 1e-6)
        if name == "c128f2":   # error of the float-pair product against the float64 one
            y64r, y64i = torch.empty_like(xr), torch.empty_like(xi)
            capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), y64r.data_ptr(), y64i.data_ptr(), sp))
            capi.check(fn(M.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))
            torch.cuda.synchronize()
            d = torch.maximum((yr - y64r).abs().max(), (yi - y64i).abs().max())
            out[name]["maxrel_vs_c128"] = float(d / torch.maximum(y64r.abs().max(), y64i.abs().max()))
    print(json.dumps({"mode": "spmv", "n_qubits": args.n, **out}), flush=True)


def _spgemm_counts(n_rows, offA, offB):
    """Result offsets and the complex multiply-adds of A B for square n_rows matrices: pair
    (da, db) contributes one per row r with r in A's diagonal da and r + da in B's diagonal db."""
    res, macs = set(), 0
    for da in offA:
        lo1, hi1 = max(0, -da), min(n_rows, n_rows - da)
        for db in offB:
            dc = da + db
            if dc <= -n_rows or dc >= n_rows:
                continue
            lo2, hi2 = max(0, -db) - da, min(n_rows, n_rows - db) - da
            macs += max(0, min(hi1, hi2) - max(lo1, lo2))
            res.add(dc)
    return sorted(res), macs


def run_ops(args):
    """The path's other operations on the named workloads, on the GPU, beside the CPU reference
    (the reference's own CPU library where it was built on this host, else its C restatement):
    12-qubit TFIM (config 1): H psi, H H (exact-zero diagonals pruned, as the CPU path does) and
    expm_negative(H, 0.1) psi; 20-qubit XXZ (config 2): the structural dry-run and the numeric
    SpGEMM of H H.  GPU times by CUDA events / wall clock around synchronous calls."""
    import torch

    from diaq_gb300 import build, capi
    from diaq_gb300 import hamiltonians as ham
    from oracle import oracle as orc
    from oracle import reference as ref

    build.build()
    L = capi.lib()
    peak, peak_kind = peaks()
    dfma_peak = 0.594e12   # FP64 FMA/s measured on a GB300 (throughput probe)
    use_ref = False
    try:
        use_ref = ref.available() and ref.lib() is not None
    except OSError:
        use_ref = False
    cpu = ref if use_ref else orc
    kind = "reference" if use_ref else "port"
    out = {"mode": "ops", "cpu_kind": kind, "cpu_threads": (ref.lib().ref_threads() if use_ref else orc.threads())}

    def gpu_wall(fn, reps=1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    def cpu_wall(fn, reps=1):
        t0 = time.perf_counter()
        for _ in range(reps):
            r = fn()
        return (time.perf_counter() - t0) / reps, r

    # ---- config 1: 12-qubit TFIM ----
    if args.ops == "xxz":
        return _ops_xxz(args, out, L, peak, peak_kind, dfma_peak, cpu, gpu_wall, cpu_wall)
    N, off, re, im = ham.tfim(12)
    H = capi.Matrix.create(N, N, off, re, im)
    Ho = orc.OMatrix(N, N, off, re, im)
    psi = ham.random_state(N, 0)
    xr = torch.from_numpy(psi.real.copy()).cuda()
    xi = torch.from_numpy(psi.imag.copy()).cuda()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    sp = torch.cuda.current_stream().cuda_stream
    spmv = lambda: capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))
    spmv()
    t_spmv = gpu_wall(spmv, 200)

    def product():
        C = ctypes.c_void_p()
        capi.check(L.diaq_spgemm(H.h, H.h, 1, None, ctypes.byref(C)))
        capi.check(L.diaq_matrix_destroy(C))

    product()
    t_prod = gpu_wall(product, 20)

    def expm():
        U = ctypes.c_void_p()
        s_o, m_o = ctypes.c_int(), ctypes.c_int()
        capi.check(L.diaq_expm_negative(H.h, 0.1, 100, 1.0, 1e-12, 1, None, ctypes.byref(U), ctypes.byref(s_o),
                                        ctypes.byref(m_o)))
        return capi.Matrix(U)

    expm()
    t0 = time.perf_counter()
    U = expm()
    torch.cuda.synchronize()
    t_expm = time.perf_counter() - t0
    nd_U = U.info()[2]
    del U
    c_spmv, _ = cpu_wall(lambda: cpu.spmv(Ho, psi), 20)
    c_prod, _ = cpu_wall(lambda: cpu.product(Ho, Ho), 3)
    # the CPU exponential at 12 qubits fills to 8191 diagonals and takes minutes: time both at 10
    N10, off10, re10, im10 = ham.tfim(10)
    H10 = capi.Matrix.create(N10, N10, off10, re10, im10)
    H10o = orc.OMatrix(N10, N10, off10, re10, im10)

    def expm10():
        U = ctypes.c_void_p()
        s_o, m_o = ctypes.c_int(), ctypes.c_int()
        capi.check(L.diaq_expm_negative(H10.h, 0.1, 100, 1.0, 1e-12, 1, None, ctypes.byref(U), ctypes.byref(s_o),
                                        ctypes.byref(m_o)))
        return capi.Matrix(U)

    expm10()
    t0 = time.perf_counter()
    U10 = expm10()
    torch.cuda.synchronize()
    t_expm10 = time.perf_counter() - t0
    c_expm10, U10c = cpu_wall(lambda: cpu.expm_negative(H10o, 0.1))
    o10, r10, i10 = U10.download()
    gd = orc.OMatrix(N10, N10, o10, r10, i10).to_dense()
    cd = U10c.to_dense()
    out["tfim12"] = {
        "spmv": {"gpu_us": 1e6 * t_spmv, "cpu_us": 1e6 * c_spmv},
        "product_HH": {"gpu_ms": 1e3 * t_prod, "cpu_ms": 1e3 * c_prod},
        "expm_negative_t0.1": {"gpu_ms": 1e3 * t_expm, "result_diagonals": nd_U,
                               "note": "CPU not timed at 12 qubits (minutes); see tfim10"},
    }
    out["tfim10"] = {"expm_negative_t0.1": {"gpu_ms": 1e3 * t_expm10, "cpu_ms": 1e3 * c_expm10,
                                            "max_rel_diff_gpu_vs_cpu": float(np.abs(gd - cd).max() / np.abs(cd).max())}}
    del H, H10, U10
    _ops_xxz(args, out, L, peak, peak_kind, dfma_peak, cpu, gpu_wall, cpu_wall)


def _live_macs(N, off, re, im):
    """Complex multiply-adds of A A (square DiaQ A, packed values) whose two factors both lie in
    32-row tiles holding a nonzero: what the numeric SpGEMM does once it skips zero tiles."""
    live_rows, pos = {}, 0
    for d in off:
        d = int(d)
        lo, L = max(0, -d), N - abs(d)
        nz = np.zeros(N, dtype=bool)
        nz[lo:lo + L] = (re[pos:pos + L] != 0) | (im[pos:pos + L] != 0)
        tiles = nz.reshape(-1, 32).any(axis=1) if N % 32 == 0 else np.add.reduceat(nz, np.arange(0, N, 32)) > 0
        row_live = np.repeat(tiles, 32)[:N]
        row_live[:lo] = False
        row_live[lo + L:] = False
        live_rows[d] = row_live
        pos += L
    macs = 0
    for da in live_rows:
        a = live_rows[da]
        for db in live_rows:
            if not -N < da + db < N:
                continue
            b = live_rows[db]
            r0, r1 = max(0, -da), min(N, N - da)   # rows r with r + da inside B
            if r1 > r0:
                macs += int(np.count_nonzero(a[r0:r1] & b[r0 + da:r1 + da]))
    return macs


def _ops_xxz(args, out, L, peak, peak_kind, dfma_peak, cpu, gpu_wall, cpu_wall):
    """Config 2's H H at args.n qubits: dry-run and numeric SpGEMM on the GPU, the CPU product."""
    import torch

    from diaq_gb300 import capi
    from oracle import oracle as orc

    # ---- config 2: 20-qubit XXZ, H H ----
    N, off, re, im = workload(args.n)
    H = capi.Matrix.create(N, N, off, re, im)
    res, macs = _spgemm_counts(N, [int(d) for d in off], [int(d) for d in off])
    live_macs = _live_macs(N, off, re, im)
    offs = np.empty(len(off) * len(off), dtype=np.int32)
    cnt = ctypes.c_int32()

    def symbolic():
        capi.check(L.diaq_spgemm_symbolic(H.h, H.h, offs.ctypes.data, ctypes.byref(cnt), None))

    symbolic()
    t_sym = gpu_wall(symbolic, 20)

    def full():
        C = ctypes.c_void_p()
        capi.check(L.diaq_spgemm(H.h, H.h, 0, None, ctypes.byref(C)))
        return capi.Matrix(C)

    C = full()
    sum_c = C.info()[3]
    del C
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    C = full()
    torch.cuda.synchronize()
    t_full = time.perf_counter() - t0
    del C
    torch.cuda.empty_cache()
    algo_bytes = 16 * (2 * int(re.size) + sum_c) + 4 * len(off) * len(off)
    Ho = orc.OMatrix(N, N, off, re, im)
    c_prod20, Wc = cpu_wall(lambda: cpu.product(Ho, Ho))
    # parity at full size: the pruned product's offsets bit-exact, its Frobenius norm (both sides
    # over every stored value) relative
    Cp = ctypes.c_void_p()
    capi.check(L.diaq_spgemm(H.h, H.h, 1, None, ctypes.byref(Cp)))
    Cp = capi.Matrix(Cp)
    fro = ctypes.c_double()
    capi.check(L.diaq_frobenius(Cp.h, ctypes.byref(fro), None))
    offs_equal = bool(np.array_equal(Cp.offsets(), np.asarray(Wc.off)))
    fro_cpu = float(np.sqrt(np.sum(np.asarray(Wc.re) ** 2) + np.sum(np.asarray(Wc.im) ** 2)))
    del Cp, Wc
    torch.cuda.empty_cache()
    out[f"xxz{args.n}"] = {
        "product_HH": {"gpu_ms": 1e3 * t_full, "symbolic_ms": 1e3 * t_sym, "cpu_ms": 1e3 * c_prod20,
                       "result_offsets": int(cnt.value), "result_stored_values": int(sum_c),
                       "offsets_equal_cpu": offs_equal, "frobenius_rel_diff_cpu": abs(fro.value - fro_cpu) / fro_cpu,
                       "complex_macs": int(macs), "complex_macs_live_tiles": int(live_macs),
                       "algorithmic_bytes": int(algo_bytes),
                       "gbs": algo_bytes / t_full / 1e9, "frac_hbm": algo_bytes / t_full / 1e9 / peak,
                       "dfma_per_s": 4 * live_macs / t_full, "frac_fp64": 4 * live_macs / t_full / dfma_peak,
                       "note": "includes the device allocation and zeroing of C and the dry-run; products "
                               "with a factor in an all-zero 32-row tile are skipped, so the FP64 rate counts "
                               "complex_macs_live_tiles (4 DFMA each); parity: the pruned product's offsets "
                               "and Frobenius norm against the CPU product"}}
    out["peak_hbm_gbs"] = peak
    out["peak_kind"] = peak_kind
    print(json.dumps(out), flush=True)


def measure_spgemm(n: int, peak: float):
    """H H of the n-qubit XXZ chain on the GPU (config 2's SpGEMM): the structural dry-run alone,
    and the whole product (dry-run, allocation of C, numeric pass), by CUDA events around
    synchronous calls.  Algorithmic bytes 16 (sum len A + sum len B + sum len C) plus the dry-run's
    4 dA dB.  Parity at full size: the result offsets against the oracle's dry-run (bit-exact), and
    C psi against the oracle's H (H psi) (a size-independent property of the product)."""
    import torch

    from diaq_gb300 import capi
    from diaq_gb300 import hamiltonians as ham
    from oracle import oracle as orc

    L = capi.lib()
    N, off, re, im = workload(n)
    H = capi.Matrix.create(N, N, off, re, im)
    offs = np.empty(len(off) * len(off), dtype=np.int32)
    cnt = ctypes.c_int32()
    stream = torch.cuda.current_stream()

    def symbolic():
        capi.check(L.diaq_spgemm_symbolic(H.h, H.h, offs.ctypes.data, ctypes.byref(cnt), None))

    def full():
        C = ctypes.c_void_p()
        capi.check(L.diaq_spgemm(H.h, H.h, 0, None, ctypes.byref(C)))
        return capi.Matrix(C)

    symbolic()
    torch.cuda.synchronize()
    reps = 10
    ms_sym = _timed(stream, lambda: [symbolic() for _ in range(reps)]) / reps
    C = full()
    del C
    torch.cuda.empty_cache()
    holder = {}
    ms_full = _timed(stream, lambda: holder.setdefault("C", full()))
    C = holder["C"]
    _, _, nd_c, sum_c, _ = C.info()
    Ho = orc.OMatrix(N, N, off, re, im)
    want_off = orc.spgemm_symbolic(Ho, Ho)
    offsets_equal = bool(np.array_equal(C.offsets(), np.asarray(want_off)))
    psi = ham.random_state(N, 0)
    xr = torch.from_numpy(psi.real.copy()).cuda()
    xi = torch.from_numpy(psi.imag.copy()).cuda()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    capi.check(L.diaq_spmv_z(C.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), None))
    torch.cuda.synchronize()
    got = yr.cpu().numpy() + 1j * yi.cpu().numpy()
    want = orc.spmv(Ho, orc.spmv(Ho, psi))
    rel = float(np.abs(got - want).max() / np.abs(want).max())
    del C, xr, xi, yr, yi
    torch.cuda.empty_cache()
    algo = 16 * (2 * int(re.size) + int(sum_c)) + 4 * len(off) * len(off)
    return {"workload": f"xxz{n}_periodic_HH", "symbolic_ms": ms_sym, "product_ms": ms_full,
            "result_offsets": int(nd_c), "result_stored_values": int(sum_c),
            "algorithmic_bytes": int(algo), "gbs": algo / ms_full / 1e6, "frac_hbm": algo / ms_full / 1e6 / peak,
            "offsets_equal_oracle_dryrun": offsets_equal, "rel_err_C_psi_vs_oracle_H_H_psi": rel,
            "note": "product_ms: dry-run + allocation of C + numeric pass (exact-zero diagonals kept, as the "
                    "reference's device product does); kernels skip products with a factor in an all-zero 32-row "
                    "tile; the bytes count every stored value of A, B and C"}


def chosen_schedule(capi, H, norm1):
    """(s, m, how) of the chosen form: the trained network's checked proposal when the package
    ships one, else the cheapest (s, m) under the remainder bound."""
    from diaq_gb300 import learn

    if os.path.exists(learn.PARAMS_PATH):
        s, m, src, rec = learn.learned_sm(H, DT, TOL_STEP)
        del rec
        import torch

        torch.cuda.empty_cache()
        if src == "learned":
            return s, m, "learned (MLP proposal, next-term check)"
    s, m = capi.select_sm_min_cost(norm1, DT, TOL_STEP, 12, 60)
    return s, m, "min-cost remainder bound"


def run_chosen_only(args):
    """Only the chosen form's evolution, W + K steps (a light command for profilers)."""
    import torch

    from diaq_gb300 import build, capi
    from diaq_gb300 import hamiltonians as ham

    build.build()
    L = capi.lib()
    N, off, re, im = workload(args.n)
    H = capi.Matrix.create(N, N, off, re, im)
    norm1 = ctypes.c_double()
    capi.check(L.diaq_norm1_est(H.h, ctypes.byref(norm1), None))
    s_c, m_c, _ = chosen_schedule(capi, H, norm1.value)
    E = capi.Evolve(H, args.states, capi.EVOLVE_HORNER if args.horner else capi.EVOLVE_MIXED)
    if args.shape:
        k, v, p = (int(x) for x in args.shape.split(","))
        E.set_config(k, v, p)
    P0 = ham.random_state(N, 0, k=args.states) if args.states > 1 else ham.random_state(N, 0)[None, :]
    pr = torch.from_numpy(np.ascontiguousarray(P0.real)).cuda()
    pi = torch.from_numpy(np.ascontiguousarray(P0.imag)).cuda()
    sp = torch.cuda.current_stream().cuda_stream
    E.run(pr, pi, N, DT, args.warmup, s_c, m_c, sp)
    ms = _timed(torch.cuda.current_stream(), lambda: E.run(pr, pi, N, DT, args.steps, s_c, m_c, sp))
    print(json.dumps({"mode": "chosen", "horner": args.horner, "n_qubits": args.n, "states": args.states, "s": s_c, "m": m_c,
                      "shape": list(E.config()) + [E.pipelined()],
                      "ms_per_step": ms / args.steps, "us_per_launch": 1e3 * ms / args.steps / E.launches_per_step()}),
          flush=True)


def _pauli_chain(model, n, rng):
    """TFIM (open; J ~ U[0.5,1.5], h ~ U[0.2,2]) or XXZ (periodic; J ~ U[0.5,1.5], Delta 0.8,
    h ~ U[-1,1]) as Pauli strings."""
    terms = []
    if model == "tfim":
        J = rng.uniform(0.5, 1.5, n - 1)
        h = rng.uniform(0.2, 2.0, n)
        terms += [(-J[i], {i: "Z", i + 1: "Z"}) for i in range(n - 1)]
        terms += [(-h[i], {i: "X"}) for i in range(n)]
    else:
        J = rng.uniform(0.5, 1.5, n)
        h = rng.uniform(-1.0, 1.0, n)
        for i in range(n):
            j = (i + 1) % n
            terms += [(J[i], {i: "X", j: "X"}), (J[i], {i: "Y", j: "Y"}), (0.8 * J[i], {i: "Z", j: "Z"})]
        terms += [(h[i], {i: "Z"}) for i in range(n)]
    return terms


def graph_launch_gap_us(n: int = 200) -> float:
    """Time per kernel node of a replayed CUDA graph of n dependent one-element kernels: what a
    graph pays between two dependent launches on this GPU (the gap a single persistent launch per
    step would save, phase by phase)."""
    import torch

    x = torch.zeros(1, device="cuda")
    x.add_(1)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(n):
            x.add_(1)
    g.replay()
    torch.cuda.synchronize()
    reps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    return 1e3 * e0.elapsed_time(e1) / (reps * n)


def measure_batched(instances=512, n_lo=10, n_hi=22, seed=4, variants=("c64",), c64_steps=50, c128_steps=3,
                    warmup=3, horner=True, planar=False, mem_gb=200.0, world=1, rank=0, dev="cuda"):
    """Config 4: many Hamiltonians of uneven size with several states each, one persistent
    work-queued launch per Taylor phase over all of them, the step recorded as a CUDA graph.
    Instances: qubit counts uniform on n_lo..n_hi, even ones TFIM and odd ones XXZ, k in {1, 4, 16}
    states each (seeded); dt = 0.02; run in groups under a device-memory budget.  Accuracy: the
    first state of up to three instances of at most 12 qubits per group against the oracle with the
    same (s, m) and steps."""
    import torch

    from diaq_gb300 import capi
    from diaq_gb300 import hamiltonians as ham
    from oracle import oracle as orc

    L = capi.lib()
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(instances):
        n = int(rng.integers(n_lo, n_hi + 1))
        model = "tfim" if i % 2 == 0 else "xxz"
        k = int(rng.choice([1, 4, 16]))
        specs.append((model, n, k, _pauli_chain(model, n, rng)))
    all_states = int(sum(k for _, _, k, _ in specs))
    mine = partition_instances([k * (2 * n + 1) * (1 << n) for _, n, k, _ in specs], world)[rank]
    specs = [specs[i] for i in mine]
    dt, tol = 0.02, TOL_STEP
    gap_us = graph_launch_gap_us()
    out = {"workload": f"batch{instances}_n{n_lo}-{n_hi}_tfim_xxz", "horner": horner, "interleaved": not planar,
           "instances": instances, "n_range": [n_lo, n_hi], "dt": dt, "states": all_states, "n_gpus": world,
           "scaling": "weak" if world > 1 else None, "graph_launch_gap_us": gap_us, "variants": {}}
    for variant in variants:
        prec = capi.C64 if variant == "c64" else capi.C128
        w = 8 if variant == "c64" else 16
        steps = c64_steps if variant == "c64" else c128_steps
        # memory per instance: matrix + states (f64) + 8 work vectors
        groups, cur, cur_bytes = [], [], 0
        for idx, (model, n, k, terms) in enumerate(specs):
            N = 1 << n
            est = w * (2 * n + 1) * N + 16 * k * N + 8 * w * k * N
            if cur and cur_bytes + est > mem_gb * 1e9:
                groups.append(cur)
                cur, cur_bytes = [], 0
            cur.append(idx)
            cur_bytes += est
        groups.append(cur)
        total_ms, total_states_steps, checks, phase_steps = 0.0, 0, [], 0
        gen = torch.Generator(device="cuda").manual_seed(7)
        cfg = (0, 0, 0)
        for grp in groups:
            mats, prs, pis, sched_s, sched_m = [], [], [], [], []
            for idx in grp:
                model, n, k, terms = specs[idx]
                M = capi.Matrix.from_pauli(n, *ham.pauli_masks(n, terms), precision=prec)
                nrm = ctypes.c_double()
                capi.check(L.diaq_norm1_est(M.h, ctypes.byref(nrm), None))
                s_i, m_i = capi.select_sm_min_cost(nrm.value, dt, tol, 12, 60)
                z = torch.randn((k, 1 << n), dtype=torch.complex128, device="cuda", generator=gen)
                z = z / torch.linalg.vector_norm(z, dim=1, keepdim=True)
                mats.append(M)
                prs.append(z.real.contiguous())
                pis.append(z.imag.contiguous())
                sched_s.append(s_i)
                sched_m.append(m_i)
            small = [j for j, idx in enumerate(grp) if specs[idx][1] <= 12][:3]
            start = {j: (prs[j][0].cpu().numpy() + 1j * pis[j][0].cpu().numpy()) for j in small}
            B = capi.Batch(mats, prs, pis)
            B.set_horner(horner)
            B.set_interleaved(not planar)
            if variant == "c128":
                B.set_config(4, 2)   # FP64-bound either way; autotuning would cost minutes of steps
            stream = torch.cuda.current_stream()
            B.run(dt, sched_s, sched_m, warmup, stream.cuda_stream)
            torch.cuda.synchronize()
            ms = _timed(stream, lambda: B.run(dt, sched_s, sched_m, steps, stream.cuda_stream))
            total_ms += ms
            total_states_steps += steps * sum(specs[idx][2] for idx in grp)
            cfg = B.config()
            phase_steps += steps * cfg[2]
            # accuracy on a few small instances: the oracle with the same (s, m), same steps
            for j in small:
                idx = grp[j]
                model, n, k, terms = specs[idx]
                N2, off, re, im = ham.pauli_sum(n, terms)
                A = orc.OMatrix(N2, N2, off, re, im)
                want = orc.ham_sim(A, start[j], dt * (warmup + steps), warmup + steps, sched_m[j],
                                   substeps=1 << sched_s[j])
                got = prs[j][0].cpu().numpy() + 1j * pis[j][0].cpu().numpy()
                checks.append(float(np.linalg.norm(got - want) / np.linalg.norm(want)))
            del B, mats, prs, pis
            torch.cuda.empty_cache()
        total_ms = _max_over_ranks(total_ms, world, dev)
        total_states_steps = _sum_over_ranks(total_states_steps, world, dev)
        gaps_ms = phase_steps * gap_us / 1e3
        out["variants"][variant] = {"value": total_states_steps / (total_ms / 1e3), "unit": "states·steps/s",
                                    "steps": steps, "groups": len(groups), "ms": total_ms,
                                    "launch_shape": {"states_per_launch": cfg[0], "rows_per_thread": cfg[1],
                                                     "phases_per_step_last_group": cfg[2]},
                                    "phase_launches": phase_steps,
                                    "launch_gaps_ms_est": gaps_ms, "launch_gap_share_est": gaps_ms / total_ms,
                                    "rel_err_vs_oracle_max": max(checks) if checks else None,
                                    "checked_instances": len(checks)}
    return out


def run_batched(args):
    """--mode batched: measure_batched with the command line's settings; one JSON line."""
    import torch

    from diaq_gb300 import build

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dev = "cuda"
    if world > 1:  # replicas: every rank evolves its share of the instances, no data exchange
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
        dev = torch.device("cuda", torch.cuda.current_device())
    build.build()
    out = measure_batched(args.instances, args.n_lo, args.n_hi, args.batch_seed,
                          ["c64", "c128"] if args.variant == "both" else [args.variant], args.batch_steps,
                          args.batch_steps_c128, args.warmup, args.horner, args.planar, args.mem_gb, world, rank, dev)
    out = {"mode": "batched", **out}
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def tile_live_values(N, off, re, im):
    """Stored values of a square DiaQ matrix (packed re/im) that lie in 32-row tiles holding a
    nonzero -- what the term kernels read; they skip the all-zero tiles of every diagonal."""
    live, pos = 0, 0
    for d in off:
        d = int(d)
        lo, L = max(0, -d), N - abs(d)
        nz = (re[pos:pos + L] != 0) | (im[pos:pos + L] != 0)
        t = (lo + np.arange(L)) // 32
        t -= t[0] if L else 0
        per_tile = np.bincount(t, minlength=1)
        live += int(per_tile[np.bincount(t, weights=nz, minlength=1) > 0].sum())
        pos += L
    return live


def measure_precision(n: int = 24, states: int = 8, ref_states: int = 2, peak: float = None):
    """Config 3: the n-qubit XXZ chain (24 by default) evolved to t = 1 in 20 steps in the
    compensated-sum (mixed) and Horner float32 forms, 8 states, against a complex128 evolution of
    the first ref_states of them at a 1e-14 step tolerance (complex128 is FP64-bound on GB300: the
    reference run covers fewer states to keep its time short).  Per form: states x steps/s, the
    relative state error and fidelity against the complex128 run, the norm drift, and the
    roofline of its term kernel (bytes of the live 32-row tiles of the c64 matrix once per launch
    plus the per-state vector traffic of the Horner form, per mean launch time)."""
    import torch

    from diaq_gb300 import capi
    from diaq_gb300 import hamiltonians as ham

    L = capi.lib()
    if peak is None:
        peak = peaks()[0]
    J, h = ham.xxz_params(n, 1)
    terms = []
    for i in range(n):
        j = (i + 1) % n
        terms += [(J[i], {i: "X", j: "X"}), (J[i], {i: "Y", j: "Y"}), (0.8 * J[i], {i: "Z", j: "Z"})]
    terms += [(h[i], {i: "Z"}) for i in range(n)]
    H = capi.Matrix.from_pauli(n, *ham.pauli_masks(n, terms))
    N, _, nd, total, _ = H.info()
    live = H.live_values()
    nrm = ctypes.c_double()
    capi.check(L.diaq_norm1_est(H.h, ctypes.byref(nrm), None))
    steps, dt, S = 20, 1.0 / 20, states
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s_c, m_c, selection = chosen_schedule(capi, H, nrm.value)
    torch.cuda.synchronize()
    selection_ms = 1e3 * (time.perf_counter() - t0)
    gen = torch.Generator(device="cuda").manual_seed(0)
    z = torch.randn((S, N), dtype=torch.complex128, device="cuda", generator=gen)
    z = z / torch.linalg.vector_norm(z, dim=1, keepdim=True)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def evolve(mode, s, m, k):
        """(final states, ms for the 20 steps, launch shape, launches per step) of one plan on the
        first k states; the plan is tuned and its step graph recorded on scratch copies first,
        outside the timed region."""
        E = capi.Evolve(H, k, mode)
        zk = z[:k]
        wr, wi = zk.real.contiguous(), zk.imag.contiguous()
        E.run(wr, wi, N, dt, 1, s, m, sp)
        del wr, wi
        pr, pi = zk.real.contiguous(), zk.imag.contiguous()
        torch.cuda.synchronize()
        ms = _timed(stream, lambda: E.run(pr, pi, N, dt, steps, s, m, sp))
        E.check()
        shape = list(E.config()) + [E.pipelined()]
        lps = E.launches_per_step()
        del E
        torch.cuda.empty_cache()
        return pr + 1j * pi, ms, shape, lps

    # complex128 reference at a 1e-14 step tolerance
    s_r, m_r = capi.select_sm(nrm.value, dt, 1e-14, 1.0, 100)
    want, ms_ref, _, _ = evolve(capi.EVOLVE_C128, s_r, m_r, ref_states)
    forms = {}
    for name, mode in (("mixed", capi.EVOLVE_MIXED), ("horner", capi.EVOLVE_HORNER)):
        got, ms, shape, lps = evolve(mode, s_c, m_c, S)
        g = got[:ref_states]
        err = (torch.linalg.vector_norm(g - want, dim=1) / torch.linalg.vector_norm(want, dim=1)).cpu().numpy()
        fid = (torch.abs((want.conj() * g).sum(dim=1)) ** 2 /
               (torch.linalg.vector_norm(g, dim=1) ** 2 * torch.linalg.vector_norm(want, dim=1) ** 2)).cpu().numpy()
        drift = (torch.linalg.vector_norm(got, dim=1) - 1).abs().cpu().numpy()
        forms[name] = {"states_steps_per_s": S * steps / (ms / 1e3), "ms": ms, "launch_shape": shape,
                       "rel_err_max": float(err.max()), "fidelity_min": float(fid.min()),
                       "norm_drift_max": float(drift.max()), "launches_per_step": lps}
        if name == "horner":
            # bytes of one step: the live c64 matrix once per launch, (24 m + 16) N per state and sub-step
            step_bytes = (1 << s_c) * m_c * 8 * live + S * (1 << s_c) * (24 * m_c + 16) * N
            ach = step_bytes / (ms / steps * 1e-3) / 1e9
            forms[name]["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                                       "frac": ach / peak, "bytes_per_step": step_bytes,
                                       "bytes_per_launch": step_bytes / max(lps, 1)}
        del got
    del z, want
    torch.cuda.empty_cache()
    return {"workload": f"xxz{n}_periodic_t1_20steps", "n_qubits": n, "rows": N, "ndiag": nd, "stored_values": total,
            "live_tile_values": live, "t": 1.0, "steps": steps, "states": S, "substeps": 1 << s_c,
            "taylor_terms": m_c, "selection": selection, "selection_ms": selection_ms,
            "mixed": forms["mixed"], "horner": forms["horner"],
            "c128_reference": {"states": ref_states, "states_steps_per_s": ref_states * steps / (ms_ref / 1e3),
                               "ms": ms_ref, "substeps": 1 << s_r, "taylor_terms": m_r,
                               "errors_over": f"the first {ref_states} of the {S} states"}}


def run_precision(args):
    """--mode precision: measure_precision at --n qubits (24 by default on the command line)."""
    from diaq_gb300 import build

    build.build()
    print(json.dumps({"mode": "precision", **measure_precision(args.n, args.states, args.ref_states)}), flush=True)


def run_ours(args, rank, world):
    import torch

    from diaq_gb300 import build, capi
    from diaq_gb300 import hamiltonians as ham

    build.build()
    L = capi.lib()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    N, off, re, im = workload(args.n)
    total = int(re.size)
    H = capi.Matrix.create(N, N, off, re, im)
    norm1 = ctypes.c_double()
    capi.check(L.diaq_norm1_est(H.h, ctypes.byref(norm1), None))
    K, W, S = args.steps, args.warmup, args.states

    # ---- plain c128 form: one state, the reference's scaling rule, remainder-bound m ----
    s_p, m_p = capi.select_sm(norm1.value, DT, TOL_STEP, 1.0, 100)
    plain = capi.Evolve(H, 1, capi.EVOLVE_C128)
    p0 = ham.random_state(N, 0)
    ppr = torch.from_numpy(p0.real.copy()).to(dev)
    ppi = torch.from_numpy(p0.imag.copy()).to(dev)
    plain.run(ppr, ppi, N, DT, W, s_p, m_p, sp)
    _barrier(world)
    ms_plain = _max_over_ranks(_timed(stream, lambda: plain.run(ppr, ppi, N, DT, K, s_p, m_p, sp)), world, dev)
    lps_plain = plain.launches_per_step()

    # ---- chosen form: all S states per launch, complex64 matrix, float32 Horner evaluation,
    # FP64 state, learned (s, m) ----
    CHOSEN_MODE = capi.EVOLVE_HORNER
    # the one-time (s, m) selection (Krylov chain of the probe state, features, network, check):
    # outside the timed region, its own time reported; the libraries it uses (cuBLAS for the chain
    # norms) are initialised first, so that their one-time start-up is not counted
    _ = torch.dot(ppr[:8], ppr[:8]).item()
    torch.cuda.synchronize()
    t_sel = time.perf_counter()
    s_c, m_c, selection = chosen_schedule(capi, H, norm1.value)
    torch.cuda.synchronize()
    selection_ms = 1e3 * (time.perf_counter() - t_sel)
    chosen = capi.Evolve(H, S, CHOSEN_MODE)
    P0 = ham.random_state(N, 0, k=S) if S > 1 else p0[None, :]
    cpr = torch.from_numpy(np.ascontiguousarray(P0.real)).to(dev)
    cpi = torch.from_numpy(np.ascontiguousarray(P0.imag)).to(dev)
    chosen.run(cpr, cpi, N, DT, W, s_c, m_c, sp)
    _barrier(world)
    with ClockSampler(dev.index) as clk:
        ms = _max_over_ranks(_timed(stream, lambda: chosen.run(cpr, cpi, N, DT, K, s_c, m_c, sp)), world, dev)
    lps = chosen.launches_per_step()
    launches = K * lps + 2

    # ---- the chosen form on one state (config 2 evolves a single psi) ----
    one = capi.Evolve(H, 1, CHOSEN_MODE)
    o_r = torch.from_numpy(np.ascontiguousarray(P0[0].real)).to(dev)
    o_i = torch.from_numpy(np.ascontiguousarray(P0[0].imag)).to(dev)
    one.run(o_r, o_i, N, DT, W, s_c, m_c, sp)
    torch.cuda.synchronize()
    ms_one = _timed(stream, lambda: one.run(o_r, o_i, N, DT, K, s_c, m_c, sp))
    one_shape = list(one.config()) + [one.pipelined()]
    del one, o_r, o_i

    # ---- accuracy of the chosen form: the same W + K steps in c128 at a tight tolerance ----
    s_r, m_r = capi.select_sm(norm1.value, DT, 1e-14, 1.0, 100)
    refp = capi.Evolve(H, S, capi.EVOLVE_C128)
    rpr = torch.from_numpy(np.ascontiguousarray(P0.real)).to(dev)
    rpi = torch.from_numpy(np.ascontiguousarray(P0.imag)).to(dev)
    refp.run(rpr, rpi, N, DT, W + K, s_r, m_r, sp)
    torch.cuda.synchronize()
    got = (cpr.double() + 1j * cpi.double())
    want = (rpr + 1j * rpi)
    errs = (torch.linalg.vector_norm(got - want, dim=1) / torch.linalg.vector_norm(want, dim=1)).cpu().numpy()
    fid = (torch.abs((want.conj() * got).sum(dim=1)) ** 2 /
           (torch.linalg.vector_norm(got, dim=1) ** 2 * torch.linalg.vector_norm(want, dim=1) ** 2)).cpu().numpy()
    del refp, rpr, rpi

    # ---- end to end through the C ABI with host buffers: every step copies the S states from
    # pinned host memory to the device, advances them one time step and copies them back ----
    host_mem = "pinned"
    try:
        pin_r = torch.from_numpy(np.ascontiguousarray(P0.real).ravel().copy()).pin_memory()
        pin_i = torch.from_numpy(np.ascontiguousarray(P0.imag).ravel().copy()).pin_memory()
        hr, hi = pin_r.numpy(), pin_i.numpy()
    except RuntimeError:
        host_mem = "pageable"
        hr = np.ascontiguousarray(P0.real).ravel().copy()
        hi = np.ascontiguousarray(P0.imag).ravel().copy()
    e2e_plan = capi.Evolve(H, S, CHOSEN_MODE)
    for _ in range(W):   # the plan's device copy of the states and its graph, outside the timed region
        e2e_plan.run_host(hr, hi, DT, 1, s_c, m_c)
    _barrier(world)
    t0 = time.perf_counter()
    for _ in range(K):
        e2e_plan.run_host(hr, hi, DT, 1, s_c, m_c)
    e2e_s = _max_over_ranks(time.perf_counter() - t0, world, dev)
    # the reference API's own pattern (hamiltonian_simulation_cuda): one call, S states up, K steps,
    # S states down
    _barrier(world)
    t0 = time.perf_counter()
    e2e_plan.run_host(hr, hi, DT, K, s_c, m_c)
    e2e_one_s = _max_over_ranks(time.perf_counter() - t0, world, dev)
    del e2e_plan

    # ---- SpMV on its own, c128 (FP64-issue bound on GB300) ----
    xr, xi = ppr.clone(), ppi.clone()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    for _ in range(3):
        capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))

    def spmv_loop():
        for i in range(args.spmv_reps):
            a, b, c, d = (xr, xi, yr, yi) if i % 2 == 0 else (yr, yi, xr, xi)
            capi.check(L.diaq_spmv_z(H.h, a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), sp))

    spmv_us = 1e3 * _timed(stream, spmv_loop) / args.spmv_reps

    # ---- the same SpMV on a c128f2 copy (float-pair values, FP32 pipes) ----
    Hf = H.convert(capi.C128F2)

    xr.copy_(ppr)
    xi.copy_(ppi)

    def spmv_f2_loop():   # y = A x from the same x each time: float pairs hold magnitudes up to ~1e38 only
        for _ in range(args.spmv_reps):
            capi.check(L.diaq_spmv_z(Hf.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))

    spmv_f2_loop()
    spmv_f2_us = 1e3 * _timed(stream, spmv_f2_loop) / args.spmv_reps
    y64r, y64i = torch.empty_like(xr), torch.empty_like(xi)
    capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), y64r.data_ptr(), y64i.data_ptr(), sp))
    capi.check(L.diaq_spmv_z(Hf.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))
    torch.cuda.synchronize()
    f2_err = float(torch.maximum((yr - y64r).abs().max(), (yi - y64i).abs().max())
                   / torch.maximum(y64r.abs().max(), y64i.abs().max()))
    del Hf, y64r, y64i

    peak, peak_kind = peaks()
    # algorithmic bytes of one chosen time step.  Every Taylor term is one launch over all S
    # states and reads the c64 matrix once (8 B per stored value) -- the values of the 32-row
    # tiles that hold a nonzero, the only ones the term kernels visit.  Per state, Horner form: the
    # first term reads fp32(psi) (8N; its window and its epilogue read the same vector) and writes
    # w (8N); a middle term reads w and fp32(psi) and writes the next w (24N); the last reads w,
    # read-modify-writes psi in float64 and writes fp32(psi) (8N + 32N + 8N) -- (24 m + 16) N per
    # sub-step for m >= 2.
    per_state_step = (1 << s_c) * (24 * m_c + 16) * N
    live = tile_live_values(N, off, re, im)
    step_bytes = (1 << s_c) * m_c * 8 * live + S * per_state_step
    achieved = step_bytes / (ms / K * 1e-3) / 1e9
    k_launch, v_launch = chosen.config()
    variant = chosen.pipelined()
    # EpiHorner*<0/1>: the middle terms' and the last term's instantiations of one kernel
    il_names = {6: "dia_spmv_il_kernel<EpiHornerT<0/1>,0,4>", 7: "dia_spmv_il_kernel<EpiHornerT<0/1>,4,4>",
                8: "dia_spmv_il_kernel<EpiHornerT<0/1>,8,4>", 9: "dia_spmv_il_kernel<EpiHornerT<0/1>,0,8>",
                10: "dia_spmv_tma_kernel<EpiHornerT<0/1>,8,true,4>",
                11: "dia_spmv_tma_kernel<EpiHornerT<0/1>,8,false,8>",
                12: "dia_spmv_il32_kernel<EpiHornerT<0/1>,8,5>"}
    kernel = (il_names.get(variant) if variant >= 6 else
              f"dia_spmv_kernel<float,{k_launch},{v_launch},EpiHornerP<0/1>>" if variant == 0 else
              f"variant {variant}, {k_launch} states x {v_launch} rows per thread")
    # DRAM bytes of one launch from the ncu capture of this workload, form and shape (profiles/);
    # null for shapes not captured
    traffic = TRAFFIC_PER_LAUNCH.get((args.n, S, "horner", k_launch, v_launch, variant))
    value = world * S * K / (ms / 1e3)
    plain_value = world * K / (ms_plain / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "states·steps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 terms + f64 state", "data": "synthetic (seeded XXZ couplings and states, built in-process)",
        "config": {"workload": f"xxz{args.n}_periodic_evolve", "form": "chosen", "evaluation": "horner", "n_qubits": args.n, "rows": N,
                   "ndiag": len(off), "stored_values": total, "live_tile_values": live, "dt": DT,
                   "states_per_gpu": S,
                   "substeps": 1 << s_c, "taylor_terms": m_c, "selection": selection,
                   "launch_shape": {"states_per_block": chosen.config()[0], "rows_per_thread": chosen.config()[1],
                                    "kernel_variant": chosen.pipelined()},
                   "tol_per_step": TOL_STEP, "norm1": norm1.value, "selection_ms": selection_ms,
                   "l2": "inputs larger than L2 (c64 matrix 327 MB, states 128 MB > 129 MB)",
                   "parallelism": f"replicas{world}"},
        "accuracy": {"rel_err_max": float(errs.max()), "fidelity_min": float(fid.min()),
                     "vs": f"c128 evolution at tol 1e-14 ({1 << s_r}x{m_r} terms/step)", "steps": W + K},
        "chosen_one_state": {"value": world * K / (ms_one / 1e3), "ms_per_step": ms_one / K,
                             "launch_shape": one_shape,
                             "speedup_over_plain": (world * K / (ms_one / 1e3)) / plain_value},
        "plain": {"value": plain_value, "ms_per_step": ms_plain / K, "substeps": 1 << s_p, "taylor_terms": m_p,
                  "launches_per_step": lps_plain, "speedup_chosen_over_plain": value / plain_value},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": kernel, "bytes_per_launch": step_bytes / lps,
                     "bytes_per_step": step_bytes, "launches_per_step": lps, "peak_kind": peak_kind,
                     "note": "achieved = algorithmic bytes per launch / mean launch time (CUDA events over the "
                             "timed steps; every launch of a step is this kernel: its middle-term and its "
                             "last-term instantiation)"},
        "spmv_c128": {"us": spmv_us, "gbs": (16 * live + 32 * N) / spmv_us / 1e3,
                      "frac": (16 * live + 32 * N) / spmv_us / 1e3 / peak,
                      "dfma_per_launch": 4 * live, "reps": args.spmv_reps,
                      "effective_gbs": (16 * total + 32 * N) / spmv_us / 1e3,
                      "note": "gbs, frac: bytes of the live 32-row tiles (all-zero tiles skipped); effective_gbs: "
                              "all stored values (w Σlen + 2 w N) per time, the dense-diagonal figure"},
        "spmv_c128f2": {"us": spmv_f2_us, "gbs": (16 * live + 32 * N) / spmv_f2_us / 1e3,
                        "frac": (16 * live + 32 * N) / spmv_f2_us / 1e3 / peak,
                        "effective_gbs": (16 * total + 32 * N) / spmv_f2_us / 1e3,
                        "maxrel_vs_c128": f2_err, "reps": args.spmv_reps,
                        "note": "same matrix as float pairs (DIAQ_C128F2), float64 vectors; includes the split of x"},
        "e2e": {"value": world * S * K / e2e_s, "unit": "states·steps/s", "h2d_bytes_per_step": 16 * N * S,
                "d2h_bytes_per_step": 16 * N * S, "host_memory": host_mem,
                "note": "K calls of diaq_evolve_run_host, each: S float64 states host to device, one time step, "
                        "S states device to host (the library runs the two halves of the states one after the "
                        "other, each half's copies overlapping the other's run)"},
        "e2e_one_call": {"value": world * S * K / e2e_one_s, "unit": "states·steps/s",
                         "h2d_bytes_per_step": 16 * N * S / K, "d2h_bytes_per_step": 16 * N * S / K,
                         "note": "one diaq_evolve_run_host call: S states up, K steps, S states down"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        # the oracle evolves state 0 for a bounded number of steps: the timed CPU baseline, and the
        # reference the chosen form's state 0 is measured against after the same steps from the same
        # states (FP64, the plain rule's (s, m)); the chosen plan reruns them on fresh copies
        base, want0, done = cpu_baseline_sample(N, off, re, im, s_p, m_p)
        line["cpu_baseline"] = base
        ar = torch.from_numpy(np.ascontiguousarray(P0.real)).to(dev)
        ai = torch.from_numpy(np.ascontiguousarray(P0.imag)).to(dev)
        chosen.run(ar, ai, N, DT, done, s_c, m_c, sp)
        torch.cuda.synchronize()
        got0 = ar[0].double().cpu().numpy() + 1j * ai[0].double().cpu().numpy()
        del ar, ai
        line["accuracy"]["rel_err_vs_oracle_state0"] = float(np.linalg.norm(got0 - want0) / np.linalg.norm(want0))
        line["accuracy"]["oracle"] = (f"C restatement of the reference's CPU time evolution, FP64, "
                                      f"{1 << s_p}x{m_p} terms/step (per-step truncation bound {TOL_STEP:g}), "
                                      f"{done} steps from the same state")
    if rank == 0 and world == 1 and not args.no_extras:
        # configs 3 and 4 and config 2's SpGEMM, on the same GPU after the headline measurement
        del chosen, plain, H
        torch.cuda.empty_cache()
        line["precision_n24"] = measure_precision(24, 8, args.ref_states, peak)
        torch.cuda.empty_cache()
        line["batched_cfg4"] = measure_batched(variants=("c64", "c128"), c64_steps=50, c128_steps=1, horner=True)
        torch.cuda.empty_cache()
        line["spgemm_xxz20"] = measure_spgemm(args.n, peak)
        line["gpu_launches_extras"] = "not counted in gpu_launches (the headline's timed region only)"
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=20)
    ap.add_argument("--spmv-reps", type=int, default=1000)
    ap.add_argument("--states", type=int, default=8, help="states evolved together by the chosen form")
    ap.add_argument("--shape", default="", help="chosen mode: force the launch shape 'states,rows,pipelined'")
    ap.add_argument("--horner", action="store_true",
                    help="chosen and batched modes: Horner-form evaluation (DIAQ_EVOLVE_HORNER, diaq_batch_set_horner)")
    ap.add_argument("--instances", type=int, default=512, help="batched mode: Hamiltonians")
    ap.add_argument("--n-lo", type=int, default=10)
    ap.add_argument("--n-hi", type=int, default=22)
    ap.add_argument("--batch-seed", type=int, default=4)
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--batch-steps-c128", type=int, default=3)
    ap.add_argument("--variant", choices=["c64", "c128", "both"], default="both")
    ap.add_argument("--mem-gb", type=float, default=200.0, help="batched mode: device memory per group")
    ap.add_argument("--planar", action="store_true",
                    help="batched mode: keep every instance's work vectors planar (no interleaved tiles)")
    ap.add_argument("--mode", choices=["evolve", "spmv", "chosen", "batched", "precision", "ops"], default="evolve",
                    help="evolve: the full measurement; spmv: the SpMV kernel alone; chosen: only the chosen "
                         "form's evolution (for profiling)")
    ap.add_argument("--ref-steps", type=int, default=10, help="time steps the CPU reference arm times at most")
    ap.add_argument("--ref-states", type=int, default=2,
                    help="precision mode: states of the complex128 reference run (the first ones)")
    ap.add_argument("--no-extras", action="store_true",
                    help="default mode: leave out the precision form, the batch and the SpGEMM keys")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--ops", choices=["all", "xxz"], default="all", help="ops mode: all operations, or the XXZ H H only")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        ap.error("--warmup must be at least 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.mode == "spmv":
        run_spmv_only(args)
        return
    if args.mode == "ops":
        run_ops(args)
        return
    if args.mode == "chosen":
        run_chosen_only(args)
        return
    if args.mode == "batched":
        run_batched(args)
        return
    if args.mode == "precision":
        run_precision(args)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    try:
        run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
