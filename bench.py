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
        self.idx = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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
        for ln in self.lines:
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
    if rank != 0:
        return
    from oracle import oracle as orc
    from diaq_gb300 import hamiltonians as ham

    N, off, re, im = workload(args.n)
    H = orc.OMatrix(N, N, off, re, im)
    norm1 = orc.norm1_est(H)
    s, m = _select_sm_py(norm1)
    psi = ham.random_state(N, 0)
    steps = max(1, min(args.steps, args.ref_steps))
    warm = min(args.warmup, 1)
    for _ in range(warm):
        psi = orc.ham_sim(H, psi, DT, 1, m, substeps=1 << s)
    t0 = time.perf_counter()
    for _ in range(steps):
        psi = orc.ham_sim(H, psi, DT, 1, m, substeps=1 << s)
    wall = time.perf_counter() - t0
    value = steps / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "states·steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * wall / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"xxz{args.n}_periodic_evolve", "n_qubits": args.n, "rows": N, "ndiag": len(off),
                   "dt": DT, "substeps": 1 << s, "taylor_terms": m, "states": 1},
        "cpu_baseline": {"value": value, "unit": "states·steps/s", "cores": orc.threads(), "kind": "port",
                         "sample": f"{steps} time step(s) of one state, {1 << s}x{m} SpMVs each, C/OpenMP restatement"},
        "e2e": {"value": value, "unit": "states·steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference CPU code cannot be built on this host (its sources are not shipped); the oracle "
                "port of the same algorithm is timed",
    }
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
def cpu_baseline_sample(N, off, re, im, s, m):
    from oracle import oracle as orc
    from diaq_gb300 import hamiltonians as ham

    H = orc.OMatrix(N, N, off, re, im)
    psi = ham.random_state(N, 0)
    # one time step = 2^s * m SpMVs; time whole steps until ~10 s have passed
    t0 = time.perf_counter()
    steps = 0
    while True:
        psi = orc.ham_sim(H, psi, DT, 1, m, substeps=1 << s)
        steps += 1
        if time.perf_counter() - t0 > 10.0 or steps >= 20:
            break
    wall = time.perf_counter() - t0
    return {"value": steps / wall, "unit": "states·steps/s", "cores": orc.threads(), "kind": "port",
            "sample": f"{steps} time step(s) of one state ({1 << s}x{m} SpMVs each) on the host, C/OpenMP"}


def run_ours(args, rank, world):
    import torch

    from diaq_gb300 import build, capi

    build.build()
    L = capi.lib()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    N, off, re, im = workload(args.n)
    total = int(re.size)
    H = capi.Matrix.create(N, N, off, re, im)
    norm1 = ctypes.c_double()
    capi.check(L.diaq_norm1_est(H.h, ctypes.byref(norm1), None))
    s, m = plain_schedule(capi, norm1.value)
    sub = 1 << s
    from diaq_gb300 import hamiltonians as ham

    psi = ham.random_state(N, 0)
    pr = torch.from_numpy(psi.real.copy()).to(dev)
    pi = torch.from_numpy(psi.imag.copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def evolve(k_steps):
        capi.check(L.diaq_ham_sim(H.h, pr.data_ptr(), pi.data_ptr(), DT * k_steps, k_steps * sub, m,
                                  pr.data_ptr(), pi.data_ptr(), sp))

    # warm-up
    evolve(args.warmup)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        e0.record(stream)
        evolve(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        torch.distributed.barrier()
    launches = args.steps * sub * m
    norm_drift = abs(float(torch.sqrt((pr * pr + pi * pi).sum()).item()) - 1.0)

    # plain SpMV (1000 repeated products of config 2, the kernel's own roofline)
    xr, xi = pr.clone(), pi.clone()
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    reps = args.spmv_reps
    for _ in range(5):
        capi.check(L.diaq_spmv_z(H.h, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), sp))
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for i in range(reps):
        a, b = (xr, xi) if i % 2 == 0 else (yr, yi)
        c, d = (yr, yi) if i % 2 == 0 else (xr, xi)
        capi.check(L.diaq_spmv_z(H.h, a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), sp))
    f1.record(stream)
    torch.cuda.synchronize()
    spmv_us = 1e3 * f0.elapsed_time(f1) / reps

    # end to end through the C ABI with host buffers: psi0 up, K steps, psi down
    hpr, hpi = np.ascontiguousarray(psi.real), np.ascontiguousarray(psi.imag)
    opr, opi = np.empty(N), np.empty(N)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    capi.check(L.diaq_ham_sim_host(H.h, hpr.ctypes.data, hpi.ctypes.data, DT * args.steps, args.steps * sub, m,
                                   opr.ctypes.data, opi.ctypes.data))
    e2e_s = time.perf_counter() - t0

    peak, peak_kind = peaks()
    w = 16
    bytes_term = w * total + 4 * w * N       # A once; term in, term out, sum read+write
    bytes_spmv = w * total + 2 * w * N       # A once; x in, y out
    us_term = 1e3 * ms / launches
    achieved = bytes_term / (us_term * 1e-6) / 1e9
    spmv_gbs = bytes_spmv / (spmv_us * 1e-6) / 1e9
    value = world * args.steps / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "states·steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded XXZ couplings and states, built in-process)",
        "config": {"workload": f"xxz{args.n}_periodic_evolve", "form": "plain", "n_qubits": args.n, "rows": N,
                   "ndiag": len(off), "stored_values": total, "dt": DT, "substeps": sub, "taylor_terms": m,
                   "states_per_gpu": 1, "precision": "c128", "norm1": norm1.value,
                   "l2": "inputs larger than L2 (matrix 654 MB c128 > 129 MB)", "parallelism": f"replicas{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "dia_spmv_kernel<double,1,EpiTaylorRhs<double>>",
                     "bytes_per_launch": bytes_term, "us_per_launch": us_term, "peak_kind": peak_kind},
        "spmv": {"us": spmv_us, "gbs": spmv_gbs, "frac": spmv_gbs / peak, "bytes": bytes_spmv, "reps": reps},
        "e2e": {"value": world * args.steps / e2e_s, "unit": "states·steps/s", "h2d_bytes_per_step": 16 * N / args.steps,
                "d2h_bytes_per_step": 16 * N / args.steps, "note": "one diaq_ham_sim_host call: psi0 up, all steps, psi down"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "norm_drift": norm_drift,
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample(N, off, re, im, s, m)
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
    ap.add_argument("--ref-steps", type=int, default=10, help="time steps the CPU reference arm times at most")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        ap.error("--warmup must be at least 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
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
