"""bench.py's reference arm runs on the host cores alone: one JSON line on rank 0 with the keys
the bench line carries, nothing on the other ranks.  No GPU needed."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _run(extra_env=None):
    env = dict(os.environ, **(extra_env or {}))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                           "--warmup", "1", "--n", "12"], capture_output=True, text=True, timeout=600, env=env,
                          cwd=ROOT)


def test_reference_arm_prints_one_line():
    p = _run()
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "states·steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"] == "xxz12_periodic_evolve" and d["config"]["rows"] == 4096
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    p = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_reference_and_port_time_the_same_step():
    """The arm's two kinds compute the same time step: the reference's rule over 2^s steps of
    dt / 2^s (oracle/_ref, where the reference sources were built) and the oracle's one step of
    dt in 2^s sub-steps."""
    import numpy as np
    import pytest

    from conftest import maxrel
    from diaq_gb300 import hamiltonians as ham
    from oracle import oracle as orc
    from oracle import reference as ref

    if not ref.available():
        pytest.skip("reference CPU library not built here")
    N, off, re, im = ham.xxz(10)
    H = orc.OMatrix(N, N, off, re, im)
    p = ham.random_state(N, 0)
    for s, m in ((0, 12), (2, 10)):
        a = ref.ham_sim(H, p, 0.05, 1 << s, m)
        b = orc.ham_sim(H, p, 0.05, 1, m, substeps=1 << s)
        assert maxrel(a, b) < 1e-13, (s, m)
        assert np.linalg.norm(a) > 0.99
