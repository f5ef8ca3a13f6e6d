"""Host-side scheduling rules, no GPU needed: the (s, m) choice of the C ABI (diaq_select_sm,
diaq_select_sm_min_cost) against independent restatements, and the same rule in bench.py's
reference arm, which runs on hosts where only the oracle is built."""
import math

import pytest


@pytest.fixture(scope="module")
def capi():
    from diaq_gb300 import build

    build.build()
    from diaq_gb300 import capi as c

    return c


def _scaling_exponent(norm1, t, cutoff=1.0):
    """s = ceil(log2((|t| ||A||_1 + 1e-12) / cutoff)) when positive (src/spME.cpp:230-295)."""
    scaled = abs(t) * norm1 + 1e-12
    return math.ceil(math.log2(scaled / cutoff)) if scaled > cutoff else 0


def _remainder(theta, k):
    """theta^(k+1) / (k+1)! e^theta: the Taylor remainder bound of degree k."""
    return math.exp((k + 1) * math.log(theta) - math.lgamma(k + 2) + theta) if theta > 0 else 0.0


GRID = [(n1, t, tol) for n1 in (0.0, 0.3, 1.0, 7.5, 54.93, 400.0) for t in (1e-3, 0.05, 1.0, 10.0)
        for tol in (1e-6, 1e-8, 1e-10, 1e-14)]


@pytest.mark.parametrize("norm1,t,tol", GRID)
def test_select_sm_follows_the_scaling_rule_and_remainder_bound(capi, norm1, t, tol):
    s, m = capi.select_sm(norm1, t, tol, 1.0, 100)
    assert s == _scaling_exponent(norm1, t)
    theta, budget = math.ldexp(t * norm1, -s), math.ldexp(tol, -s)
    assert 1 <= m <= 100
    if m < 100:
        # the smallest degree whose remainder bound meets the per-sub-step budget (a relative
        # margin for the bound built up term by term against lgamma here)
        assert _remainder(theta, m) <= budget * (1 + 1e-9)
        if m > 1:
            assert _remainder(theta, m - 1) > budget * (1 - 1e-9)


@pytest.mark.parametrize("norm1,t,tol", GRID)
def test_reference_arm_rule_equals_the_c_abi(capi, norm1, t, tol, monkeypatch):
    """bench.py's Python copy of the rule (the reference arm's schedule) picks the C ABI's (s, m)
    at the bench's time step and per-step tolerance."""
    import bench

    monkeypatch.setattr(bench, "DT", t)
    monkeypatch.setattr(bench, "TOL_STEP", tol)
    assert bench._select_sm_py(norm1) == capi.select_sm(norm1, t, tol, 1.0, 100)


@pytest.mark.parametrize("norm1,t,tol", [(54.93, 0.05, 1e-8), (7.5, 1.0, 1e-10), (400.0, 0.05, 1e-6),
                                         (0.3, 10.0, 1e-14)])
def test_min_cost_is_the_cheapest_admissible_pair(capi, norm1, t, tol):
    """diaq_select_sm_min_cost: 2^s m is minimal over every (s, m) whose remainder bound meets
    tol 2^-s, by brute force."""
    max_s, max_m = 12, 60
    s, m = capi.select_sm_min_cost(norm1, t, tol, max_s, max_m)
    best = min(2 ** s2 * m2 for s2 in range(max_s + 1) for m2 in range(1, max_m + 1)
               if _remainder(math.ldexp(t * norm1, -s2), m2) <= math.ldexp(tol, -s2) * (1 + 1e-9))
    assert 2 ** s * m == best
    assert _remainder(math.ldexp(t * norm1, -s), m) <= math.ldexp(tol, -s) * (1 + 1e-9)


def test_selection_rejects_bad_arguments(capi):
    with pytest.raises(capi.DiaqError):
        capi.select_sm(-1.0, 0.05, 1e-8)
    with pytest.raises(capi.DiaqError):
        capi.select_sm(1.0, 0.05, 0.0)
    with pytest.raises(capi.DiaqError):
        capi.select_sm(1.0, 0.05, 1e-8, 0.0)
    with pytest.raises(capi.DiaqError):
        capi.select_sm_min_cost(1.0, 0.05, 1e-8, 31, 60)
    with pytest.raises(capi.DiaqError):   # no (s, m) within 2^0 x 1 meets 1e-300
        capi.select_sm_min_cost(100.0, 1.0, 1e-300, 0, 1)
