"""Batched solves (igaos_pdhg_solve_batch): thousands of uneven LPs in one
persistent launch, each with its own restarts and termination.

* Every golden LP solved inside one batch reaches the reference simplex
  optimum (tests/golden, made by the reference's own simplex) within 1e-5 at
  1e-6 relative KKT (FP32 iterates).
* C3-shaped instances (m log-uniform, n = 2.5 m, Bernoulli pattern, box
  [0,5]) agree with the single-LP engine (FP64, 1e-8).
* A spread of the 4,096-LP set itself (16 ranks of m, the 8 largest
  instances up to m = 2,000, and the slowest instance) reaches scipy-HiGHS
  optima (tests/golden/make_c3_golden.py) within 1e-5 at 1e-6.
* Per-instance results do not depend on the batch's composition or order
  (CTAs never share an instance) and repeat bit for bit.
"""
import json
import os

import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))


def golden_lps():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import make_lp
    names = sorted(k for k in GOLD if not k.startswith("zipf"))
    return names, [make_lp(GOLD[k]["generator"], GOLD[k]["kwargs"]) for k in names]


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def c3_like(count, seed, m_hi=400):
    rng = np.random.default_rng(seed)
    ms = np.rint(np.exp(rng.uniform(np.log(20), np.log(m_hi), count))).astype(int)
    return [G.bernoulli_lp(rng, int(m), int(round(2.5 * m)), 0.01 if m >= 100 else 0.05, 5.0)
            for m in ms]


def test_batch_reaches_simplex_optimum(native):
    from igaos_gb300 import capi
    names, lps = golden_lps()
    out = capi.solve_batch(lps, tolerance=1e-6, max_iterations=400000)
    for name, lp, r in zip(names, lps, out):
        assert r["status_name"] == "near-optimal", (name, r)
        assert rel(r["objective"], GOLD[name]["simplex_objective"]) <= 1e-5, (name, r["objective"])
        assert max(r["pinf"], r["dinf"], r["rel_gap"], r["prow"]) <= 1e-6


def test_batch_matches_single_lp_engine(native):
    from igaos_gb300 import capi
    lps = c3_like(48, 3)
    out = capi.solve_batch(lps, tolerance=1e-6, max_iterations=400000)
    for lp, r in zip(lps, out):
        assert r["status_name"] == "near-optimal"
        single = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0)
        assert single["status_name"] == "near-optimal"
        assert rel(r["objective"], single["objective"]) <= 2e-5


def test_handoff_is_bounded_and_finishes_in_fp64(native, monkeypatch):
    """With the hand-off at 1,000 iterations and at most 3 instances, exactly
    3 of the instances still running at 1,000 iterations stop there and are
    finished in FP64 (each to the tolerance, with more than 1,000 iterations
    counted); the rest run to the tolerance in the launch, as without a
    hand-off, bit for bit."""
    from igaos_gb300 import capi
    lps = c3_like(24, 11)
    monkeypatch.setenv("IGAOS_PDHG_BATCH_HANDOFF", "0")
    base = capi.solve_batch(lps, tolerance=1e-6, max_iterations=400000)
    assert all(r["finished_fp64"] == 0 for r in base)
    slow = [i for i, r in enumerate(base) if r["iterations"] > 1000]
    assert len(slow) > 3
    monkeypatch.setenv("IGAOS_PDHG_BATCH_HANDOFF", "1000")
    monkeypatch.setenv("IGAOS_PDHG_BATCH_HANDOFF_MAX", "3")
    out = capi.solve_batch(lps, tolerance=1e-6, max_iterations=400000)
    handed = [i for i, r in enumerate(out) if r["finished_fp64"]]
    assert len(handed) == 3 and set(handed) <= set(slow), handed
    for i, (a, r) in enumerate(zip(base, out)):
        assert r["status_name"] == "near-optimal", (i, r["status_name"])
        if i in handed:
            assert r["iterations"] > 1000
            assert rel(r["objective"], a["objective"]) <= 2e-5
        else:
            assert r["iterations"] == a["iterations"] and r["objective"] == a["objective"]


def test_batch_full_size_range_reaches_highs_optimum(native):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import same_checksum
    from igaos_gb300 import capi
    gold = json.load(open(os.path.join(HERE, "golden", "c3_objectives.json")))
    lps = G.config3(**gold["kwargs"])
    idx = sorted(gold["instances"], key=int)
    batch = [lps[int(i)] for i in idx]
    assert max(lp.m for lp in batch) >= 1990
    for i, lp in zip(idx, batch):
        assert same_checksum(lp, gold["instances"][i]["checksum"]), "generator drift"
    out = capi.solve_batch(batch, tolerance=1e-6)
    for i, r in zip(idx, out):
        want = gold["instances"][i]["highs_ds_objective"]
        assert r["status_name"] == "near-optimal", (i, r["status_name"])
        assert max(r["pinf"], r["dinf"], r["rel_gap"], r["prow"]) <= 1e-6, i
        assert rel(r["objective"], want) <= 1e-5, (i, r["objective"], want)


def test_batch_order_independent_and_deterministic(native):
    from igaos_gb300 import capi
    lps = c3_like(40, 9)
    a = capi.solve_batch(lps, tolerance=1e-6, max_iterations=400000)
    b = capi.solve_batch(lps, tolerance=1e-6, max_iterations=400000)
    perm = np.random.default_rng(1).permutation(len(lps))
    c = capi.solve_batch([lps[i] for i in perm], tolerance=1e-6, max_iterations=400000)
    for i in range(len(lps)):
        assert a[i]["objective"] == b[i]["objective"] and a[i]["iterations"] == b[i]["iterations"]
        assert np.array_equal(a[i]["x"], b[i]["x"])
    for k, i in enumerate(perm):
        assert c[k]["objective"] == a[i]["objective"] and c[k]["iterations"] == a[i]["iterations"]


def test_batch_iteration_cap_and_validation(native):
    from igaos_gb300 import capi
    lps = c3_like(4, 5)
    out = capi.solve_batch(lps, tolerance=1e-12, max_iterations=100)
    # left at the cap by the launch, then by the FP64 finish under the same cap
    assert all(r["status_name"] == "iteration-limit" and r["finished_fp64"] == 1 and
               r["iterations"] == 200 for r in out)
    bad = G.random_lp(10, 20, 10, 0)
    bad.ai = bad.ai.copy()
    bad.ai[0] = 99
    with pytest.raises(capi.EngineError, match="column index out of range"):
        capi.solve_batch([bad])


def test_instance_left_at_the_cap_is_finished_in_fp64(native):
    """Instance 1018 of the 4,096-LP set (m 1,747, n 4,368, 1 % density)
    needs ~256k FP32 + refinement iterations but far fewer in FP64. Under a
    cap of 120,000 the persistent launch hands it off at 100,000 iterations;
    the single-LP engine then solves it in FP64 within the same cap, and the
    batch result reports that finish and the FP64 engine's optimum. A batch
    whose instances all converge early in the launch has no such finish."""
    from igaos_gb300 import capi
    lp = G.config3(seed=0, count=4096)[1018]
    assert (lp.m, lp.n) == (1747, 4368)
    want = capi.solve_lp(lp, tolerance=1e-6, time_limit=1e9, max_iterations=120000,
                         precision="fp64")
    assert want["status_name"] == "near-optimal", want["message"]
    (got,) = capi.solve_batch([lp], tolerance=1e-6, max_iterations=120000)
    assert got["finished_fp64"] == 1 and got["status_name"] == "near-optimal", got
    assert got["iterations"] > 120000
    assert rel(got["objective"], want["objective"]) <= 1e-9
    names, lps = golden_lps()
    out = capi.solve_batch(lps[:4], tolerance=1e-6, max_iterations=200000)
    assert all(r["finished_fp64"] == 0 for r in out)
