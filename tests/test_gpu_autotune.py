"""Schedule autotuner (igaos_pdhg_options.schedule = autotune): at the first
solve of a precision on a handle, the A and A^T attempt kernels are timed on
warp schedules of 2, 4, 8, 16 and 32 entries per lane and the fastest is kept.

* The choice is one of the candidates and is reported in the result
  (entries_a, entries_at); the fixed schedule reports 8 and 8.
* Solves on the chosen schedules reach the reference simplex optimum to 1e-6
  at 1e-8 relative KKT, in FP64 and FP32 + refinement (a schedule changes
  only the order of each row's sum).
* A handle keeps its choice: a second autotuned solve repeats the first bit
  for bit; a fixed-schedule solve on a tuned handle repeats a fresh handle's
  fixed solve bit for bit (captured graphs are kept per schedule).
* An unknown schedule value is refused.
"""
import json
import os
import sys

import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))
sys.path.insert(0, os.path.join(HERE, "golden"))


def make(name):
    from make_golden import make_lp
    e = GOLD[name]
    return make_lp(e["generator"], e["kwargs"]), e["simplex_objective"]


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
@pytest.mark.parametrize("name", ["rand200x500-s0", "bern300-s3", "grid6x6-k2"])
def test_autotuned_solve_matches_simplex(native, name, precision):
    from igaos_gb300 import capi
    lp, ref = make(name)
    with capi.Problem(lp) as P:
        a = P.solve(tolerance=1e-8, time_limit=60.0, precision=precision, schedule="autotune")
        b = P.solve(tolerance=1e-8, time_limit=60.0, precision=precision, schedule="autotune")
        f = P.solve(tolerance=1e-8, time_limit=60.0, precision=precision)
    assert a["status_name"] == "near-optimal", a["message"]
    assert abs(a["objective"] - ref) / max(1.0, abs(ref)) <= 1e-6, (a["objective"], ref)
    assert a["entries_a"] in (2, 4, 8, 16, 32) and a["entries_at"] in (2, 4, 8, 16, 32)
    assert (b["entries_a"], b["entries_at"]) == (a["entries_a"], a["entries_at"])
    assert b["objective"] == a["objective"] and b["iterations"] == a["iterations"]
    assert np.array_equal(a["x"], b["x"])
    assert (f["entries_a"], f["entries_at"]) == (8, 8)
    with capi.Problem(lp) as Q:
        g = Q.solve(tolerance=1e-8, time_limit=60.0, precision=precision)
    assert g["objective"] == f["objective"] and g["iterations"] == f["iterations"]
    assert np.array_equal(g["x"], f["x"])


def test_autotune_on_a_large_shape(native):
    """The Zipf / log-uniform shape (3,000 x 8,000): the grid-wide kernels
    run, all three candidates are timed, and a fixed budget of iterations
    lands within rounding of the fixed schedule's point."""
    from igaos_gb300 import capi
    lp = G.config2(seed=2, m=3000, n=8000, target_nnz=60000)
    with capi.Problem(lp) as P:
        a = P.solve(tolerance=1e-12, time_limit=1e9, max_iterations=128, schedule="autotune")
        f = P.solve(tolerance=1e-12, time_limit=1e9, max_iterations=128)
    assert a["iterations"] == f["iterations"] == 128
    assert a["entries_a"] in (2, 4, 8, 16, 32) and a["entries_at"] in (2, 4, 8, 16, 32)
    assert abs(a["objective"] - f["objective"]) <= 1e-5 * max(1.0, abs(f["objective"]))


def test_unknown_schedule_is_refused(native):
    from igaos_gb300 import capi
    r = capi.solve_lp(G.random_lp(20, 40, 60, 0), schedule=5)
    assert r["rc"] == capi.ERR_INVALID and "unknown schedule" in capi.last_error()
