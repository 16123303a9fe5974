"""Start points (igaos_pdhg_set_start; no reference counterpart: its iterates
start at zero, src/pdhg/pdhg.cu:576-580).

* Started at its own 1e-8 answer, an FP64 solve ends within two KKT
  checks, at the same optimum. FP32 + refinement takes the point as its first
  anchor; its FP32 deltas over FP32-rounded residual data need a few
  re-anchoring restarts to hold 1e-8 again, still fewer iterations than
  from zero.
* Started near the optimum it needs fewer iterations than from zero, and
  reaches the reference simplex's optimum (tests/golden).
* Clearing the start point gives back the cold solve bit for bit; a start
  outside the box is projected onto it; a presolved handle and a half-given
  start are refused.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))


def golden(name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import make_lp
    return make_lp(GOLD[name]["generator"], GOLD[name]["kwargs"]), GOLD[name]["simplex_objective"]


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
def test_start_at_the_answer_ends_at_once(native, precision):
    from igaos_gb300 import capi
    lp, want = golden("rand200x500-s0")
    with capi.Problem(lp) as P:
        cold = P.solve(precision=precision, tolerance=1e-8, time_limit=60.0)
        assert cold["status_name"] == "near-optimal"
        P.set_start(cold["x"], cold["y"])
        warm = P.solve(precision=precision, tolerance=1e-8, time_limit=60.0)
        assert warm["status_name"] == "near-optimal"
        if precision == "fp64":
            assert warm["iterations"] <= 128 < cold["iterations"]
        else:
            assert warm["iterations"] < cold["iterations"], (warm["iterations"], cold["iterations"])
        assert rel(warm["objective"], want) <= 1e-6
        P.set_start()
        again = P.solve(precision=precision, tolerance=1e-8, time_limit=60.0)
        assert again["iterations"] == cold["iterations"]
        assert again["objective"] == cold["objective"]
        assert np.array_equal(again["x"], cold["x"])


def test_start_near_the_optimum_saves_iterations(native):
    from igaos_gb300 import capi
    lp, want = golden("rand200x500-s1")
    with capi.Problem(lp) as P:
        cold = P.solve(precision="fp64", tolerance=1e-8, time_limit=60.0)
        rough = P.solve(precision="fp64", tolerance=1e-4, time_limit=60.0)
        assert rough["status_name"] == "near-optimal"
        P.set_start(rough["x"], rough["y"])
        warm = P.solve(precision="fp64", tolerance=1e-8, time_limit=60.0)
    assert warm["status_name"] == "near-optimal"
    assert rel(warm["objective"], want) <= 1e-6
    assert warm["iterations"] < cold["iterations"], (warm["iterations"], cold["iterations"])


def test_start_is_projected_and_validated(native):
    from igaos_gb300 import capi
    lp, want = golden("rand60x150-s0")
    with capi.Problem(lp) as P:
        big = np.full(lp.n, 1e30)
        P.set_start(big, np.zeros(lp.m))  # projected onto the box
        r = P.solve(precision="fp64", tolerance=1e-8, time_limit=60.0)
        assert r["status_name"] == "near-optimal" and rel(r["objective"], want) <= 1e-6
        with pytest.raises(capi.EngineError, match="both given or both NULL"):
            capi._check(capi.lib().igaos_pdhg_set_start(P.h, capi._d(big), None))
    with capi.Problem(lp, pdhg_presolve=1) as P:
        with pytest.raises(capi.EngineError, match="presolved handle"):
            P.set_start(np.zeros(lp.n), np.zeros(lp.m))
