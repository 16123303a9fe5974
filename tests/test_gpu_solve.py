"""End-to-end parity of GPU solves through the C ABI against the reference
simplex optimum (golden fixtures made by tests/golden/make_golden.py from the
reference's own simplex) and against the CPU oracle of the reference PDHG.

Objective parity bar: |obj - obj_ref| / max(1, |obj_ref|) <= 1e-6 at a
relative-KKT tolerance of 1e-8 (FP64, FP32+refine); FP32 without refinement
is only held to its own tolerance.
"""
import json
import os

import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))


def make(name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import make_lp, same_checksum
    e = GOLD[name]
    lp = make_lp(e["generator"], e["kwargs"])
    assert same_checksum(lp, e["checksum"]), "generator drift: regenerate tests/golden"
    return lp, e["simplex_objective"]


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


# The reference's PDHG does not reach 1e-8 on the Zipf / log-uniform shape in
# any practical budget (its own oracle plateaus at dinf ~1e-1 after 3.5M
# iterations); that instance is covered by fixed-budget tracking below.
CONVERGING = sorted(k for k in GOLD if not k.startswith("zipf"))


@pytest.mark.parametrize("name", CONVERGING)
def test_fp64_matches_simplex(native, name):
    from igaos_gb300 import capi
    lp, ref = make(name)
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0)
    assert r["status_name"] == "near-optimal", r["message"]
    assert rel(r["objective"], ref) <= 1e-6, (r["objective"], ref)
    assert r["pinf"] <= 1e-8 and r["dinf"] <= 1e-8 and r["rel_gap"] <= 1e-8 and r["prow"] <= 1e-8


@pytest.mark.parametrize("name", ["rand60x150-s0", "mixed80x200-s1"])
def test_fp64_tracks_oracle_pdhg(native, orc, name):
    """Same algorithm on both sides: both certify, the objectives agree to the
    tolerance and the iteration counts are of the same size (rounding-level
    differences in the sums can move a restart check by an epoch, so the
    trajectories are not identical)."""
    from igaos_gb300 import capi
    lp, ref = make(name)
    want = orc.pdhg_solve(orc.lp_from(lp), tolerance=1e-6, time_limit=60.0)
    got = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0)
    assert got["status_name"] == want["status_name"] == "near-optimal"
    assert rel(got["objective"], want["objective"]) <= 1e-5
    assert 0.5 * want["iterations"] <= got["iterations"] <= 2.0 * want["iterations"]


def test_fp64_fixed_budget_tracks_oracle_on_zipf(native, orc):
    """On the shape where neither side converges, a fixed budget of the same
    algorithm (checks, restarts and all) lands on the same point. The
    trajectory there is chaotic -- a 1-ulp change of c moves the oracle's own
    objective by 1e-7 after 256 iterations and by 4e-4 after 640 -- so the
    budget is 256 iterations (four checks)."""
    from igaos_gb300 import capi
    lp, _ = make("zipf400x1000")
    want = orc.pdhg_solve(orc.lp_from(lp), tolerance=1e-12, time_limit=1e9, max_iterations=256)
    got = capi.solve_lp(lp, tolerance=1e-12, time_limit=1e9, max_iterations=256)
    assert got["iterations"] == want["iterations"] == 256
    assert got["restarts"] == want["restarts"]
    assert rel(got["objective"], want["objective"]) <= 1e-5


def test_solution_vectors_certify(native, orc):
    """x, y returned in original units reproduce the reported metrics under the
    oracle's evaluate()."""
    from igaos_gb300 import capi
    lp, ref = make("rand200x500-s0")
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0)
    olp = orc.lp_from(lp)
    Ax = orc.spmv(olp.ap, olp.ai, olp.ax, r["x"])
    d = lp.c + orc.spmv(olp.cp, olp.ci, olp.acx, r["y"])
    m = orc.evaluate(olp, r["x"], r["y"], Ax, d)
    assert m["pinf"] <= 1e-8 and m["prow"] <= 1e-8 and m["gap"] <= 1e-8 and m["dinf"] <= 1e-8
    assert rel(m["op"] + lp.obj_const, ref) <= 1e-6


def test_deterministic_repeat(native):
    from igaos_gb300 import capi
    lp, _ = make("zipf400x1000")
    with capi.Problem(lp) as P:
        a = P.solve(tolerance=1e-12, time_limit=1e9, max_iterations=3000)
        b = P.solve(tolerance=1e-12, time_limit=1e9, max_iterations=3000)
    assert a["objective"] == b["objective"] and a["iterations"] == b["iterations"]
    assert np.array_equal(a["x"], b["x"])


def test_graphs_and_direct_launch_agree(native):
    from igaos_gb300 import capi
    lp, _ = make("mixed80x200-s0")
    a = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0, use_graphs=1)
    b = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0, use_graphs=0)
    assert a["objective"] == b["objective"] and a["iterations"] == b["iterations"]


def test_fp32_reaches_its_tolerance(native):
    from igaos_gb300 import capi
    lp, ref = make("rand200x500-s1")
    r = capi.solve_lp(lp, tolerance=1e-4, time_limit=60.0, precision="fp32")
    assert r["status_name"] == "near-optimal", r["message"]
    assert rel(r["objective"], ref) <= 1e-3


@pytest.mark.parametrize("name", CONVERGING)
def test_fp32_refine_matches_simplex(native, name):
    """FP32 attempts with FP64 anchors reach the FP64 bar: 1e-8 relative KKT
    and the reference simplex optimum to 1e-6."""
    from igaos_gb300 import capi
    lp, ref = make(name)
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0, precision="fp32-refine")
    assert r["status_name"] == "near-optimal", r["message"]
    assert rel(r["objective"], ref) <= 1e-6, (r["objective"], ref)
    assert r["refinements"] >= 1


def test_fp32_refine_vectors_certify(native, orc):
    from igaos_gb300 import capi
    lp, ref = make("mixed80x200-s2")
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0, precision="fp32-refine")
    olp = orc.lp_from(lp)
    Ax = orc.spmv(olp.ap, olp.ai, olp.ax, r["x"])
    d = lp.c + orc.spmv(olp.cp, olp.ci, olp.acx, r["y"])
    m = orc.evaluate(olp, r["x"], r["y"], Ax, d)
    assert max(m["pinf"], m["prow"], m["dinf"], m["gap"]) <= 1e-8
    assert rel(m["op"] + lp.obj_const, ref) <= 1e-6


def test_iteration_limit_and_time_limit(native):
    from igaos_gb300 import capi
    lp, _ = make("rand200x500-s0")
    # max_iterations binds only without a finite time limit (src/pdhg/pdhg.cu:669-671)
    r = capi.solve_lp(lp, tolerance=1e-12, time_limit=1e9, max_iterations=200)
    assert r["status_name"] == "iteration-limit" and r["iterations"] == 200
    r = capi.solve_lp(lp, tolerance=1e-14, time_limit=0.05)
    assert r["status_name"] == "time-limit"
    assert r["message"] == "wall-clock budget exhausted"


def test_short_run_without_check_is_not_certified(native):
    """Fewer iterations than one check period: the final iterate is evaluated
    (the reference would report its zero-initialised metrics as certified)."""
    from igaos_gb300 import capi
    lp, _ = make("rand200x500-s0")
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=1e9, max_iterations=10)
    assert r["iterations"] == 10 and r["status_name"] == "iteration-limit"


def test_c1_full_size_matches_simplex(native):
    path = os.path.join(HERE, "golden", "c1_objectives.json")
    if not os.path.exists(path):
        pytest.skip("c1 golden not generated")
    from igaos_gb300 import capi
    gold = json.load(open(path))
    e = gold["c1-s0"]
    lp = G.config1(seed=0)
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=120.0)
    assert r["status_name"] == "near-optimal", r["message"]
    assert rel(r["objective"], e["simplex_objective"]) <= 1e-6
