"""The pdhg_presolve option on the GPU engine (igaos_pdhg_options.pdhg_presolve,
CLI --pdhg-presolve, igaos_gb300.solve(pdhg_presolve=True)).

* LPs with every planted reduction solve to the HiGHS optimum at 1e-6 in
  FP64 and FP32 + refinement; the reported metrics are those of the ORIGINAL
  LP (the oracle's evaluate of the returned pair agrees with them).
* An LP presolve removes entirely is answered without a PDHG iteration.
* Presolve outcomes (infeasible, unbounded) become the solve's status.
* A presolved handle refuses the inspection entry points.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from igaos_gb300 import generators as G
from test_presolve_cpu import highs, metrics, tiny
from test_gpu_surfaces import write_mps

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INF = float("inf")


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
@pytest.mark.parametrize("seed", [0, 1])
def test_presolved_solve_reaches_the_optimum(native, orc, precision, seed):
    from igaos_gb300 import capi
    tol = 1e-6
    lp = G.presolvable_lp(60, 150, 250, seed)
    _, _, ref = highs(lp)
    r = capi.solve_lp(lp, tolerance=tol, time_limit=60.0, precision=precision, pdhg_presolve=1)
    assert r["status_name"] == "near-optimal", r["message"]
    assert "presolve" in r["message"]
    assert max(r["pinf"], r["prow"], r["dinf"], r["rel_gap"]) <= tol
    assert abs(r["objective"] - ref) <= 10 * tol * max(1.0, abs(ref)), (r["objective"], ref)
    mt = metrics(orc, lp, r["x"], r["y"])
    for k, rk in (("pinf", "pinf"), ("prow", "prow"), ("dinf", "dinf"), ("gap", "rel_gap")):
        assert mt[k] == pytest.approx(r[rk], rel=1e-9, abs=1e-13), (k, mt[k], r[rk])
    # the same LP without presolve reaches the same optimum
    s = capi.solve_lp(lp, tolerance=tol, time_limit=60.0, precision=precision)
    assert s["status_name"] == "near-optimal"
    assert abs(s["objective"] - ref) <= 10 * tol * max(1.0, abs(ref))


def test_lp_removed_by_presolve(native, orc):
    from igaos_gb300 import capi
    lp = tiny([0], [0], [2.0], [1.0], [-INF], [INF], [4.0], [INF])
    r = capi.solve_lp(lp, tolerance=1e-8, pdhg_presolve=1)
    assert r["status_name"] == "near-optimal" and r["iterations"] == 0, r
    assert r["objective"] == 2.0 and np.array_equal(r["x"], [2.0]) and np.array_equal(r["y"], [-0.5])
    assert max(r["pinf"], r["prow"], r["dinf"], r["rel_gap"]) == 0.0


@pytest.mark.parametrize("status, lp", [
    ("infeasible", tiny([0, 1], [0, 0], [1.0, 1.0], [1.0], [0.0], [10.0], [-INF, 3.0], [1.0, INF])),
    ("unbounded", tiny([0], [0], [1.0], [1.0, -1.0], [0.0, 0.0], [1.0, INF], [0.0], [1.0])),
])
def test_presolve_outcome_is_the_status(native, status, lp):
    from igaos_gb300 import capi
    r = capi.solve_lp(lp, tolerance=1e-6, pdhg_presolve=1)
    assert r["rc"] == capi.OK and r["status_name"] == status, r
    assert r["message"].startswith("presolve") and r["iterations"] == 0


def test_presolved_handle_refuses_inspection(native):
    from igaos_gb300 import capi
    lp = G.presolvable_lp(60, 150, 250, 0)
    with capi.Problem(lp, pdhg_presolve=1) as P:
        with pytest.raises(capi.EngineError, match="presolved handle"):
            P.scaling()
        with pytest.raises(capi.EngineError, match="presolved handle"):
            P.spmv(np.zeros(lp.n))
        r = P.solve(tolerance=1e-6, time_limit=60.0)
        assert r["status_name"] == "near-optimal" and len(r["x"]) == lp.n


def test_cli_and_pybind_pdhg_presolve(native, tmp_path):
    import igaos_gb300 as ig
    lp = G.presolvable_lp(60, 150, 250, 1)
    _, _, ref = highs(lp)
    p = tmp_path / "p.mps"
    write_mps(lp, p)
    cli = os.path.join(ROOT, "igaos_gb300", "igaos")
    out = subprocess.run([cli, "solve", str(p), "--engine", "pdhg", "--tol", "1e-6",
                          "--time-limit", "60", "--pdhg-presolve"], capture_output=True, text=True,
                         check=True).stdout
    rec = json.loads(out)
    assert rec["status"] == "near-optimal" and "presolve" in rec["message"], rec["message"]
    assert abs(rec["objective"] - ref) <= 1e-5 * max(1.0, abs(ref))
    s = ig.solve(str(p), time_limit=60.0, tolerance=1e-6, engine="pdhg", pdhg_presolve=True)
    assert s.status == "near-optimal" and len(s.x) == lp.n and len(s.y) == lp.m
    assert abs(s.objective - ref) <= 1e-5 * max(1.0, abs(ref))


def test_rays_come_back_as_certificates_of_the_original(native):
    """Rays through a presolved solve. x1 + x2 >= 3 with x1 <= 1 and x2 <= 1
    as singleton rows, x free: presolve proves it infeasible (largest
    activity 2 < 3) and the answer's y is that row's ray mapped back through
    the singleton rows, a certificate of the ORIGINAL LP. And presolve's own
    unbounded column comes back as a primal ray with its substituted column
    following."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 1, 2], [0, 1, 0, 1], [1.0] * 4, [1.0, 1.0], [-INF, -INF], [INF, INF],
              [3.0, -INF, -INF], [INF, 1.0, 1.0])
    r = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0, detect_infeasibility=1,
                      pdhg_presolve=1)
    assert r["status_name"] == "infeasible" and "reduced LP" not in r["message"], r["message"]
    assert capi.ray_certificate(lp, np.zeros(2), r["y"])[0] == 1
    lp = tiny([0, 0, 0], [0, 1, 2], [1.0, 1.0, 1.0], [0.0, 1.0, 0.5], [0.0, -INF, 0.0],
              [5.0, INF, INF], [2.0], [2.0])
    r = capi.solve_lp(lp, tolerance=1e-6, pdhg_presolve=1)
    assert r["status_name"] == "unbounded" and np.array_equal(r["x"], [0.0, -1.0, 1.0]), r
