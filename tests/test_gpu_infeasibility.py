"""Infeasibility certificates (igaos_pdhg_options.detect_infeasibility; no
counterpart in the reference engine, which ends such LPs at its iteration
cap): the change between consecutive restart points is tested as a dual ray
(the LP is infeasible) or a primal ray (its dual is; a feasible LP is
unbounded). Each reported ray is re-checked here with numpy in original
units, and feasible LPs are solved exactly as without the test.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
INF = float("inf")


def check_dual_ray(lp, y):
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    assert np.max(np.abs(y)) == pytest.approx(1.0)
    d = A.T @ y
    obj = 0.0
    for j in range(lp.n):
        if d[j] > 0:
            assert np.isfinite(lp.cl[j]) or d[j] <= 1e-9
            obj += d[j] * lp.cl[j] if np.isfinite(lp.cl[j]) else 0.0
        elif d[j] < 0:
            assert np.isfinite(lp.cu[j]) or -d[j] <= 1e-9
            obj += d[j] * lp.cu[j] if np.isfinite(lp.cu[j]) else 0.0
    for i in range(lp.m):
        if y[i] > 0:
            assert np.isfinite(lp.rmax[i]) or y[i] <= 1e-9
            obj -= y[i] * lp.rmax[i] if np.isfinite(lp.rmax[i]) else 0.0
        elif y[i] < 0:
            assert np.isfinite(lp.rmin[i]) or -y[i] <= 1e-9
            obj -= y[i] * lp.rmin[i] if np.isfinite(lp.rmin[i]) else 0.0
    assert obj > 0.0, obj


def check_primal_ray(lp, x):
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    assert np.max(np.abs(x)) == pytest.approx(1.0)
    assert lp.c @ x < 0.0
    ax = A @ x
    tol = 1e-9 * max(1.0, np.max(np.abs(ax)))
    assert np.all((x >= -1e-9) | ~np.isfinite(lp.cl))
    assert np.all((x <= 1e-9) | ~np.isfinite(lp.cu))
    assert np.all((ax >= -tol) | ~np.isfinite(lp.rmin))
    assert np.all((ax <= tol) | ~np.isfinite(lp.rmax))


def two_rows_infeasible():
    # x1 + x2 <= 1 and x1 + x2 >= 3 on [0, 5]^2
    return G.from_triplets(2, 2, [0, 0, 1, 1], [0, 1, 0, 1], [1.0, 1.0, 1.0, 1.0],
                           [1.0, 1.0], [0.0, 0.0], [5.0, 5.0], [-INF, 3.0], [1.0, INF])


def contradictory_rows(seed=2):
    """A feasible random LP (m 1,500) plus two rows that contradict each
    other (the sum of the first 40 columns <= 10 and >= 30)."""
    base = G.random_lp(1500, 3750, 6000, seed)
    rows = np.repeat(np.arange(base.m), np.diff(base.ap))
    k = np.arange(40)
    rows = np.concatenate([rows, np.full(40, base.m), np.full(40, base.m + 1)])
    cols = np.concatenate([base.ai, k, k])
    vals = np.concatenate([base.ax, np.ones(80)])
    return G.from_triplets(base.m + 2, base.n, rows, cols, vals, base.c, base.cl, base.cu,
                           np.concatenate([base.rmin, [-INF, 30.0]]),
                           np.concatenate([base.rmax, [10.0, INF]]))


def unbounded_lp():
    # min -x1 - 0.5 x3 s.t. x1 - x2 <= 1, x2 - x3 <= 2, x1 + x3 >= 1; x >= 0
    return G.from_triplets(3, 3, [0, 0, 1, 1, 2, 2], [0, 1, 1, 2, 0, 2],
                           [1.0, -1.0, 1.0, -1.0, 1.0, 1.0], [-1.0, 0.0, -0.5],
                           [0.0, 0.0, 0.0], [INF, INF, INF], [-INF, -INF, 1.0], [1.0, 2.0, INF])


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
@pytest.mark.parametrize("make", [two_rows_infeasible, contradictory_rows])
def test_infeasible_lp_gets_a_dual_ray(native, precision, make):
    from igaos_gb300 import capi
    lp = make()
    r = capi.solve_lp(lp, tolerance=1e-6, time_limit=120.0, max_iterations=400000,
                      precision=precision, detect_infeasibility=1)
    assert r["status_name"] == "infeasible", (r["status_name"], r["message"], r["iterations"])
    assert "dual ray" in r["message"]
    check_dual_ray(lp, r["y"])


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
def test_unbounded_lp_gets_a_primal_ray(native, precision):
    from igaos_gb300 import capi
    lp = unbounded_lp()
    r = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0, max_iterations=400000,
                      precision=precision, detect_infeasibility=1)
    assert r["status_name"] == "unbounded", (r["status_name"], r["message"], r["iterations"])
    check_primal_ray(lp, r["x"])


@pytest.mark.parametrize("name,make", [
    ("random", lambda: G.random_lp(300, 700, 2500, 1)),
    ("free-cost", lambda: G.free_cost_lp(80, 200, 400, 3)),
    ("mixed", lambda: G.mixed_bounds_lp(120, 300, 700, 4)),
])
def test_feasible_lps_unchanged_by_the_test(native, name, make):
    from igaos_gb300 import capi
    lp = make()
    a = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0)
    b = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0, detect_infeasibility=1)
    assert a["status_name"] == b["status_name"] == "near-optimal", (a["message"], b["message"])
    assert a["iterations"] == b["iterations"]
    assert a["objective"] == b["objective"]


def test_cli_flag_reports_infeasible(native, tmp_path):
    """`igaos solve m.mps --engine pdhg --detect-infeasibility` prints the
    reference's JSON record with status "infeasible"; without the flag the
    record says "iteration-limit", as the reference engine would."""
    import json
    import os
    import subprocess
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_gpu_surfaces import write_mps
    lp = contradictory_rows()
    p = tmp_path / "inf.mps"
    write_mps(lp, p)
    cli = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "igaos_gb300",
                       "igaos")
    base = [cli, "solve", str(p), "--engine", "pdhg", "--tol", "1e-6", "--time-limit", "1e9"]
    rec = json.loads(subprocess.run(base + ["--max-iter", "400000", "--detect-infeasibility"],
                                    capture_output=True, text=True, check=True).stdout)
    assert rec["status"] == "infeasible", rec["message"]
    rec = json.loads(subprocess.run(base + ["--max-iter", "20000"], capture_output=True, text=True,
                                    check=True).stdout)
    assert rec["status"] == "iteration-limit", rec["message"]


def test_pybind_solve_reports_infeasible(native, tmp_path):
    """igaos_gb300.solve(path, engine="pdhg", detect_infeasibility=True)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_gpu_surfaces import write_mps
    import igaos_gb300 as ig
    p = tmp_path / "inf.mps"
    write_mps(two_rows_infeasible(), p)
    s = ig.solve(str(p), time_limit=60.0, tolerance=1e-6, engine="pdhg", detect_infeasibility=True)
    assert s.status == "infeasible", s.message
