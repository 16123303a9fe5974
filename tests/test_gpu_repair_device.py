"""Matrix-free dual repair on the device (igaos_pdhg_dual_repair_device), the
solve loop's repair step at every m.

The reference's dual_repair (src/pdhg/pdhg.cu:288-448) needs a dense m x m
Cholesky factor; the device path projects onto the same three sets
matrix-free, so its duals differ from the reference's. What is checked is
the certificate itself, recomputed by the oracle's restatement of
evaluate() (src/pdhg/pdhg.cu:173-254): every dual the device path reports
certified has a finite gap <= tol at the candidate x.

* LPs with a known optimal pair (x*, y*) and a perturbed dual (gap -inf):
  certified at m = 3,000 and m = 40,000.
* Duals the reference's dense repair certifies on the golden cases are
  certified by the device path as well (at the reference's own gap, or 1e-6).
* A candidate off the feasible set is reported uncertified.
* In a solve with m = 5,000 the scheduled repair step runs on the device and
  certifies the gap.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def oracle_metrics(orc, lp, x, y):
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    return orc.evaluate_arrays(lp.rmin, lp.rmax, lp.cl, lp.cu, lp.c, x, y, A @ x, lp.c + A.T @ y)


def noisy(y, seed, scale=1e-6):
    rng = np.random.default_rng(seed)
    return y + scale * rng.standard_normal(y.shape[0]) * (1.0 + np.abs(y))


@pytest.mark.parametrize("m,seed", [(3000, 1), (3000, 2), (40000, 0)])
def test_device_repair_certifies_perturbed_optimum(native, orc, m, seed):
    from igaos_gb300 import capi
    lp, xs, ys = G.known_optimum_lp(m, int(2.5 * m), 2 * m, seed)
    yn = noisy(ys, seed)
    assert oracle_metrics(orc, lp, xs, ys)["gap"] <= 1e-12
    assert not np.isfinite(oracle_metrics(orc, lp, xs, yn)["gap"])
    tol = 1e-6
    with capi.Problem(lp) as P:
        ok, y, mt = P.dual_repair_device(xs, yn, 1e-6, tol)
    assert ok, mt
    check = oracle_metrics(orc, lp, xs, y)
    assert np.isfinite(check["gap"]) and check["gap"] <= tol, check
    assert abs(check["gap"] - mt["gap"]) <= 1e-9 + 1e-6 * check["gap"], (check, mt)
    # the certified dual stays close to the optimal one
    assert np.max(np.abs(y - ys)) <= 1e-3 * (1.0 + np.max(np.abs(ys)))


def test_device_repair_certifies_what_the_dense_repair_certifies(native, orc):
    from igaos_gb300 import capi
    gold = np.load(os.path.join(HERE, "golden", "dual_repair_cases.npz"))
    checked = 0
    for k in range(int(gold["count"])):
        if not bool(gold[f"ok_{k}"]):
            continue
        m, n, e, seed = (int(v) for v in gold[f"lp_{k}"])
        lp = G.free_cost_lp(m, n, e, seed)
        x, y_it, col_tol = gold[f"x_{k}"], gold[f"y_it_{k}"], float(gold[f"tol_{k}"])
        ref = oracle_metrics(orc, lp, x, gold[f"y_{k}"])
        base = oracle_metrics(orc, lp, x, y_it)
        # pinf and prow depend on x alone; the device's KKT sums may round
        # their last digits differently
        tol = max(1e-6, ref["gap"], base["pinf"], base["prow"]) * (1.0 + 1e-9)
        with capi.Problem(lp) as P:
            ok, y, mt = P.dual_repair_device(x, y_it, col_tol, tol)
        assert ok, (k, mt, ref)
        check = oracle_metrics(orc, lp, x, y)
        assert np.isfinite(check["gap"]) and check["gap"] <= tol, (k, check)
        checked += 1
    assert checked >= 2


def test_device_repair_reports_uncertified_duals(native, orc):
    """A candidate x off the feasible set (pinf above tol) can never be
    certified: the call says so and its metrics are those of the dual it
    returns."""
    from igaos_gb300 import capi
    lp, xs, ys = G.known_optimum_lp(2000, 5000, 4000, 5)
    x = xs + 0.01 * np.random.default_rng(3).standard_normal(lp.n)
    with capi.Problem(lp) as P:
        ok, y, mt = P.dual_repair_device(x, noisy(ys, 5), 1e-6, 1e-9)
    assert not ok
    check = oracle_metrics(orc, lp, x, y)
    assert check["pinf"] > 1e-9
    assert check["pinf"] == pytest.approx(mt["pinf"], rel=1e-9, abs=1e-15)


def test_solve_certified_by_device_repair(native, orc):
    """m = 5,000: the solve loop's scheduled repair step runs on the device
    and certifies the gap; the reported pair passes the oracle's
    evaluate() at tol and the objective matches the known optimum."""
    from igaos_gb300 import capi
    lp, xs, ys = G.known_optimum_lp(5000, 12500, 10000, 0)
    opt = float(lp.c @ xs)
    tol = 1e-4
    r = capi.solve_lp(lp, tolerance=tol, time_limit=60.0, precision="fp64")
    assert r["status_name"] == "near-optimal", r["message"]
    assert "dual repair" in r["message"], r["message"]
    check = oracle_metrics(orc, lp, r["x"], r["y"])
    assert np.isfinite(check["gap"]) and check["gap"] <= tol, check
    assert max(check["pinf"], check["prow"]) <= tol, check
    assert abs(r["objective"] - opt) <= 10 * tol * max(1.0, abs(opt)), (r["objective"], opt)
