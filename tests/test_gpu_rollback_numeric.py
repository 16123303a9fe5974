"""Two rarely taken branches of the solve loop, driven from the host.

* Rollback to the incumbent (src/pdhg/pdhg.cu:965-988): when the current
  iterate's pinf reaches 0.5 after an incumbent (pinf <= 1e-4) exists and
  more than 2,000 iterations after the last rollback, the incumbent is
  restored, the averaging restarts there and eta is capped at eta0 / 2. No
  LP of the test sets blows up by itself (the oracle counts no rollback on
  the golden and Netlib LPs), so the testing knob IGAOS_PDHG_PERTURB_AT adds
  1e6 to every entry of the current x at the first check at or after
  iteration 3,000 -- on the host's command, no device fault involved. The
  oracle's restatement, given the same perturbation, takes the same single
  rollback at the same check; both then converge to the simplex optimum.
* Numerical failure (IGAOS_PDHG_ERR_NUMERIC): a cost that is finite in FP64
  but overflows the attempt arithmetic (1e39 beyond FP32's range; 1e300
  squared in FP64) makes the step's dot products non-finite; the device step
  decision raises its NaN flag, the loop stops, and the result carries the
  error code and status "error" instead of a number.
"""
import json
import os
import re
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))
sys.path.insert(0, os.path.join(HERE, "golden"))

pytestmark = pytest.mark.gpu


def make(name):
    from make_golden import make_lp
    e = GOLD[name]
    return make_lp(e["generator"], e["kwargs"]), e["simplex_objective"]


@pytest.mark.parametrize("name", ["rand200x500-s0", "bern300-s3"])
@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
def test_rollback_restores_incumbent(native, orc, monkeypatch, capfd, name, precision):
    from igaos_gb300 import capi
    lp, ref = make(name)
    want = orc.pdhg_solve(orc.lp_from(lp), tolerance=1e-8, time_limit=60.0, perturb_at=3000)
    assert want["rollbacks"] == 1 and want["status_name"] == "near-optimal"
    monkeypatch.setenv("IGAOS_PDHG_PERTURB_AT", "3000")
    with capi.Problem(lp) as P:
        eta0 = P.step_init()[1]  # (lambda, eta0, omega0)
        r = P.solve(tolerance=1e-8, time_limit=60.0, precision=precision, verbosity=2)
    err = capfd.readouterr().err
    assert r["rollbacks"] == 1, r
    hits = re.findall(r"rollback @k=(\d+) to the incumbent, eta (\S+)", err)
    assert len(hits) == 1 and int(hits[0][0]) == 3008, hits  # first check at or after 3000
    assert r["status_name"] == "near-optimal", r["message"]
    assert abs(r["objective"] - ref) / max(1.0, abs(ref)) <= 1e-6, (r["objective"], ref)
    assert float(hits[0][1]) <= 0.5 * eta0 * (1 + 1e-12)


def test_no_rollback_without_perturbation(native, monkeypatch):
    from igaos_gb300 import capi
    monkeypatch.delenv("IGAOS_PDHG_PERTURB_AT", raising=False)
    lp, _ = make("rand200x500-s0")
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0)
    assert r["rollbacks"] == 0 and r["status_name"] == "near-optimal"


@pytest.mark.parametrize("precision, cost", [("fp32", 1e39), ("fp32-refine", 1e39),
                                             ("fp64", 1e300)])
def test_overflow_reports_numeric_error(native, precision, cost):
    from igaos_gb300 import capi, generators as G
    lp = G.random_lp(40, 90, 150, 2)
    lp.c = lp.c.copy()
    lp.cl = lp.cl.copy()
    lp.cu = lp.cu.copy()
    lp.c[0] = cost
    lp.cl[0], lp.cu[0] = -np.inf, np.inf
    r = capi.solve_lp(lp, tolerance=1e-6, time_limit=30.0, precision=precision)
    assert r["error_code"] == capi.ERR_NUMERIC, (r["error_code"], r["message"])
    assert r["status_name"] == "error"
    assert "NaN/Inf" in r["message"]
