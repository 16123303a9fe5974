"""Multicommodity-flow LPs (generators.config5: grid arcs both ways,
8 commodities, shared capacities) against an independent solver's optimum
(scipy's HiGHS interior point, tests/golden/make_mcf_golden.py):

* the 100 x 100 grid (119,600 x 316,800) in both precisions to 1e-8;
* the full 300 x 300 grid (1,078,800 x 2,870,400, 8.6M nonzeros) in FP32 +
  FP64 refinement to 1e-8.

The objective agrees with HiGHS to 1e-6 relative, and the returned pair
passes the oracle's evaluate() at the tolerance.
"""
import json
import os

import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "mcf_objectives.json")))


def check(orc, name, precision, tol=1e-8):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import same_checksum
    from igaos_gb300 import capi
    e = GOLD[name]
    lp = G.config5(**e["kwargs"])
    assert same_checksum(lp, e["checksum"]), "generator drift: regenerate tests/golden"
    ref = e["highs_ipm_objective"]
    r = capi.solve_lp(lp, tolerance=tol, time_limit=120.0, precision=precision)
    assert r["status_name"] == "near-optimal", r["message"]
    assert abs(r["objective"] - ref) / max(1.0, abs(ref)) <= 1e-6, (r["objective"], ref)
    import scipy.sparse as sp
    olp = orc.lp_from(lp)
    A = sp.csr_matrix((olp.ax, olp.ai, olp.ap), shape=(olp.m, olp.n))
    m = orc.evaluate(olp, r["x"], r["y"], A @ r["x"], olp.c + A.T @ r["y"])
    assert max(m["pinf"], m["prow"], m["dinf"]) <= tol and np.isfinite(m["gap"]) and m["gap"] <= tol, m


@pytest.mark.parametrize("precision", ["fp32-refine", "fp64"])
def test_mcf_100_grid_reaches_highs_optimum(native, orc, precision):
    check(orc, "mcf100x8-s0", precision)


def test_mcf_full_size_reaches_highs_optimum(native, orc):
    if "mcf300x8-s0" not in GOLD:
        pytest.skip("no independent optimum recorded for the 300 x 300 grid")
    check(orc, "mcf300x8-s0", "fp32-refine")
