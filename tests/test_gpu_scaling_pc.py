"""Opt-in Pock-Chambolle scaling (igaos_pdhg_options.scaling =
IGAOS_PDHG_SCALING_RUIZ_PC): after the reference's 10 Ruiz sweeps
(src/pdhg/pdhg.cu:472-492), one pass with alpha = 1 divides every row and
column of the scaled matrix by the square root of its 1-norm (PDLP's
default scaling; the reference has none, its cost scale is 1 at :494-498).

* The factors equal the oracle's restatement (oracle.pock_chambolle applied
  to the oracle's Ruiz factors) to 1e-13 relative: the 1-norms are sums, so
  their order differs from the sequential loop.
* The default stays the reference's Ruiz scaling, bit for bit.
* With the pass on, FP64 and FP32 + refinement solves reach the reference
  simplex optimum to 1e-6 at 1e-8 relative KKT (the metrics are always
  those of the original LP, so the scaling changes the path, not the bar).
"""
import json
import os

import numpy as np
import pytest

from igaos_gb300 import generators as G

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))

MATS = {
    "rand": lambda: G.random_lp(300, 700, 2500, 1),
    "zipf": lambda: G.config2(seed=2, m=3000, n=8000, target_nnz=60000),
    "grid": lambda: G.config5(seed=3, side=12, commodities=3),
    "mixed": lambda: G.mixed_bounds_lp(120, 300, 700, 4),
}


def test_unknown_scaling_is_rejected(native):
    from igaos_gb300 import capi
    with pytest.raises(capi.EngineError, match="unknown scaling"):
        capi.Problem(G.random_lp(20, 40, 60, 0), scaling=7)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MATS))
def test_pc_factors_match_oracle(native, orc, name):
    from igaos_gb300 import capi
    lp = MATS[name]()
    olp = orc.lp_from(lp)
    rdr, rdc = orc.ruiz(olp)
    want_r, want_c = orc.pock_chambolle(olp, rdr, rdc)
    with capi.Problem(lp, scaling="ruiz-pc") as P:
        dr, dc = P.scaling()
    np.testing.assert_allclose(dr, want_r, rtol=1e-13, atol=0)
    np.testing.assert_allclose(dc, want_c, rtol=1e-13, atol=0)
    with capi.Problem(lp) as P:
        dr, dc = P.scaling()
    assert np.array_equal(dr, rdr) and np.array_equal(dc, rdc)


def make(name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import make_lp, same_checksum
    e = GOLD[name]
    lp = make_lp(e["generator"], e["kwargs"])
    assert same_checksum(lp, e["checksum"])
    return lp, e["simplex_objective"]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
@pytest.mark.parametrize("name", sorted(k for k in GOLD if not k.startswith("zipf")))
def test_pc_solves_match_simplex(native, name, precision):
    from igaos_gb300 import capi
    lp, ref = make(name)
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0, precision=precision,
                      scaling="ruiz-pc")
    assert r["status_name"] == "near-optimal", r["message"]
    assert abs(r["objective"] - ref) / max(1.0, abs(ref)) <= 1e-6, (r["objective"], ref)
    assert max(r["pinf"], r["prow"], r["dinf"], r["rel_gap"]) <= 1e-8
