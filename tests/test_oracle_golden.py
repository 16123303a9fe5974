"""Pins the CPU oracle to the reference (no GPU).

* evaluate(): bit-identical to the reference's own evaluate()
  (src/pdhg/pdhg.cu:173-254) on the committed golden cases.
* counting_sort(): bit-identical to src/io/model.hpp:39-67.
* The oracle PDHG reaches the reference simplex optimum (golden, produced by
  the reference's own simplex) on seeded LPs, and -- where the reference tree
  is present -- the reference's recorded PDHG objectives on Netlib
  (docs/research/final_battery_2026-08-29.txt:57-64; exact HiGHS values from
  docs/research/sweep_results.csv; afiro asserted in tests/warm_smoke.cpp:76).
"""
import json
import os

import numpy as np
import pytest

from conftest import reference_dir

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_evaluate_bit_identical_to_reference(orc):
    z = np.load(os.path.join(GOLD, "evaluate_cases.npz"))
    finite_gaps = 0
    for k in range(int(z["count"])):
        a = [z[f"{k}_{q}"] for q in ("rmin", "rmax", "cl", "cu", "c", "x", "y", "Ax", "d")]
        got = orc.evaluate_arrays(*a)
        want = z[f"{k}_out"]
        for i, key in enumerate(("pinf", "dinf", "gap", "op", "od", "prow")):
            assert got[key] == want[i] or (np.isnan(got[key]) and np.isnan(want[i])), (k, key)
        finite_gaps += np.isfinite(want[2])
    assert finite_gaps >= 2  # both the certified-gap and the -inf-bound branches


def test_counting_sort_bit_identical_to_reference(orc):
    z = np.load(os.path.join(GOLD, "counting_sort.npz"))
    for k in range(int(z["count"])):
        rows, cols = (int(v) for v in z[f"{k}_shape"])
        got = orc.counting_sort(z[f"{k}_ti"], z[f"{k}_tj"], z[f"{k}_tv"], rows, cols)
        for g, name in zip(got, ("ap", "ai", "ax", "cp", "ci", "acx")):
            assert np.array_equal(g, z[f"{k}_{name}"]), (k, name)


def test_transpose_equals_counting_sort_of_row_ordered_triplets(orc):
    rng = np.random.default_rng(5)
    rows, cols = 40, 55
    ti = np.sort(rng.integers(0, rows, 300))
    tj = rng.integers(0, cols, 300)
    tv = rng.standard_normal(300)
    ap, ai, ax, cp, ci, acx = orc.counting_sort(ti, tj, tv, rows, cols)
    tcp, tci, tacx = orc.transpose(rows, cols, ap, ai, ax)
    assert np.array_equal(tcp, cp) and np.array_equal(tci, ci) and np.array_equal(tacx, acx)


def _golden_lp(name):
    import sys
    sys.path.insert(0, GOLD)
    from make_golden import make_lp, same_checksum
    e = json.load(open(os.path.join(GOLD, "lp_objectives.json")))[name]
    lp = make_lp(e["generator"], e["kwargs"])
    assert same_checksum(lp, e["checksum"])
    return lp, e


@pytest.mark.parametrize("name", ["rand60x150-s0", "rand60x150-s1", "mixed80x200-s0",
                                  "bern50-s1", "grid6x6-k2"])
def test_oracle_pdhg_reaches_reference_simplex_optimum(orc, name):
    lp, e = _golden_lp(name)
    assert e["simplex_status"] == "optimal"
    if e["highs_objective"] is not None:
        assert abs(e["simplex_objective"] - e["highs_objective"]) <= 1e-7 * max(1, abs(e["highs_objective"]))
    r = orc.pdhg_solve(orc.lp_from(lp), tolerance=1e-8, time_limit=60.0)
    assert r["status_name"] == "near-optimal"
    ref = e["simplex_objective"]
    assert abs(r["objective"] - ref) / max(1.0, abs(ref)) <= 1e-6


# Netlib instances shipped with the reference, with the reference's recorded
# PDHG objective at tol 1e-3 / 16 s and the exact optimum it was compared to.
NETLIB = {
    "afiro": (-464.7531, -464.7531429),
    "kb2": (-1749.9002, -1749.90013),
    "sc50a": (-64.5751, -64.57507706),
}


@pytest.mark.skipif(reference_dir() is None, reason="reference tree not present")
@pytest.mark.parametrize("name", sorted(NETLIB))
def test_oracle_on_reference_netlib_fixtures(orc, name):
    path = os.path.join(reference_dir(), "demo", "models", "netlib_full", name + ".mps")
    if not os.path.exists(path) or not orc.ref_available():
        pytest.skip("netlib file or reference helpers missing")
    lp = orc.ref_parse_mps(path)
    recorded, exact = NETLIB[name]
    r = orc.pdhg_solve(lp, tolerance=1e-6, time_limit=60.0)
    assert abs(r["objective"] - exact) / max(1.0, abs(exact)) <= 1e-4
    assert abs(r["objective"] - recorded) / max(1.0, abs(recorded)) <= 1e-3
