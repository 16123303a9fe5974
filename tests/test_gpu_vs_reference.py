"""Parity with the reference's own GPU PDHG (src/pdhg/pdhg.cu:457-1156, the
cuSPARSE path) run on the same GB300.

tests/golden/ref_gpu_pdhg.json holds the reference's results, recorded on a
GB300 by tests/golden/make_ref_gpu_golden.py with the reference compiled from
its sources (oracle/Makefile `ref`): the seeded golden LPs and the small
random LP shape (m 2000, n 5000, seed 0) at 1e-8 relative KKT (C1 also at
1e-4), and the eight Netlib LPs of the reference's PDHG spike set at its
battery tolerance 1e-3 and at 1e-8.

Bars (FP64 and FP32 + refinement):
* wherever the reference certifies, this engine certifies at the same
  tolerance; at 1e-8 the objectives agree to 1e-6 relative
  (|a - b| / max(1, |b|)), at 1e-3 both lie within 2e-3 of the exact
  optimum (HiGHS, from the reference's own records);
* the FP64 engine runs the same algorithm, so its iteration count is of the
  reference's size (within 4x either way; rounding differences in the sums
  move restart checks, so the trajectories are not identical);
* the one case the reference does not certify, share2b (time-limit at 16 s
  and 30 s), is named below and checked against the exact optimum instead.

Where the reference library is built on this machine, a live run of it on a
few cases reproduces the recorded results (same iterations and objective):
the fixture is the reference's own deterministic output.
"""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
REF = json.load(open(os.path.join(GOLD, "ref_gpu_pdhg.json")))
sys.path.insert(0, GOLD)

# cases the reference's PDHG leaves uncertified on the GB300 (recorded status)
REF_UNCERTIFIED = {"netlib-share2b@0.001": "time-limit", "netlib-share2b@1e-08": "time-limit"}


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def load_case(name):
    import make_golden as MG
    import make_netlib_golden as MN
    from igaos_gb300 import generators as G
    from oracle import oracle as O
    if name.startswith("netlib-"):
        lp, exact, _ = MN.load(name[len("netlib-"):])
        return lp, exact
    if name == "c1-s0":
        c1 = json.load(open(os.path.join(GOLD, "c1_objectives.json")))["c1-s0"]
        return O.lp_from(G.config1(seed=0)), c1["simplex_objective"]
    e = json.load(open(os.path.join(GOLD, "lp_objectives.json")))[name]
    return O.lp_from(MG.make_lp(e["generator"], e["kwargs"])), e["simplex_objective"]


KEYS = sorted(k for k in REF if not k.startswith("_"))


def test_fixture_records_what_the_reference_certifies():
    for k in KEYS:
        want = REF_UNCERTIFIED.get(k, "near-optimal")
        assert REF[k]["status_name"] == want, (k, REF[k]["status_name"], REF[k]["message"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
@pytest.mark.parametrize("key", KEYS)
def test_engine_matches_reference_gpu_pdhg(native, key, precision):
    from igaos_gb300 import capi
    name, tol = key.split("@")
    tol = float(tol)
    ref = REF[key]
    lp, exact = load_case(name)
    r = capi.solve_lp(lp, tolerance=tol, time_limit=60.0, precision=precision)
    assert r["status_name"] == "near-optimal", (key, r["message"])
    if ref["status_name"] == "near-optimal":
        if tol <= 1e-8:
            assert rel(r["objective"], ref["objective"]) <= 1e-6, (r["objective"], ref["objective"])
        else:
            assert rel(r["objective"], exact) <= 2 * tol and rel(ref["objective"], exact) <= 2 * tol
        if precision == "fp64":
            assert ref["iterations"] / 4 <= r["iterations"] <= 4 * ref["iterations"], \
                (r["iterations"], ref["iterations"])
    else:
        assert key in REF_UNCERTIFIED
        assert rel(r["objective"], exact) <= max(1e-6, 2 * tol), (r["objective"], exact)


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["rand60x150-s0@1e-08", "netlib-afiro@1e-08",
                                 "netlib-grow22@1e-08", "mixed80x200-s2@1e-08"])
def test_live_reference_reproduces_fixture(orc, key):
    if not orc.ref_pdhg_available():
        pytest.skip("reference GPU PDHG not built here (oracle/_ref)")
    name, tol = key.split("@")
    lp, _ = load_case(name)
    got = orc.ref_pdhg_solve(lp, tolerance=float(tol), time_limit=60.0)
    want = REF[key]
    assert got["status_name"] == want["status_name"]
    assert got["iterations"] == want["iterations"]
    assert rel(got["objective"], want["objective"]) <= 1e-12
