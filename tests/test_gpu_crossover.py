"""The crossover option on the GPU engine (igaos_pdhg_options.crossover, CLI
--crossover, igaos_gb300.solve(crossover=True)): the PDHG answer is finished
on the host at an optimal vertex, status "optimal".

* From answers at 1e-6 (FP64, FP32 + refinement) and a rough one at 1e-3 the
  vertex has HiGHS's objective and metrics at rounding level on the original
  LP; with pdhg_presolve the vertex is the original LP's.
* Above 2,048 rows the option is inert: the PDHG answer stands.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from igaos_gb300 import generators as G
from test_presolve_cpu import highs, metrics
from test_gpu_surfaces import write_mps

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("precision, tol, presolve", [
    ("fp64", 1e-6, 0), ("fp32-refine", 1e-6, 0), ("fp64", 1e-3, 0), ("fp64", 1e-6, 1),
])
@pytest.mark.parametrize("kind", ["mixed", "presolvable"])
def test_solve_ends_at_an_optimal_vertex(native, orc, precision, tol, presolve, kind):
    from igaos_gb300 import capi
    lp = G.mixed_bounds_lp(40, 90, 150, 3) if kind == "mixed" else G.presolvable_lp(60, 150, 250, 3)
    _, _, ref = highs(lp)
    r = capi.solve_lp(lp, tolerance=tol, time_limit=60.0, precision=precision, crossover=1,
                      pdhg_presolve=presolve)
    assert r["status_name"] == "optimal", r["message"]
    assert "crossover: optimal vertex" in r["message"]
    assert abs(r["objective"] - ref) <= 1e-9 * (1.0 + abs(ref)), (r["objective"], ref)
    mt = metrics(orc, lp, r["x"], r["y"])
    assert max(mt["pinf"], mt["prow"], mt["dinf"], mt["gap"]) <= 1e-9, mt
    assert max(r["pinf"], r["prow"], r["dinf"], r["rel_gap"]) <= 1e-9


def test_crossover_is_inert_above_its_size(native):
    from igaos_gb300 import capi
    lp = G.random_lp(2100, 5000, 12000, 0)
    r = capi.solve_lp(lp, tolerance=1e-4, time_limit=60.0, crossover=1)
    assert r["status_name"] == "near-optimal" and "crossover" not in r["message"], r


def test_cli_and_pybind_crossover(native, tmp_path):
    import igaos_gb300 as ig
    lp = G.mixed_bounds_lp(40, 90, 150, 4)
    _, _, ref = highs(lp)
    p = tmp_path / "x.mps"
    write_mps(lp, p)
    cli = os.path.join(ROOT, "igaos_gb300", "igaos")
    out = subprocess.run([cli, "solve", str(p), "--engine", "pdhg", "--tol", "1e-6",
                          "--time-limit", "60", "--crossover"], capture_output=True, text=True,
                         check=True).stdout
    rec = json.loads(out)
    assert rec["status"] == "optimal", rec["message"]
    assert abs(rec["objective"] - ref) <= 1e-9 * (1.0 + abs(ref))
    s = ig.solve(str(p), time_limit=60.0, tolerance=1e-6, engine="pdhg", crossover=True)
    assert s.status == "optimal" and len(s.x) == lp.n
    assert abs(s.objective - ref) <= 1e-9 * (1.0 + abs(ref))
