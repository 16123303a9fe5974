"""The drop-in surfaces on the GPU, end to end from an MPS file, and edge
cases of the LP shape.

* `igaos solve model.mps --engine pdhg` (CLI JSON record) and
  `igaos_gb300.solve(path, engine="pdhg")` (pybind) reach the reference
  simplex optimum of golden LPs written as MPS.
* LPs with empty rows and empty columns, a 1 x 1 LP, and LPs with every
  bound type solve to the optimum of an independent LP solver.
* An infeasible LP ends at its iteration cap with finite, honest metrics.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = json.load(open(os.path.join(HERE, "golden", "lp_objectives.json")))
INF = float("inf")


def write_mps(lp, path):
    """Free-format MPS of an LPData (rows E/L/G, ranged rows as E + RANGES)."""
    rows, rhs, ranges = [], [], []
    for i in range(lp.m):
        lo, hi = float(lp.rmin[i]), float(lp.rmax[i])
        if np.isfinite(lo) and np.isfinite(hi):
            rows.append(f" E  R{i}")
            rhs.append(f"    RHS  R{i}  {lo!r}")
            if hi != lo:
                ranges.append(f"    RNG  R{i}  {hi - lo!r}")
        elif np.isfinite(hi):
            rows.append(f" L  R{i}")
            rhs.append(f"    RHS  R{i}  {hi!r}")
        else:
            rows.append(f" G  R{i}")
            rhs.append(f"    RHS  R{i}  {lo!r}")
    cols = []
    for j in range(lp.n):
        cols.append(f"    C{j}  OBJ  {float(lp.c[j])!r}")
        for p in range(lp.cp[j], lp.cp[j + 1]):
            cols.append(f"    C{j}  R{lp.ci[p]}  {float(lp.acx[p])!r}")
    bounds = []
    for j in range(lp.n):
        lo, hi = float(lp.cl[j]), float(lp.cu[j])
        if lo == -INF and hi == INF:
            bounds.append(f" FR BND  C{j}")
        elif lo == hi:
            bounds.append(f" FX BND  C{j}  {lo!r}")
        else:
            if lo == -INF:
                bounds.append(f" MI BND  C{j}")
            elif lo != 0.0:
                bounds.append(f" LO BND  C{j}  {lo!r}")
            if hi != INF:
                bounds.append(f" UP BND  C{j}  {hi!r}")
    text = ["NAME T", "ROWS", " N  OBJ", *rows, "COLUMNS", *cols, "RHS", *rhs]
    if ranges:
        text += ["RANGES", *ranges]
    text += ["BOUNDS", *bounds, "ENDATA"]
    path.write_text("\n".join(text) + "\n")


def golden(name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import make_lp
    e = GOLD[name]
    return make_lp(e["generator"], e["kwargs"]), e["simplex_objective"]


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


@pytest.mark.parametrize("name", ["rand60x150-s0", "mixed80x200-s1"])
def test_cli_solve_from_mps(native, tmp_path, name):
    lp, ref = golden(name)
    p = tmp_path / "m.mps"
    write_mps(lp, p)
    cli = os.path.join(ROOT, "igaos_gb300", "igaos")
    out = subprocess.run([cli, "solve", str(p), "--engine", "pdhg", "--tol", "1e-8",
                          "--time-limit", "60"], capture_output=True, text=True, check=True).stdout
    rec = json.loads(out)
    assert rec["status"] == "near-optimal", rec["message"]
    assert rec["m"] == lp.m and rec["n"] == lp.n and rec["nnz"] == lp.nnz
    assert rel(rec["objective"], ref) <= 1e-6, (rec["objective"], ref)
    assert len(rec["x"]) == lp.n


def test_pybind_solve_from_mps(native, tmp_path):
    import igaos_gb300 as ig
    lp, ref = golden("mixed80x200-s0")
    p = tmp_path / "m.mps"
    write_mps(lp, p)
    s = ig.solve(str(p), time_limit=60.0, tolerance=1e-8, engine="pdhg")
    assert s.status == "near-optimal", s.message
    assert rel(s.objective, ref) <= 1e-6
    assert len(s.x) == lp.n and len(s.y) == lp.m


def linprog(lp):
    scipy_opt = pytest.importorskip("scipy.optimize")
    import scipy.sparse as sp
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    fh, fl = np.isfinite(lp.rmax), np.isfinite(lp.rmin)
    eq = fh & fl & (lp.rmin == lp.rmax)
    A_ub = sp.vstack([A[fh & ~eq], -A[fl & ~eq]])
    b_ub = np.concatenate([lp.rmax[fh & ~eq], -lp.rmin[fl & ~eq]])
    bounds = [(None if not np.isfinite(a) else a, None if not np.isfinite(b) else b)
              for a, b in zip(lp.cl, lp.cu)]
    return scipy_opt.linprog(lp.c, A_ub=A_ub, b_ub=b_ub, A_eq=A[eq], b_eq=lp.rmin[eq],
                             bounds=bounds, method="highs")


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
def test_empty_rows_and_columns(native, precision):
    """Rows with no entries (bounds containing 0) and columns with no entries
    (their optimum is the bound their cost points at)."""
    from igaos_gb300 import capi
    base = G.random_lp(40, 90, 150, 7)
    rows = np.repeat(np.arange(base.m), np.diff(base.ap))
    m, n = base.m + 3, base.n + 4
    rmin = np.concatenate([base.rmin, [-1.0, -INF, 0.0]])
    rmax = np.concatenate([base.rmax, [2.0, 5.0, INF]])
    c = np.concatenate([base.c, [1.0, -2.0, 0.0, -0.5]])
    cl = np.concatenate([base.cl, [0.0, -3.0, 1.0, -INF]])
    cu = np.concatenate([base.cu, [4.0, 3.0, 1.0, 8.0]])
    lp = G.from_triplets(m, n, rows, base.ai, base.ax, c, cl, cu, rmin, rmax)
    ref = linprog(lp)
    assert ref.status == 0
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=60.0, precision=precision)
    assert r["status_name"] == "near-optimal", r["message"]
    assert rel(r["objective"], ref.fun) <= 1e-6
    x = r["x"]
    assert x[base.n] == pytest.approx(0.0, abs=1e-9)      # cost +1 on [0, 4]
    assert x[base.n + 1] == pytest.approx(3.0, abs=1e-9)  # cost -2 on [-3, 3]
    assert x[base.n + 2] == pytest.approx(1.0, abs=1e-12)  # fixed
    assert x[base.n + 3] == pytest.approx(8.0, abs=1e-8)  # cost -0.5 on (-inf, 8]


def test_one_by_one(native):
    from igaos_gb300 import capi
    lp = G.from_triplets(1, 1, [0], [0], [2.0], [-1.0], [0.0], [10.0], [-INF], [6.0])
    r = capi.solve_lp(lp, tolerance=1e-8, time_limit=30.0)
    assert r["status_name"] == "near-optimal"
    assert r["objective"] == pytest.approx(-3.0, rel=1e-8)
    assert r["x"][0] == pytest.approx(3.0, rel=1e-8)


def test_infeasible_lp_stops_at_cap(native):
    """x1 + x2 <= 1 and x1 + x2 >= 3 on [0, 5]^2: no feasible point. The
    reference engine has no infeasibility certificate; the engine stops at
    the iteration cap and reports the residuals it reached."""
    from igaos_gb300 import capi
    lp = G.from_triplets(2, 2, [0, 0, 1, 1], [0, 1, 0, 1], [1.0, 1.0, 1.0, 1.0],
                         [1.0, 1.0], [0.0, 0.0], [5.0, 5.0], [-INF, 3.0], [1.0, INF])
    r = capi.solve_lp(lp, tolerance=1e-6, time_limit=1e9, max_iterations=2048)
    assert r["status_name"] in ("iteration-limit", "error"), r
    assert r["status_name"] != "near-optimal"
    if r["status_name"] == "iteration-limit":
        assert r["pinf"] > 1e-3 and np.isfinite(r["pinf"])
