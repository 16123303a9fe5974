"""Generates the committed golden fixtures of the parity tests.

Runs where the reference tree is present: it builds the reference helpers
(oracle/Makefile `ref`: the reference's own evaluate(), counting_sort(),
parse_mps() and CPU simplex, compiled from the reference sources) and records
their outputs on seeded inputs:

  evaluate_cases.npz     reference evaluate() (src/pdhg/pdhg.cu:173-254)
  counting_sort.npz      reference counting_sort() (src/io/model.hpp:39-67)
  mps_cases.npz          reference parse_mps() on hand-written MPS texts
  lp_objectives.json     reference simplex optimum (+ scipy-HiGHS) of seeded
                         synthetic LPs, with a data checksum per LP
  c1_objectives.json     the same for the full-size small-LP shape
                         (m=2000, n=5000; minutes per seed) -- `--c1`

Usage: python tests/golden/make_golden.py [--c1]
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from igaos_gb300 import generators as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

INF = np.inf


def checksum(lp) -> dict:
    return dict(m=int(lp.m), n=int(lp.n), nnz=int(lp.ap[lp.m]),
                ax_sum=float(np.sum(lp.ax)), c_sum=float(np.sum(lp.c)),
                rmax_fin=float(np.sum(lp.rmax[np.isfinite(lp.rmax)])))


def same_checksum(lp, want: dict) -> bool:
    """Sizes exactly, sums to 1e-12 relative: numpy's summation order (and
    so the last bits of a float sum) differs between x86 and Arm builds."""
    got = checksum(lp)
    if any(got[k] != want[k] for k in ("m", "n", "nnz")):
        return False
    return all(abs(got[k] - want[k]) <= 1e-12 * max(1.0, abs(want[k]))
               for k in ("ax_sum", "c_sum", "rmax_fin"))


# ------------------------------------------------------------ LP catalogue
# name -> (generator name, kwargs); every generator is seeded and pure.
CATALOGUE = {}
for s in range(4):
    CATALOGUE[f"rand60x150-s{s}"] = ("random_lp", dict(m=60, n=150, extra_nnz=300, seed=s))
for s in range(2):
    CATALOGUE[f"rand200x500-s{s}"] = ("random_lp", dict(m=200, n=500, extra_nnz=1500, seed=s))
for s in range(3):
    CATALOGUE[f"mixed80x200-s{s}"] = ("mixed_bounds_lp", dict(m=80, n=200, extra_nnz=400, seed=s))
for s, m in enumerate((20, 50, 120, 300)):
    CATALOGUE[f"bern{m}-s{s}"] = ("bernoulli", dict(m=m, seed=s))
CATALOGUE["grid6x6-k2"] = ("config5", dict(seed=1, side=6, commodities=2))
CATALOGUE["zipf400x1000"] = ("config2", dict(seed=3, m=400, n=1000, target_nnz=6000))


def make_lp(gen: str, kw: dict):
    kw = dict(kw)
    if gen == "random_lp":
        return G.random_lp(kw["m"], kw["n"], kw["extra_nnz"], kw["seed"])
    if gen == "mixed_bounds_lp":
        return G.mixed_bounds_lp(kw["m"], kw["n"], kw["extra_nnz"], kw["seed"])
    if gen == "bernoulli":
        rng = np.random.default_rng(kw["seed"])
        m = kw["m"]
        return G.bernoulli_lp(rng, m, int(round(2.5 * m)), 0.01 if m >= 100 else 0.05, 5.0)
    if gen == "config5":
        return G.config5(**kw)
    if gen == "config2":
        return G.config2(**kw)
    if gen == "config1":
        return G.config1(**kw)
    raise KeyError(gen)


def highs(lp):
    import scipy.sparse as sp
    from scipy.optimize import linprog
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    eq = lp.rmin == lp.rmax
    ub = ~eq & np.isfinite(lp.rmax)
    lb = ~eq & np.isfinite(lp.rmin)
    Aub = sp.vstack([A[ub], -A[lb]])
    bub = np.concatenate([lp.rmax[ub], -lp.rmin[lb]])
    r = linprog(lp.c, A_ub=Aub, b_ub=bub, A_eq=A[eq], b_eq=lp.rmin[eq],
                bounds=list(zip(np.where(np.isfinite(lp.cl), lp.cl, None),
                                np.where(np.isfinite(lp.cu), lp.cu, None))),
                method="highs")
    return float(r.fun) + float(lp.obj_const) if r.status == 0 else None


def solve_entry(item):
    name, (gen, kw) = item
    lp = make_lp(gen, kw)
    s = O.ref_simplex_solve(O.lp_from(lp), time_limit=3600.0)
    return name, dict(generator=gen, kwargs=kw, checksum=checksum(lp),
                      simplex_status=s["status"], simplex_objective=s["objective"],
                      highs_objective=highs(lp))


# ------------------------------------------------------------ evaluate cases
def evaluate_cases(rng, count=10):
    cases = {}
    for k in range(count):
        m, n = int(rng.integers(5, 40)), int(rng.integers(5, 50))
        rmin = rng.standard_normal(m)
        rmax = rmin + rng.uniform(0, 1, m)
        cl = rng.standard_normal(n)
        cu = cl + rng.uniform(0, 2, n)
        if k % 2:  # some infinite bounds
            rmin[rng.random(m) < .3] = -INF
            rmax[rng.random(m) < .3] = INF
            cl[rng.random(n) < .2] = -INF
            cu[rng.random(n) < .2] = INF
        c = rng.standard_normal(n)
        x = np.clip(rng.standard_normal(n), cl, cu)
        at_lo = (rng.random(n) < .3) & np.isfinite(cl)
        x[at_lo] = cl[at_lo]
        y = rng.standard_normal(m) * (rng.random(m) < .6)
        Ax = rng.standard_normal(m)
        d = rng.standard_normal(n) * (rng.random(n) < .5)
        if k % 3 == 0:  # signs matching finite bounds: a finite dual bound
            y = np.where(y > 0, np.where(np.isfinite(rmax), y, 0.0),
                         np.where(np.isfinite(rmin), y, 0.0))
            d = np.where(d >= 0, np.where(np.isfinite(cl), d, 0.0),
                         np.where(np.isfinite(cu), d, 0.0))
        ref = O.ref_evaluate(rmin, rmax, cl, cu, c, x, y, Ax, d)
        for key, arr in dict(rmin=rmin, rmax=rmax, cl=cl, cu=cu, c=c, x=x, y=y, Ax=Ax, d=d).items():
            cases[f"{k}_{key}"] = arr
        cases[f"{k}_out"] = np.array([ref[q] for q in ("pinf", "dinf", "gap", "op", "od", "prow")])
    cases["count"] = np.array(count)
    return cases


def counting_sort_cases(rng, count=4):
    out = {}
    for k in range(count):
        rows, cols = int(rng.integers(1, 30)), int(rng.integers(1, 30))
        nt = int(rng.integers(0, 120))
        ti = rng.integers(0, rows, nt)
        tj = rng.integers(0, cols, nt)
        tv = rng.standard_normal(nt)
        ap, ai, ax, cp, ci, acx = O.ref_counting_sort(ti, tj, tv, rows, cols)
        for key, arr in dict(ti=ti, tj=tj, tv=tv, ap=ap, ai=ai, ax=ax, cp=cp, ci=ci,
                             acx=acx, shape=np.array([rows, cols])).items():
            out[f"{k}_{key}"] = arr
    out["count"] = np.array(count)
    return out


# Hand-written MPS texts covering every section and bound type the reader
# handles (negative UP, MI, PL, FR, FX, BV/LI/UI, RANGES on E/L/G rows with
# both signs, objective constant, integer markers, QUADOBJ, free N rows).
MPS_TEXTS = {
    "bounds": """NAME BOUNDS
ROWS
 N cost
 L lim1
 G lim2
 E eq1
 N spare
COLUMNS
    x1 cost 1.5 lim1 2.0
    x1 eq1 1.0 spare 9.0
    x2 cost -2.0 lim2 1.0
    x3 cost 0.5 lim1 -1.0 eq1 3.0
    x4 lim2 4.0
    x5 cost 1.0 eq1 -1.0
    x6 cost 2.0 lim1 1.0
RHS
    rhs cost 7.25 lim1 10.0
    rhs lim2 -3.0 eq1 4.0
BOUNDS
 UP bnd x1 -2.0
 MI bnd x2
 FR bnd x3
 FX bnd x4 3.5
 LO bnd x5 -1.0
 PL bnd x5
 UP bnd x6 8.0
ENDATA
""",
    "ranges": """NAME RANGES
ROWS
 N obj
 E e1
 E e2
 L l1
 G g1
COLUMNS
    a obj 1.0 e1 1.0
    a l1 1.0 g1 1.0
    b obj 2.0 e2 1.0
    b l1 1.0 g1 -2.0
RHS
    r e1 1.0 e2 2.0
    r l1 5.0 g1 -1.0
RANGES
    rg e1 2.0 e2 -3.0
    rg l1 4.0 g1 -6.0
ENDATA
""",
    "integer": """NAME INTS
ROWS
 N obj
 L c1
COLUMNS
    MARKER 'MARKER' 'INTORG'
    y obj -1.0 c1 2.0
    MARKER 'MARKER' 'INTEND'
    z obj 1.0 c1 1.0
RHS
    r c1 5.0
BOUNDS
 BV b y
 UI b z 9.0
ENDATA
""",
}


def mps_cases():
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, text in MPS_TEXTS.items():
            p = os.path.join(td, name + ".mps")
            with open(p, "w") as f:
                f.write(text)
            lp = O.ref_parse_mps(p)
            out[f"{name}_text"] = np.array(text)
            for k in ("ap", "ai", "ax", "cp", "ci", "acx", "c", "cl", "cu", "rmin", "rmax"):
                out[f"{name}_{k}"] = getattr(lp, k)
            out[f"{name}_obj_const"] = np.array(lp.obj_const)
    return out


def main():
    O.build(ref=True)
    assert O.ref_available() and O.ref_simplex_available(), "reference helpers not built"
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "evaluate_cases.npz"), **evaluate_cases(rng))
    np.savez_compressed(os.path.join(HERE, "counting_sort.npz"), **counting_sort_cases(rng))
    np.savez_compressed(os.path.join(HERE, "mps_cases.npz"), **mps_cases())
    with ProcessPoolExecutor(max_workers=6) as ex:
        res = dict(ex.map(solve_entry, CATALOGUE.items()))
    with open(os.path.join(HERE, "lp_objectives.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print("lp_objectives:", {k: (v["simplex_status"], v["simplex_objective"]) for k, v in res.items()})
    if "--c1" in sys.argv:
        items = {f"c1-s{s}": ("config1", dict(seed=s)) for s in range(2)}
        with ProcessPoolExecutor(max_workers=2) as ex:
            res1 = dict(ex.map(solve_entry, items.items()))
        with open(os.path.join(HERE, "c1_objectives.json"), "w") as f:
            json.dump(res1, f, indent=1, sort_keys=True)
        print("c1:", res1)


if __name__ == "__main__":
    main()
