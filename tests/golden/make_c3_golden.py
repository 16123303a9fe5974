"""Optima of a spread of instances from the 4,096-LP small-batch set
(generators.config3(seed=0, count=4096): m log-uniform in [20, 2000],
n = 2.5 m, 1 % Bernoulli pattern, N(0,1) values, box [0, 5]): the
instances at 16 evenly spaced ranks of m, the 8 largest, and instance 1018
(m 1,747, the one that needs the most PDHG iterations). Solved by scipy's
HiGHS dual simplex (not reference code; the reference's simplex takes
minutes per 2,000-row LP). Each objective is stored with a checksum of the
generated data. Writes tests/golden/c3_objectives.json.

Usage: python tests/golden/make_c3_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from igaos_gb300 import generators as G  # noqa: E402
from make_golden import checksum  # noqa: E402

SEED, COUNT = 0, 4096


def picks(lps) -> list:
    ms = np.array([lp.m for lp in lps])
    order = np.argsort(ms, kind="stable")
    ranks = np.rint(np.linspace(0, COUNT - 1, 16)).astype(int)
    chosen = set(int(order[r]) for r in ranks) | set(int(i) for i in order[-8:]) | {1018}
    return sorted(chosen)


def main():
    import scipy.sparse as sp
    from scipy.optimize import linprog
    lps = G.config3(seed=SEED, count=COUNT)
    out = {"generator": "config3", "kwargs": {"seed": SEED, "count": COUNT}, "instances": {}}
    for i in picks(lps):
        lp = lps[i]
        A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
        eq = np.isfinite(lp.rmin) & np.isfinite(lp.rmax) & (lp.rmin == lp.rmax)
        ub = ~eq & np.isfinite(lp.rmax)
        lb = ~eq & np.isfinite(lp.rmin) & ~np.isfinite(lp.rmax)
        A_ub = sp.vstack([A[ub], -A[lb]]).tocsr()
        b_ub = np.concatenate([lp.rmax[ub], -lp.rmin[lb]])
        both = ~eq & np.isfinite(lp.rmin) & np.isfinite(lp.rmax)
        if both.any():
            A_ub = sp.vstack([A_ub, -A[both]]).tocsr()
            b_ub = np.concatenate([b_ub, -lp.rmin[both]])
        t = time.time()
        r = linprog(lp.c, A_ub=A_ub, b_ub=b_ub, A_eq=A[eq], b_eq=lp.rmin[eq],
                    bounds=list(zip(lp.cl, lp.cu)), method="highs-ds")
        assert r.status == 0, (i, r.message)
        out["instances"][str(i)] = {"checksum": checksum(lp), "highs_ds_objective": float(r.fun)}
        print(i, lp.m, lp.n, r.fun, f"{time.time() - t:.1f} s", flush=True)
    with open(os.path.join(HERE, "c3_objectives.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
