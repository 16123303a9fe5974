"""Optima of LPs of the large sparse shape (column degrees Zipf(1.5)
rescaled to the target nonzero count, |A_ij| log-uniform in [1e-3, 1e3],
box [0, 10], half equality / half <= rows), seed 5, at two sizes an
independent solver finishes:

* m = 5,000, n = 12,500, ~128k nonzeros: scipy's HiGHS interior-point and
  dual-simplex methods (~13 s and ~24 s on one x86 core);
* m = 20,000, n = 50,000, ~522k nonzeros (the 20k x 50k, 500k-nonzero
  size of the large LP's scaled-down parity case): HiGHS interior point
  only (~21 minutes on one x86 core).

Neither is reference code; the reference's simplex takes minutes per
2,000-row LP and is not run at these sizes. Each objective is stored with a
checksum of the generated data. Writes (merges into)
tests/golden/zipf_objectives.json.

Usage: python tests/golden/make_zipf_golden.py [name ...]   (default: all)
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

CASES = {
    "zipf5000x12500-s5": (dict(seed=5, m=5000, n=12500, target_nnz=125000),
                          ("highs-ipm", "highs-ds")),
    "zipf20000x50000-s5": (dict(seed=5, m=20000, n=50000, target_nnz=500000),
                           ("highs-ipm",)),
}
OUT = os.path.join(HERE, "zipf_objectives.json")


def solve(name):
    import scipy.sparse as sp
    from scipy.optimize import linprog
    kwargs, methods = CASES[name]
    lp = G.config2(**kwargs)
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    eq = np.isfinite(lp.rmin) & np.isfinite(lp.rmax) & (lp.rmin == lp.rmax)
    ub = ~eq & np.isfinite(lp.rmax)
    out = {"generator": "config2", "kwargs": kwargs, "checksum": checksum(lp)}
    for meth in methods:
        t = time.time()
        r = linprog(lp.c, A_ub=A[ub], b_ub=lp.rmax[ub], A_eq=A[eq], b_eq=lp.rmin[eq],
                    bounds=list(zip(lp.cl, lp.cu)), method=meth)
        assert r.status == 0, r.message
        out[meth.replace("-", "_") + "_objective"] = float(r.fun)
        print(name, meth, r.fun, f"{time.time() - t:.1f} s", flush=True)
    return out


def main():
    names = sys.argv[1:] or list(CASES)
    gold = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for name in names:
        gold[name] = solve(name)
    with open(OUT, "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
