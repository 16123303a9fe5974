"""Optimum of a mid-size LP of the large sparse shape (column degrees
Zipf(1.5) rescaled to the target nonzero count, |A_ij| log-uniform in
[1e-3, 1e3], box [0, 10], half equality / half <= rows): m = 5,000,
n = 12,500, ~125k nonzeros, seed 5. Solved by scipy's HiGHS interior-point
and dual-simplex methods (not reference code; the reference's simplex takes
minutes per 2,000-row LP and is not run at this size); both objectives are
stored with a checksum of the generated data. Writes
tests/golden/zipf_objectives.json.

Usage: python tests/golden/make_zipf_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from igaos_gb300 import generators as G  # noqa: E402
from make_golden import checksum  # noqa: E402

KWARGS = dict(seed=5, m=5000, n=12500, target_nnz=125000)


def main():
    import scipy.sparse as sp
    from scipy.optimize import linprog
    lp = G.config2(**KWARGS)
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    eq = np.isfinite(lp.rmin) & np.isfinite(lp.rmax) & (lp.rmin == lp.rmax)
    ub = ~eq & np.isfinite(lp.rmax)
    out = {"generator": "config2", "kwargs": KWARGS, "checksum": checksum(lp)}
    for meth in ("highs-ipm", "highs-ds"):
        r = linprog(lp.c, A_ub=A[ub], b_ub=lp.rmax[ub], A_eq=A[eq], b_eq=lp.rmin[eq],
                    bounds=list(zip(lp.cl, lp.cu)), method=meth)
        assert r.status == 0, r.message
        out[meth.replace("-", "_") + "_objective"] = float(r.fun)
        print(meth, r.fun)
    with open(os.path.join(HERE, "zipf_objectives.json"), "w") as f:
        json.dump({"zipf5000x12500-s5": out}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
