"""Optima of the multicommodity-flow LP (generators.config5: a side x side
4-neighbour grid, 8 commodities, shared arc capacities), seed 0, from
scipy's HiGHS interior-point method (not reference code):

* side 300: the full 1,078,800 x 2,870,400 LP (8.6M nonzeros);
* side 100: 119,600 x 316,800 (950k nonzeros), the same construction at a
  ninth of the size.

Each objective is stored with a checksum of the generated data and the
solve time. Writes (merges into) tests/golden/mcf_objectives.json.

Usage: python tests/golden/make_mcf_golden.py [name ...]   (default: all)
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
    "mcf100x8-s0": dict(seed=0, side=100, commodities=8),
    "mcf300x8-s0": dict(seed=0, side=300, commodities=8),
}
OUT = os.path.join(HERE, "mcf_objectives.json")


def solve(name):
    import scipy.sparse as sp
    from scipy.optimize import linprog
    kwargs = CASES[name]
    lp = G.config5(**kwargs)
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    eq = np.isfinite(lp.rmin) & np.isfinite(lp.rmax) & (lp.rmin == lp.rmax)
    ub = ~eq & np.isfinite(lp.rmax)
    assert not (~eq & np.isfinite(lp.rmin)).any(), "only = and <= rows expected"
    t = time.time()
    r = linprog(lp.c, A_ub=A[ub], b_ub=lp.rmax[ub], A_eq=A[eq], b_eq=lp.rmin[eq],
                bounds=np.stack([lp.cl, lp.cu], axis=1), method="highs-ipm")
    assert r.status == 0, r.message
    s = time.time() - t
    print(name, lp.m, lp.n, r.fun, f"{s:.1f} s", flush=True)
    return {"generator": "config5", "kwargs": kwargs, "checksum": checksum(lp),
            "highs_ipm_objective": float(r.fun), "highs_ipm_s": round(s, 1)}


def main():
    names = sys.argv[1:] or list(CASES)
    for name in names:
        out = solve(name)
        gold = json.load(open(OUT)) if os.path.exists(OUT) else {}
        gold[name] = out
        with open(OUT, "w") as f:
            json.dump(gold, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
