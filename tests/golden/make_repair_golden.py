"""Golden cases of the reference dual_repair (src/pdhg/pdhg.cu:257-448).

Runs where the reference tree is present: builds the reference helpers
(oracle/Makefile `ref`) and records the reference's own dual_repair output
on LPs with free and one-sided columns (generators.free_cost_lp) at
candidates taken from short runs of the oracle PDHG, for both col_tol tiers
the reference uses (1e-6, 1e-1).

  dual_repair_cases.npz   per case k: lp_k (generator arguments), x_k, Ax_k,
                          y_it_k, tol_k, ok_k, y_k

Usage: python tests/golden/make_repair_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from igaos_gb300 import generators as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

# (m, n, extra_nnz, seed, oracle iterations before the candidate is taken)
CASES = [(30, 70, 120, 0, 3000), (30, 70, 120, 1, 3000), (40, 100, 200, 2, 640),
         (40, 100, 200, 3, 6000), (60, 150, 300, 4, 4000), (25, 60, 80, 5, 128)]


def candidate(lp, iters):
    r = O.pdhg_solve(lp, tolerance=1e-12, time_limit=1e9, max_iterations=iters)
    x, y = r["x"], r["y"]
    Ax = np.zeros(lp.m)
    for i in range(lp.m):  # sequential per row, storage order
        s = 0.0
        for p in range(lp.ap[i], lp.ap[i + 1]):
            s += lp.ax[p] * x[lp.ai[p]]
        Ax[i] = s
    return x, Ax, y


def main():
    O.build(ref=True)
    out = {}
    k = 0
    for (m, n, e, seed, iters) in CASES:
        lp = O.lp_from(G.free_cost_lp(m, n, e, seed))
        x, Ax, y_it = candidate(lp, iters)
        for tol in (1e-6, 1e-1):
            ok, y = O.ref_dual_repair(lp, x, Ax, y_it, tol)
            out.update({f"lp_{k}": np.array([m, n, e, seed]), f"x_{k}": x, f"Ax_{k}": Ax,
                        f"y_it_{k}": y_it, f"tol_{k}": np.array(tol), f"ok_{k}": np.array(ok),
                        f"y_{k}": y})
            print(k, (m, n, e, seed, iters), tol, "certified" if ok else "not certified")
            k += 1
    out["count"] = np.array(k)
    np.savez_compressed(os.path.join(HERE, "dual_repair_cases.npz"), **out)


if __name__ == "__main__":
    main()
