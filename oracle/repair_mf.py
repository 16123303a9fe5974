"""Matrix-free dual repair, restated in numpy (test infrastructure).

The algorithm of the engine's device repair (igaos_gb300/csrc/repair_dev.cuh,
engine.cu: repair_dev) in original units, for CPU tests: from two anchors
(the candidate dual, then 0), rounds of
  1. the regularised least-squares step onto {A_J^T y = -c_J} (J: columns
     strictly inside their bounds by col_tol (1 + |bound|)) by CGLS, moving
     only two-sided rows and one-sided rows whose dual is off 0;
  2. all violated sign half-spaces of the columns with an infinite bound at
     once, each row averaging the steps of the violated columns it meets;
  3. the row cone;
stopping at the first dual whose pair passes pinf, prow and a finite gap
<= tol under the restatement of the reference evaluate() (oracle.evaluate).
The reference's own repair (src/pdhg/pdhg.cu:288-448) projects onto the same
sets with a dense Cholesky solve and one column at a time; the device form
exists for LPs whose m x m normal matrix does not fit.
"""
import numpy as np
import scipy.sparse as sp

from . import oracle as O

INF = np.inf


def _cone(lp):
    fl, fh = np.isfinite(lp.rmin), np.isfinite(lp.rmax)
    ylo = np.where(fl & fh, -INF, np.where(fh, 0.0, np.where(fl, -INF, 0.0)))
    yhi = np.where(fl & fh, INF, np.where(fh, INF, np.where(fl, 0.0, 0.0)))
    return ylo, yhi


def _cgls(A, J, R, b, ridge, iters, rtol):
    """min ||(A^T z)_J - b||^2 + ridge ||z||^2 over z supported on the rows
    where R is 1."""
    z = np.zeros(A.shape[0])
    r = b.copy()

    def mt(rj):
        full = np.zeros(A.shape[1])
        full[J] = rj
        return (A @ full) * R

    s = mt(r)
    p = s.copy()
    g = g0 = s @ s
    for _ in range(iters):
        if g <= rtol * rtol * g0 or g == 0.0:
            break
        q = (A.T @ p)[J]
        dl = q @ q + ridge * (p @ p)
        if not (dl > 0.0 and np.isfinite(dl)):
            break
        a = g / dl
        z += a * p
        r -= a * q
        s = mt(r) - ridge * z
        gn = s @ s
        p = s + (gn / g) * p
        g = gn
    return z


def repair(lp, x, y_it, col_tol, tol, rounds=150, stall=40, cg_iters=40, cg_rtol=1e-10):
    """(certified, y, metrics) for the candidate x and dual estimate y_it."""
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    Ax = A @ x
    ylo, yhi = _cone(lp)
    two = np.isfinite(lp.rmin) & np.isfinite(lp.rmax)
    one = np.isfinite(lp.rmin) ^ np.isfinite(lp.rmax)
    up_inf, lo_inf = ~np.isfinite(lp.cu), ~np.isfinite(lp.cl)
    sign = np.where(up_inf & lo_inf, 2, np.where(up_inf, 0, np.where(lo_inf, 1, 3)))
    norm2 = np.asarray(A.multiply(A).sum(axis=0)).ravel()
    band = lambda b: col_tol * (1 + np.where(np.isfinite(b), np.abs(b), 0.0))
    J = np.nonzero((x - lp.cl > band(lp.cl)) & (lp.cu - x > band(lp.cu)))[0]
    trace = norm2[J].sum()
    ridge = 1e-10 * trace / lp.m if trace > 0 else 1e-14
    best = (INF, None, None)
    for anchor in (0, 1):
        y = np.clip(y_it if anchor == 0 else np.zeros(lp.m), ylo, yhi)
        finite_seen = False
        for it in range(rounds):
            if it == stall and not finite_seen:
                break
            if len(J):
                d = lp.c + A.T @ y
                R = (two | (one & (y != 0))).astype(float)
                y = y + _cgls(A, J, R, -d[J], ridge, cg_iters, cg_rtol)
            d = lp.c + A.T @ y
            v = np.zeros(lp.n)
            v = np.where((sign == 0) & (d < 0), -d, v)
            v = np.where((sign == 1) & (d > 0), -d, v)
            v = np.where((sign == 2) & (d != 0), -d, v)
            step = np.where((v != 0) & (norm2 > 0), v / np.where(norm2 > 0, norm2, 1.0), 0.0)
            hit = (step != 0).astype(float)
            cnt = abs(A).sign() @ hit
            y = np.clip(y + (A @ step) / np.maximum(cnt, 1.0), ylo, yhi)
            mt = O.evaluate_arrays(lp.rmin, lp.rmax, lp.cl, lp.cu, lp.c, x, y, Ax, lp.c + A.T @ y)
            finite_seen = finite_seen or np.isfinite(mt["gap"])
            if np.isfinite(mt["gap"]) and mt["gap"] < best[0]:
                best = (mt["gap"], y.copy(), mt)
                if mt["pinf"] <= tol and mt["prow"] <= tol and mt["gap"] <= tol:
                    return True, y, mt
    return False, best[1], best[2]
