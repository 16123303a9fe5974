"""The engine's presolve on host arrays (igaos_pdhg_presolve / _postsolve; no
GPU needed).

The bar is the one the solve needs: an optimal pair of the reduced LP maps
back to an optimal pair of the original, duals included. The optimal pair of
the reduced LP comes from HiGHS (scipy), and the postsolved pair is checked
with the oracle's restatement of the reference evaluate() on the ORIGINAL LP
(primal and row infeasibility, reduced-cost complementarity and the duality
gap), and its objective against HiGHS on the original LP.
"""
import os

import numpy as np
import pytest

from conftest import reference_dir
from igaos_gb300 import generators as G

INF = float("inf")


def highs(lp):
    """(x, y, objective) of an optimal pair by HiGHS; y in the engine's sign
    convention (reduced cost d = c + A^T y: y >= 0 pushes a row down to rmax,
    y <= 0 up to rmin)."""
    opt = pytest.importorskip("scipy.optimize")
    import scipy.sparse as sp
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    hi, lo = np.isfinite(lp.rmax), np.isfinite(lp.rmin)
    eq = hi & lo & (lp.rmin == lp.rmax)
    up, dn = hi & ~eq, lo & ~eq
    bounds = [(l if np.isfinite(l) else None, u if np.isfinite(u) else None)
              for l, u in zip(lp.cl, lp.cu)]
    kw = {}
    if up.any() or dn.any():
        kw.update(A_ub=sp.vstack([A[up], -A[dn]]), b_ub=np.concatenate([lp.rmax[up], -lp.rmin[dn]]))
    if eq.any():
        kw.update(A_eq=A[eq], b_eq=lp.rmin[eq])
    r = opt.linprog(lp.c, bounds=bounds, method="highs",
                    options=dict(primal_feasibility_tolerance=1e-10,
                                 dual_feasibility_tolerance=1e-10), **kw)
    assert r.status == 0, r.message
    y = np.zeros(lp.m)
    if up.any() or dn.any():
        mu = r.ineqlin.marginals
        y[np.nonzero(up)[0]] -= mu[:up.sum()]
        y[np.nonzero(dn)[0]] += mu[up.sum():]
    if eq.any():
        y[np.nonzero(eq)[0]] -= r.eqlin.marginals
    return r.x, y, r.fun


def metrics(orc, lp, x, y):
    import scipy.sparse as sp
    A = sp.csr_matrix((lp.ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    return orc.evaluate(lp, x, y, A @ x, lp.c + A.T @ y)


def assert_optimal(mt, tol):
    assert max(mt["pinf"], mt["prow"], mt["dinf"]) <= tol, mt
    assert np.isfinite(mt["gap"]) and mt["gap"] <= tol, mt


def tiny(rows, cols, vals, c, cl, cu, rmin, rmax):
    return G.from_triplets(len(rmin), len(c), rows, cols, vals, c, cl, cu, rmin, rmax)


def test_highs_pair_is_optimal_under_evaluate(native, orc):
    """Pins the checker: the HiGHS pair, converted to the engine's sign
    convention, is optimal for the oracle's evaluate."""
    for lp in (G.presolvable_lp(60, 150, 250, 0), G.mixed_bounds_lp(40, 90, 150, 1)):
        x, y, _ = highs(lp)
        assert_optimal(metrics(orc, lp, x, y), 1e-9)


@pytest.mark.parametrize("seed", range(8))
def test_postsolve_of_an_optimal_reduced_pair_is_optimal(native, orc, seed):
    from igaos_gb300 import capi
    lp = G.presolvable_lp(60, 150, 250, seed)
    P = capi.Presolved(lp)
    assert P.outcome == "reduced"
    assert P.lp.m < lp.m and P.lp.n < lp.n
    xr, yr, fr = highs(P.lp)
    x, y = P.postsolve(xr, yr)
    assert_optimal(metrics(orc, lp, x, y), 1e-9)
    _, _, f = highs(lp)
    assert abs((fr + P.lp.obj_const) - f) <= 1e-8 * (1.0 + abs(f))
    assert abs(lp.c @ x - f) <= 1e-8 * (1.0 + abs(f))


def test_every_reduction_is_made(native):
    from igaos_gb300 import capi
    tot = dict.fromkeys(capi.PRESOLVE_COUNTS, 0)
    for seed in range(4):
        for k, v in capi.Presolved(G.presolvable_lp(60, 150, 250, seed)).counts.items():
            tot[k] += v
    assert all(v > 0 for v in tot.values()), tot


def test_implied_bound_moves_into_the_singleton_row_dual(native, orc):
    """min x s.t. 2x >= 4, x free: the row becomes x >= 2, the column is then
    empty and fixed at 2, and the whole LP is gone. Postsolve moves the
    reduced cost 1 into the row: y = -1/2 (d = 1 + 2 y = 0)."""
    from igaos_gb300 import capi
    lp = tiny([0], [0], [2.0], [1.0], [-INF], [INF], [4.0], [INF])
    P = capi.Presolved(lp)
    assert (P.lp.m, P.lp.n) == (0, 0)
    assert P.lp.obj_const == 2.0
    x, y = P.postsolve(np.zeros(0), np.zeros(0))
    assert np.array_equal(x, [2.0]) and np.array_equal(y, [-0.5])
    assert_optimal(metrics(orc, lp, x, y), 0.0)


def test_singleton_rows_on_both_sides(native, orc):
    """x in [0, 10] with rows x >= 3 (a = 1) and -x >= -5 (x <= 5): the
    implied side that binds carries the dual, for either cost sign."""
    from igaos_gb300 import capi
    for cost, xs, ys in ((1.0, 3.0, [-1.0, 0.0]), (-1.0, 5.0, [0.0, -1.0])):
        lp = tiny([0, 1], [0, 0], [1.0, -1.0], [cost], [0.0], [10.0], [3.0, -5.0], [INF, INF])
        P = capi.Presolved(lp)
        assert P.counts["singleton_rows"] == 2 and (P.lp.m, P.lp.n) == (0, 0)
        x, y = P.postsolve(np.zeros(0), np.zeros(0))
        assert np.array_equal(x, [xs]) and np.array_equal(y, ys), (x, y)
        assert_optimal(metrics(orc, lp, x, y), 0.0)


def test_free_singleton_substitution(native, orc):
    """min x1 + 2 x2 + 3 x3 s.t. x1 + x2 + x3 = 4, x1, x2 in [0, 10], x3
    free: x3 takes up the row (y = -3), x1 and x2 then cost -2 and -1 and go
    to 10, x3 = -16; objective -18."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 0], [0, 1, 2], [1.0, 1.0, 1.0], [1.0, 2.0, 3.0], [0.0, 0.0, -INF],
              [10.0, 10.0, INF], [4.0], [4.0])
    P = capi.Presolved(lp)
    assert P.counts["free_singletons"] == 1
    x, y = P.postsolve(np.zeros(P.lp.n), np.zeros(P.lp.m))
    assert np.allclose(x, [10.0, 10.0, -16.0]) and np.allclose(y, [-3.0])
    assert_optimal(metrics(orc, lp, x, y), 1e-12)
    assert lp.c @ x == -18.0


@pytest.mark.parametrize("case, outcome", [
    ("empty row excludes 0", "infeasible"),
    ("singleton rows cross", "infeasible"),
    ("cost runs to an infinite bound", "unbounded"),
    ("free singleton against an open row", "unbounded"),
])
def test_outcomes(native, case, outcome):
    from igaos_gb300 import capi
    lps = {
        "empty row excludes 0": tiny([0], [0], [1.0], [1.0], [0.0], [1.0], [0.0, 1.0], [1.0, 2.0]),
        "singleton rows cross": tiny([0, 1], [0, 0], [1.0, 1.0], [1.0], [0.0], [10.0],
                                     [-INF, 3.0], [1.0, INF]),
        "cost runs to an infinite bound": tiny([0], [0], [1.0], [1.0, -1.0], [0.0, 0.0],
                                               [1.0, INF], [0.0], [1.0]),
        "free singleton against an open row": tiny([0, 0], [0, 1], [1.0, 1.0], [0.0, 1.0],
                                                   [0.0, -INF], [1.0, INF], [-INF], [1.0]),
    }
    P = capi.Presolved(lps[case])
    assert P.outcome == outcome and P.lp is None


def test_invalid_input_is_refused(native):
    from igaos_gb300 import capi
    with pytest.raises(capi.EngineError, match="lower bound above upper"):
        capi.Presolved(tiny([0], [0], [1.0], [1.0], [2.0], [1.0], [0.0], [1.0]))


def test_no_reduction_leaves_the_lp_unchanged(native):
    """A dense LP with boxed columns and two-sided rows that bind: nothing to
    reduce, and the reduced LP is the input, array for array."""
    from igaos_gb300 import capi
    rng = np.random.default_rng(5)
    m, n = 6, 9
    r, c_ = np.nonzero(np.ones((m, n)))
    lp = tiny(r, c_, rng.uniform(0.5, 1.5, m * n), rng.standard_normal(n), np.zeros(n),
              np.full(n, 10.0), np.full(m, 1.0), np.full(m, 3.0))
    P = capi.Presolved(lp)
    assert sum(P.counts.values()) == 0
    for k in ("ap", "ai", "ax", "c", "cl", "cu", "rmin", "rmax"):
        assert np.array_equal(getattr(P.lp, k), getattr(lp, k)), k
    x, y = P.postsolve(np.arange(n, dtype=float), np.arange(m, dtype=float))
    assert np.array_equal(x, np.arange(n)) and np.array_equal(y, np.arange(m))


NETLIB = ["afiro", "kb2", "sc50a", "adlittle", "bandm", "grow22", "boeing1", "degen2",
          "etamacro", "forplan", "agg", "brandy", "e226", "scfxm1", "capri", "stocfor1",
          "scagr25", "sc205", "share2b", "israel"]


@pytest.mark.skipif(reference_dir() is None, reason="reference tree not present")
@pytest.mark.parametrize("name", NETLIB)
def test_netlib_postsolve(native, orc, name):
    """Netlib LPs read by the engine's MPS reader: the postsolved HiGHS pair
    of the reduced LP is optimal for the original."""
    from igaos_gb300 import build, capi
    path = os.path.join(reference_dir(), "demo", "models", "netlib_full", name + ".mps")
    if not os.path.exists(path):
        pytest.skip("netlib file missing")
    build.build()
    from igaos_gb300 import _core
    M = _core.read_mps(path)
    a = lambda v, t=float: np.asarray(v, t)
    lp = G.LPData(M.m, M.n, a(M.ap, np.int32), a(M.ai, np.int32), a(M.ax), a(M.cp, np.int32),
                  a(M.ci, np.int32), a(M.acx), a(M.c), a(M.cl), a(M.cu), a(M.rmin), a(M.rmax),
                  float(M.obj_const))
    P = capi.Presolved(lp)
    assert P.outcome == "reduced"
    xr, yr, _ = highs(P.lp)
    x, y = P.postsolve(xr, yr)
    assert_optimal(metrics(orc, lp, x, y), 1e-8)
    _, _, f = highs(lp)
    assert abs(lp.c @ x - f) <= 1e-8 * (1.0 + abs(f))


def test_dual_ray_of_the_reduced_lp_maps_to_a_certificate(native):
    """x1 + x2 >= 3 and x1 - x2 >= 2 (together x1 >= 2.5) with x1 <= 2 as a
    singleton row, x free: no single row shows the infeasibility, so the
    reduced LP keeps both rows, with x1 <= 2 as a column bound, and has the
    dual ray y = (-1, -1). Scattered with zeros it is no certificate of the
    original (x1 is free there); mapped like a postsolve with zero costs,
    the reduced cost -2 of x1 moves into the singleton row: y = (-1, -1, 2)."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 1, 1, 2], [0, 1, 0, 1, 0], [1.0, 1.0, 1.0, -1.0, 1.0], [1.0, 1.0],
              [-INF, -INF], [INF, INF], [3.0, 2.0, -INF], [INF, INF, 2.0])
    P = capi.Presolved(lp)
    assert P.outcome == "reduced" and (P.lp.m, P.lp.n) == (2, 2)
    assert P.counts["singleton_rows"] == 1 and P.lp.cu[0] == 2.0
    yr = np.array([-1.0, -1.0])
    assert capi.ray_certificate(P.lp, np.zeros(2), yr)[0] == 1
    assert capi.ray_certificate(lp, np.zeros(2), np.array([-1.0, -1.0, 0.0]))[0] == 0
    x, y = P.postsolve_ray(np.zeros(2), yr)
    assert np.array_equal(y, [-1.0, -1.0, 2.0]) and not x.any()
    assert capi.ray_certificate(lp, x, y)[0] == 1


def test_presolve_infeasibility_comes_with_a_dual_ray(native):
    """x1 + x2 >= 3 with x1 <= 1 and x2 <= 1 as singleton rows, x free: after
    the singleton rows, the row's largest activity is 2 < 3 and presolve
    stops. Its ray, -1 on that row mapped back through the singleton rows,
    is y = (-1, 1, 1): a certificate of the original LP. The same for an
    empty row outside its bounds and for crossing singleton rows."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 1, 2], [0, 1, 0, 1], [1.0] * 4, [1.0, 1.0], [-INF, -INF], [INF, INF],
              [3.0, -INF, -INF], [INF, 1.0, 1.0])
    P = capi.Presolved(lp)
    assert P.outcome == "infeasible"
    x, y = P.ray()
    assert np.array_equal(y, [-1.0, 1.0, 1.0]) and not x.any()
    assert capi.ray_certificate(lp, x, y)[0] == 1
    for lp in (tiny([0, 1], [0, 0], [1.0, 1.0], [1.0], [0.0], [10.0], [-INF, 3.0], [1.0, INF]),
               tiny([0, 1], [0, 0], [2.0, -1.0], [1.0], [-INF], [INF], [-INF, -INF], [2.0, -3.0]),
               tiny([0, 1], [0, 1], [1.0, 1.0], [1.0, 1.0], [2.0, 0.0], [2.0, 1.0],
                    [0.0, -INF], [1.0, INF])):
        P = capi.Presolved(lp)
        assert P.outcome == "infeasible"
        x, y = P.ray()
        assert capi.ray_certificate(lp, x, y)[0] == 1, (lp.rmin, lp.rmax, y)


def test_parallel_rows_with_disjoint_ranges_come_with_a_dual_ray(native):
    """x0 + x1 in [0, 1] and 2 x0 + 2 x1 in [4, 5] (x free): the second row
    is twice the first, and in the first row's units it asks for [2, 2.5],
    which misses [0, 1]. Presolve stops at the parallel-row merge; its ray
    is +1 on the kept row and -1/2 on the other (A^T y = 0, bound 1 > 0).
    The same with the ratio negative and with the other side crossing."""
    from igaos_gb300 import capi
    for vals, rmin, rmax in (([1.0, 1.0, 2.0, 2.0], [0.0, 4.0], [1.0, 5.0]),
                             ([1.0, 1.0, -2.0, -2.0], [0.0, -5.0], [1.0, -4.0]),
                             ([1.0, 1.0, 3.0, 3.0], [4.0, -3.0], [5.0, 6.0])):
        lp = tiny([0, 0, 1, 1], [0, 1, 0, 1], vals, [1.0, 1.0], [-INF, -INF], [INF, INF],
                  rmin, rmax)
        P = capi.Presolved(lp)
        assert P.outcome == "infeasible"
        x, y = P.ray()
        assert not x.any() and np.count_nonzero(y) == 2, y
        assert capi.ray_certificate(lp, x, y)[0] == 1, (vals, rmin, rmax, y)


def test_unbounded_column_ray_follows_substitutions(native):
    """min x2 + 0.5 x4 s.t. x1 + x2 + x4 = 2, x1 in [0, 5], x2 free, x4 >= 0:
    substituting the free singleton x2 leaves x4 empty at cost -0.5 with no
    upper bound. Its ray x4 = +1 needs x2 = -1 to keep the row: the ray
    presolve returns is a primal certificate of the original LP."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 0], [0, 1, 2], [1.0, 1.0, 1.0], [0.0, 1.0, 0.5], [0.0, -INF, 0.0],
              [5.0, INF, INF], [2.0], [2.0])
    P = capi.Presolved(lp)
    assert P.outcome == "unbounded" and P.lp is None
    r, yr = P.ray()
    assert np.array_equal(r, [0.0, -1.0, 1.0]) and not yr.any()
    assert capi.ray_certificate(lp, r, np.zeros(1))[0] == 2
    with pytest.raises(capi.EngineError, match="only its ray"):
        P.postsolve(np.zeros(1), np.zeros(1))


def test_implied_free_singleton_is_substituted(native, orc):
    """min x1 + 2 x2 - s s.t. x1 + x2 + s = 5, x1, x2 in [0, 2], s in [0, 10]:
    the row keeps s in [1, 5], inside its bounds, so s is substituted like a
    free column (y = 1; x1, x2 then cost 2 and 3 and go to 0, s = 5)."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 0], [0, 1, 2], [1.0, 1.0, 1.0], [1.0, 2.0, -1.0], [0.0, 0.0, 0.0],
              [2.0, 2.0, 10.0], [5.0], [5.0])
    P = capi.Presolved(lp)
    assert P.counts["free_singletons"] == 1 and (P.lp.m, P.lp.n) == (0, 0)
    x, y = P.postsolve(np.zeros(0), np.zeros(0))
    assert np.array_equal(x, [0.0, 0.0, 5.0]) and np.array_equal(y, [1.0])
    assert_optimal(metrics(orc, lp, x, y), 0.0)
    # with s in [0, 4] the row could need s = 5: the bounds bind, no substitution
    lp = tiny([0, 0, 0], [0, 1, 2], [1.0, 1.0, 1.0], [1.0, 2.0, -1.0], [0.0, 0.0, 0.0],
              [2.0, 2.0, 4.0], [5.0], [5.0])
    assert capi.Presolved(lp).counts["free_singletons"] == 0


def test_implied_free_singletons_keep_postsolve_exact(native, orc):
    """Seeded LPs with a slack-like singleton column of wide bounds in every
    row: those of the equality rows qualify (a <= row leaves the column's
    lower side open), and the postsolved HiGHS pair stays optimal."""
    from igaos_gb300 import capi
    for seed in range(4):
        base = G.random_lp(40, 90, 150, seed)
        rows = np.repeat(np.arange(base.m), np.diff(base.ap))
        m, n = base.m, base.n + base.m
        lp = G.from_triplets(m, n, np.concatenate([rows, np.arange(m)]),
                             np.concatenate([base.ai, base.n + np.arange(m)]),
                             np.concatenate([base.ax, np.ones(m)]),
                             np.concatenate([base.c, np.full(m, 0.1)]),
                             np.concatenate([base.cl, np.full(m, -1e4)]),
                             np.concatenate([base.cu, np.full(m, 1e4)]), base.rmin, base.rmax)
        P = capi.Presolved(lp)
        assert P.counts["free_singletons"] >= m // 4
        xr, yr, _ = highs(P.lp)
        x, y = P.postsolve(xr, yr)
        assert_optimal(metrics(orc, lp, x, y), 1e-9)
        _, _, f = highs(lp)
        assert abs(lp.c @ x - f) <= 1e-8 * (1.0 + abs(f))


def test_parallel_rows_merge_and_hand_over_the_dual(native, orc):
    """min -x1 - x2 s.t. x1 + 2 x2 <= 4, 2 x1 + 4 x2 <= 6 (the same row at
    ratio 2, tighter), -x1 - 2 x2 >= -5 (ratio -1, looser), x in [0, 2]: the
    first row keeps x1 + 2 x2 <= 3 and the others go. At the optimum (2,
    0.5) the binding side came from the second row, which gets the dual."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 1, 1, 2, 2], [0, 1, 0, 1, 0, 1], [1.0, 2.0, 2.0, 4.0, -1.0, -2.0],
              [-1.0, -1.0], [0.0, 0.0], [2.0, 2.0], [-INF, -INF, -5.0], [4.0, 6.0, INF])
    P = capi.Presolved(lp)
    assert P.counts["redundant_rows"] == 2 and P.lp.m == 1 and P.lp.rmax[0] == 3.0
    xr, yr, _ = highs(P.lp)
    x, y = P.postsolve(xr, yr)
    assert np.allclose(x, [2.0, 0.5]) and y[0] == 0.0 and y[2] == 0.0 and y[1] > 0.0
    assert_optimal(metrics(orc, lp, x, y), 1e-12)


def test_repeated_entries_are_summed(native, orc):
    """A column entered twice in a row (2 x1 and -1 x1: x1 in total) with
    x2: x1 + x2 <= 0 on [0, 1]^2 forces both to 0. Were the entries taken
    apart, the row's least activity would be 2*0 - 1*1 = -1 and nothing
    forced; summed, the row forces, and the postsolved pair is optimal."""
    from igaos_gb300 import capi
    lp = tiny([0, 0, 0, 1], [0, 0, 1, 1], [2.0, -1.0, 1.0, 1.0], [-1.0, -2.0], [0.0, 0.0],
              [1.0, 1.0], [-INF, -INF], [0.0, 1.0])
    P = capi.Presolved(lp)
    assert P.outcome == "reduced" and P.counts["redundant_rows"] >= 1
    xr, yr, _ = highs(P.lp) if P.lp.m else (np.zeros(P.lp.n), np.zeros(0), 0.0)
    x, y = P.postsolve(xr, yr)
    assert np.array_equal(x, [0.0, 0.0])
    assert_optimal(metrics(orc, lp, x, y), 1e-12)
