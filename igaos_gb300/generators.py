"""Seeded synthetic LP generators for the engine's workload shapes.

Every LP is returned in the engine's form (rmin <= A x <= rmax,
cl <= x <= cu, minimise c^T x) with A held both as CSR (ap, ai, ax) and as
CSC (cp, ci, acx) -- the two orientations the reference's model reader
builds (src/io/model.hpp:16-37, counting_sort :39-67). Triplets are ordered
column-major then row-major, as an MPS COLUMNS section lists them, so CSR
rows hold their entries in increasing column order and CSC columns in
increasing row order, exactly what counting_sort yields from that order.

Feasibility follows the x*-construction: x* drawn inside the box, b = A x*
for equality rows and b = A x* + U[0,1] slack for <= rows.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

INF = float("inf")


@dataclass
class LPData:
    m: int
    n: int
    ap: np.ndarray
    ai: np.ndarray
    ax: np.ndarray
    cp: np.ndarray
    ci: np.ndarray
    acx: np.ndarray
    c: np.ndarray
    cl: np.ndarray
    cu: np.ndarray
    rmin: np.ndarray
    rmax: np.ndarray
    obj_const: float = 0.0
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def nnz(self) -> int:
        return int(self.ap[self.m])

    def dense(self) -> np.ndarray:
        A = np.zeros((self.m, self.n))
        rows = np.repeat(np.arange(self.m), np.diff(self.ap))
        np.add.at(A, (rows, self.ai), self.ax)
        return A


def from_triplets(m: int, n: int, rows, cols, vals, c, cl, cu, rmin, rmax,
                  obj_const=0.0, name="", presorted=False) -> LPData:
    """CSR + CSC from (row, col, val) triplets, ordered column-major first
    (stable), the counting-sort result for MPS-ordered triplets."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    vals = np.asarray(vals, np.float64)
    if not presorted:
        o = np.lexsort((rows, cols))
        rows, cols, vals = rows[o], cols[o], vals[o]
    # CSR: stable by row keeps the column-major order inside each row
    o = np.argsort(rows, kind="stable")
    ap = np.zeros(m + 1, np.int64)
    np.add.at(ap, rows + 1, 1)
    ap = np.cumsum(ap).astype(np.int32)
    cp = np.zeros(n + 1, np.int64)
    np.add.at(cp, cols + 1, 1)
    cp = np.cumsum(cp).astype(np.int32)
    return LPData(m=m, n=n, ap=ap, ai=cols[o].astype(np.int32), ax=vals[o].copy(),
                  cp=cp, ci=rows.astype(np.int32), acx=vals.copy(),
                  c=np.asarray(c, np.float64), cl=np.asarray(cl, np.float64),
                  cu=np.asarray(cu, np.float64), rmin=np.asarray(rmin, np.float64),
                  rmax=np.asarray(rmax, np.float64), obj_const=obj_const, name=name)


def _csr_matvec(lp: LPData, x: np.ndarray) -> np.ndarray:
    rows = np.repeat(np.arange(lp.m), np.diff(lp.ap))
    return np.bincount(rows, weights=lp.ax * x[lp.ai], minlength=lp.m)


def _feasible_rows(rng, lp_rows, ax_star, n_eq):
    """Row bounds: first n_eq rows equality at A x*, the rest <= A x* + U[0,1]."""
    m = ax_star.shape[0]
    rmin = np.full(m, -INF)
    rmax = ax_star.copy()
    rmin[:n_eq] = ax_star[:n_eq]
    rmax[n_eq:] = ax_star[n_eq:] + rng.uniform(0.0, 1.0, m - n_eq)
    return rmin, rmax


def _dedupe(rows, cols):
    key = cols.astype(np.int64) * (1 << 31) + rows.astype(np.int64)
    key = np.unique(key)
    return (key % (1 << 31)).astype(np.int64), (key // (1 << 31)).astype(np.int64)


def random_lp(m: int, n: int, extra_nnz: int, seed: int, hi: float = 10.0,
              name="random") -> LPData:
    """Small random LP: every column gets one entry at a uniform row, plus
    `extra_nnz` uniform (row, col) entries, de-duplicated; A_ij ~ N(0,1);
    first half of the rows equality, second half <=; box [0, hi]; c ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    r0 = rng.integers(0, m, n)
    c0 = np.arange(n)
    r1 = rng.integers(0, m, extra_nnz)
    c1 = rng.integers(0, n, extra_nnz)
    rows, cols = _dedupe(np.concatenate([r0, r1]), np.concatenate([c0, c1]))
    vals = rng.standard_normal(rows.shape[0])
    xs = rng.uniform(0.0, hi, n)
    c = rng.standard_normal(n)
    lp = from_triplets(m, n, rows, cols, vals, c, np.zeros(n), np.full(n, hi),
                       np.zeros(m), np.zeros(m), name=name, presorted=True)
    ax_star = _csr_matvec(lp, xs)
    lp.rmin, lp.rmax = _feasible_rows(rng, None, ax_star, m // 2)
    lp.meta = dict(seed=seed, x_star=xs)
    return lp


def config1(seed: int = 0) -> LPData:
    """Small random LP: m=2,000 (1,000 equality, 1,000 <=), n=5,000,
    0<=x<=10, ~20k nnz (one per column + 15k uniform, de-duplicated)."""
    return random_lp(2000, 5000, 15000, seed, 10.0, name=f"c1-seed{seed}")


def config2(seed: int = 0, m: int = 200_000, n: int = 500_000,
            target_nnz: int = 5_000_000) -> LPData:
    """Large sparse LP: column degrees Zipf(1.5) clipped to [1,2000] and
    rescaled to ~target_nnz total (>= 1 per column), rows uniform,
    |A_ij| log-uniform in [1e-3, 1e3] with a random sign; half equality,
    half <= rows; box [0,10]; c ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    deg = np.minimum(rng.zipf(1.5, n), 2000).astype(np.float64)
    s = target_nnz / deg.sum()
    deg = np.maximum(1, np.rint(deg * s)).astype(np.int64)
    cols = np.repeat(np.arange(n, dtype=np.int64), deg)
    rows = rng.integers(0, m, cols.shape[0])
    rows, cols = _dedupe(rows, cols)
    k = rows.shape[0]
    mag = 10.0 ** rng.uniform(-3.0, 3.0, k)
    vals = np.where(rng.random(k) < 0.5, -mag, mag)
    xs = rng.uniform(0.0, 10.0, n)
    c = rng.standard_normal(n)
    lp = from_triplets(m, n, rows, cols, vals, c, np.zeros(n), np.full(n, 10.0),
                       np.zeros(m), np.zeros(m), name=f"c2-seed{seed}", presorted=True)
    lp.rmin, lp.rmax = _feasible_rows(rng, None, _csr_matvec(lp, xs), m // 2)
    lp.meta = dict(seed=seed, degree_scale=s)
    return lp


def bernoulli_lp(rng, m: int, n: int, density: float, hi: float, name="") -> LPData:
    """Bernoulli(density) sparsity pattern drawn by geometric skips,
    N(0,1) values, x* ~ U[0,hi], half equality / half <= rows, box [0,hi]."""
    cells = m * n
    expect = cells * density
    draw = int(expect + 6.0 * np.sqrt(expect) + 16)
    gaps = rng.geometric(density, draw)
    pos = np.cumsum(gaps) - 1
    while pos[-1] < cells:  # extremely unlikely top-up
        more = np.cumsum(rng.geometric(density, draw)) + pos[-1]
        pos = np.concatenate([pos, more])
    pos = pos[pos < cells]
    # column-major cell numbering: pos = col*m + row
    cols = pos // m
    rows = pos % m
    vals = rng.standard_normal(pos.shape[0])
    xs = rng.uniform(0.0, hi, n)
    c = rng.standard_normal(n)
    lp = from_triplets(m, n, rows, cols, vals, c, np.zeros(n), np.full(n, hi),
                       np.zeros(m), np.zeros(m), name=name, presorted=True)
    lp.rmin, lp.rmax = _feasible_rows(rng, None, _csr_matvec(lp, xs), m // 2)
    return lp


def config3(seed: int = 0, count: int = 4096, m_lo: int = 20, m_hi: int = 2000,
            density: float = 0.01) -> list:
    """Batch of uneven random LPs: m log-uniform in [m_lo, m_hi], n = 2.5 m,
    Bernoulli(density) pattern, N(0,1) values, box [0,5]."""
    rng = np.random.default_rng(seed)
    ms = np.rint(np.exp(rng.uniform(np.log(m_lo), np.log(m_hi), count))).astype(int)
    out = []
    for b, m in enumerate(ms):
        n = int(round(2.5 * m))
        out.append(bernoulli_lp(rng, int(m), n, density, 5.0, name=f"c3-{seed}-{b}"))
    return out


def config4(seed: int = 0, count: int = 256, m: int = 500, n: int = 1000,
            density: float = 0.02) -> list:
    """Batch for the differentiable layer: m=500, n=1000, 2% density,
    N(0,1) values, box [0,10], c ~ N(0,1). The ridge weight (0.005) is a
    property of the layer, not of the data."""
    rng = np.random.default_rng(seed)
    return [bernoulli_lp(rng, m, n, density, 10.0, name=f"c4-{seed}-{b}")
            for b in range(count)]


def config5(seed: int = 0, side: int = 300, commodities: int = 8) -> LPData:
    """Multicommodity flow on a side x side 4-neighbour grid (directed arcs
    both ways): per-commodity conservation equalities, shared arc capacity
    rows sum_k x_ka <= U[20,60], arc cost U[1,10], demand U[1,10] between a
    random source/sink pair per commodity; the implied box 0 <= x_ka <= cap_a
    keeps the dual bound finite."""
    rng = np.random.default_rng(seed)
    V = side * side
    idx = np.arange(V).reshape(side, side)
    tails, heads = [], []
    for a, b in ((idx[:, :-1], idx[:, 1:]), (idx[:-1, :], idx[1:, :])):
        tails += [a.ravel(), b.ravel()]
        heads += [b.ravel(), a.ravel()]
    tail = np.concatenate(tails)
    head = np.concatenate(heads)
    E = tail.shape[0]
    cap = rng.uniform(20.0, 60.0, E)
    cost = rng.uniform(1.0, 10.0, E)
    K = commodities
    src = np.empty(K, np.int64)
    dst = np.empty(K, np.int64)
    for k in range(K):
        s, t = rng.choice(V, 2, replace=False)
        src[k], dst[k] = s, t
    dem = rng.uniform(1.0, 10.0, K)
    m = K * V + E
    n = K * E
    # column k*E + a: +1 in row k*V + tail (outflow), -1 in row k*V + head,
    # +1 in capacity row K*V + a. Rows per column are increasing.
    kk = np.repeat(np.arange(K, dtype=np.int64), E)
    aa = np.tile(np.arange(E, dtype=np.int64), K)
    r_out = kk * V + tail[aa]
    r_in = kk * V + head[aa]
    r_cap = K * V + aa
    R = np.stack([r_out, r_in, r_cap], 1)
    Vv = np.stack([np.ones(n), -np.ones(n), np.ones(n)], 1)
    o = np.argsort(R, axis=1, kind="stable")
    R = np.take_along_axis(R, o, 1)
    Vv = np.take_along_axis(Vv, o, 1)
    cols = np.repeat(np.arange(n, dtype=np.int64), 3)
    rows = R.ravel()
    vals = Vv.ravel()
    rhs = np.zeros(K * V)
    rhs[np.arange(K) * V + src] += dem
    rhs[np.arange(K) * V + dst] -= dem
    rmin = np.concatenate([rhs, np.full(E, -INF)])
    rmax = np.concatenate([rhs, cap])
    c = np.tile(cost, K)
    cu = np.tile(cap, K)
    lp = from_triplets(m, n, rows, cols, vals, c, np.zeros(n), cu, rmin, rmax,
                       name=f"c5-seed{seed}", presorted=True)
    lp.meta = dict(seed=seed, arcs=E, nodes=V, commodities=K)
    return lp


def mixed_bounds_lp(m: int, n: int, extra_nnz: int, seed: int) -> LPData:
    """Random LP exercising every bound type the engine handles: free,
    lower-only, upper-only, boxed and fixed columns; equality, <=, >= and
    ranged rows. Feasible by construction around x*; bounded objective is
    ensured by giving free / one-sided columns a cost pushing into a bound
    only when that bound exists (free columns get zero cost)."""
    rng = np.random.default_rng(seed)
    r0 = rng.integers(0, m, n)
    r1 = rng.integers(0, m, extra_nnz)
    c1 = rng.integers(0, n, extra_nnz)
    rows, cols = _dedupe(np.concatenate([r0, r1]), np.concatenate([np.arange(n), c1]))
    vals = rng.standard_normal(rows.shape[0])
    kind = rng.integers(0, 5, n)  # 0 free, 1 lower, 2 upper, 3 box, 4 fixed
    xs = rng.uniform(-2.0, 2.0, n)
    cl = np.full(n, -INF)
    cu = np.full(n, INF)
    c = rng.standard_normal(n)
    lo_set = (kind == 1) | (kind == 3)
    up_set = (kind == 2) | (kind == 3)
    cl[lo_set] = xs[lo_set] - rng.uniform(0, 1, lo_set.sum())
    cu[up_set] = xs[up_set] + rng.uniform(0, 1, up_set.sum())
    cl[kind == 4] = cu[kind == 4] = xs[kind == 4]
    c[kind == 0] = 0.0
    c[kind == 1] = np.abs(c[kind == 1])
    c[kind == 2] = -np.abs(c[kind == 2])
    lp = from_triplets(m, n, rows, cols, vals, c, cl, cu, np.zeros(m), np.zeros(m),
                       name=f"mixed-{seed}", presorted=True)
    ax = _csr_matvec(lp, xs)
    rk = rng.integers(0, 4, m)  # 0 E, 1 L, 2 G, 3 ranged
    rmin = np.full(m, -INF)
    rmax = np.full(m, INF)
    e = rk == 0
    rmin[e] = rmax[e] = ax[e]
    l_ = rk == 1
    rmax[l_] = ax[l_] + rng.uniform(0, 1, l_.sum())
    g_ = rk == 2
    rmin[g_] = ax[g_] - rng.uniform(0, 1, g_.sum())
    r_ = rk == 3
    rmin[r_] = ax[r_] - rng.uniform(0, 1, r_.sum())
    rmax[r_] = ax[r_] + rng.uniform(0, 1, r_.sum())
    lp.rmin, lp.rmax = rmin, rmax
    lp.meta = dict(seed=seed)
    return lp


def known_optimum_lp(m: int, n: int, extra_nnz: int, seed: int):
    """LP with the sparsity, bound and row types of mixed_bounds_lp and a
    known optimal pair (x*, y*): columns strictly inside their bounds (all
    free ones) have zero reduced cost, columns at a bound a reduced cost of
    the sign that bound allows; rows with y*_i != 0 are tight at the bound
    matching its sign, the others slack. Returns (lp, x*, y*); in the
    convention d = c + A^T y the gap of (x*, y*) is zero."""
    rng = np.random.default_rng(seed)
    r0 = rng.integers(0, m, n)
    r1 = rng.integers(0, m, extra_nnz)
    c1 = rng.integers(0, n, extra_nnz)
    rows, cols = _dedupe(np.concatenate([r0, r1]), np.concatenate([np.arange(n), c1]))
    vals = rng.standard_normal(rows.shape[0])
    kind = rng.integers(0, 5, n)  # 0 free, 1 lower, 2 upper, 3 box, 4 fixed
    base = rng.uniform(-2.0, 2.0, n)
    cl = np.full(n, -INF)
    cu = np.full(n, INF)
    lo_set = (kind == 1) | (kind == 3)
    up_set = (kind == 2) | (kind == 3)
    cl[lo_set] = base[lo_set] - rng.uniform(0.5, 1.5, lo_set.sum())
    cu[up_set] = base[up_set] + rng.uniform(0.5, 1.5, up_set.sum())
    cl[kind == 4] = cu[kind == 4] = base[kind == 4]
    # where x* sits: 0 inside, 1 at the lower bound, 2 at the upper bound
    at = np.zeros(n, np.int64)
    pick = rng.integers(0, 3, n)
    at[(kind == 1) & (pick > 0)] = 1
    at[(kind == 2) & (pick > 0)] = 2
    at[kind == 3] = pick[kind == 3]
    at[kind == 4] = 1
    xs = base.copy()
    xs[at == 1] = cl[at == 1]
    xs[at == 2] = cu[at == 2]
    lp = from_triplets(m, n, rows, cols, vals, np.zeros(n), cl, cu, np.zeros(m), np.zeros(m),
                       name=f"known-{seed}", presorted=True)
    ax = _csr_matvec(lp, xs)
    rk = rng.integers(0, 4, m)  # 0 E, 1 L, 2 G, 3 ranged
    tight = rng.integers(0, 2, m) == 1
    ys = np.zeros(m)
    rmin = np.full(m, -INF)
    rmax = np.full(m, INF)
    e = rk == 0
    rmin[e] = rmax[e] = ax[e]
    ys[e] = rng.standard_normal(e.sum())
    for k, sgn in ((1, 1.0), (2, -1.0)):
        sel = rk == k
        t, f = sel & tight, sel & ~tight
        ys[t] = sgn * rng.uniform(0.1, 2.0, t.sum())
        if k == 1:
            rmax[t] = ax[t]
            rmax[f] = ax[f] + rng.uniform(0.1, 1.0, f.sum())
        else:
            rmin[t] = ax[t]
            rmin[f] = ax[f] - rng.uniform(0.1, 1.0, f.sum())
    r_ = rk == 3
    side = rng.integers(0, 3, m)  # 0 slack, 1 tight at rmax, 2 tight at rmin
    rmin[r_] = ax[r_] - rng.uniform(0.1, 1.0, r_.sum())
    rmax[r_] = ax[r_] + rng.uniform(0.1, 1.0, r_.sum())
    hi_t, lo_t = r_ & (side == 1), r_ & (side == 2)
    rmax[hi_t] = ax[hi_t]
    ys[hi_t] = rng.uniform(0.1, 2.0, hi_t.sum())
    rmin[lo_t] = ax[lo_t]
    ys[lo_t] = -rng.uniform(0.1, 2.0, lo_t.sum())
    aty = np.zeros(n)
    rr = np.repeat(np.arange(m), np.diff(lp.ap))
    np.add.at(aty, lp.ai, lp.ax * ys[rr])
    s = np.zeros(n)
    s[at == 1] = rng.uniform(0.1, 2.0, (at == 1).sum())
    s[at == 2] = -rng.uniform(0.1, 2.0, (at == 2).sum())
    s[kind == 4] = rng.standard_normal((kind == 4).sum())
    lp.c = s - aty
    lp.rmin, lp.rmax = rmin, rmax
    lp.meta = dict(seed=seed)
    return lp, xs, ys


def free_cost_lp(m: int, n: int, extra_nnz: int, seed: int) -> LPData:
    """The bound and row structure of mixed_bounds_lp, with costs that give
    free and one-sided columns nonzero reduced-cost pressure: c = -A^T y* + s
    for a dual point y* in the row cone (y* >= 0 on <= rows, <= 0 on >=
    rows) and s = 0 (free), s >= 0 (lower bound only), s <= 0 (upper bound
    only), s ~ N(0,1) (boxed, fixed). Primal feasible around x*, dual
    feasible at y*, so bounded. The dual objective stays -inf until the
    iterate's reduced costs of the columns with an infinite bound are within
    1e-8 (1 + max|c|) of their sign -- the case dual_repair certifies."""
    lp = mixed_bounds_lp(m, n, extra_nnz, seed)
    rng = np.random.default_rng(seed + 7919)
    fin_lo, fin_hi = np.isfinite(lp.rmin), np.isfinite(lp.rmax)
    ys = rng.standard_normal(m)
    ys[fin_hi & ~fin_lo] = np.abs(ys[fin_hi & ~fin_lo])
    ys[fin_lo & ~fin_hi] = -np.abs(ys[fin_lo & ~fin_hi])
    ys[~fin_lo & ~fin_hi] = 0.0
    aty = np.zeros(n)
    rows = np.repeat(np.arange(m), np.diff(lp.ap))
    np.add.at(aty, lp.ai, lp.ax * ys[rows])
    lo_f, up_f = np.isfinite(lp.cl), np.isfinite(lp.cu)
    s = rng.standard_normal(n)
    s[~lo_f & ~up_f] = 0.0
    s[lo_f & ~up_f] = np.abs(s[lo_f & ~up_f])
    s[~lo_f & up_f] = -np.abs(s[~lo_f & up_f])
    lp.c = -aty + s
    lp.name = f"freecost-{seed}"
    return lp


def presolvable_lp(m: int, n: int, extra_nnz: int, seed: int) -> LPData:
    """random_lp(m, n, extra_nnz, seed) with every reduction of the engine's
    presolve planted, feasible and bounded by construction: fixed columns in
    base rows (row bounds shifted by their contribution), empty columns (cost
    sign matched to a finite bound, or zero cost), empty rows around 0, free
    columns held by two singleton rows (x >= lo and x <= hi, so the implied
    bounds decide the optimum), free columns fixed by an equality singleton
    row, free singleton columns in base equality rows (some with zero cost)
    and redundant rows over boxed base columns. Rows and columns are then
    permuted so that the planted parts are spread through the LP."""
    rng = np.random.default_rng(seed + 7919)
    base = random_lp(m, n, extra_nnz, seed)
    xs = base.meta["x_star"]
    R = list(np.repeat(np.arange(m), np.diff(base.ap)))
    Cc = list(base.ai)
    V = list(base.ax)
    c, cl, cu = list(base.c), list(base.cl), list(base.cu)
    rmin, rmax = list(base.rmin), list(base.rmax)

    def col(cost, lo, hi):
        c.append(cost)
        cl.append(lo)
        cu.append(hi)
        return len(c) - 1

    def row(lo, hi):
        rmin.append(lo)
        rmax.append(hi)
        return len(rmin) - 1

    def put(i, j, a):
        R.append(i)
        Cc.append(j)
        V.append(a)

    def in_base_rows(j, value, count):
        for i in rng.choice(m, count, replace=False):
            a = rng.standard_normal()
            put(i, j, a)
            rmin[i] += a * value  # -inf stays -inf
            rmax[i] += a * value

    k = max(2, n // 20)
    for _ in range(k):  # fixed columns
        v = rng.uniform(-3.0, 3.0)
        in_base_rows(col(rng.standard_normal(), v, v), v, 3)
    for t in range(k):  # empty columns
        g = abs(rng.standard_normal()) + 0.1
        if t % 4 == 0:
            col(g, rng.uniform(-2.0, 0.0), INF)
        elif t % 4 == 1:
            col(-g, -INF, rng.uniform(0.0, 2.0))
        elif t % 4 == 2:
            col(0.0, -INF, INF)
        else:
            col(rng.standard_normal(), -1.0, 1.0)
    for t in range(k):  # empty rows
        if t % 3 == 0:
            row(0.0, 0.0)
        elif t % 3 == 1:
            row(-INF, rng.uniform(0.0, 1.0))
        else:
            row(-rng.uniform(0.0, 1.0), rng.uniform(0.0, 1.0))
    for _ in range(k):  # free columns bounded by two singleton rows
        lo = rng.uniform(-2.0, 0.0)
        hi = lo + rng.uniform(0.5, 2.0)
        j = col(2.0 * rng.standard_normal(), -INF, INF)
        in_base_rows(j, 0.5 * (lo + hi), 2)
        a1 = rng.uniform(0.5, 2.0)
        put(row(a1 * lo, INF), j, a1)       # a1 x >= a1 lo
        a2 = -rng.uniform(0.5, 2.0)
        put(row(a2 * hi, INF), j, a2)       # a2 x >= a2 hi, i.e. x <= hi
    for _ in range(k // 2 + 1):  # free columns fixed by an equality singleton row
        v = rng.uniform(-1.0, 1.0)
        j = col(rng.standard_normal(), -INF, INF)
        in_base_rows(j, v, 2)
        a = rng.uniform(1.0, 3.0) * rng.choice([-1.0, 1.0])
        put(row(a * v, a * v), j, a)
    eq = rng.permutation(m // 2)[:k]  # free singleton columns in equality rows
    for t, i in enumerate(eq):
        j = col(0.0 if t % 3 == 0 else rng.standard_normal(), -INF, INF)
        put(i, j, rng.uniform(0.5, 2.0) * rng.choice([-1.0, 1.0]))
    for t in range(k):  # redundant rows over boxed base columns [0, 10]
        js = rng.choice(n, 4, replace=False)
        a = rng.standard_normal(4)
        L = float(np.minimum(0.0, 10.0 * a).sum())
        U = float(np.maximum(0.0, 10.0 * a).sum())
        i = row(L - 1.0, U + 1.0) if t % 2 == 0 else row(-INF, U + 0.5)
        for jj, aa in zip(js, a):
            put(i, int(jj), float(aa))
    M, N = len(rmin), len(c)
    pr, pc = rng.permutation(M), rng.permutation(N)  # new index of each old one
    lp = from_triplets(M, N, pr[np.asarray(R)], pc[np.asarray(Cc)], V,
                       np.asarray(c)[np.argsort(pc)], np.asarray(cl)[np.argsort(pc)],
                       np.asarray(cu)[np.argsort(pc)], np.asarray(rmin)[np.argsort(pr)],
                       np.asarray(rmax)[np.argsort(pr)], name=f"presolvable-{seed}")
    lp.meta = dict(seed=seed, planted=k)
    return lp
