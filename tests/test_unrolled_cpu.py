"""Differentiable layer, CPU side: the dense FP64 checker against central
finite differences and the envelope theorem, the batch pattern (CSC with CSR
positions) and the C layout struct. No GPU needed."""
import ctypes as C

import numpy as np
import pytest
import torch

from igaos_gb300 import capi
from igaos_gb300 import generators as G
from igaos_gb300.layer import BatchPattern
from oracle import unrolled_dense as U

RIDGE = 0.005


def tiny(seed=3, m=8, n=16, density=0.3):
    return G.bernoulli_lp(np.random.default_rng(seed), m, n, density, 10.0)


def fd(lp, tau, sigma, K, name, d, h=1e-6, weights=None):
    base = np.asarray(getattr(lp, name), float)

    def f(v):
        kw = {"ax": v} if name == "ax" else {name: v}
        x, y, obj = U.forward(lp, tau, sigma, K, RIDGE, **kw)
        return obj if weights is None else float(weights @ x)
    return (f(base + h * d) - f(base - h * d)) / (2 * h)


@pytest.mark.parametrize("name", ["c", "rmin", "rmax", "ax", "cl", "cu"])
def test_dense_checker_matches_central_fd(name):
    lp = tiny()
    if name in ("cl", "cu"):
        # keep x0 = clamp(0, cl, cu) off its kink: a lower bound above 0
        lp.cl = np.full(lp.n, 0.25)
    tau, sigma = U.power_steps(lp)
    K = 40
    wx = np.random.default_rng(7).standard_normal(lp.n)
    _, g_obj = U.gradients(lp, tau, sigma, K, RIDGE)
    _, g_x = U.gradients(lp, tau, sigma, K, RIDGE, gx=wx, gobj=0.0)
    base = np.asarray(getattr(lp, name), float)
    d = np.random.default_rng(11).standard_normal(base.shape)
    d[~np.isfinite(base)] = 0.0
    for g, w in ((g_obj, None), (g_x, wx)):
        num = fd(lp, tau, sigma, K, name, d, weights=w)
        ana = float(g[name] @ d)
        assert abs(num - ana) <= 1e-6 * max(1.0, abs(ana)), (name, num, ana)


def test_dense_checker_envelope_theorem():
    """At convergence, d obj/d c = x*, d obj/d b_i = -y_i, d obj/d A_ij =
    y_i x*_j (reduced cost d = c + A^T y)."""
    lp = tiny()
    tau, sigma = U.power_steps(lp)
    out, g = U.gradients(lp, tau, sigma, 10000, RIDGE)
    x, y = out["x"], out["y"]
    rows = np.repeat(np.arange(lp.m), np.diff(lp.ap))
    eq = np.isfinite(lp.rmin)
    gb = np.where(eq, g["rmin"] + g["rmax"], g["rmax"])
    assert np.abs(g["c"] - x).max() <= 1e-6
    assert np.abs(gb + y).max() <= 1e-6
    assert np.abs(g["ax"] - y[rows] * x[lp.ai]).max() <= 1e-6


def test_pattern_transpose_and_positions():
    rng = np.random.default_rng(0)
    lps = [G.bernoulli_lp(rng, m, n, 0.2, 10.0) for m, n in ((5, 9), (12, 7), (1, 3))]
    P = BatchPattern.from_lps(lps, device="cpu")
    assert P.total_m == 18 and P.total_n == 19 and P.max_m == 12 and P.max_n == 9
    cp, ci, perm = P.t_cp.numpy(), P.t_ci.numpy(), P.t_cperm.numpy()
    for b, lp in enumerate(lps):
        z0, z1 = P.nz_off[b], P.nz_off[b + 1]
        c0 = P.col_off[b] + b
        assert np.array_equal(cp[c0:c0 + lp.n + 1], lp.cp)
        assert np.array_equal(ci[z0:z1], lp.ci)
        assert np.array_equal(lp.ax[perm[z0:z1]], lp.acx)


def test_pattern_rejects_bad_input():
    lp = tiny()
    ai = lp.ai.copy()
    ai[0] = lp.n
    with pytest.raises(ValueError, match="column index out of range"):
        BatchPattern([lp.m], [lp.n], [lp.ap], [ai], device="cpu")
    with pytest.raises(ValueError, match="m >= 1"):
        BatchPattern([0], [3], [np.zeros(1, np.int32)], [np.zeros(0, np.int32)], device="cpu")


def test_layout_struct_matches_header():
    # 4 ints, 1 double, 2 ints, 4 int64, 8 pointers
    assert C.sizeof(capi.UnrolledLayout) == 16 + 8 + 8 + 32 + 8 * 8
    assert capi.UnrolledLayout.row_off.offset == 64
    P = BatchPattern.from_lps([tiny()], device="cpu")
    L = P.layout(torch.float64, 1000, 50, RIDGE)
    assert L.precision == capi.FP64 and L.iterations == 1000 and L.checkpoint == 50
    assert L.ap == P.t_ap.data_ptr()


def test_layout_sizes_without_device(native):
    """Buffer-size queries are pure host arithmetic."""
    P = BatchPattern.from_lps([tiny(), tiny(4, 6, 20)], device="cpu")
    L = P.layout(torch.float32, 1000, 50, RIDGE)
    lib = capi.lib()
    assert lib.igaos_pdhg_unrolled_checkpoint_elems(C.byref(L)) == 20 * (P.total_n + P.total_m)
    per = 50 * (P.total_n + P.total_m)
    assert lib.igaos_pdhg_unrolled_workspace_bytes(C.byref(L)) == (per * 4 + 255) // 256 * 256 + per
    L.checkpoint = 0
    assert lib.igaos_pdhg_unrolled_checkpoint_elems(C.byref(L)) == -1
    assert "checkpoint" in capi.last_error()
