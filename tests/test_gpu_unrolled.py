"""Differentiable LP layer on the GPU (igaos_pdhg_unrolled_*): K unrolled
fixed-step PDHG iterations of ridge-regularised LPs and their reverse mode.

* FP64 forward and gradients equal the dense FP64 checker (torch autograd
  through the same iterations) on ragged batches and on C4-shaped instances
  (m 500, n 1000, 2% density, box [0,10], ridge 0.005, K 1000, checkpoints
  every 50).
* FP64 gradients of obj and of a projection of x* with respect to c, b and
  A's values agree with central finite differences (h = 1e-6).
* At convergence they satisfy the envelope theorem.
* The checkpoint interval changes nothing (bit for bit); runs repeat bit for
  bit; FP32 stays close to FP64.
"""
import numpy as np
import pytest
import torch

from igaos_gb300 import capi
from igaos_gb300 import generators as G
from igaos_gb300.layer import BatchPattern, UnrolledPDHG, pdhg_steps, stack_lps, unrolled_lp
from oracle import unrolled_dense as U

pytestmark = pytest.mark.gpu
RIDGE = 0.005
DEV = "cuda"


def ragged(seed=0):
    rng = np.random.default_rng(seed)
    return [G.bernoulli_lp(rng, m, n, d, 10.0) for m, n, d in
            ((8, 16, 0.3), (30, 60, 0.1), (12, 20, 0.2), (1, 4, 0.9))]


def c4(count, seed=0):
    return G.config4(seed=seed, count=count)


def run(lps, K, ck, dtype=torch.float64, seed=1, tau=None, sigma=None):
    """Forward + backward with random output cotangents; numpy results."""
    P = BatchPattern.from_lps(lps, DEV)
    data = [t.clone().requires_grad_(True) for t in stack_lps(lps, dtype, DEV)]
    if tau is None:
        tau, sigma = pdhg_steps(P, data[5].detach())
    x, y, obj = UnrolledPDHG.apply(*data, tau, sigma, P, K, ck, RIDGE)
    rng = np.random.default_rng(seed)
    wx = torch.tensor(rng.standard_normal(P.total_n), dtype=dtype, device=DEV)
    wy = torch.tensor(rng.standard_normal(P.total_m), dtype=dtype, device=DEV)
    wo = torch.tensor(rng.standard_normal(P.count), dtype=dtype, device=DEV)
    ((wx * x).sum() + (wy * y).sum() + (wo * obj).sum()).backward()
    names = ("c", "cl", "cu", "rmin", "rmax", "ax")
    grads = {k: t.grad.double().cpu().numpy() for k, t in zip(names, data)}
    fw = {"x": x.detach().double().cpu().numpy(), "y": y.detach().double().cpu().numpy(),
          "obj": obj.detach().double().cpu().numpy()}
    w = {"x": wx.double().cpu().numpy(), "y": wy.double().cpu().numpy(),
         "obj": wo.double().cpu().numpy()}
    return P, fw, grads, w, tau.double().cpu().numpy(), sigma.double().cpu().numpy()


def split(P, v, kind):
    off = {"n": P.col_off, "m": P.row_off, "nz": P.nz_off}[kind]
    return [v[off[b]:off[b + 1]] for b in range(P.count)]


def relerr(a, b):
    """Norm-wise error relative to max(1, ||b||)."""
    return float(np.linalg.norm(a - b) / max(1.0, np.linalg.norm(b)))


def check_against_dense(lps, K, ck, tol_fw, tol_g):
    P, fw, g, w, tau, sigma = run(lps, K, ck)
    xs, ys = split(P, fw["x"], "n"), split(P, fw["y"], "m")
    for b, lp in enumerate(lps):
        ref_tau, ref_sigma = U.power_steps(lp)
        assert abs(tau[b] - ref_tau) <= 1e-6 * ref_tau
        out, rg = U.gradients(lp, tau[b], sigma[b], K, RIDGE, gx=split(P, w["x"], "n")[b],
                              gy=split(P, w["y"], "m")[b], gobj=w["obj"][b])
        assert relerr(xs[b], out["x"]) <= tol_fw
        assert relerr(ys[b], out["y"]) <= tol_fw
        assert abs(fw["obj"][b] - out["obj"]) <= tol_fw * max(1.0, abs(out["obj"]))
        for k, kind in (("c", "n"), ("cl", "n"), ("cu", "n"), ("rmin", "m"), ("rmax", "m"),
                        ("ax", "nz")):
            e = relerr(split(P, g[k], kind)[b], rg[k])
            assert e <= tol_g, (b, k, e)


def test_ragged_batch_matches_dense_fp64(native):
    check_against_dense(ragged(), K=200, ck=50, tol_fw=1e-11, tol_g=1e-9)


def test_c4_instance_matches_dense_fp64(native):
    check_against_dense(c4(2), K=1000, ck=50, tol_fw=1e-10, tol_g=1e-8)


def test_c4_gradients_match_central_fd(native):
    """Central differences (h = 1e-6, FP64 forward on the GPU) of obj and of
    <w, x_K> on a C4 instance (K = 1000) along single-coordinate and dense
    random directions in c, b (both bounds of an equality row, the finite
    one of an inequality row) and A's values. The unrolled map is smooth
    only between clamp kinks; a direction whose +-h points change a clamp
    outcome somewhere in the K iterations (the oracle's clamp trace) is not
    a fair check and is skipped. Every other direction must agree to 1e-6,
    and each class needs at least 4 of its 8 directions kink-free."""
    lp = c4(2, seed=5)[1]
    K, h = 1000, 1e-6
    rng = np.random.default_rng(2)
    c, cl, cu, rmin, rmax, ax = (np.asarray(getattr(lp, k), np.float64)
                                 for k in ("c", "cl", "cu", "rmin", "rmax", "ax"))
    P1 = BatchPattern.from_lps([lp], DEV)
    tau, sigma = pdhg_steps(P1, torch.tensor(ax, device=DEV))
    t0, s0 = float(tau[0]), float(sigma[0])
    wx = rng.standard_normal(lp.n)
    grads = {}
    for target in ("obj", "x"):
        data = [torch.tensor(v, device=DEV, requires_grad=True) for v in (c, cl, cu, rmin, rmax, ax)]
        x, y, obj = UnrolledPDHG.apply(*data, tau, sigma, P1, K, 50, RIDGE)
        (obj.sum() if target == "obj" else (torch.tensor(wx, device=DEV) * x).sum()).backward()
        grads[target] = [t.grad.cpu().numpy() for t in data]
    eq = rmin == rmax
    fin_hi = np.isfinite(rmax)
    dirs = []
    for cls, size in (("c", lp.n), ("b", lp.m), ("ax", lp.nnz)):
        for r in range(8):
            if r < 6:
                d = np.zeros(size)
                d[rng.integers(size)] = 1.0
            else:
                d = rng.standard_normal(size)
            z = lambda v: np.zeros_like(v)
            dirs.append((cls, d if cls == "c" else z(c),
                         np.where(eq, d, 0.0) if cls == "b" else z(rmin),
                         np.where(fin_hi, d, 0.0) if cls == "b" else z(rmax),
                         d if cls == "ax" else z(ax)))
    # every perturbed point in one batch: direction k at 2k (+h), 2k+1 (-h)
    pts = []
    for _, dc, dlo, dhi, dax in dirs:
        for sg in (1.0, -1.0):
            pts.append((c + sg * h * dc, cl, cu, rmin + sg * h * dlo, rmax + sg * h * dhi,
                        ax + sg * h * dax))
    P = BatchPattern.from_lps([lp] * len(pts), DEV)
    stack = [torch.tensor(np.concatenate([p[k] for p in pts]), device=DEV) for k in range(6)]
    T = torch.full((P.count,), t0, dtype=torch.float64, device=DEV)
    S = torch.full((P.count,), s0, dtype=torch.float64, device=DEV)
    with torch.no_grad():
        x, y, obj = UnrolledPDHG.apply(*stack, T, S, P, K, 50, RIDGE)
    vals = {"obj": obj.cpu().numpy(), "x": x.cpu().numpy().reshape(P.count, lp.n) @ wx}
    base_trace = U.clamp_trace(lp, t0, s0, K, RIDGE)
    free = {"c": 0, "b": 0, "ax": 0}
    for k, (cls, dc, dlo, dhi, dax) in enumerate(dirs):
        kinks = sum(U.kinks_crossed(lp, base_trace, U.clamp_trace(
            lp, t0, s0, K, RIDGE, ax=ax + sg * h * dax, c=c + sg * h * dc,
            rmin=rmin + sg * h * dlo, rmax=rmax + sg * h * dhi)) for sg in (1.0, -1.0))
        if kinks:
            continue
        free[cls] += 1
        for target in ("obj", "x"):
            g = grads[target]
            ana = g[0] @ dc + g[3] @ dlo + g[4] @ dhi + g[5] @ dax
            num = (vals[target][2 * k] - vals[target][2 * k + 1]) / (2 * h)
            assert abs(num - ana) <= 1e-6 * max(1.0, abs(ana)), (cls, k, target, num, ana)
    assert min(free.values()) >= 4, free


def test_envelope_theorem_at_convergence(native):
    lp = G.bernoulli_lp(np.random.default_rng(3), 8, 16, 0.3, 10.0)
    P = BatchPattern.from_lps([lp], DEV)
    data = [t.clone().requires_grad_(True) for t in stack_lps([lp], torch.float64, DEV)]
    x, y, obj = unrolled_lp(P, *data, iterations=10000, checkpoint=50, ridge=RIDGE)
    obj.sum().backward()
    xs, ys = x.detach().cpu().numpy(), y.detach().cpu().numpy()
    g = [t.grad.cpu().numpy() for t in data]
    rows = np.repeat(np.arange(lp.m), np.diff(lp.ap))
    eq = np.isfinite(lp.rmin)
    assert np.abs(g[0] - xs).max() <= 1e-6
    assert np.abs(np.where(eq, g[3] + g[4], g[4]) + ys).max() <= 1e-6
    assert np.abs(g[5] - ys[rows] * xs[lp.ai]).max() <= 1e-6


@pytest.mark.parametrize("K", [95, 200])
def test_checkpoint_interval_changes_nothing(native, K):
    lps = ragged(4)
    ref = run(lps, K, 50)
    for ck in (1, 7, K, 1000):
        got = run(lps, K, ck, tau=torch.tensor(ref[4], device=DEV),
                  sigma=torch.tensor(ref[5], device=DEV))
        for k in ref[2]:
            assert np.array_equal(got[2][k], ref[2][k]), (ck, k)
        assert np.array_equal(got[1]["x"], ref[1]["x"])


def test_repeatable_bit_for_bit(native):
    a = run(c4(3), 300, 50)
    b = run(c4(3), 300, 50)
    for k in a[2]:
        assert np.array_equal(a[2][k], b[2][k])


def test_fp32_close_to_fp64(native):
    lps = c4(4, seed=7)
    P64, f64, g64, _, tau, sigma = run(lps, 1000, 50, torch.float64)
    P32, f32, g32, _, _, _ = run(lps, 1000, 50, torch.float32,
                                 tau=torch.tensor(tau, dtype=torch.float32, device=DEV),
                                 sigma=torch.tensor(sigma, dtype=torch.float32, device=DEV))
    assert relerr(f32["x"], f64["x"]) <= 1e-4
    assert relerr(f32["obj"], f64["obj"]) <= 1e-4
    for k in ("c", "rmax", "ax"):
        assert relerr(g32[k], g64[k]) <= 1e-3, (k, relerr(g32[k], g64[k]))


def test_rejects_bad_inputs(native):
    lp = ragged()[0]
    P = BatchPattern.from_lps([lp], DEV)
    data = stack_lps([lp], torch.float16, DEV)
    with pytest.raises(TypeError):
        unrolled_lp(P, *data, tau=torch.ones(1, device=DEV), sigma=torch.ones(1, device=DEV))
    data = stack_lps([lp], torch.float64, DEV)
    with pytest.raises(ValueError, match="shape"):
        unrolled_lp(P, data[0][:-1], *data[1:], tau=torch.ones(1, dtype=torch.float64, device=DEV),
                    sigma=torch.ones(1, dtype=torch.float64, device=DEV))
    big = G.from_triplets(4000, 4000, np.arange(4000), np.arange(4000), np.ones(4000),
                          np.zeros(4000), np.zeros(4000), np.ones(4000), np.zeros(4000),
                          np.ones(4000))
    Pb = BatchPattern.from_lps([big], DEV)
    with pytest.raises(capi.EngineError, match="too large"):
        pdhg_steps(Pb, stack_lps([big], torch.float64, DEV)[5])
