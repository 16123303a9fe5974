"""Dense FP64 checker of the differentiable LP layer (test infrastructure).

Only tests, smoke() and bench.py's CPU baseline use this module; the product
never imports it.

It restates, with dense torch FP64 tensors on the CPU, the K fixed-step PDHG
iterations that the layer unrolls -- the reference engine's primal and dual
steps (kern_primal, kern_dual in src/pdhg/pdhg.cu:33-58) with the ridge term
ridge ||x||^2 folded into the primal prox -- and lets torch autograd
differentiate them. Clamps use the layer's convention: the gradient passes to
the argument where it lies inside the bounds (ties included) and to the
bound where it lies strictly outside.
"""
from __future__ import annotations

import numpy as np
import torch


def _clamp(v, lo, hi):
    return torch.where(v < lo, lo, torch.where(v > hi, hi, v))


def unrolled(A, c, cl, cu, rmin, rmax, tau, sigma, iterations, ridge):
    """x_K, y_K, obj of one instance (dense A, all float64 tensors)."""
    kappa = 1.0 / (1.0 + 2.0 * ridge * tau)
    x = _clamp(torch.zeros_like(c), cl, cu)
    y = torch.zeros_like(rmin)
    for _ in range(iterations):
        g = c + A.T @ y
        xn = _clamp((x - tau * g) * kappa, cl, cu)
        xb = 2.0 * xn - x
        t = y + sigma * (A @ xb)
        y = t - sigma * _clamp(t / sigma, rmin, rmax)
        x = xn
    obj = c @ x + ridge * (x @ x)
    return x, y, obj


def dense_of(lp):
    """Dense A of an LPData plus the CSR coordinates of its nonzeros."""
    rows = np.repeat(np.arange(lp.m), np.diff(lp.ap))
    A = np.zeros((lp.m, lp.n))
    A[rows, lp.ai] = lp.ax
    return A, rows, np.asarray(lp.ai)


def gradients(lp, tau, sigma, iterations, ridge, gx=None, gy=None, gobj=1.0):
    """Forward outputs and gradients of <gx,x_K> + <gy,y_K> + gobj*obj with
    respect to (c, cl, cu, rmin, rmax, ax) for one LPData instance."""
    A0, rows, cols = dense_of(lp)
    f64 = lambda a: torch.tensor(np.asarray(a, np.float64), requires_grad=True)
    A = torch.tensor(A0, requires_grad=True)
    c, cl, cu, rmin, rmax = (f64(getattr(lp, k)) for k in ("c", "cl", "cu", "rmin", "rmax"))
    x, y, obj = unrolled(A, c, cl, cu, rmin, rmax, float(tau), float(sigma), iterations, ridge)
    loss = gobj * obj
    if gx is not None:
        loss = loss + torch.as_tensor(gx, dtype=torch.float64) @ x
    if gy is not None:
        loss = loss + torch.as_tensor(gy, dtype=torch.float64) @ y
    loss.backward()
    g = {k: v.grad.numpy().copy() for k, v in
         (("c", c), ("cl", cl), ("cu", cu), ("rmin", rmin), ("rmax", rmax))}
    g["ax"] = A.grad.numpy()[rows, cols].copy()
    out = {"x": x.detach().numpy(), "y": y.detach().numpy(), "obj": float(obj.detach())}
    return out, g


def forward(lp, tau, sigma, iterations, ridge, ax=None, **override):
    """Forward only (no graph); `ax`/`override` replace data (finite differences)."""
    A0, rows, cols = dense_of(lp)
    if ax is not None:
        A0 = np.zeros_like(A0)
        A0[rows, cols] = ax
    t = lambda k: torch.tensor(np.asarray(override.get(k, getattr(lp, k)), np.float64))
    with torch.no_grad():
        x, y, obj = unrolled(torch.tensor(A0), t("c"), t("cl"), t("cu"), t("rmin"), t("rmax"),
                             float(tau), float(sigma), iterations, ridge)
    return x.numpy(), y.numpy(), float(obj)


def clamp_trace(lp, tau, sigma, iterations, ridge, ax=None, **override):
    """Clamp outcomes of every iteration (0 inside, 1 below, 2 above) for the
    primal (K x n) and the dual (K x m) prox, FP64 sparse arithmetic. Two
    parameter points whose traces agree lie on one smooth piece of the
    unrolled map, where central differences are exact to O(h^2)."""
    import scipy.sparse as sp
    A = sp.csr_matrix((lp.ax if ax is None else ax, lp.ai, lp.ap), shape=(lp.m, lp.n))
    AT = A.T.tocsr()
    g = lambda k: np.asarray(override.get(k, getattr(lp, k)), np.float64)
    c, cl, cu, rmin, rmax = g("c"), g("cl"), g("cu"), g("rmin"), g("rmax")
    kappa = 1.0 / (1.0 + 2.0 * ridge * tau)
    x = np.where(0.0 < cl, cl, np.where(0.0 > cu, cu, 0.0))
    y = np.zeros(lp.m)
    fx = np.empty((iterations, lp.n), np.int8)
    fy = np.empty((iterations, lp.m), np.int8)
    for k in range(iterations):
        v = (x - tau * (c + AT @ y)) * kappa
        fx[k] = np.where(v < cl, 1, np.where(v > cu, 2, 0))
        xn = np.where(fx[k] == 1, cl, np.where(fx[k] == 2, cu, v))
        t = y + sigma * (A @ (2.0 * xn - x))
        q = t / sigma
        fy[k] = np.where(q < rmin, 1, np.where(q > rmax, 2, 0))
        y = t - sigma * np.where(fy[k] == 1, rmin, np.where(fy[k] == 2, rmax, q))
        x = xn
    return fx, fy


def kinks_crossed(lp, a, b):
    """Clamp outcomes that differ between traces a and b; a dual row with
    rmin == rmax flipping between below and above is no kink (the prox is
    the same affine map on both sides)."""
    eq = np.asarray(lp.rmin) == np.asarray(lp.rmax)
    dy = (a[1] != b[1]) & ~(eq[None, :] & (a[1] != 0) & (b[1] != 0))
    return int((a[0] != b[0]).sum() + dy.sum())


def power_steps(lp, omega=1.0, its=100):
    """eta = 0.9/||A||_2 by the layer's power iteration (dense FP64)."""
    A, _, _ = dense_of(lp)
    v = np.full(lp.n, 1.0 / np.sqrt(lp.n))
    lam = 0.0
    for _ in range(its):
        u = A.T @ (A @ v)
        lam = float(np.linalg.norm(u))
        if not lam > 0:
            break
        v = u / lam
    eta = 0.9 / np.sqrt(lam) if lam > 0 else 1.0
    return eta / omega, eta * omega
