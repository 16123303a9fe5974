"""Differentiable LP layer over the engine's unrolled-PDHG entry points.

A batch of ridge-regularised LPs

    min c^T x + ridge ||x||^2   s.t.  rmin <= A x <= rmax,  cl <= x <= cu

is run for K PDHG iterations with fixed steps (one CTA per instance, CUDA
kernels behind ``igaos_pdhg_unrolled_forward``); the backward is the exact
reverse mode of those K iterations (``igaos_pdhg_unrolled_backward``), with
checkpoints every ``checkpoint`` iterations and replay in between. Outputs
are x_K, y_K and obj = c^T x_K + ridge ||x_K||^2 per instance; gradients flow
to c, cl, cu, rmin, rmax and the CSR values of A. The sign convention is the
reference engine's (reduced cost d = c + A^T y, src/pdhg/pdhg.cu:33-58), so
at convergence d obj/d c = x*, d obj/d b_i = -y_i, d obj/d A_ij = y_i x*_j.

Vectors are flat concatenations over the batch (instance b's columns at
col_off[b]:col_off[b+1], rows at row_off[b]:row_off[b+1], nonzeros at
nz_off[b]:nz_off[b+1]); float32 and float64 tensors select the FP32 and FP64
kernels. PyTorch supplies device memory and the stream only; there is no CPU
path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import capi


class BatchPattern:
    """Sparsity layout of a batch (fixed across calls): per-instance CSR
    (row pointers local to the instance) and its transpose as CSC with each
    entry's CSR position, uploaded once as int32 device tensors."""

    def __init__(self, ms, ns, aps, ais, device="cuda"):
        self.count = len(ms)
        if self.count == 0:
            raise ValueError("empty batch")
        ms = [int(v) for v in ms]
        ns = [int(v) for v in ns]
        if min(ms) < 1 or min(ns) < 1:
            raise ValueError("every instance needs m >= 1 and n >= 1")
        nnz = [int(np.asarray(a)[-1]) for a in aps]
        self.row_off = np.concatenate([[0], np.cumsum(ms)]).astype(np.int64)
        self.col_off = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        self.nz_off = np.concatenate([[0], np.cumsum(nnz)]).astype(np.int64)
        if max(self.row_off[-1], self.col_off[-1], self.nz_off[-1]) >= 2 ** 31:
            raise ValueError("batch too large for int32 offsets")
        cps, cis, cperms = [], [], []
        for m, n, ap, ai in zip(ms, ns, aps, ais):
            ap = np.asarray(ap, np.int64)
            ai = np.asarray(ai, np.int64)
            if ap.shape[0] != m + 1 or ap[0] != 0 or np.any(np.diff(ap) < 0):
                raise ValueError("bad row pointer")
            if ai.size and (ai.min() < 0 or ai.max() >= n):
                raise ValueError("column index out of range")
            rows = np.repeat(np.arange(m), np.diff(ap))
            perm = np.lexsort((rows, ai))  # by column, then row
            cnt = np.bincount(ai, minlength=n)
            cps.append(np.concatenate([[0], np.cumsum(cnt)]))
            cis.append(rows[perm])
            cperms.append(perm)
        i32 = lambda parts: torch.from_numpy(np.concatenate(parts).astype(np.int32)).to(device)
        self.t_row_off = i32([self.row_off])
        self.device = self.t_row_off.device  # with its index ("cuda" -> "cuda:0")
        self.t_col_off = i32([self.col_off])
        self.t_nz_off = i32([self.nz_off])
        self.t_ap = i32([np.asarray(a, np.int64) for a in aps])
        self.t_ai = i32([np.asarray(a, np.int64) for a in ais])
        self.t_cp = i32(cps)
        self.t_ci = i32(cis)
        self.t_cperm = i32(cperms)
        self.max_m, self.max_n, self.max_nnz = max(ms), max(ns), max(nnz)
        self.total_m, self.total_n = int(self.row_off[-1]), int(self.col_off[-1])
        self.total_nnz = int(self.nz_off[-1])

    @classmethod
    def from_lps(cls, lps, device="cuda"):
        return cls([lp.m for lp in lps], [lp.n for lp in lps], [lp.ap for lp in lps],
                   [lp.ai for lp in lps], device)

    def layout(self, dtype, iterations, checkpoint, ridge) -> capi.UnrolledLayout:
        L = capi.UnrolledLayout()
        L.count = self.count
        L.precision = capi.FP64 if dtype == torch.float64 else capi.FP32
        L.iterations = int(iterations)
        L.checkpoint = int(checkpoint)
        L.ridge = float(ridge)
        L.max_m, L.max_n, L.max_nnz = self.max_m, self.max_n, self.max_nnz
        L.total_m, L.total_n, L.total_nnz = self.total_m, self.total_n, self.total_nnz
        for f in ("row_off", "col_off", "nz_off", "ap", "ai", "cp", "ci", "cperm"):
            setattr(L, f, getattr(self, "t_" + f).data_ptr())
        return L


def stack_lps(lps, dtype=torch.float32, device="cuda"):
    """(c, cl, cu, rmin, rmax, ax) of a list of LPData as flat device tensors."""
    cat = lambda f: torch.from_numpy(np.concatenate([getattr(lp, f) for lp in lps])).to(
        device=device, dtype=dtype)
    return tuple(cat(f) for f in ("c", "cl", "cu", "rmin", "rmax", "ax"))


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(device):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _check_vec(name, t, n, dtype, device):
    if not isinstance(t, torch.Tensor) or t.device != device or t.dtype != dtype:
        raise TypeError(f"{name} must be a {dtype} tensor on {device}")
    if t.dim() != 1 or t.shape[0] != n:
        raise ValueError(f"{name} must have shape ({n},), got {tuple(t.shape)}")
    return t.contiguous()


def pdhg_steps(pattern: BatchPattern, ax: torch.Tensor, omega: float = 1.0):
    """Fixed steps per instance: eta = 0.9 / ||A||_2 (power iteration),
    tau = eta / omega, sigma = eta * omega. Not differentiated."""
    dtype = ax.dtype
    ax = _check_vec("ax", ax.detach(), pattern.total_nnz, dtype, pattern.device)
    tau = torch.empty(pattern.count, dtype=dtype, device=pattern.device)
    sigma = torch.empty_like(tau)
    L = pattern.layout(dtype, 1, 1, 0.0)
    capi._check(capi.lib().igaos_pdhg_unrolled_steps(C.byref(L), _ptr(ax), float(omega),
                                                     _ptr(tau), _ptr(sigma),
                                                     _stream(pattern.device)))
    return tau, sigma


class UnrolledPDHG(torch.autograd.Function):
    """(c, cl, cu, rmin, rmax, ax, tau, sigma) -> (x_K, y_K, obj)."""

    @staticmethod
    def forward(ctx, c, cl, cu, rmin, rmax, ax, tau, sigma, pattern, iterations, checkpoint,
                ridge):
        P = pattern
        dtype, dev = c.dtype, P.device
        if dtype not in (torch.float32, torch.float64):
            raise TypeError("the layer computes in float32 or float64")
        c = _check_vec("c", c, P.total_n, dtype, dev)
        cl = _check_vec("cl", cl, P.total_n, dtype, dev)
        cu = _check_vec("cu", cu, P.total_n, dtype, dev)
        rmin = _check_vec("rmin", rmin, P.total_m, dtype, dev)
        rmax = _check_vec("rmax", rmax, P.total_m, dtype, dev)
        ax = _check_vec("ax", ax, P.total_nnz, dtype, dev)
        tau = _check_vec("tau", tau.detach(), P.count, dtype, dev)
        sigma = _check_vec("sigma", sigma.detach(), P.count, dtype, dev)
        L = P.layout(dtype, iterations, checkpoint, ridge)
        lib = capi.lib()
        nck = lib.igaos_pdhg_unrolled_checkpoint_elems(C.byref(L))
        if nck < 0:
            raise capi.EngineError(capi.ERR_INVALID, capi.last_error())
        x = torch.empty(P.total_n, dtype=dtype, device=dev)
        y = torch.empty(P.total_m, dtype=dtype, device=dev)
        obj = torch.empty(P.count, dtype=dtype, device=dev)
        ckpt = torch.empty(nck, dtype=dtype, device=dev)
        capi._check(lib.igaos_pdhg_unrolled_forward(
            C.byref(L), _ptr(c), _ptr(cl), _ptr(cu), _ptr(rmin), _ptr(rmax), _ptr(ax),
            _ptr(tau), _ptr(sigma), _ptr(x), _ptr(y), _ptr(obj), _ptr(ckpt), _stream(dev)))
        ctx.save_for_backward(c, cl, cu, rmin, rmax, ax, tau, sigma, ckpt, x)
        ctx.cfg = (P, iterations, checkpoint, ridge)
        return x, y, obj

    @staticmethod
    def backward(ctx, gx, gy, gobj):
        c, cl, cu, rmin, rmax, ax, tau, sigma, ckpt, x = ctx.saved_tensors
        P, iterations, checkpoint, ridge = ctx.cfg
        dtype, dev = c.dtype, P.device
        L = P.layout(dtype, iterations, checkpoint, ridge)
        lib = capi.lib()
        fix = lambda g: None if g is None else g.to(dtype).contiguous()
        gx, gy, gobj = fix(gx), fix(gy), fix(gobj)
        outs = [torch.empty(P.total_n, dtype=dtype, device=dev) for _ in range(3)]
        outs += [torch.empty(P.total_m, dtype=dtype, device=dev) for _ in range(2)]
        outs.append(torch.empty(P.total_nnz, dtype=dtype, device=dev))
        wb = lib.igaos_pdhg_unrolled_workspace_bytes(C.byref(L))
        if wb < 0:
            raise capi.EngineError(capi.ERR_INVALID, capi.last_error())
        work = torch.empty(max(1, wb), dtype=torch.uint8, device=dev)
        capi._check(lib.igaos_pdhg_unrolled_backward(
            C.byref(L), _ptr(c), _ptr(cl), _ptr(cu), _ptr(rmin), _ptr(rmax), _ptr(ax),
            _ptr(tau), _ptr(sigma), _ptr(ckpt), _ptr(x), _ptr(gx), _ptr(gy), _ptr(gobj),
            *[_ptr(o) for o in outs], _ptr(work), _stream(dev)))
        gc, gcl, gcu, grmin, grmax, gax = outs
        return gc, gcl, gcu, grmin, grmax, gax, None, None, None, None, None, None


def unrolled_lp(pattern: BatchPattern, c, cl, cu, rmin, rmax, ax, iterations: int = 1000,
                checkpoint: int = 50, ridge: float = 0.005, omega: float = 1.0, tau=None,
                sigma=None):
    """K = `iterations` PDHG iterations of the ridge-regularised batch;
    returns (x_K, y_K, obj). Steps default to pdhg_steps(pattern, ax, omega)."""
    if tau is None or sigma is None:
        tau, sigma = pdhg_steps(pattern, ax, omega)
    return UnrolledPDHG.apply(c, cl, cu, rmin, rmax, ax, tau, sigma, pattern, int(iterations),
                              int(checkpoint), float(ridge))
