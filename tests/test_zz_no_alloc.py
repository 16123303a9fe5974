"""igaos_pdhg_evaluate_noalloc: the allocation-free KKT evaluation for
callers that cannot call cudaMalloc (their device memory belongs to a
framework allocator or a fixed pool, or an allocation's device
synchronisation is not acceptable where they run). The caller owns every
buffer -- here torch allocates them, as such a caller's framework would --
and the engine adds none.

Checked through the C ABI against the existing entry point
igaos_pdhg_evaluate on the same candidates, twice in a row (the scratch array
is shared between calls and keeps the previous call's contents), and against
the oracle's restatement of the reference evaluate() (src/pdhg/pdhg.cu:
173-254) on A x and c + A^T y formed in FP64 by numpy. This file
sorts last so that a run stopping at the first failure has run every other
test first; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _candidates(lp, seed):
    rng = np.random.default_rng(seed)
    lo = np.where(np.isfinite(lp.cl), lp.cl, -3.0)
    hi = np.where(np.isfinite(lp.cu), lp.cu, 3.0)
    out = []
    for trial in range(2):
        x = rng.uniform(lo, hi)
        pick = rng.random(lp.n) < 0.3
        x[pick & np.isfinite(lp.cl)] = lp.cl[pick & np.isfinite(lp.cl)]
        y = rng.standard_normal(lp.m) * (rng.random(lp.m) < 0.5)
        if trial == 0:  # sign-consistent dual: a finite bound and gap
            y = np.where(y > 0, np.where(np.isfinite(lp.rmax), y, 0),
                         np.where(np.isfinite(lp.rmin), y, 0))
        out.append((x, y))
    return out


def test_noalloc_evaluate_matches_evaluate_twice(native, orc):
    import scipy.sparse as sp
    import torch
    from igaos_gb300 import capi, generators as G
    assert torch.cuda.is_available()
    dev = torch.device("cuda", 0)
    lp = G.mixed_bounds_lp(120, 300, 700, 4)
    gen = G.config2(seed=2, m=3000, n=8000, target_nnz=60000)
    for prob in (lp, gen):
        t = {k: torch.as_tensor(np.ascontiguousarray(getattr(prob, k)), device=dev)
             for k in ("ap", "ai", "cp", "ci")}
        t.update({k: torch.as_tensor(np.ascontiguousarray(getattr(prob, k), np.float64), device=dev)
                  for k in ("ax", "acx", "c", "cl", "cu", "rmin", "rmax")})
        for k in ("ap", "ai", "cp", "ci"):
            t[k] = t[k].to(torch.int32)
        out = torch.empty(6, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        olp = orc.lp_from(prob)
        A = sp.csr_matrix((olp.ax, olp.ai, olp.ap), shape=(olp.m, olp.n))
        with capi.Problem(prob) as P:
            for x, y in _candidates(prob, 7):
                want = P.evaluate(x, y)
                ref = orc.evaluate(olp, x, y, A @ x, olp.c + A.T @ y)
                tx = torch.as_tensor(x, dtype=torch.float64, device=dev)
                ty = torch.as_tensor(y, dtype=torch.float64, device=dev)
                got_runs = []
                for _ in range(2):
                    out.fill_(float("nan"))
                    ptrs = [t[k].data_ptr() for k in ("ap", "ai", "ax", "cp", "ci", "acx", "c",
                                                      "cl", "cu", "rmin", "rmax")]
                    rc = native.igaos_pdhg_evaluate_noalloc(
                        prob.m, prob.n, *[C.c_void_p(p) for p in ptrs],
                        C.c_void_p(tx.data_ptr()), C.c_void_p(ty.data_ptr()),
                        C.c_void_p(out.data_ptr()), C.c_void_p(stream))
                    assert rc == capi.OK, capi.last_error()
                    torch.cuda.synchronize(dev)
                    got_runs.append(dict(zip(("pinf", "dinf", "gap", "op", "od", "prow"),
                                             out.cpu().tolist())))
                assert got_runs[0] == got_runs[1]  # deterministic, scratch reuse is clean
                got = got_runs[0]
                for k in ("pinf", "prow", "dinf", "op", "od", "gap"):
                    for w in (want, ref):
                        if np.isinf(w[k]):
                            assert got[k] == w[k], k
                        else:
                            assert got[k] == pytest.approx(w[k], rel=1e-9, abs=1e-9), (k, got[k], w[k])


def test_noalloc_rejects_sizes_beyond_its_scratch(native):
    from igaos_gb300 import capi
    null = [C.c_void_p(0)] * 15
    rc = native.igaos_pdhg_evaluate_noalloc(5_000_000, 10, *null)
    assert rc == capi.ERR_INVALID
    assert "4,194,304" in capi.last_error()
