"""Kernel-level parity of the CUDA engine against the CPU oracle, through the
C ABI (include/igaos_pdhg.h). Integer/structure work must be bit-exact; FP64
arithmetic within stated tolerances (summation order differs from a
sequential loop); FP32 arithmetic within FP32 rounding of its inputs.

Reference items covered: Ruiz scaling (src/pdhg/pdhg.cu:472-492), scaled
problem (:499-513), A^T build (src/io/model.hpp:39-67), SpMV (:143-157),
power iteration (:605-631), step init (:642-663), the iteration with its
line search and averaging (:748-799), evaluate (:173-254).
"""
import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu


def _matrices():
    rng = np.random.default_rng(7)
    out = {
        "rand": G.random_lp(300, 700, 2500, 1),
        "zipf": G.config2(seed=2, m=3000, n=8000, target_nnz=60000),
        "grid": G.config5(seed=3, side=12, commodities=3),
        "mixed": G.mixed_bounds_lp(120, 300, 700, 4),
    }
    # long rows (> one 2048-nonzero tile) and empty rows/columns
    m, n = 40, 6000
    rows = np.concatenate([np.zeros(5000, int), np.full(3000, 7), rng.integers(10, 40, 800)])
    cols = np.concatenate([rng.permutation(n)[:5000], rng.permutation(n)[:3000],
                           rng.integers(0, n, 800)])
    key = np.unique(cols * 1000 + rows)
    rows, cols = key % 1000, key // 1000
    lp = G.from_triplets(m, n, rows, cols, rng.standard_normal(rows.size), rng.standard_normal(n),
                         np.zeros(n), np.full(n, 2.0), np.full(m, -1.0), np.full(m, 1.0),
                         presorted=True)
    out["longrows"] = lp
    return out


MATS = _matrices()


@pytest.fixture(scope="module", params=sorted(MATS))
def case(request, native, orc):
    from igaos_gb300 import capi
    lp = MATS[request.param]
    olp = orc.lp_from(lp)
    with capi.Problem(lp) as P:
        yield request.param, lp, olp, P


def test_ruiz_scaling_bit_exact(case, orc):
    _, lp, olp, P = case
    dr, dc = P.scaling()
    rdr, rdc = orc.ruiz(olp)
    assert np.array_equal(dr, rdr)
    assert np.array_equal(dc, rdc)


def test_transpose_and_scaled_values_bit_exact(case, orc, native):
    from igaos_gb300 import capi
    name, lp, olp, P = case
    sd = orc.scale(olp, *orc.ruiz(olp))
    cp, ci, acx = P.transpose()
    assert np.array_equal(cp, olp.cp) and np.array_equal(ci, olp.ci)
    assert np.array_equal(acx, sd["sacx"])
    # the same when A^T is built by the engine from the CSR alone
    with capi.Problem(lp, with_transpose=False) as Q:
        cp2, ci2, acx2 = Q.transpose()
    tcp, tci, tacx = orc.transpose(lp.m, lp.n, lp.ap, lp.ai, lp.ax)
    assert np.array_equal(cp2, tcp) and np.array_equal(ci2, tci)
    assert np.array_equal(acx2, orc.scale(orc.LP(**{**olp.__dict__, "cp": tcp, "ci": tci,
                                                    "acx": tacx}), *orc.ruiz(olp))["sacx"])


def test_spmv_fp64_and_fp32(case, orc):
    name, lp, olp, P = case
    sd = orc.scale(olp, *orc.ruiz(olp))
    rng = np.random.default_rng(3)
    for transpose in (False, True):
        ptr, idx, val = (olp.cp, olp.ci, sd["sacx"]) if transpose else (olp.ap, olp.ai, sd["sax"])
        x = rng.standard_normal(lp.m if transpose else lp.n)
        ref = orc.spmv(ptr, idx, val, x)
        mag = orc.spmv(ptr, idx, np.abs(val), np.abs(x)) + 1e-300
        y64 = P.spmv(x, transpose=transpose, precision="fp64")
        assert np.all(np.abs(y64 - ref) <= 1e-14 * mag), np.max(np.abs(y64 - ref) / mag)
        y32 = P.spmv(x, transpose=transpose, precision="fp32")
        # inputs rounded to FP32 (2 x 2^-24 relative per product) + one final
        # rounding of the compensated sum
        tol = 2.5 * 2.0 ** -24 * mag + 2.0 ** -24 * np.abs(ref)
        assert np.all(np.abs(y32 - ref) <= tol), np.max(np.abs(y32 - ref) / mag)


@pytest.mark.parametrize("name", sorted(MATS))
def test_spmv_grid_kernels_padded_rows(native, orc, monkeypatch, name):
    """With the cluster path off, the FP32 copy of A has rows padded to 4k
    entries and lanes read 4-entry chunks with 16-byte loads (dealt to the
    G lanes of a row in turn; the long-row case has G = 32). Same bounds as
    the unpadded products."""
    from igaos_gb300 import capi
    monkeypatch.setenv("IGAOS_PDHG_CLUSTER", "0")
    lp = MATS[name]
    olp = orc.lp_from(lp)
    sd = orc.scale(olp, *orc.ruiz(olp))
    rng = np.random.default_rng(5)
    with capi.Problem(lp) as P:
        for transpose in (False, True):
            ptr, idx, val = (olp.cp, olp.ci, sd["sacx"]) if transpose else (olp.ap, olp.ai, sd["sax"])
            x = rng.standard_normal(lp.m if transpose else lp.n)
            ref = orc.spmv(ptr, idx, val, x)
            mag = orc.spmv(ptr, idx, np.abs(val), np.abs(x)) + 1e-300
            y32 = P.spmv(x, transpose=transpose, precision="fp32")
            tol = 2.5 * 2.0 ** -24 * mag + 2.0 ** -24 * np.abs(ref)
            assert np.all(np.abs(y32 - ref) <= tol), np.max(np.abs(y32 - ref) / mag)
            y64 = P.spmv(x, transpose=transpose, precision="fp64")
            assert np.all(np.abs(y64 - ref) <= 1e-14 * mag)


def test_step_init(case, orc):
    _, lp, olp, P = case
    sd = orc.scale(olp, *orc.ruiz(olp))
    lam = orc.power_iteration(olp, sd)
    lam_g, eta0, omega0 = P.step_init()
    assert lam_g == pytest.approx(lam, rel=1e-9)
    assert eta0 == pytest.approx(1.2 / np.sqrt(lam), rel=1e-9)
    sc = sd["sc"]
    q = np.where(np.isfinite(sd["srmax"]), sd["srmax"], np.where(np.isfinite(sd["srmin"]), sd["srmin"], 0.0))
    cn, qn = float(sc @ sc), float(q @ q)
    want = np.clip(np.sqrt(cn / qn), 0.3, 3.0) if cn > 1e-24 and qn > 1e-24 else 1.0
    assert omega0 == pytest.approx(want, rel=1e-12)


@pytest.mark.parametrize("iters", [1, 7, 64])
def test_iterations_fp64_match_oracle(case, orc, iters):
    name, lp, olp, P = case
    sd = orc.scale(olp, *orc.ruiz(olp))
    _, eta0, omega0 = P.step_init()
    z = lambda k: np.zeros(k)
    st0 = dict(x=z(lp.n), y=z(lp.m), xavg=z(lp.n), yavg=z(lp.m), axcur=z(lp.m), eta=eta0,
               omega=omega0, k=1, hn=0)
    want, att = orc.iterate(olp, sd, st0, iters)
    got = P.iterate(st0, iters, "fp64")
    assert got["k"] == want["k"] and got["hn"] == want["hn"]
    assert got["attempts"] == att  # same accept/reject sequence
    assert got["eta"] == pytest.approx(want["eta"], rel=1e-9)
    for key in ("x", "y", "xavg", "yavg", "axcur"):
        scale = max(1.0, float(np.max(np.abs(want[key]))))
        assert np.max(np.abs(got[key] - want[key])) <= 1e-9 * scale, key


def test_iterations_fp32_track_oracle(case, orc):
    name, lp, olp, P = case
    sd = orc.scale(olp, *orc.ruiz(olp))
    _, eta0, omega0 = P.step_init()
    z = lambda k: np.zeros(k)
    st0 = dict(x=z(lp.n), y=z(lp.m), xavg=z(lp.n), yavg=z(lp.m), axcur=z(lp.m), eta=eta0,
               omega=omega0, k=1, hn=0)
    want, _ = orc.iterate(olp, sd, st0, 5)
    got = P.iterate(st0, 5, "fp32")
    assert got["k"] == want["k"]
    for key in ("x", "y"):
        scale = max(1.0, float(np.max(np.abs(want[key]))))
        assert np.max(np.abs(got[key] - want[key])) <= 2e-4 * scale, key


def test_evaluate_matches_oracle(case, orc):
    name, lp, olp, P = case
    rng = np.random.default_rng(11)
    A = lp.dense() if lp.m * lp.n < 3e6 else None
    for trial in range(3):
        lo = np.where(np.isfinite(lp.cl), lp.cl, -3.0)
        hi = np.where(np.isfinite(lp.cu), lp.cu, 3.0)
        x = rng.uniform(lo, hi)
        pick = rng.random(lp.n) < 0.3
        x[pick & np.isfinite(lp.cl)] = lp.cl[pick & np.isfinite(lp.cl)]
        y = rng.standard_normal(lp.m) * (rng.random(lp.m) < 0.5)
        if trial == 0:  # sign-consistent dual: finite bound
            y = np.where(y > 0, np.where(np.isfinite(lp.rmax), y, 0), np.where(np.isfinite(lp.rmin), y, 0))
        Ax = orc.spmv(olp.ap, olp.ai, olp.ax, x)
        d = lp.c + orc.spmv(olp.cp, olp.ci, olp.acx, y)
        want = orc.evaluate(olp, x, y, Ax, d)
        got = P.evaluate(x, y)
        for k in ("pinf", "prow", "dinf", "op", "od", "gap"):
            w, g = want[k], got[k]
            if np.isinf(w):
                assert g == w, k
            else:
                assert g == pytest.approx(w, rel=1e-9, abs=1e-9), (k, g, w)


def test_gather_rate_calibration(native):
    """The gather-bound roofline's ceiling: random reads of an L1-resident
    vector are served faster than of an L2-resident one, and those faster
    than of an HBM-resident one; all rates are positive and finite."""
    from igaos_gb300 import capi
    l1, l2, hbm = capi.gather_rate(14), capi.gather_rate(19), capi.gather_rate(28)
    assert all(np.isfinite(v) and v > 1e9 for v in (l1, l2, hbm)), (l1, l2, hbm)
    assert l1 > l2 > hbm, (l1, l2, hbm)


def test_spmv_fp64_matches_cusparse(case, orc):
    """The reference computes A x and A^T y with cusparseSpMV (FP64 CSR,
    src/pdhg/pdhg.cu:143-157). The same products through cuSPARSE (torch's
    CSR matvec) on the same scaled matrices agree with the engine's FP64
    products to 1e-14 of the sum of |terms| (only the summation order
    differs)."""
    torch = pytest.importorskip("torch")
    name, lp, olp, P = case
    sd = orc.scale(olp, *orc.ruiz(olp))
    rng = np.random.default_rng(5)
    dev = torch.device("cuda:0")
    for transpose in (False, True):
        ptr, idx, val = (olp.cp, olp.ci, sd["sacx"]) if transpose else (olp.ap, olp.ai, sd["sax"])
        rows, cols = (lp.n, lp.m) if transpose else (lp.m, lp.n)
        x = rng.standard_normal(cols)
        A = torch.sparse_csr_tensor(torch.as_tensor(np.asarray(ptr, np.int64), device=dev),
                                    torch.as_tensor(np.asarray(idx, np.int64), device=dev),
                                    torch.as_tensor(np.asarray(val, np.float64), device=dev),
                                    size=(rows, cols))
        want = (A @ torch.as_tensor(x, device=dev)).cpu().numpy()
        mag = orc.spmv(ptr, idx, np.abs(val), np.abs(x)) + 1e-300
        got = P.spmv(x, transpose=transpose, precision="fp64")
        assert np.all(np.abs(got - want) <= 1e-14 * mag), np.max(np.abs(got - want) / mag)
