"""Small LPs run each chunk of line-search attempts in one thread-block
cluster with the LP in shared memory (k_attempts_cluster, csrc/cluster.cuh):
FP32 attempts by default, FP64 ones with IGAOS_PDHG_CLUSTER=all;
IGAOS_PDHG_CLUSTER=0 keeps the grid-wide kernels. Both paths are held to the oracle's iteration
(src/pdhg/pdhg.cu:748-799): the same accept/reject sequence and FP64
iterates within 1e-9, and both solve to the same optimum.
"""
import numpy as np
import pytest

from igaos_gb300 import generators as G

pytestmark = pytest.mark.gpu

CASES = {
    "rand": lambda: G.random_lp(300, 700, 2500, 1),
    "mixed": lambda: G.mixed_bounds_lp(120, 300, 700, 4),
    "small": lambda: G.config1(seed=1),
}


def use_path(monkeypatch, path):
    # FP32 attempts take the cluster path by default, FP64 ones only with "all"
    monkeypatch.setenv("IGAOS_PDHG_CLUSTER", "all" if path == "cluster" else "0")


@pytest.fixture(params=["cluster", "grid"])
def path(request, monkeypatch):
    use_path(monkeypatch, request.param)
    return request.param


@pytest.mark.parametrize("name", sorted(CASES))
def test_iterations_match_oracle_on_both_paths(native, orc, path, name):
    from igaos_gb300 import capi
    lp = CASES[name]()
    olp = orc.lp_from(lp)
    sd = orc.scale(olp, *orc.ruiz(olp))
    with capi.Problem(lp) as P:
        _, eta0, omega0 = P.step_init()
        z = lambda k: np.zeros(k)
        st0 = dict(x=z(lp.n), y=z(lp.m), xavg=z(lp.n), yavg=z(lp.m), axcur=z(lp.m), eta=eta0,
                   omega=omega0, k=1, hn=0)
        got = P.iterate(st0, 64, "fp64")
    want, att = orc.iterate(olp, sd, st0, 64)
    assert got["k"] == want["k"] and got["hn"] == want["hn"]
    assert got["attempts"] == att
    for key in ("x", "y", "xavg", "yavg", "axcur"):
        scale = max(1.0, float(np.max(np.abs(want[key]))))
        assert np.max(np.abs(got[key] - want[key])) <= 1e-9 * scale, key


@pytest.mark.parametrize("precision", ["fp64", "fp32-refine"])
def test_small_lp_solves_alike_on_both_paths(native, monkeypatch, precision):
    """The 2,000 x 5,000 LP: both paths reach 1e-6 at the same objective; the
    cluster path takes one launch per chunk instead of two per attempt."""
    from igaos_gb300 import capi
    lp = G.config1(seed=0)
    out = {}
    for p in ("cluster", "grid"):
        use_path(monkeypatch, p)
        out[p] = capi.solve_lp(lp, tolerance=1e-6, time_limit=60.0, precision=precision)
        assert out[p]["status_name"] == "near-optimal", (p, out[p]["message"])
    a, b = out["cluster"], out["grid"]
    assert abs(a["objective"] - b["objective"]) <= 1e-5 * max(1.0, abs(b["objective"]))
    assert a["launches"] * 10 < b["launches"], (a["launches"], b["launches"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_iterations_track_oracle_on_both_paths(native, orc, path, name):
    from igaos_gb300 import capi
    lp = CASES[name]()
    olp = orc.lp_from(lp)
    sd = orc.scale(olp, *orc.ruiz(olp))
    with capi.Problem(lp) as P:
        _, eta0, omega0 = P.step_init()
        z = lambda k: np.zeros(k)
        st0 = dict(x=z(lp.n), y=z(lp.m), xavg=z(lp.n), yavg=z(lp.m), axcur=z(lp.m), eta=eta0,
                   omega=omega0, k=1, hn=0)
        got = P.iterate(st0, 5, "fp32")
    want, _ = orc.iterate(olp, sd, st0, 5)
    assert got["k"] == want["k"]
    for key in ("x", "y"):
        scale = max(1.0, float(np.max(np.abs(want[key]))))
        assert np.max(np.abs(got[key] - want[key])) <= 2e-4 * scale, key
