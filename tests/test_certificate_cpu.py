"""The infeasibility-certificate test of detect_infeasibility on host arrays
(igaos_pdhg_ray_certificate; no GPU needed): planted dual and primal rays are
accepted and normalised, vectors that are not rays are refused, and no
candidate of a feasible bounded LP is taken for a certificate.
"""
import numpy as np

from igaos_gb300 import generators as G

INF = float("inf")


def two_rows(extra=None):
    """x1 + x2 <= 1 and x1 + x2 >= 3 on [0, 5]^2 (infeasible); extra =
    coefficient of a free column x3 in the first row (None: no x3)."""
    if extra is None:
        return G.from_triplets(2, 2, [0, 0, 1, 1], [0, 1, 0, 1], [1.0] * 4, [1.0, 1.0],
                               [0.0, 0.0], [5.0, 5.0], [-INF, 3.0], [1.0, INF])
    return G.from_triplets(2, 3, [0, 0, 0, 1, 1], [0, 1, 2, 0, 1], [1.0, 1.0, extra, 1.0, 1.0],
                           [1.0, 1.0, 0.0], [0.0, 0.0, -INF], [5.0, 5.0, INF], [-INF, 3.0],
                           [1.0, INF])


def unbounded():
    # min -x1 - 0.5 x3 s.t. x1 - x2 <= 1, x2 - x3 <= 2, x1 + x3 >= 1; x >= 0
    return G.from_triplets(3, 3, [0, 0, 1, 1, 2, 2], [0, 1, 1, 2, 0, 2],
                           [1.0, -1.0, 1.0, -1.0, 1.0, 1.0], [-1.0, 0.0, -0.5],
                           [0.0, 0.0, 0.0], [INF, INF, INF], [-INF, -INF, 1.0], [1.0, 2.0, INF])


def test_dual_ray_accepted_and_normalised(native):
    from igaos_gb300 import capi
    lp = two_rows()
    kind, _, yr = capi.ray_certificate(lp, np.zeros(2), np.array([4.0, -4.0]))
    assert kind == 1
    assert np.array_equal(yr, [1.0, -1.0])


def test_not_a_dual_ray(native):
    from igaos_gb300 import capi
    lp = two_rows()
    # y2 > 0 on a row without a finite upper bound
    assert capi.ray_certificate(lp, np.zeros(2), np.array([1.0, 1.0]))[0] == 0
    # sign-feasible but with a non-positive objective along it
    assert capi.ray_certificate(lp, np.zeros(2), np.array([1.0, -0.2]))[0] == 0


def test_free_column_tolerance(native):
    """A free column makes d_3 = y_1 a; |a| = 1e-12 is within the tolerance
    (the LP stays infeasible up to that), |a| = 1e-3 is not (x3 -> -inf
    satisfies both rows: the LP is feasible)."""
    from igaos_gb300 import capi
    y = np.array([1.0, -1.0])
    assert capi.ray_certificate(two_rows(1e-12), np.zeros(3), y)[0] == 1
    assert capi.ray_certificate(two_rows(1e-3), np.zeros(3), y)[0] == 0


def test_primal_ray(native):
    from igaos_gb300 import capi
    lp = unbounded()
    kind, xr, _ = capi.ray_certificate(lp, np.array([3.0, 3.0, 3.0]), np.zeros(3))
    assert kind == 2 and np.array_equal(xr, [1.0, 1.0, 1.0])
    # A x leaves the recession cone of row 0 (x1 - x2 <= 1)
    assert capi.ray_certificate(lp, np.array([1.0, 0.0, 0.0]), np.zeros(3))[0] == 0
    # x3 < 0 against its finite lower bound
    assert capi.ray_certificate(lp, np.array([1.0, 1.0, -1.0]), np.zeros(3))[0] == 0


def test_no_certificate_for_feasible_lps(native):
    """Random candidates of feasible LPs: boxed (every nonzero x leaves its
    box; a dual ray cannot exist) and with every bound type."""
    from igaos_gb300 import capi
    rng = np.random.default_rng(0)
    for seed in range(6):
        for lp in (G.random_lp(40, 90, 150, seed), G.mixed_bounds_lp(40, 90, 150, seed)):
            for _ in range(20):
                x = rng.standard_normal(lp.n) * (rng.random(lp.n) < 0.5)
                y = rng.standard_normal(lp.m) * (rng.random(lp.m) < 0.5)
                assert capi.ray_certificate(lp, x, y)[0] == 0
