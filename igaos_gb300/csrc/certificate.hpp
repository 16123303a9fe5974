// Infeasibility certificates from a ray candidate, in original units (host).
//
// A candidate pair (x, y) -- in the solve loop the change between two
// consecutive restart points -- with ax = A x and aty = A^T y, normalised to
// max-norm 1, is tested as
//   a dual ray y (returns 1; the LP is infeasible): with d = A^T y (no cost),
//     d_j > 0 needs a finite lower bound, d_j < 0 a finite upper one, y_i > 0
//     a finite rmax and y_i < 0 a finite rmin, and the dual objective along
//     the ray, sum_j d_j (l_j or u_j) - sum_i y_i (rmax_i or rmin_i), must be
//     positive (the dual is unbounded);
//   a primal ray x (returns 2; the dual is infeasible, so a feasible LP is
//     unbounded): x_j < 0 needs l_j = -inf, x_j > 0 needs u_j = +inf,
//     (A x)_i < 0 needs rmin_i = -inf, (A x)_i > 0 needs rmax_i = +inf, and
//     c^T x < 0.
// Sign violations may not exceed kRayViolRel of the ray's scale (1, or the
// largest |d_j| / |(A x)_i|) and the objective must exceed kRayObjRel of the
// magnitude of its terms. The dual ray is tested first. The normalised ray
// goes to yray (m) or xray (n) when non-null; 0 means no certificate.
#pragma once

namespace igx {

constexpr double kRayViolRel = 1e-9;
constexpr double kRayObjRel = 1e-6;

int ray_certificate(int m, int n, const double* x, const double* ax, const double* y,
                    const double* aty, const double* c, const double* cl, const double* cu,
                    const double* rmin, const double* rmax, double* xray, double* yray);

}  // namespace igx
