// Dual repair: a certifiable dual for a primal candidate, so that LPs with
// infinite bounds can terminate on a finite duality gap (the reference
// engine's dual_repair, src/pdhg/pdhg.cu:257-448, tried from the solve loop
// at :854-931). Host code on the original (unscaled) LP, dense m x m normal
// equations: the engine keeps a host copy of the LP and enables the step only
// for m <= kRepairMaxRows.
#pragma once

#include <vector>

namespace igx {

// dense factor of A_J A_J^T: 128 MiB at the limit
constexpr int kRepairMaxRows = 4096;

struct HostLP {
    int m = 0, n = 0;
    std::vector<int> ap, ai, cp, ci;
    std::vector<double> ax, acx, c, cl, cu, rmin, rmax;
};

struct HostMetrics {
    double pinf, dinf, gap, op, od, prow;
};

// evaluate() of the reference (src/pdhg/pdhg.cu:173-254) on host vectors.
HostMetrics host_evaluate(const HostLP& lp, const double* x, const double* y, const double* Ax,
                          const double* d);

// y = a dual near y_it whose objective is finite for candidate x (Ax = A x),
// via alternating projections: onto {A_J^T y = -c_J} for the columns J
// strictly inside their bounds (col_tol band), onto the sign half-spaces of
// the columns with an infinite bound, onto the row cone. Returns true when a
// y with a finite gap was found (y = the smallest-gap one); otherwise y is
// the point of least sign violation, or empty if the factorisation failed.
bool dual_repair(const HostLP& lp, const double* x, const double* Ax, const double* y_it,
                 double col_tol, std::vector<double>& y);

}  // namespace igx
