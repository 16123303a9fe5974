// Host-side LP in original units and its KKT metrics, for the parts of the
// C ABI that work on the caller's LP on the host (presolve's postsolved
// answer, crossover's vertex): the same six metrics the device KKT pass
// computes (the reference's evaluate(), src/pdhg/pdhg.cu:173-254).
#pragma once

#include <vector>

namespace igx {

struct HostLP {
    int m = 0, n = 0;
    std::vector<int> ap, ai, cp, ci;
    std::vector<double> ax, acx, c, cl, cu, rmin, rmax;
};

struct HostMetrics {
    double pinf, dinf, gap, op, od, prow;
};

// Metrics of (x, y) with Ax = A x and d = c + A^T y, all in original units:
//   pinf  max row violation / (1 + max |Ax projected onto the row box|)
//   prow  max over rows of violation / (1 + the row's own scale)
//   dinf  max reduced cost not excused by an active bound (band 1e-9 of the
//         bound) / (1 + max |c|)
//   op    c^T x
//   od    the Lagrangian bound at y; -inf when a reduced cost or dual
//         presses on an infinite bound beyond a 1e-8 noise slack
//   gap   max(0, op - od) / (1 + |op|); +inf when od is -inf
HostMetrics host_evaluate(const HostLP& lp, const double* x, const double* y, const double* Ax,
                          const double* d);

}  // namespace igx
