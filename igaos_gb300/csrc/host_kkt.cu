// KKT metrics of a candidate pair on the host (see host_kkt.hpp).
#include "host_kkt.hpp"

#include <algorithm>
#include <cmath>
#include <limits>

namespace igx {
namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();

struct RowPart {
    double worst = 0.0;  // largest signed excursion outside [rmin, rmax]
    double scale = 0.0;  // largest |Ax_i| clipped into its row box
    double rel = 0.0;    // largest per-row violation / (1 + row scale)
};

RowPart rows(const HostLP& lp, const double* Ax) {
    RowPart r;
    for (int i = 0; i < lp.m; ++i) {
        const double lo = lp.rmin[i], hi = lp.rmax[i], a = Ax[i];
        const double out = std::max(lo - a, a - hi);
        r.worst = std::max(r.worst, out);
        r.scale = std::max(r.scale, std::fabs(std::min(std::max(a, lo), hi)));
        double own = std::fabs(a);
        if (std::isfinite(lo)) own = std::max(own, std::fabs(lo));
        if (std::isfinite(hi)) own = std::max(own, std::fabs(hi));
        r.rel = std::max(r.rel, std::max(0.0, out) / (1.0 + own));
    }
    return r;
}

// largest |d_j| of a column not sitting at the bound its sign points to
double unexcused_reduced_cost(const HostLP& lp, const double* x, const double* d) {
    double worst = 0.0;
    for (int j = 0; j < lp.n; ++j) {
        const double l = lp.cl[j], u = lp.cu[j];
        const double band = 1e-9 * (1.0 + std::fabs(std::isfinite(u) ? u : l));
        const bool excused = (d[j] > 0 && x[j] <= l + band) || (d[j] < 0 && x[j] >= u - band);
        if (!excused) worst = std::max(worst, std::fabs(d[j]));
    }
    return worst;
}

// min over the column box of d^T x minus max over the row box of y^T z
double lagrangian_bound(const HostLP& lp, const double* y, const double* d, double cmax) {
    double ymax = 0.0;
    for (int i = 0; i < lp.m; ++i) ymax = std::max(ymax, std::fabs(y[i]));
    const double dslack = 1e-8 * (1.0 + cmax), yslack = 1e-8 * (1.0 + ymax);
    double b = 0.0;
    for (int j = 0; j < lp.n; ++j) {
        const double bound = d[j] >= 0 ? lp.cl[j] : lp.cu[j];
        if (std::isfinite(bound)) b += d[j] * bound;
        else if (std::fabs(d[j]) > dslack) return -kInf;
    }
    for (int i = 0; i < lp.m; ++i) {
        if (std::fabs(y[i]) <= yslack) continue;
        const double side = y[i] > 0 ? lp.rmax[i] : lp.rmin[i];
        if (!std::isfinite(side)) return -kInf;
        b -= y[i] * side;
    }
    return b;
}

}  // namespace

HostMetrics host_evaluate(const HostLP& lp, const double* x, const double* y, const double* Ax,
                          const double* d) {
    HostMetrics r{};
    const RowPart rp = rows(lp, Ax);
    r.pinf = std::max(rp.worst, 0.0) / (1.0 + rp.scale);
    r.prow = rp.rel;
    double cmax = 0.0;
    for (int j = 0; j < lp.n; ++j) cmax = std::max(cmax, std::fabs(lp.c[j]));
    r.dinf = unexcused_reduced_cost(lp, x, d) / (1.0 + cmax);
    r.op = 0.0;
    for (int j = 0; j < lp.n; ++j) r.op += lp.c[j] * x[j];
    r.od = lagrangian_bound(lp, y, d, cmax);
    r.gap = std::isfinite(r.od) ? std::max(0.0, r.op - r.od) / (1.0 + std::fabs(r.op)) : kInf;
    return r;
}

}  // namespace igx
