// Dual repair (host code; see repair.hpp). Compiled without floating-point
// contraction so that its arithmetic is the reference host code's on every
// host: the certified duals are bit-identical to the reference's.
#include "repair.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace igx {
namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();

// std::max / std::min operand order (they differ from fmax/fmin on NaN)
inline double vmax(double a, double b) { return (a < b) ? b : a; }
inline double vmin(double a, double b) { return (b < a) ? b : a; }

// c_j + sum over column j of a_ij y_i, in column storage order
inline double reduced_cost(const HostLP& lp, int j, const double* y) {
    double d = lp.c[j];
    for (int p = lp.cp[j]; p < lp.cp[j + 1]; ++p) d += lp.acx[p] * y[lp.ci[p]];
    return d;
}

// Lower Cholesky factor in place (row-major, lower triangle used); false
// when a pivot is not positive.
bool cholesky(std::vector<double>& G, int m) {
    for (int i = 0; i < m; ++i) {
        double* gi = G.data() + (size_t)i * m;
        for (int j = 0; j <= i; ++j) {
            const double* gj = G.data() + (size_t)j * m;
            double s = gi[j];
            for (int t = 0; t < j; ++t) s -= gi[t] * gj[t];
            if (i == j) {
                if (!(s > 0)) return false;
                gi[i] = std::sqrt(s);
            } else {
                gi[j] = s / gj[j];
            }
        }
    }
    return true;
}

// b <- (L L^T)^-1 b
void cholesky_solve(const std::vector<double>& L, int m, double* b) {
    for (int i = 0; i < m; ++i) {
        const double* li = L.data() + (size_t)i * m;
        double s = b[i];
        for (int t = 0; t < i; ++t) s -= li[t] * b[t];
        b[i] = s / li[i];
    }
    for (int i = m - 1; i >= 0; --i) {
        double s = b[i];
        for (int t = i + 1; t < m; ++t) s -= L[(size_t)t * m + i] * b[t];
        b[i] = s / L[(size_t)i * m + i];
    }
}

// sign requirement on a column's reduced cost from its bounds
enum : char { kNonNeg = 0, kNonPos = 1, kZero = 2, kAny = 3 };

double band(double tol, double b) { return tol * (1.0 + (std::isfinite(b) ? std::fabs(b) : 0.0)); }

}  // namespace

HostMetrics host_evaluate(const HostLP& lp, const double* x, const double* y, const double* Ax,
                          const double* d) {
    const int m = lp.m, n = lp.n;
    HostMetrics r{};
    double pv = 0.0, pa = 0.0, prow = 0.0;
    for (int i = 0; i < m; ++i) {
        const double lo = lp.rmin[i], hi = lp.rmax[i], a = Ax[i];
        pv = vmax(pv, vmax(lo - a, a - hi));
        pa = vmax(pa, std::fabs(vmin(vmax(a, lo), hi)));
        const double viol = vmax(0.0, vmax(lo - a, a - hi));
        double sc = std::fabs(a);
        if (std::isfinite(lo)) sc = vmax(sc, std::fabs(lo));
        if (std::isfinite(hi)) sc = vmax(sc, std::fabs(hi));
        prow = vmax(prow, viol / (1.0 + sc));
    }
    r.pinf = vmax(pv, 0.0) / (1.0 + pa);
    r.prow = prow;
    double dv = 0.0;
    for (int j = 0; j < n; ++j) {
        const double tol = 1e-9 * (1.0 + std::fabs(std::isfinite(lp.cu[j]) ? lp.cu[j] : lp.cl[j]));
        double v;
        if (x[j] <= lp.cl[j] + tol && d[j] > 0) v = 0.0;
        else if (x[j] >= lp.cu[j] - tol && d[j] < 0) v = 0.0;
        else v = std::fabs(d[j]);
        dv = vmax(dv, v);
    }
    double cmax = 0.0;
    for (int j = 0; j < n; ++j) cmax = vmax(cmax, std::fabs(lp.c[j]));
    r.dinf = dv / (1.0 + cmax);
    r.op = 0.0;
    for (int j = 0; j < n; ++j) r.op += lp.c[j] * x[j];
    double ymax = 0.0;
    for (int i = 0; i < m; ++i) ymax = vmax(ymax, std::fabs(y[i]));
    const double dz = 1e-8 * (1.0 + cmax), yz = 1e-8 * (1.0 + ymax);
    double od = 0.0;
    bool bounded = true;
    for (int j = 0; j < n && bounded; ++j) {
        if (d[j] >= 0) {
            if (std::isfinite(lp.cl[j])) od += d[j] * lp.cl[j];
            else if (d[j] > dz) bounded = false;
        } else {
            if (std::isfinite(lp.cu[j])) od += d[j] * lp.cu[j];
            else if (-d[j] > dz) bounded = false;
        }
    }
    for (int i = 0; i < m && bounded; ++i) {
        if (y[i] > yz) {
            if (std::isfinite(lp.rmax[i])) od -= y[i] * lp.rmax[i];
            else bounded = false;
        } else if (y[i] < -yz) {
            if (std::isfinite(lp.rmin[i])) od -= y[i] * lp.rmin[i];
            else bounded = false;
        }
    }
    r.od = bounded ? od : -kInf;
    r.gap = bounded ? vmax(0.0, r.op - od) / (1.0 + std::fabs(r.op)) : kInf;
    return r;
}

bool dual_repair(const HostLP& lp, const double* x, const double* Ax, const double* y_it,
                 double col_tol, std::vector<double>& y) {
    const int m = lp.m, n = lp.n;
    // row cone of the dual: free on two-sided rows, signed on one-sided
    // rows, zero on free rows
    std::vector<double> ylo(m), yhi(m);
    for (int i = 0; i < m; ++i) {
        const bool fl = std::isfinite(lp.rmin[i]), fh = std::isfinite(lp.rmax[i]);
        ylo[i] = (fl && fh) ? -kInf : fh ? 0.0 : fl ? -kInf : 0.0;
        yhi[i] = (fl && fh) ? kInf : fh ? kInf : fl ? 0.0 : 0.0;
    }
    std::vector<char> sign(n);
    std::vector<double> norm2(n, 0.0);
    std::vector<int> inner;  // columns strictly inside their bounds: d_j = 0
    for (int j = 0; j < n; ++j) {
        const bool up_inf = !std::isfinite(lp.cu[j]), lo_inf = !std::isfinite(lp.cl[j]);
        sign[j] = (up_inf && lo_inf) ? kZero : up_inf ? kNonNeg : lo_inf ? kNonPos : kAny;
        for (int p = lp.cp[j]; p < lp.cp[j + 1]; ++p) norm2[j] += lp.acx[p] * lp.acx[p];
        if (x[j] - lp.cl[j] > band(col_tol, lp.cl[j]) && lp.cu[j] - x[j] > band(col_tol, lp.cu[j]))
            inner.push_back(j);
    }
    const int k = (int)inner.size();
    // normal matrix A_J A_J^T plus a ridge, factored once
    std::vector<double> L;
    if (k > 0) {
        L.assign((size_t)m * m, 0.0);
        for (int j : inner)
            for (int p = lp.cp[j]; p < lp.cp[j + 1]; ++p) {
                double* row = L.data() + (size_t)lp.ci[p] * m;
                const double a = lp.acx[p];
                for (int q = lp.cp[j]; q < lp.cp[j + 1]; ++q) row[lp.ci[q]] += a * lp.acx[q];
            }
        double trace = 0.0;
        for (int i = 0; i < m; ++i) trace += L[(size_t)i * m + i];
        double ridge = trace > 0 ? 1e-10 * trace / m : 1e-14;
        bool factored = false;
        for (int attempt = 0; attempt < 6 && !factored; ++attempt) {
            std::vector<double> F = L;
            for (int i = 0; i < m; ++i) F[(size_t)i * m + i] += ridge;
            factored = cholesky(F, m);
            if (factored) L.swap(F);
            else ridge = ridge > 0 ? ridge * 100.0 : 1e-14;
        }
        if (!factored) {
            y.clear();
            return false;
        }
    }
    double best_gap = kInf, best_viol = kInf;
    bool have = false;
    std::vector<double> d(n), rhs(m), yc(m), ybest, yviol;
    for (int anchor = 0; anchor < 2; ++anchor) {
        for (int i = 0; i < m; ++i) yc[i] = vmin(vmax(anchor == 0 ? y_it[i] : 0.0, ylo[i]), yhi[i]);
        double vref = -1.0;
        for (int it = 0; it < 300; ++it) {
            if (k > 0) {  // affine: y += (A_J A_J^T + ridge)^-1 (-A_J d_J)
                std::fill(rhs.begin(), rhs.end(), 0.0);
                double res2 = 0.0;
                for (int j : inner) {
                    const double dj = reduced_cost(lp, j, yc.data());
                    res2 += dj * dj;
                    if (dj != 0.0)
                        for (int p = lp.cp[j]; p < lp.cp[j + 1]; ++p) rhs[lp.ci[p]] -= lp.acx[p] * dj;
                }
                if (res2 > 0.0) {
                    cholesky_solve(L, m, rhs.data());
                    for (int i = 0; i < m; ++i) yc[i] += rhs[i];
                }
            }
            // sign half-spaces, one column at a time (Hildreth)
            for (int j = 0; j < n; ++j) {
                if (sign[j] == kAny || norm2[j] == 0.0) continue;
                const double dj = reduced_cost(lp, j, yc.data());
                double v = 0.0;
                if (sign[j] == kNonNeg && dj < 0.0) v = -dj;
                else if (sign[j] == kNonPos && dj > 0.0) v = -dj;
                else if (sign[j] == kZero && dj != 0.0) v = -dj;
                if (v != 0.0) {
                    const double step = v / norm2[j];
                    for (int p = lp.cp[j]; p < lp.cp[j + 1]; ++p) yc[lp.ci[p]] += step * lp.acx[p];
                }
            }
            for (int i = 0; i < m; ++i) yc[i] = vmin(vmax(yc[i], ylo[i]), yhi[i]);
            for (int j = 0; j < n; ++j) d[j] = reduced_cost(lp, j, yc.data());
            if (it % 25 == 0) {
                // worst sign violation; a projection that stalls is abandoned
                double viol = 0.0;
                for (int j = 0; j < n; ++j) {
                    double v = 0.0;
                    if (sign[j] == kNonNeg && d[j] < 0) v = -d[j];
                    else if (sign[j] == kNonPos && d[j] > 0) v = d[j];
                    else if (sign[j] == kZero) v = std::fabs(d[j]);
                    viol = vmax(viol, v);
                }
                for (int i = 0; i < m; ++i) {
                    double v = 0.0;
                    if (ylo[i] == 0.0 && yhi[i] == 0.0) v = std::fabs(yc[i]);
                    else if (yhi[i] == 0.0 && yc[i] > 0) v = yc[i];
                    else if (ylo[i] == 0.0 && yc[i] < 0) v = -yc[i];
                    viol = vmax(viol, v);
                }
                if (it == 25) vref = viol;
                if (viol < best_viol) {
                    best_viol = viol;
                    yviol = yc;
                }
                if (it == 100 && vref > 0 && viol > 0.25 * vref) break;
            }
            const HostMetrics t = host_evaluate(lp, x, yc.data(), Ax, d.data());
            if (std::isfinite(t.gap) && t.gap < best_gap) {
                best_gap = t.gap;
                ybest = yc;
                have = true;
            }
        }
    }
    y = have ? ybest : yviol;
    return have;
}

}  // namespace igx
