// Presolve for the PDHG engine (host code; see presolve.hpp).
#include "presolve.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace igx {
namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr int kMaxRounds = 64;
constexpr double kFeasTol = 1e-9;
constexpr double kForceTol = 1e-12;  // activity bound this close to a row bound: forcing
constexpr double kParallelTol = 1e-12;  // rows proportional to within this (relative)

inline double mag(double b) { return std::isfinite(b) ? std::fabs(b) : 0.0; }

// splitmix64 finaliser
inline uint64_t mix64(uint64_t x) {
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

}  // namespace

int presolve(int m, int n, const int* ap, const int* ai, const double* ax, const double* c,
             const double* cl, const double* cu, const double* rmin, const double* rmax,
             double obj_const, Presolved& P) {
    P = Presolved();
    P.m0 = m;
    P.n0 = n;
    // row-wise copy with repeated (row, column) entries summed (the activity
    // bounds below treat every entry as its own term) and exact zeros
    // dropped, and its column-wise counterpart
    std::vector<int> rp(m + 1, 0), rj;
    std::vector<double> ra;
    rj.reserve(ap[m]);
    ra.reserve(ap[m]);
    {
        std::vector<int> at(n, -1);  // position of column j in the current row
        for (int i = 0; i < m; ++i) {
            const int start = (int)rj.size();
            for (int p = ap[i]; p < ap[i + 1]; ++p) {
                const int j = ai[p];
                if (at[j] >= start) {
                    ra[at[j]] += ax[p];
                    continue;
                }
                at[j] = (int)rj.size();
                rj.push_back(j);
                ra.push_back(ax[p]);
            }
            int w = start;
            for (int q = start; q < (int)rj.size(); ++q)
                if (ra[q] != 0.0) {
                    rj[w] = rj[q];
                    ra[w] = ra[q];
                    ++w;
                }
            rj.resize(w);
            ra.resize(w);
            rp[i + 1] = w;
        }
    }
    const int64_t nz = rp[m];
    std::vector<int>& cp = P.cp0;
    std::vector<int>& ci = P.ci0;
    std::vector<double>& ca = P.acx0;
    cp.assign(n + 1, 0);
    ci.resize(nz);
    ca.resize(nz);
    for (int64_t p = 0; p < nz; ++p) cp[rj[p] + 1]++;
    for (int j = 0; j < n; ++j) cp[j + 1] += cp[j];
    {
        std::vector<int> next(cp.begin(), cp.end() - 1);
        for (int i = 0; i < m; ++i)
            for (int p = rp[i]; p < rp[i + 1]; ++p) {
                const int q = next[rj[p]]++;
                ci[q] = i;
                ca[q] = ra[p];
            }
    }
    P.c0.assign(c, c + n);

    std::vector<double> lo(cl, cl + n), hi(cu, cu + n), cost(c, c + n);
    std::vector<double> rlo(rmin, rmin + m), rhi(rmax, rmax + m), rscale(m);
    for (int j = 0; j < n; ++j)
        if (lo[j] == kInf || hi[j] == -kInf) return kPresolveInfeasible;
    for (int i = 0; i < m; ++i) {
        if (rlo[i] == kInf || rhi[i] == -kInf) return kPresolveInfeasible;
        rscale[i] = 1.0 + mag(rlo[i]) + mag(rhi[i]);
    }
    std::vector<char> ralive(m, 1), calive(n, 1);
    std::vector<int> rcnt(m), ccnt(n);
    for (int i = 0; i < m; ++i) rcnt[i] = rp[i + 1] - rp[i];
    for (int j = 0; j < n; ++j) ccnt[j] = cp[j + 1] - cp[j];
    double shift = 0.0;
    PresolveCounts& K = P.counts;

    auto kill_row = [&](int i) {
        ralive[i] = 0;
        for (int p = rp[i]; p < rp[i + 1]; ++p)
            if (calive[rj[p]]) --ccnt[rj[p]];
    };
    auto kill_col = [&](int j) {
        calive[j] = 0;
        for (int p = cp[j]; p < cp[j + 1]; ++p)
            if (ralive[ci[p]]) --rcnt[ci[p]];
    };
    auto fix_col = [&](int j, double v) {
        for (int p = cp[j]; p < cp[j + 1]; ++p) {
            const int i = ci[p];
            if (!ralive[i]) continue;
            const double t = ca[p] * v;
            rlo[i] -= t;  // -inf and +inf stay as they are
            rhi[i] -= t;
            rscale[i] += std::fabs(t);
        }
        shift += cost[j] * v;
        PresolveRec r;
        r.kind = PresolveRec::FixVal;
        r.j = j;
        r.val = v;
        P.recs.push_back(r);
        kill_col(j);
    };
    auto infeasible = [&](int i, int side) {
        P.infeasible_row = i;
        P.infeasible_side = side;
        return kPresolveInfeasible;
    };
    auto empty_row = [&](int i) -> bool {  // false: 0 is outside the row's range
        const double t = kFeasTol * rscale[i];
        if (rlo[i] > t || rhi[i] < -t) {
            P.infeasible_row = i;
            P.infeasible_side = rlo[i] > t ? -1 : 1;
            return false;
        }
        kill_row(i);
        ++K.empty_rows;
        return true;
    };
    auto empty_col = [&](int j) -> bool {  // false: the cost runs to an infinite bound
        double v;
        if (cost[j] > 0.0) {
            if (!std::isfinite(lo[j])) {
                P.unbounded_col = j;
                P.ray_step = -1.0;
                return false;
            }
            v = lo[j];
        } else if (cost[j] < 0.0) {
            if (!std::isfinite(hi[j])) {
                P.unbounded_col = j;
                P.ray_step = 1.0;
                return false;
            }
            v = hi[j];
        } else {
            v = std::isfinite(lo[j]) ? lo[j] : (std::isfinite(hi[j]) ? hi[j] : 0.0);
        }
        fix_col(j, v);
        ++K.empty_cols;
        return true;
    };

    // a singleton column j of row i whose bounds the row implies: with the
    // other columns inside their bounds and the activity inside [rlo, rhi],
    // x_j = (activity - others) / a already lies in [lo_j, hi_j], so those
    // bounds never bind and j is substituted like a free column
    auto implied_free = [&](int i, int j, double a) -> bool {
        // a finite lower bound of x_j can only be implied through the row
        // bound on its side (rmin for a > 0, rmax for a < 0), an upper one
        // through the other: without it, no scan is needed
        const double below = a > 0.0 ? rlo[i] : rhi[i], above = a > 0.0 ? rhi[i] : rlo[i];
        if ((std::isfinite(lo[j]) && !std::isfinite(below)) ||
            (std::isfinite(hi[j]) && !std::isfinite(above)))
            return false;
        double L = 0.0, U = 0.0;  // activity range of the row's other columns
        for (int s = rp[i]; s < rp[i + 1]; ++s) {
            const int k = rj[s];
            if (k == j || !calive[k]) continue;
            const double b = ra[s];
            L += b > 0.0 ? b * lo[k] : b * hi[k];
            U += b > 0.0 ? b * hi[k] : b * lo[k];
            if (L == -kInf && U == kInf) return false;  // unbounded both ways
        }
        const double ilo = a > 0.0 ? (rlo[i] - U) / a : (rhi[i] - L) / a;
        const double ihi = a > 0.0 ? (rhi[i] - L) / a : (rlo[i] - U) / a;
        return ilo >= lo[j] && ihi <= hi[j];
    };

    // Parallel rows: rows with the same live columns and proportional values
    // (grouped by a hash of the columns and the values over the first one),
    // the later merged into the earlier.
    std::vector<std::pair<int, double>> ea, eb;  // (column, value) of two rows
    auto live = [&](int i, std::vector<std::pair<int, double>>& e) {
        e.clear();
        for (int q = rp[i]; q < rp[i + 1]; ++q)
            if (calive[rj[q]]) e.push_back({rj[q], ra[q]});
        std::sort(e.begin(), e.end());
    };
    auto parallel_rows = [&](bool& changed_out) -> int {
        // one key per row: an order-free hash (a sum of per-entry hashes) of
        // its live columns and their values over the entry of the smallest
        // column; sorted by (key, row), equal keys form the candidate groups
        std::vector<std::pair<uint64_t, int>> keys;
        for (int i = 0; i < m; ++i) {
            if (!ralive[i] || rcnt[i] < 2) continue;
            int jmin = n;
            double vmin = 0.0;
            for (int q = rp[i]; q < rp[i + 1]; ++q)
                if (calive[rj[q]] && rj[q] < jmin) {
                    jmin = rj[q];
                    vmin = ra[q];
                }
            uint64_t h = 0;
            for (int q = rp[i]; q < rp[i + 1]; ++q) {
                if (!calive[rj[q]]) continue;
                // hash only: two ratios within 1e-12 that straddle a 1e-9
                // rounding boundary land in different groups, so such a
                // pair is not merged (a reduction missed, never a wrong one)
                const double r = std::round(ra[q] / vmin * 1e9) / 1e9;
                uint64_t bits;
                std::memcpy(&bits, &r, sizeof(bits));
                h += mix64(((uint64_t)(uint32_t)rj[q] << 32) ^ mix64(bits));
            }
            keys.push_back({h, i});
        }
        std::sort(keys.begin(), keys.end());
        for (size_t g0 = 0, g1; g0 < keys.size(); g0 = g1) {
            for (g1 = g0 + 1; g1 < keys.size() && keys[g1].first == keys[g0].first; ++g1) {
            }
            for (size_t u = g0 + 1; u < g1; ++u) {
                const int i = keys[u].second;  // candidate to remove
                if (!ralive[i]) continue;
                live(i, ea);
                for (size_t v = g0; v < u; ++v) {
                    const int k = keys[v].second;  // earlier row: candidate to keep
                    if (!ralive[k]) continue;
                    live(k, eb);
                    if (ea.size() != eb.size()) continue;
                    const double sr = ea[0].second / eb[0].second;
                    bool same = true;
                    for (size_t t = 0; t < ea.size() && same; ++t)
                        same = ea[t].first == eb[t].first &&
                               std::fabs(ea[t].second - sr * eb[t].second) <=
                                   kParallelTol * std::fabs(ea[t].second);
                    if (!same) continue;
                    // row i's range in row k's units
                    const double ilo = sr > 0.0 ? rlo[i] / sr : rhi[i] / sr;
                    const double ihi = sr > 0.0 ? rhi[i] / sr : rlo[i] / sr;
                    const bool tl = ilo > rlo[k], th = ihi < rhi[k];
                    double nlo = tl ? ilo : rlo[k], nhi = th ? ihi : rhi[k];
                    if (nlo > nhi) {
                        if (nlo - nhi > kFeasTol * (1.0 + mag(nlo) + mag(nhi))) {
                            // row i needs row k's activity above rhi[k]
                            // (side +1) or below rlo[k] (side -1): the dual
                            // ray y_k = side, y_i = -side / sr has A^T y = 0
                            // on the live columns and a positive bound
                            P.infeasible_row2 = i;
                            P.infeasible_ratio = sr;
                            return infeasible(k, ilo > rhi[k] ? 1 : -1);
                        }
                        if (tl && !th) nlo = nhi;
                        else nhi = nlo;
                    }
                    rlo[k] = nlo;
                    rhi[k] = nhi;
                    rscale[k] = std::max(rscale[k], rscale[i] / std::fabs(sr));
                    PresolveRec r;
                    r.kind = PresolveRec::ParallelRow;
                    r.i = i;
                    r.j = k;
                    r.a = sr;
                    r.lo_from_row = tl;
                    r.hi_from_row = th;
                    P.recs.push_back(r);
                    kill_row(i);
                    ++K.redundant_rows;
                    changed_out = true;
                    break;
                }
            }
        }
        return kPresolveReduced;
    };

    bool changed = true;
    while (changed && P.rounds < kMaxRounds) {
        changed = false;
        ++P.rounds;
        for (int i = 0; i < m; ++i) {
            if (!ralive[i]) continue;
            if (rcnt[i] == 0) {
                if (!empty_row(i)) return kPresolveInfeasible;
                changed = true;
                continue;
            }
            if (rcnt[i] == 1) {
                int p = rp[i];
                while (!calive[rj[p]]) ++p;
                const int j = rj[p];
                const double a = ra[p];
                // a x_j in [rlo, rhi]  <=>  x_j in [blo, bhi]
                const double blo = a > 0.0 ? rlo[i] / a : rhi[i] / a;
                const double bhi = a > 0.0 ? rhi[i] / a : rlo[i] / a;
                const bool tl = blo > lo[j], th = bhi < hi[j];
                double nlo = tl ? blo : lo[j], nhi = th ? bhi : hi[j];
                if (nlo > nhi) {
                    // the row's own range is not empty: it crosses a column
                    // bound from the side it tightened
                    if (nlo - nhi > kFeasTol * (1.0 + mag(nlo) + mag(nhi)))
                        return infeasible(i, tl ? (a > 0.0 ? -1 : 1) : (a > 0.0 ? 1 : -1));
                    if (tl && !th) nlo = nhi;  // crossing by rounding only
                    else nhi = nlo;
                }
                lo[j] = nlo;
                hi[j] = nhi;
                PresolveRec r;
                r.kind = PresolveRec::SingletonRow;
                r.i = i;
                r.j = j;
                r.a = a;
                r.lo_from_row = tl;
                r.hi_from_row = th;
                P.recs.push_back(r);
                kill_row(i);
                ++K.singleton_rows;
                changed = true;
                continue;
            }
            // activity range over the current column bounds
            double L = 0.0, U = 0.0;
            for (int p = rp[i]; p < rp[i + 1]; ++p) {
                const int j = rj[p];
                if (!calive[j]) continue;
                const double a = ra[p];
                L += a > 0.0 ? a * lo[j] : a * hi[j];
                U += a > 0.0 ? a * hi[j] : a * lo[j];
            }
            if (L >= rlo[i] && U <= rhi[i]) {
                kill_row(i);
                ++K.redundant_rows;
                changed = true;
                continue;
            }
            const double tf = kFeasTol * rscale[i], te = kForceTol * rscale[i];
            if (L > rhi[i] + tf) return infeasible(i, 1);
            if (U < rlo[i] - tf) return infeasible(i, -1);
            const int side = std::fabs(L - rhi[i]) <= te ? 1 : (std::fabs(U - rlo[i]) <= te ? -1 : 0);
            if (side == 0) continue;
            // forcing: least activity at rmax (side +1) or largest at rmin (-1)
            PresolveRec r;
            r.kind = PresolveRec::Forcing;
            r.i = i;
            r.side = side;
            r.t0 = (int64_t)P.term_col.size();
            for (int q = rp[i]; q < rp[i + 1]; ++q) {
                const int k = rj[q];
                if (!calive[k]) continue;
                const double b = ra[q];
                const bool upper = (b > 0.0) == (side < 0);  // the bound that achieves it
                P.term_col.push_back(k);
                P.term_a.push_back(b);
                P.term_at.push_back(lo[k] == hi[k] ? 2 : (upper ? 1 : 0));
                if (upper) lo[k] = hi[k];
                else hi[k] = lo[k];
            }
            r.t1 = (int64_t)P.term_col.size();
            P.recs.push_back(r);
            kill_row(i);
            ++K.redundant_rows;
            changed = true;
        }
        if (parallel_rows(changed) != kPresolveReduced) return kPresolveInfeasible;
        for (int j = 0; j < n; ++j) {
            if (!calive[j]) continue;
            if (lo[j] == hi[j]) {
                fix_col(j, lo[j]);
                ++K.fixed_cols;
                changed = true;
                continue;
            }
            if (ccnt[j] == 0) {
                if (!empty_col(j)) return kPresolveUnbounded;
                changed = true;
                continue;
            }
            if (ccnt[j] != 1) continue;
            int p = cp[j];
            while (!ralive[ci[p]]) ++p;
            const int i = ci[p];
            const double a = ca[p];
            if ((lo[j] != -kInf || hi[j] != kInf) && !implied_free(i, j, a)) continue;
            const double q = cost[j] / a;
            double t;
            // unbounded: x_j alone moves the row's activity toward its open
            // side, and the cost falls (c_j dx_j = q a dx_j < 0)
            if (q > 0.0) {
                if (!std::isfinite(rlo[i])) {
                    P.unbounded_col = j;
                    P.ray_step = -1.0 / a;
                    return kPresolveUnbounded;
                }
                t = rlo[i];
            } else if (q < 0.0) {
                if (!std::isfinite(rhi[i])) {
                    P.unbounded_col = j;
                    P.ray_step = 1.0 / a;
                    return kPresolveUnbounded;
                }
                t = rhi[i];
            } else {
                t = std::isfinite(rlo[i]) ? rlo[i] : (std::isfinite(rhi[i]) ? rhi[i] : 0.0);
            }
            PresolveRec r;
            r.kind = PresolveRec::FreeSingleton;
            r.i = i;
            r.j = j;
            r.a = a;
            r.q = q;
            r.val = t;
            r.t0 = (int64_t)P.term_col.size();
            for (int s = rp[i]; s < rp[i + 1]; ++s) {
                const int k = rj[s];
                if (k == j || !calive[k]) continue;
                P.term_col.push_back(k);
                P.term_a.push_back(ra[s]);
                P.term_at.push_back(2);
                cost[k] -= q * ra[s];
            }
            r.t1 = (int64_t)P.term_col.size();
            shift += q * t;
            P.recs.push_back(r);
            kill_col(j);
            kill_row(i);
            ++K.free_singletons;
            changed = true;
        }
    }
    // a round cap can leave empty rows and columns behind: clear them so that
    // the reduced LP has rows exactly when it has columns
    for (int i = 0; i < m; ++i)
        if (ralive[i] && rcnt[i] == 0 && !empty_row(i)) return kPresolveInfeasible;
    for (int j = 0; j < n; ++j)
        if (calive[j] && ccnt[j] == 0 && !empty_col(j)) return kPresolveUnbounded;

    // reduced LP
    P.row_red.assign(m, -1);
    P.col_red.assign(n, -1);
    for (int i = 0; i < m; ++i)
        if (ralive[i]) P.row_red[i] = P.m++;
    for (int j = 0; j < n; ++j)
        if (calive[j]) P.col_red[j] = P.n++;
    P.ap.assign(P.m + 1, 0);
    P.ai.reserve(nz);
    P.ax.reserve(nz);
    P.rmin.resize(P.m);
    P.rmax.resize(P.m);
    for (int i = 0; i < m; ++i) {
        const int r = P.row_red[i];
        if (r < 0) continue;
        P.rmin[r] = rlo[i];
        P.rmax[r] = rhi[i];
        for (int p = rp[i]; p < rp[i + 1]; ++p)
            if (calive[rj[p]]) {
                P.ai.push_back(P.col_red[rj[p]]);
                P.ax.push_back(ra[p]);
            }
        P.ap[r + 1] = (int)P.ai.size();
    }
    P.c.resize(P.n);
    P.cl.resize(P.n);
    P.cu.resize(P.n);
    for (int j = 0; j < n; ++j) {
        const int k = P.col_red[j];
        if (k < 0) continue;
        P.c[k] = cost[j];
        P.cl[k] = lo[j];
        P.cu[k] = hi[j];
    }
    P.obj_const = obj_const + shift;
    return kPresolveReduced;
}

namespace {

// x, y: the reduced LP's pair scattered to the original (0 elsewhere). ray:
// costs, fixed values and row targets taken as 0
void undo(const Presolved& P, double* x, double* y, bool ray) {
    // the duals of substituted rows do not depend on the solution; every
    // reduced cost below needs them
    if (!ray)
        for (const PresolveRec& r : P.recs)
            if (r.kind == PresolveRec::FreeSingleton) y[r.i] = -r.q;
    for (auto it = P.recs.rbegin(); it != P.recs.rend(); ++it) {
        const PresolveRec& r = *it;
        switch (r.kind) {
            case PresolveRec::FixVal:
                x[r.j] = ray ? 0.0 : r.val;
                break;
            case PresolveRec::FreeSingleton: {
                double s = 0.0;
                for (int64_t t = r.t0; t < r.t1; ++t) s += P.term_a[t] * x[P.term_col[t]];
                x[r.j] = ((ray ? 0.0 : r.val) - s) / r.a;
                break;
            }
            case PresolveRec::SingletonRow: {
                // rows removed before this one still hold y = 0 here
                double d = ray ? 0.0 : P.c0[r.j];
                for (int p = P.cp0[r.j]; p < P.cp0[r.j + 1]; ++p) d += P.acx0[p] * y[P.ci0[p]];
                if ((r.lo_from_row && d > 0.0) || (r.hi_from_row && d < 0.0)) y[r.i] = -d / r.a;
                break;
            }
            case PresolveRec::ParallelRow: {
                // the kept row's dual moves to the removed one when it
                // presses on a side that row set (a_i = s a_k: the same
                // reduced costs)
                const double yk = y[r.j];
                if ((yk > 0.0 && r.hi_from_row) || (yk < 0.0 && r.lo_from_row)) {
                    y[r.i] = yk / r.a;
                    y[r.j] = 0.0;
                }
                break;
            }
            case PresolveRec::Forcing: {
                // y_i on the row's active side (>= 0 at rmax, <= 0 at rmin)
                // with d_k + a_ik y_i >= 0 for columns at lower, <= 0 at upper
                double ylo = r.side > 0 ? 0.0 : -kInf, yhi = r.side > 0 ? kInf : 0.0;
                for (int64_t t = r.t0; t < r.t1; ++t) {
                    if (P.term_at[t] == 2) continue;
                    const int k = P.term_col[t];
                    const double a = P.term_a[t];
                    double d = ray ? 0.0 : P.c0[k];
                    for (int p = P.cp0[k]; p < P.cp0[k + 1]; ++p) d += P.acx0[p] * y[P.ci0[p]];
                    const double v = -d / a;
                    if ((P.term_at[t] == 0) == (a > 0.0)) ylo = std::max(ylo, v);
                    else yhi = std::min(yhi, v);
                }
                // nearest 0 inside [ylo, yhi]; rounding can cross them: midpoint
                y[r.i] = ylo > yhi ? 0.5 * (ylo + yhi) : std::min(std::max(0.0, ylo), yhi);
                break;
            }
        }
    }
}

void scatter(const Presolved& P, const double* x_red, const double* y_red, double* x, double* y) {
    for (int j = 0; j < P.n0; ++j) x[j] = P.col_red[j] >= 0 ? x_red[P.col_red[j]] : 0.0;
    for (int i = 0; i < P.m0; ++i) y[i] = P.row_red[i] >= 0 ? y_red[P.row_red[i]] : 0.0;
}

}  // namespace

void postsolve(const Presolved& P, const double* x_red, const double* y_red, double* x, double* y) {
    scatter(P, x_red, y_red, x, y);
    undo(P, x, y, false);
}

void postsolve_ray(const Presolved& P, const double* x_red, const double* y_red, double* x,
                   double* y) {
    scatter(P, x_red, y_red, x, y);
    undo(P, x, y, true);
}

bool infeasible_ray(const Presolved& P, double* y) {
    if (P.infeasible_row < 0) return false;
    std::vector<double> x(P.n0, 0.0);
    std::fill(y, y + P.m0, 0.0);
    y[P.infeasible_row] = P.infeasible_side;
    if (P.infeasible_row2 >= 0) y[P.infeasible_row2] = -P.infeasible_side / P.infeasible_ratio;
    undo(P, x.data(), y, true);
    return true;
}

bool unbounded_ray(const Presolved& P, double* x) {
    if (P.unbounded_col < 0) return false;
    std::fill(x, x + P.n0, 0.0);
    x[P.unbounded_col] = P.ray_step;
    for (auto it = P.recs.rbegin(); it != P.recs.rend(); ++it) {
        if (it->kind != PresolveRec::FreeSingleton) continue;
        double s = 0.0;
        for (int64_t t = it->t0; t < it->t1; ++t) s += P.term_a[t] * x[P.term_col[t]];
        x[it->j] = -s / it->a;
    }
    return true;
}

}  // namespace igx
