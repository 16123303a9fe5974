// Presolve for the PDHG engine (host code). No counterpart on the reference's
// PDHG path, whose solve ignores Options.presolve; the reference's own
// presolve (src/simplex/presolve.hpp:176-600, Andersen & Andersen 1995) is
// simplex-only and maps back x alone, setting y = 0 on every removed row.
//
// The reductions here are the subset of Andersen & Andersen whose optimal
// duals are recovered exactly, so that postsolve turns an optimal pair of the
// reduced LP into an optimal pair of the original (the engine's termination
// test is on both):
//   empty row        -- 0 must lie in [rmin, rmax]; y_i = 0;
//   singleton row    -- a x_j in [rmin, rmax] becomes a bound of x_j; the
//                       side(s) it tightened are recorded, and postsolve
//                       moves a reduced cost d_j pressing on such a side
//                       into y_i = -d_j / a;
//   redundant row    -- its activity range over the column bounds lies in
//                       [rmin, rmax]; y_i = 0;
//   parallel row     -- row i = s row k (same columns, values in ratio s):
//                       row k keeps the intersection of both ranges and
//                       row i goes; postsolve hands k's dual to i (y_i =
//                       y_k / s, y_k = 0) when it presses on a side i set;
//   forcing row      -- its least activity is rmax (or its largest rmin):
//                       every column goes to the bound that achieves it and
//                       the row is removed; postsolve takes y_i nearest 0 on
//                       the row's active side with every such column's
//                       reduced cost of the sign its bound needs (an
//                       activity range beyond the row's bounds: infeasible);
//   fixed column     -- l_j = u_j: removed, row bounds shifted by a x_j;
//   empty column     -- x_j at the bound its cost prefers (the LP is
//                       unbounded or infeasible when that bound is infinite);
//   free singleton   -- a column j met by one row i, free or with bounds
//                       the row implies (the other columns' bounds and the
//                       row's keep x_j inside them): x_j takes up the row
//                       (activity pinned at the row bound the sign of
//                       q = c_j / a selects), the row's other columns pay
//                       c_k -= q a_ik, and y_i = -q.
// Exact zeros of A are dropped. Rounds repeat until nothing changes.
#pragma once

#include <cstdint>
#include <vector>

namespace igx {

struct PresolveCounts {
    // forcing and parallel rows are counted with the redundant ones
    int64_t empty_rows = 0, singleton_rows = 0, redundant_rows = 0;
    int64_t fixed_cols = 0, empty_cols = 0, free_singletons = 0;
};

// Outcome codes share the values of IGAOS_STATUS_INFEASIBLE / _UNBOUNDED.
constexpr int kPresolveReduced = 0;
constexpr int kPresolveInfeasible = 3;
constexpr int kPresolveUnbounded = 4;  // dual infeasible: unbounded if feasible

struct PresolveRec {
    enum Kind : unsigned char {
        FixVal = 0, SingletonRow = 1, FreeSingleton = 2, Forcing = 3, ParallelRow = 4
    } kind;
    // SingletonRow: the sides of x_j's bounds the row set; ParallelRow: the
    // sides of the kept row's bounds the removed row set
    bool lo_from_row = false, hi_from_row = false;
    int i = -1, j = -1;  // ParallelRow: i removed, j the row kept
    double a = 0.0;    // SingletonRow / FreeSingleton: the entry a_ij; ParallelRow:
                       // the ratio s of the rows (row i = s row j)
    double val = 0.0;  // FixVal: x_j; FreeSingleton: the row target t
    double q = 0.0;    // FreeSingleton: c_j / a_ij (y_i = -q)
    int64_t t0 = 0, t1 = 0;  // FreeSingleton: its row's other entries in terms;
                             // Forcing: the row's columns (term_at: the bound)
    int side = 0;            // Forcing: +1 activity pinned at rmax, -1 at rmin
};

struct Presolved {
    // original LP, column-wise (reduced costs in postsolve) and its costs
    int m0 = 0, n0 = 0;
    std::vector<int> cp0, ci0;
    std::vector<double> acx0, c0;
    // reduced LP (CSR), its constant, and the index maps original -> reduced
    int m = 0, n = 0;
    std::vector<int> ap, ai;
    std::vector<double> ax, c, cl, cu, rmin, rmax;
    double obj_const = 0.0;
    std::vector<int> row_red, col_red;
    // reductions in the order they were made
    std::vector<PresolveRec> recs;
    std::vector<int> term_col;
    std::vector<double> term_a;
    std::vector<signed char> term_at;  // Forcing: 0 lower, 1 upper, 2 fixed
    PresolveCounts counts;
    int rounds = 0;
    // kPresolveUnbounded: the column whose cost runs to an infinite bound and
    // its primal ray (x_j moves by ray_step per unit; every other entry 0)
    int unbounded_col = -1;
    double ray_step = 0.0;
    // kPresolveInfeasible: the row whose bounds the activity cannot meet and
    // the sign of its dual ray (+1 at rmax, -1 at rmin); -1 when none. When
    // two parallel rows (row infeasible_row2 = infeasible_ratio x row
    // infeasible_row) have ranges that do not meet, the ray also holds
    // y[infeasible_row2] = -infeasible_side / infeasible_ratio, which cancels
    // their columns.
    int infeasible_row = -1;
    int infeasible_side = 0;
    int infeasible_row2 = -1;
    double infeasible_ratio = 0.0;
};

// Reduces the LP (CSR, original units). Returns kPresolveReduced (out holds
// the reduced LP, possibly with no rows and no columns), kPresolveInfeasible
// or kPresolveUnbounded. Bounds must satisfy cl <= cu and rmin <= rmax.
int presolve(int m, int n, const int* ap, const int* ai, const double* ax, const double* c,
             const double* cl, const double* cu, const double* rmin, const double* rmax,
             double obj_const, Presolved& out);

// x (n0) and y (m0) of the original LP from x_red (n) and y_red (m) of the
// reduced one: records undone in reverse order.
void postsolve(const Presolved& p, const double* x_red, const double* y_red, double* x, double* y);

// The same map for a ray of the reduced LP (a direction: zero costs, fixed
// values and row targets): a dual ray y_red maps to a dual ray of the
// original (reduced costs pressing on a bound a singleton row set move into
// that row), a primal ray x_red to a primal ray (substituted columns follow
// their rows).
void postsolve_ray(const Presolved& p, const double* x_red, const double* y_red, double* x,
                   double* y);

// kPresolveUnbounded: x (n0) = the primal ray of the column presolve found
// running to an infinite bound, with the columns substituted before it
// following their rows. False for the other outcomes.
bool unbounded_ray(const Presolved& p, double* x);

// kPresolveInfeasible: y (m0) = a dual ray of the original LP: the row that
// proved it (y_i = +-1 in the LP presolve had reduced so far; for two
// parallel rows with disjoint ranges, +-1 on the kept row and the opposite
// multiple on the other), mapped back through the records made before it.
// False when no row proved it.
bool infeasible_ray(const Presolved& p, double* y);

}  // namespace igx
