// Crossover from a PDHG point to an optimal vertex (host code). No
// counterpart on the reference's PDHG path; the reference's simplex
// (src/simplex/simplex.hpp:12-28) solves from scratch and takes no start
// point.
//
// The LP is put in the bounded form [A  -I] (x, s) = 0 with x in [cl, cu]
// and the row activities s in [rmin, rmax]. From the slack basis (B = -I)
// and the start point x0 (values within 1e-9 of a bound are snapped to it),
//   1. crash: the structurals strictly inside their bounds enter the basis
//      at once in place of the slacks of rows at a bound (1e-6, relative);
//   2. primal push: every variable still inside its bounds moves along
//      the edge its phase-2 reduced cost improves (either way when that cost
//      is 0) until it reaches a bound or a basic variable blocks, which
//      then leaves the basis (the moving variable enters);
//   3. a composite primal simplex: phase 1 minimises the sum of the basic
//      variables' bound violations (a violated basic blocks at the bound it
//      reaches), phase 2 the cost; Devex pricing, a two-pass (Harris)
//      ratio test preferring large pivots, Bland's rule after 100
//      consecutive degenerate steps; repeated until a fresh factorisation's
//      values and duals are clean;
//   4. a last push of variables still inside their bounds (reduced cost
//      0, so the objective does not move).
// An unbounded edge or a stuck phase 1 is confirmed on a fresh factorisation
// before it ends the run, and a run from the crash basis that does not end
// optimal is repeated once from the slack basis.
// B^-1 is kept explicitly (dense, m x m; product-form updates, Gauss-Jordan
// refactorisation with partial pivoting every m pivots), so the host work
// per pivot is O(m^2), split over up to 16 host threads: LPs up to
// kCrossoverMaxRows rows.
#pragma once

#include <cstdint>

namespace igx {

constexpr int kCrossoverMaxRows = 2048;

// outcome codes
constexpr int kXoOptimal = 0;     // optimal basis; x, y, basis filled
constexpr int kXoIterLimit = 1;   // pivot cap reached
constexpr int kXoSingular = 2;    // a refactorisation met a singular basis
constexpr int kXoUnbounded = 3;   // phase 2 found an unbounded edge
constexpr int kXoInfeasible = 4;  // phase 1 ended with violations left
constexpr int kXoTooLarge = 5;    // m > kCrossoverMaxRows

// basis codes of the n structurals followed by the m row activities
constexpr signed char kAtLower = 0, kAtUpper = 1, kBasic = 2, kSuperbasic = 3;

struct CrossoverInfo {
    int status = kXoOptimal;
    int64_t pushes = 0, pivots = 0, bound_flips = 0, phase1_iters = 0, refactors = 0;
    int64_t basis_repairs = 0;    // dependent basis columns swapped for slacks
    int64_t superbasic_left = 0;  // variables not at a bound and not basic
    double time_ms = 0.0;
};

// A (m x n) as CSC. x (n), y (m; reduced cost d = c + A^T y) and basis
// (n + m, may be NULL) are written for every outcome but kXoTooLarge; they
// hold an optimal vertex pair only for kXoOptimal.
int crossover(int m, int n, const int* cp, const int* ci, const double* acx, const double* c,
              const double* cl, const double* cu, const double* rmin, const double* rmax,
              const double* x0, double* x, double* y, signed char* basis, CrossoverInfo& info);

}  // namespace igx
