/*
 * CPU oracle for the PDHG LP engine -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference engine's algorithm
 * (src/pdhg/pdhg.cu and src/io/model.hpp of IGAOS). It exists to check the
 * CUDA engine: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg (and its --impl reference arm) may load it. The product
 * (igaos_gb300/) never links, imports or falls back to it.
 *
 * Parity pins: orc_evaluate and orc_counting_sort are compared bit-for-bit
 * against the reference's own evaluate() / counting_sort() compiled from the
 * reference sources (oracle/Makefile -> oracle/_ref), through the fixtures in
 * tests/golden/. The full orc_pdhg_solve is pinned against the reference
 * simplex optimum (also compiled from the reference sources) and the
 * reference's recorded Netlib PDHG objectives.
 */
#ifndef IGAOS_PDHG_ORACLE_H
#define IGAOS_PDHG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double pinf, dinf, gap, op, od, prow;
} orc_metrics;

typedef struct {
    int m, n;
    int64_t nnz;
    const int *ap, *ai;
    const double* ax; /* CSR of A, m x n */
    const int *cp, *ci;
    const double* acx; /* CSC of A (CSR of A^T) */
    const double *c, *cl, *cu, *rmin, *rmax;
    double obj_const;
} orc_lp;

typedef struct {
    double time_limit_s;
    double tolerance;
    int64_t max_iterations;
    int check_period; /* 64 in the reference */
    int threads;      /* OpenMP threads for SpMV / vector loops (1 = serial) */
    int verbosity;
    /* test perturbation: at the first check at or after this iteration, 1e6
     * is added to every entry of the current (scaled) x before its metrics
     * are taken, as the engine's IGAOS_PDHG_PERTURB_AT does; 0: never */
    int64_t perturb_at;
} orc_options;

typedef struct {
    int status; /* 1 near-optimal, 5 iteration-limit, 6 time-limit, 7 error */
    double objective, pinf, dinf, gap, prow;
    int64_t iterations, attempts, restarts, checks;
    double seconds;      /* power iteration + iteration loop */
    double loop_seconds; /* iteration loop only */
    double eta, omega; /* final step controller state (scaled units) */
    int64_t rollbacks; /* incumbent restores (reference :965-988) */
} orc_result;

/* reference src/pdhg/pdhg.cu:173-254 */
void orc_evaluate(int m, int n, const double* rmin, const double* rmax,
                  const double* cl, const double* cu, const double* c,
                  const double* x, const double* y, const double* Ax,
                  const double* d, orc_metrics* out);

/* reference src/io/model.hpp:39-67 */
void orc_counting_sort(int64_t nt, const int* ti, const int* tj,
                       const double* tv, int rows, int cols, int* ap, int* ai,
                       double* ax, int* cp, int* ci, double* acx);

/* CSR -> CSR of the transpose, stable in CSR order (entries of each column
 * in increasing row order, row ties in CSR position order). */
void orc_transpose(int rows, int cols, const int* ap, const int* ai,
                   const double* ax, int* cp, int* ci, double* acx);

/* y = A x over CSR, sequential sum per row in storage order. */
void orc_spmv(int rows, const int* ptr, const int* idx, const double* val,
              const double* x, double* y, int threads);

/* reference src/pdhg/pdhg.cu:472-492 (10 sweeps) + :491-492 */
void orc_ruiz(const orc_lp* lp, int sweeps, double* dr, double* dc);

/* reference src/pdhg/pdhg.cu:499-513: scaled copies of the problem. */
void orc_scale(const orc_lp* lp, const double* dr, const double* dc,
               double* sax, double* sacx, double* sc, double* scl,
               double* scu, double* srmin, double* srmax);

/* reference src/pdhg/pdhg.cu:605-631: lambda ~ ||A~||_2^2 by 30 power
 * iterations on A~^T A~ starting from 1/sqrt(n). */
double orc_power_iteration(int m, int n, const int* ap, const int* ai,
                           const double* sax, const int* cp, const int* ci,
                           const double* sacx, int iters, int threads);

/* One line-search attempt (reference kern_primal / kern_dual / kern_dots,
 * src/pdhg/pdhg.cu:33-125), on scaled data. ata = A~^T y must be given. */
void orc_primal(int n, double tau, const double* x, const double* c,
                const double* ata, const double* lo, const double* hi,
                double* xnew, double* xbar, double* dx);
void orc_dual(int m, double sigma, const double* y, const double* axb,
              const double* rmin, const double* rmax, const double* axcur,
              double* ynew, double* dy, double* adx);
void orc_dots(int n, int m, const double* dx, const double* dy,
              const double* adx, double out[3]);

/* Iterate state of the scaled problem (for stepwise parity tests). */
typedef struct {
    double *x, *y, *xavg, *yavg, *axcur; /* scaled units */
    double eta, omega;
    int64_t k;  /* next iteration index (starts at 1) */
    int64_t hn; /* Halpern counter */
} orc_state;

/* Runs `iters` accepted PDHG iterations (line search + averaging, reference
 * src/pdhg/pdhg.cu:748-799) on the scaled problem, no checks or restarts.
 * Returns the number of attempts made. */
int64_t orc_iterate(int m, int n, const int* ap, const int* ai,
                    const double* sax, const int* cp, const int* ci,
                    const double* sacx, const double* sc, const double* scl,
                    const double* scu, const double* srmin,
                    const double* srmax, orc_state* st, int64_t iters,
                    int threads);

/* Full solve, reference src/pdhg/pdhg.cu:457-1156 minus dual_repair
 * (:288-448, :854-931). x (n) and y (m) receive the original-unit answer. */
int orc_pdhg_solve(const orc_lp* lp, const orc_options* opt, orc_result* res,
                   double* x, double* y);

void orc_default_options(orc_options* o);

/* reference src/pdhg/pdhg.cu:257-448: certifiable dual near y_it for the
 * primal candidate x (original units, Ax = A x). Returns 1 when a dual with a
 * finite gap was found (y = the best-gap one), else 0 (y = the point of least
 * sign violation, or NaN when the dense factorisation failed). */
int orc_dual_repair(const orc_lp* lp, const double* x, const double* Ax,
                    const double* y_it, double col_tol, double* y);

#ifdef __cplusplus
}
#endif
#endif
