/*
 * igaos_pdhg -- C ABI of the GB300 PDHG LP engine.
 *
 * This is the boundary the reference's PDHG path sits behind: the reference
 * exposes `igaos::Solution igaos::pdhg::solve(const io::Model&, const
 * Options&)` (src/pdhg/pdhg.hpp:9), called only from
 * igaos::solve_with_engine(model, opts, "pdhg") (src/api/engine.hpp:32-38).
 * Every entry point here takes plain pointers and sizes, never throws, and
 * reports failure as a nonzero IGAOS_PDHG_ERR_* code with a message readable
 * through igaos_pdhg_last_error(). The C++ igaos::pdhg::solve of this repo is
 * a thin wrapper over igaos_pdhg_create / igaos_pdhg_solve.
 *
 * Conventions shared with the reference model (src/io/model.hpp:16-37):
 *   minimise c^T x + obj_const  s.t.  rmin <= A x <= rmax,  cl <= x <= cu,
 *   A is m x n, CSR (ap[m+1], ai[nnz], ax[nnz]) with int32 indices, FP64
 *   values; absent bounds are +-INFINITY. The dual y follows the reference
 *   sign convention: reduced cost d = c + A^T y.
 */
#ifndef IGAOS_PDHG_H
#define IGAOS_PDHG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IGAOS_PDHG_ABI_VERSION 4

/* Return codes of every entry point. */
enum {
    IGAOS_PDHG_OK = 0,
    IGAOS_PDHG_ERR_INVALID = 1,  /* bad argument: sizes, NULL, NaN in data */
    IGAOS_PDHG_ERR_CUDA = 2,     /* CUDA runtime failure */
    IGAOS_PDHG_ERR_NOMEM = 3,    /* device allocation failed */
    IGAOS_PDHG_ERR_NODEVICE = 4, /* no usable CUDA device */
    IGAOS_PDHG_ERR_NUMERIC = 5,  /* NaN/Inf appeared in the iterates */
    IGAOS_PDHG_ERR_TIMEOUT = 6   /* a bounded device wait ran out */
};

/* Solution status, same order and meaning as igaos::Status
 * (include/igaos/status.h:5-14 of the reference). */
enum {
    IGAOS_STATUS_OPTIMAL = 0,
    IGAOS_STATUS_NEAR_OPTIMAL = 1,
    IGAOS_STATUS_FEASIBLE = 2,
    IGAOS_STATUS_INFEASIBLE = 3,
    IGAOS_STATUS_UNBOUNDED = 4,
    IGAOS_STATUS_ITERATION_LIMIT = 5,
    IGAOS_STATUS_TIME_LIMIT = 6,
    IGAOS_STATUS_ERROR = 7
};

/* Arithmetic of the iteration loop. */
enum {
    IGAOS_PDHG_FP64 = 0,        /* reference algorithm, all FP64 */
    IGAOS_PDHG_FP32_REFINE = 1, /* FP32 iterates + FP64 residual refinement */
    IGAOS_PDHG_FP32 = 2         /* FP32 iterates, FP64 checks, no refinement */
};

/* Options. The first seven fields mirror igaos::Options
 * (include/igaos/options.h:5-13 of the reference) with the same defaults;
 * the rest are engine controls. As in the reference engine
 * (src/pdhg/pdhg.cu:669-671), max_iterations only binds when the time limit
 * is not finite (<= 0 or >= 1e6); otherwise the cap is 20,000,000. */
typedef struct igaos_pdhg_options {
    double time_limit_s;      /* 120 */
    double tolerance;         /* 1e-4: relative KKT (pinf, prow, dinf, gap) */
    int64_t max_iterations;   /* 500000 */
    int seed;                 /* ignored, as in the reference engine */
    int presolve;             /* ignored, as in the reference engine (see pdhg_presolve) */
    int restarts;             /* ignored: the engine always restarts */
    int verbosity;            /* 0 quiet, 1 progress, 2 debug (stderr) */
    int precision;            /* IGAOS_PDHG_FP64 (default) / FP32_REFINE / FP32 */
    int check_period;         /* 64: iterations between KKT checks */
    double inner_tolerance;   /* FP32_REFINE: tolerance of each FP32 solve (1e-4) */
    int max_refinements;      /* FP32_REFINE: outer rounds (12) */
    int use_graphs;           /* 1: replay captured CUDA graphs of attempts */
    int device;               /* CUDA device ordinal (-1: current) */
    /* 1: at every restart, test the change between consecutive restart
     * points as an infeasibility certificate (a dual ray: the LP is
     * infeasible; a primal ray: its dual is, so a feasible LP is unbounded),
     * in original units, and stop with IGAOS_STATUS_INFEASIBLE /
     * IGAOS_STATUS_UNBOUNDED when the same kind holds at two consecutive
     * restarts; the ray is returned in y / x (max-norm 1). 0 (default): off,
     * as the reference engine, which has no such test. Added in ABI 2. */
    int detect_infeasibility;
    /* 1: reduce the LP on the host before the upload (empty, singleton,
     * redundant, forcing and parallel rows; fixed, empty and free or
     * implied-free singleton columns; see igaos_pdhg_presolve) and map the
     * answer back with exact duals; the
     * result's metrics are then those of the ORIGINAL LP. The handle's
     * inspection entry points (get_scaling ... spmv) refuse it. A ray of
     * detect_infeasibility, and the ray behind a presolve outcome of
     * infeasible / unbounded, are mapped to the original LP and checked there with
     * igaos_pdhg_ray_certificate's test; if that check fails, x / y hold
     * the reduced LP's ray on the surviving rows and columns (0 elsewhere).
     * 0 (default): off, as the reference engine, which ignores `presolve`.
     * Read by igaos_pdhg_create. Added in ABI 3. */
    int pdhg_presolve;
    /* 1: after the solve, run igaos_pdhg_crossover on the host from the
     * answer's x (LPs with m <= 2048); when it ends at an optimal basis whose
     * pair passes the tolerance on the original LP, that vertex replaces the
     * answer and the status is IGAOS_STATUS_OPTIMAL (the PDHG answer alone is
     * NEAR_OPTIMAL). Read by igaos_pdhg_create. 0 (default): off. Added in
     * ABI 3. */
    int crossover;
    /* Diagonal scaling of the LP before the iterations:
     * IGAOS_PDHG_SCALING_RUIZ (0, default): 10 Ruiz sweeps, as the reference
     * (src/pdhg/pdhg.cu:472-492, cost scale 1 at :494-498).
     * IGAOS_PDHG_SCALING_RUIZ_PC (1): the same sweeps, then one
     * Pock-Chambolle pass with alpha = 1 (rows divided by the square root of
     * their scaled 1-norm, columns likewise, both from the same matrix), the
     * scaling of PDLP (Applegate et al. 2021). Read by igaos_pdhg_create.
     * Added in ABI 4. */
    int scaling;
    /* Warp schedule of the attempt kernels (how many lanes share a row of
     * each length, and so how many rows a warp item holds):
     * IGAOS_PDHG_SCHEDULE_FIXED (0, default): about 8 entries per lane.
     * IGAOS_PDHG_SCHEDULE_AUTOTUNE (1): at the first solve of each precision
     * on a handle, the A and A^T attempt kernels are timed on schedules of 2, 4,
     * 8, 16 and 32 entries per lane (8 launches each; FP64 kernels
     * also at 3 and 4 resident CTAs per SM) and the fastest is kept for that
     * handle and precision; the result's entries_a / entries_at report the
     * choice. The schedule changes the order of each
     * row's sum, so results match the fixed schedule's to rounding, not bit
     * for bit, and two handles may choose differently. Added in ABI 4. */
    int schedule;
} igaos_pdhg_options;

/* Values of igaos_pdhg_options.schedule. */
enum {
    IGAOS_PDHG_SCHEDULE_FIXED = 0,
    IGAOS_PDHG_SCHEDULE_AUTOTUNE = 1
};

/* Values of igaos_pdhg_options.scaling. */
enum {
    IGAOS_PDHG_SCALING_RUIZ = 0,
    IGAOS_PDHG_SCALING_RUIZ_PC = 1
};

typedef struct igaos_pdhg_result {
    int status;               /* IGAOS_STATUS_* */
    int error_code;           /* IGAOS_PDHG_OK or IGAOS_PDHG_ERR_* */
    double objective;         /* c^T x + obj_const, original units */
    double pinf, dinf, rel_gap, prow;
    int64_t iterations;       /* accepted PDHG iterations (all rounds) */
    int64_t attempts;         /* line-search attempts */
    int64_t kkt_checks;       /* KKT evaluations */
    int64_t restarts;
    int64_t kkt_passes;       /* matrix passes: one A + one A^T product each */
    int refinements;          /* FP32_REFINE outer rounds taken */
    double solve_time_ms;     /* solve loop wall time (setup excluded) */
    double setup_time_ms;     /* upload + scaling + power iteration */
    double device_time_ms;    /* solve, CUDA events on the engine stream */
    double attempt_time_ms;   /* of which in line-search attempt launches */
    int64_t launches;         /* engine kernel launches during the solve */
    int64_t rollbacks;        /* restores of the incumbent after a blow-up
                                 (src/pdhg/pdhg.cu:965-988); added in ABI 4 */
    int32_t entries_a;        /* entries per lane of the schedules used for A */
    int32_t entries_at;       /* ... and for A^T (ABI 4; see options.schedule) */
    char message[160];
} igaos_pdhg_result;

typedef struct igaos_pdhg_problem igaos_pdhg_problem;

/* ABI version (IGAOS_PDHG_ABI_VERSION). No reference counterpart. */
int igaos_pdhg_abi_version(void);

/* Calibration of the gather-bound roofline (no reference counterpart): the
 * rate, in 4-byte gathers per second for the whole GPU, at which the device
 * serves random reads of a resident zero vector of 2^log2_words floats
 * (10..28), with 8 independent gathers in flight per thread and 8 CTAs of
 * 256 threads per SM; best of 3 launches after a warming one. */
int igaos_pdhg_gather_rate(int log2_words, int device, double* gathers_per_s);

/* The infeasibility-certificate test of detect_infeasibility, on host arrays
 * (no device needed; no reference counterpart). A candidate (x, y) with
 * ax = A x and aty = A^T y, ORIGINAL units, is normalised to max-norm 1 and
 * tested as a dual ray y (*kind = 1: with d = A^T y, every d_j and y_i has a
 * sign its finite bound allows and sum_j d_j (l_j or u_j) - sum_i y_i (rmax_i
 * or rmin_i) > 0: the LP is infeasible) or a primal ray x (*kind = 2: x and
 * A x in the recession cones of the column and row bounds and c^T x < 0: the
 * dual is infeasible). Sign violations up to 1e-9 of the ray's scale are
 * tolerated; the objective must exceed 1e-6 of its terms' magnitude.
 * *kind = 0: neither. The normalised ray goes to yray (m) / xray (n) when
 * non-NULL. */
int igaos_pdhg_ray_certificate(int m, int n, const double* x, const double* ax, const double* y,
                               const double* aty, const double* c, const double* cl,
                               const double* cu, const double* rmin, const double* rmax,
                               double* xray, double* yray, int* kind);

/* ---- presolve (host only; no device needed) ----------------------------
 * The reductions of the pdhg_presolve option, callable on their own. The
 * reference's PDHG path has none (its solve ignores Options.presolve); its
 * simplex presolve (src/simplex/presolve.hpp:176-600) maps back x only. Here
 * every reduction has an exact dual postsolve: an optimal pair of the reduced
 * LP maps to an optimal pair of the original.
 * igaos_pdhg_presolve reduces the CSR LP; *outcome = 0 (reduced: *out holds
 * it, possibly with no rows and no columns), IGAOS_STATUS_INFEASIBLE (a row
 * whose bounds its activity cannot meet) or IGAOS_STATUS_UNBOUNDED (a column
 * whose cost runs to an infinite bound: the LP is unbounded if it is
 * feasible). *out is a handle for every outcome; for the last two only
 * igaos_pdhg_presolved_ray and _destroy accept it. */
typedef struct igaos_pdhg_presolved igaos_pdhg_presolved;

int igaos_pdhg_presolve(int m, int n, int64_t nnz, const int* ap, const int* ai,
                        const double* ax, const double* c, const double* cl,
                        const double* cu, const double* rmin, const double* rmax,
                        double obj_const, igaos_pdhg_presolved** out, int* outcome);

/* Sizes and constant of the reduced LP; counts6 (may be NULL) = empty rows,
 * singleton rows, redundant rows (forcing and parallel ones included), fixed
 * columns, empty columns and free or implied-free singleton columns
 * removed. */
int igaos_pdhg_presolved_info(const igaos_pdhg_presolved* p, int* m, int* n, int64_t* nnz,
                              double* obj_const, int64_t* counts6);

/* The reduced LP: ap (m+1), ai, ax (nnz), c, cl, cu (n), rmin, rmax (m). */
int igaos_pdhg_presolved_lp(const igaos_pdhg_presolved* p, int* ap, int* ai, double* ax,
                            double* c, double* cl, double* cu, double* rmin, double* rmax);

/* x (original n) and y (original m) from x_red, y_red of the reduced LP. */
int igaos_pdhg_postsolve(const igaos_pdhg_presolved* p, const double* x_red,
                         const double* y_red, double* x, double* y);

/* The same map for a ray of the reduced LP (costs, fixed values and row
 * targets taken as 0): a dual ray y_red (reduced costs pressing on a bound a
 * singleton row set move into that row) and a primal ray x_red map to rays
 * of the original LP. */
int igaos_pdhg_postsolve_ray(const igaos_pdhg_presolved* p, const double* x_red,
                             const double* y_red, double* x, double* y);

/* The certificate behind presolve's outcome, in the original LP: for
 * IGAOS_STATUS_UNBOUNDED, x (n) = the primal ray of the column whose cost
 * runs to an infinite bound (columns substituted before it follow their
 * rows); for IGAOS_STATUS_INFEASIBLE, y (m) = a dual ray: +-1 on the row
 * that proved it, mapped back through the reductions made before (e.g. onto
 * the singleton rows that set the bounds it crossed). The other vector is
 * 0. IGAOS_PDHG_ERR_INVALID when presolve found no such ray. */
int igaos_pdhg_presolved_ray(const igaos_pdhg_presolved* p, double* x, double* y);

void igaos_pdhg_presolved_destroy(igaos_pdhg_presolved* p);

/* ---- crossover (host only; no device needed) ----------------------------
 * From a start point x0 (n; a PDHG answer, or any point) to an optimal
 * vertex of the LP: primal push of the structurals inside their bounds from
 * the slack basis, then a composite primal simplex (phase 1 on the basic
 * bound violations, phase 2 on the cost) with a dense explicit basis
 * inverse, so m <= 2048. No reference counterpart: the reference's PDHG
 * returns its last iterate, its simplex (src/simplex/simplex.hpp:12-28)
 * takes no start point. On status 0, x (n) and y (m; d = c + A^T y) are an
 * optimal basic pair and basis (n + m, may be NULL) holds 0 at lower, 1 at
 * upper, 2 basic, 3 inside its bounds (nonbasic with reduced cost 0) for
 * the structurals and then the row activities. */
typedef struct igaos_pdhg_crossover_info {
    int status;               /* 0 optimal vertex, 1 pivot cap, 2 singular basis,
                                 3 unbounded edge, 4 infeasible (phase 1), 5 m > 2048 */
    int pad;
    int64_t pushes, pivots, bound_flips, phase1_iterations, refactorizations;
    int64_t basis_repairs;    /* dependent basis columns swapped for row slacks */
    int64_t superbasic_left;  /* variables left inside their bounds, nonbasic */
    double time_ms;
} igaos_pdhg_crossover_info;

int igaos_pdhg_crossover(int m, int n, int64_t nnz, const int* ap, const int* ai,
                         const double* ax, const double* c, const double* cl,
                         const double* cu, const double* rmin, const double* rmax,
                         const double* x0, double* x, double* y, signed char* basis,
                         igaos_pdhg_crossover_info* info);

/* Number of visible CUDA devices (0 when none). Replaces the handle-creation
 * probe of src/pdhg/pdhg.cu:459-465. */
int igaos_pdhg_device_count(void);

/* Fills *o with the defaults above. Mirrors igaos::Options{} defaults. */
void igaos_pdhg_default_options(igaos_pdhg_options* o);

/* Copies the calling thread's last error message into buf (NUL-terminated,
 * truncated to len); returns the last error code. Replaces Solution.message
 * on failure paths ("CUDA error in PDHG engine", src/pdhg/pdhg.cu:14-23). */
int igaos_pdhg_last_error(char* buf, size_t len);

/* Uploads an LP and prepares it on the device: Ruiz scaling (10 sweeps,
 * src/pdhg/pdhg.cu:472-492), scaled FP64/FP32 copies (:499-513), SpMV tile
 * schedules, power iteration (:605-631). Replaces the upload block
 * src/pdhg/pdhg.cu:515-603. cp/ci/acx may all be NULL: A^T is then built from
 * the CSR by a stable counting sort (bit-identical values, the orientation
 * src/io/model.hpp:39-67 builds). Host buffers are only read during the call. */
int igaos_pdhg_create(igaos_pdhg_problem** out, int m, int n, int64_t nnz,
                      const int* ap, const int* ai, const double* ax,
                      const int* cp, const int* ci, const double* acx,
                      const double* c, const double* cl, const double* cu,
                      const double* rmin, const double* rmax, double obj_const,
                      const igaos_pdhg_options* opt);

/* Solves the uploaded LP. x (n) and y (m) may be NULL; else they receive the
 * answer in original units. Replaces the solve loop + unscale of
 * src/pdhg/pdhg.cu:605-1141; result fields mirror igaos::Solution
 * (include/igaos/solution.h:10-22). The problem can be solved again. */
int igaos_pdhg_solve(igaos_pdhg_problem* p, const igaos_pdhg_options* opt,
                     igaos_pdhg_result* res, double* x, double* y);

/* Frees every device buffer of the problem (src/pdhg/pdhg.cu:1143-1154). */
void igaos_pdhg_destroy(igaos_pdhg_problem* p);

/* Convenience: create + solve + destroy in one call, the shape of the
 * reference's pdhg::solve(Model, Options). */
int igaos_pdhg_solve_csr(int m, int n, int64_t nnz, const int* ap,
                         const int* ai, const double* ax, const int* cp,
                         const int* ci, const double* acx, const double* c,
                         const double* cl, const double* cu,
                         const double* rmin, const double* rmax,
                         double obj_const, const igaos_pdhg_options* opt,
                         igaos_pdhg_result* res, double* x, double* y);

/* ---- inspection entry points (parity tests, tooling) --------------------
 * Row/column scaling factors dr (m), dc (n) computed at create: the Ruiz
 * vectors of src/pdhg/pdhg.cu:472-492. */
int igaos_pdhg_get_scaling(const igaos_pdhg_problem* p, double* dr, double* dc);

/* Power-iteration estimate of ||A~||_2^2 (src/pdhg/pdhg.cu:605-631) and the
 * initial step eta0 = 1.2/sqrt(lambda) and weight omega0 (:642-663). */
int igaos_pdhg_get_step_init(const igaos_pdhg_problem* p, double* lambda,
                             double* eta0, double* omega0);

/* The device-built A^T (CSR of the transpose of the scaled A): pointers,
 * indices and FP64 values (src/io/model.hpp:39-67 orientation). */
int igaos_pdhg_get_transpose(const igaos_pdhg_problem* p, int* cp, int* ci,
                             double* acx_scaled);

/* Runs exactly `iters` accepted PDHG iterations (adaptive line search +
 * Halpern averaging, src/pdhg/pdhg.cu:748-799) from the given scaled-unit
 * state, without KKT checks or restarts, in the given precision, and returns
 * the new state. state6 = {eta, omega, k, hn, attempts(out), parity(out)};
 * x, y, xavg, yavg, axcur are read and overwritten (scaled units, FP64). */
int igaos_pdhg_iterate(igaos_pdhg_problem* p, int precision, int64_t iters,
                       double* x, double* y, double* xavg, double* yavg,
                       double* axcur, double* state6);

/* Matrix-free dual repair on the device, for any m (the solve loop runs the
 * same step on the reference's schedule, src/pdhg/pdhg.cu:854-931: from
 * k = 5000, spacing 2000 tripling up to 30000; col_tol tiers 1e-6, 1e-1).
 * Replaces the reference's dual_repair (src/pdhg/pdhg.cu:257-448).
 * Same three sets as the reference's dual_repair (src/pdhg/pdhg.cu:288-448)
 * on the Ruiz-scaled LP: the regularised least-squares step onto
 * {A_J^T y = -c_J} by CGLS instead of a dense Cholesky solve, all violated
 * sign half-spaces at once (component-averaged) instead of one at a time,
 * then the row cone; two anchors (y_it, 0), up to 150 rounds each, stopping
 * at the first dual certified at `tol`. x and y_it in ORIGINAL units, the
 * caller's numbering. *certified = 1 when pinf, prow and a finite gap of
 * (x, y) are all <= tol; y = the dual with the smallest finite gap seen
 * (else the last iterate). metrics6 (may be NULL) = pinf, dinf, gap, op, od,
 * prow of (x, y). Unlike the reference's dense m x m factor it needs no
 * memory beyond a few n- and m-vectors. */
int igaos_pdhg_dual_repair_device(igaos_pdhg_problem* p, const double* x, const double* y_it,
                                  double col_tol, double tol, double* y, int* certified,
                                  double* metrics6);

/* Start point of the following solves on this handle (until replaced; two
 * NULLs clear it): x0 (n) and y0 (m) in ORIGINAL units, the caller's
 * numbering. The iterates start there instead of at zero (x0 projected onto
 * the column bounds; the reference starts at zero, src/pdhg/pdhg.cu:576-580);
 * FP32 + refinement takes it as its first anchor. Step size and primal
 * weight start as usual. Not available on a presolved handle. */
int igaos_pdhg_set_start(igaos_pdhg_problem* p, const double* x0, const double* y0);

/* FP64 KKT metrics of (x, y) given in ORIGINAL units, evaluated on the
 * device (the fused pass replacing src/pdhg/pdhg.cu:173-254 + :698-733).
 * out6 = {pinf, dinf, gap, op, od, prow}. */
int igaos_pdhg_evaluate(igaos_pdhg_problem* p, const double* x,
                        const double* y, double* out6);

/* y = A~ x or A~^T x (transpose != 0) with the engine's tiled SpMV on the
 * scaled matrix, in FP64 (precision 0) or FP32 (precision 2; x and y are
 * still passed as FP64 host arrays). Replaces Spmv::mv (cuSPARSE,
 * src/pdhg/pdhg.cu:143-157). */
int igaos_pdhg_spmv(igaos_pdhg_problem* p, int transpose, int precision,
                    const double* x, double* y);

/* ---- batched solve ------------------------------------------------------
 * Per-instance outcome of igaos_pdhg_solve_batch. */
typedef struct igaos_pdhg_batch_result {
    int status;              /* IGAOS_STATUS_* */
    int finished_fp64;       /* 1: the persistent launch handed this instance off
                                or left it at max_iterations, and the
                                single-LP engine finished it in FP64 (ABI 4;
                                was padding) */
    double objective;        /* c^T x of the instance */
    double pinf, dinf, rel_gap, prow;
    int64_t iterations, attempts, restarts;
    double kernel_time_ms;   /* the whole batch's persistent kernel (same for all) */
    double total_time_ms;    /* the whole call: upload, kernel, download */
    double instance_time_ms; /* this instance, from its CTA taking it to its answer
                                (plus its FP64 finish, if it had one) */
} igaos_pdhg_batch_result;

/* Solves `count` independent LPs of uneven sizes in one persistent kernel
 * launch: instance b is m[b] x n[b]; its CSR row pointer (m[b]+1 entries,
 * starting at 0) follows the previous instance's in `ap`, its column indices
 * (local, 0..n[b]-1, no duplicate (row, column) entries) and values follow in
 * `ai`/`ax`, its c/cl/cu in the concatenated n-vectors and rmin/rmax in the
 * concatenated m-vectors. Each instance runs the engine's iteration (Ruiz,
 * power iteration, adaptive line search, averaging, restarts, primal weight;
 * FP32 iterates, termination metrics combined in FP64) to `tolerance` or
 * `max_iterations` on its own, with its own restarts and termination; the
 * reference has no batched path (its engine is one LP per call,
 * src/pdhg/pdhg.hpp:9). FP32 iterates can stall where FP64 ones do not:
 * the first 16 instances still running at 100,000 iterations stop there
 * (environment IGAOS_PDHG_BATCH_HANDOFF / _MAX change both numbers; 0
 * iterations turns the hand-off off), and those, with any instance the
 * launch leaves at max_iterations, are solved again by the single-LP engine
 * in FP64 (the reference's arithmetic) under the same tolerance and
 * iteration cap, up to 8 at once on their own streams. Their results say so
 * (finished_fp64), and `iterations` counts both runs. x (sum n) and y
 * (sum m) may be NULL. */
int igaos_pdhg_solve_batch(int count, const int* m, const int* n,
                           const int* ap, const int* ai, const double* ax,
                           const double* c, const double* cl, const double* cu,
                           const double* rmin, const double* rmax,
                           const igaos_pdhg_options* opt,
                           igaos_pdhg_batch_result* res, double* x, double* y);

/* Allocation-free FP64 KKT metrics, for callers that cannot call cudaMalloc
 * (device memory owned by a framework allocator or a fixed pool, or loops
 * where an allocation's device synchronisation is not acceptable). No
 * counterpart in the reference. Every pointer is a DEVICE pointer owned by
 * the caller: A in original units as CSR (ap, ai, ax) and CSC (cp, ci, acx),
 * c, cl, cu (n), rmin, rmax (m), the candidate x (n), y (m), and out6, which
 * receives {pinf, dinf, gap, op, od, prow} as evaluate() defines them
 * (src/pdhg/pdhg.cu:173-254). Work is enqueued on `stream` (a cudaStream_t,
 * NULL = default stream); the caller synchronises before reading out6.
 * Scratch is a fixed 1 MiB array in device memory that every GPU loading the
 * library holds until exit; m and n are limited to 4,194,304 (larger sizes
 * return IGAOS_PDHG_ERR_INVALID). The first call on a device looks up that
 * array's device address (no allocation); make that first call before any
 * stream capture. All calls share the array: calls that overlap on the GPU
 * (other streams, other threads) race and must be serialised by the caller.
 * Nothing is allocated: no cudaMalloc, cudaFree or allocating library call. */
int igaos_pdhg_evaluate_noalloc(int m, int n, const int* ap, const int* ai,
                                const double* ax, const int* cp, const int* ci,
                                const double* acx, const double* c,
                                const double* cl, const double* cu,
                                const double* rmin, const double* rmax,
                                const double* x, const double* y, double* out6,
                                void* stream);

/* ---- Differentiable LP layer: K unrolled PDHG iterations ----------------
 * No counterpart in the reference (its engine has no gradient path). A batch
 * of ridge-regularised LPs
 *     min c^T x + ridge ||x||^2   s.t.  rmin <= A x <= rmax,  cl <= x <= cu
 * is run for exactly K PDHG iterations with fixed steps (tau, sigma) per
 * instance, from x0 = clamp(0, cl, cu), y0 = 0, in the reference's sign
 * convention (reduced cost d = c + A^T y, src/pdhg/pdhg.cu:33-58):
 *     x+ = clamp((x - tau (c + A^T y)) / (1 + 2 ridge tau), cl, cu)
 *     t  = y + sigma A (2 x+ - x),   y+ = t - sigma clamp(t / sigma, rmin, rmax)
 * The outputs are x_K, y_K and obj = c^T x_K + ridge ||x_K||^2. The backward
 * entry is the exact reverse mode of those K iterations (clamps
 * differentiated almost everywhere: the gradient passes where the argument is
 * strictly inside the bounds), replaying each `checkpoint`-long segment from
 * its stored iterate. Every pointer is a DEVICE pointer owned by the caller;
 * value arrays hold float (precision IGAOS_PDHG_FP32) or double
 * (IGAOS_PDHG_FP64). Work is enqueued on `stream`; nothing is allocated. */
typedef struct igaos_pdhg_unrolled_layout {
    int count;          /* instances (one CTA each) */
    int precision;      /* IGAOS_PDHG_FP32 or IGAOS_PDHG_FP64 */
    int iterations;     /* K >= 1 */
    int checkpoint;     /* checkpoint interval >= 1 */
    double ridge;       /* >= 0 */
    int max_m, max_n;   /* largest instance (shared-memory sizing) */
    int64_t max_nnz;    /* most nonzeros of one instance */
    int64_t total_m, total_n, total_nnz;
    const int* row_off; /* count+1 prefix offsets into the m-vectors */
    const int* col_off; /* count+1 prefix offsets into the n-vectors */
    const int* nz_off;  /* count+1 prefix offsets into the nonzeros */
    const int* ap;      /* local row pointers, instance b at row_off[b] + b */
    const int* ai;      /* local column indices, instance b at nz_off[b] */
    const int* cp;      /* local column pointers, instance b at col_off[b] + b */
    const int* ci;      /* local row index of each CSC entry, at nz_off[b] */
    const int* cperm;   /* local CSR position of each CSC entry, at nz_off[b] */
} igaos_pdhg_unrolled_layout;

/* Elements (of the layout's type) of the checkpoint buffer the forward fills
 * and the backward reads: ceil(K / checkpoint) * (total_n + total_m). */
int64_t igaos_pdhg_unrolled_checkpoint_elems(const igaos_pdhg_unrolled_layout* L);
/* Bytes of backward scratch: checkpoint * (total_n + total_m) * (size + 1). */
int64_t igaos_pdhg_unrolled_workspace_bytes(const igaos_pdhg_unrolled_layout* L);
/* Fixed steps per instance: tau = eta / omega, sigma = eta * omega with
 * eta = 0.9 / ||A||_2 (power iteration, 100 products of A^T A). */
int igaos_pdhg_unrolled_steps(const igaos_pdhg_unrolled_layout* L, const void* ax,
                              double omega, void* tau, void* sigma, void* stream);
/* x (total_n), y (total_m), obj (count), ckpt (checkpoint_elems). */
int igaos_pdhg_unrolled_forward(const igaos_pdhg_unrolled_layout* L, const void* c,
                                const void* cl, const void* cu, const void* rmin,
                                const void* rmax, const void* ax, const void* tau,
                                const void* sigma, void* x, void* y, void* obj,
                                void* ckpt, void* stream);
/* Gradients of <gx, x_K> + <gy, y_K> + <gobj, obj> with respect to c, cl,
 * cu, rmin, rmax and the CSR values ax (each overwritten). gx, gy, gobj may
 * be NULL (zero). x is the forward's x_K; ckpt its checkpoints; work holds
 * workspace_bytes. Steps are constants (no gradient through tau, sigma). */
int igaos_pdhg_unrolled_backward(const igaos_pdhg_unrolled_layout* L, const void* c,
                                 const void* cl, const void* cu, const void* rmin,
                                 const void* rmax, const void* ax, const void* tau,
                                 const void* sigma, const void* ckpt, const void* x,
                                 const void* gx, const void* gy, const void* gobj,
                                 void* gc, void* gcl, void* gcu, void* grmin,
                                 void* grmax, void* gax, void* work, void* stream);

#ifdef __cplusplus
}
#endif
#endif
