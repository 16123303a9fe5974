// C ABI of the GB300 PDHG engine (declared in include/igaos_pdhg.h).
// No exception crosses this boundary: every failure becomes an
// IGAOS_PDHG_ERR_* code plus a thread-local message.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "engine.hpp"
#include "certificate.hpp"
#include "crossover.hpp"
#include "presolve.hpp"
#include "host_kkt.hpp"

struct igaos_pdhg_problem {
    igx::Engine* eng = nullptr;  // NULL when presolve removed the whole LP
    // pdhg_presolve: the reductions and their outcome, the original LP's
    // costs and bounds (metrics of the postsolved answer), the presolve time
    igx::Presolved* pre = nullptr;
    int pre_outcome = 0;
    igx::HostLP orig;
    double obj_const = 0.0;
    double presolve_ms = 0.0;
    // crossover: requested at create (m <= 2048); orig then also holds A as CSC
    bool xo = false;
};

struct igaos_pdhg_presolved {
    igx::Presolved p;
};

namespace {
thread_local int g_code = IGAOS_PDHG_OK;
thread_local char g_msg[512] = "";

int fail(int code, const char* msg) {
    g_code = code;
    std::snprintf(g_msg, sizeof(g_msg), "%s", msg);
    return code;
}
int ok() {
    g_code = IGAOS_PDHG_OK;
    g_msg[0] = 0;
    return IGAOS_PDHG_OK;
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return ok();
    } catch (const igx::CudaError& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(IGAOS_PDHG_ERR_NOMEM, "host allocation failed");
    } catch (const std::invalid_argument& e) {
        return fail(IGAOS_PDHG_ERR_INVALID, e.what());
    } catch (const std::exception& e) {
        return fail(IGAOS_PDHG_ERR_CUDA, e.what());
    }
}

// Structural and numeric validation of the input LP, before any upload.
void validate(int m, int n, int64_t nnz, const int* ap, const int* ai, const double* ax,
              const int* cp, const int* ci, const double* acx, const double* c,
              const double* cl, const double* cu, const double* rmin, const double* rmax) {
    auto bad = [](const char* s) { throw std::invalid_argument(s); };
    if (m <= 0 || n <= 0) bad("problem must have at least one row and one column");
    if (nnz < 0 || nnz > 0x7fffffffLL) bad("nnz must be in [0, 2^31)");
    if (!ap || (nnz > 0 && (!ai || !ax))) bad("CSR arrays must not be NULL");
    if (!c || !cl || !cu || !rmin || !rmax) bad("cost and bound arrays must not be NULL");
    const bool have_t = cp || ci || acx;
    if (have_t && (!cp || (nnz > 0 && (!ci || !acx))))
        bad("pass all of cp, ci, acx or none of them");
    if (ap[0] != 0 || ap[m] != nnz) bad("row pointer must start at 0 and end at nnz");
    for (int i = 0; i < m; ++i)
        if (ap[i + 1] < ap[i]) bad("row pointer must be non-decreasing");
    for (int64_t p = 0; p < nnz; ++p) {
        if (ai[p] < 0 || ai[p] >= n) bad("column index out of range");
        if (!std::isfinite(ax[p])) bad("matrix values must be finite");
    }
    if (have_t) {
        if (cp[0] != 0 || cp[n] != nnz) bad("column pointer must start at 0 and end at nnz");
        for (int j = 0; j < n; ++j)
            if (cp[j + 1] < cp[j]) bad("column pointer must be non-decreasing");
        for (int64_t p = 0; p < nnz; ++p) {
            if (ci[p] < 0 || ci[p] >= m) bad("row index out of range");
            if (!std::isfinite(acx[p])) bad("matrix values must be finite");
        }
    }
    for (int j = 0; j < n; ++j) {
        if (!std::isfinite(c[j])) bad("cost must be finite");
        if (std::isnan(cl[j]) || std::isnan(cu[j])) bad("column bounds must not be NaN");
        if (cl[j] > cu[j]) bad("column lower bound above upper bound");
    }
    for (int i = 0; i < m; ++i) {
        if (std::isnan(rmin[i]) || std::isnan(rmax[i])) bad("row bounds must not be NaN");
        if (rmin[i] > rmax[i]) bad("row lower bound above upper bound");
    }
}

// Stable counting sort of the CSR by column: the CSC orientation that
// src/io/model.hpp:39-67 builds from row-ordered triplets.
void transpose_host(int m, int n, const int* ap, const int* ai, const double* ax,
                    std::vector<int>& cp, std::vector<int>& ci, std::vector<double>& acx) {
    const int64_t nnz = ap[m];
    cp.assign(n + 1, 0);
    ci.resize(nnz);
    acx.resize(nnz);
    for (int64_t p = 0; p < nnz; ++p) cp[ai[p] + 1]++;
    for (int j = 0; j < n; ++j) cp[j + 1] += cp[j];
    std::vector<int> next(cp.begin(), cp.end() - 1);
    for (int i = 0; i < m; ++i)
        for (int p = ap[i]; p < ap[i + 1]; ++p) {
            const int j = ai[p];
            ci[next[j]] = i;
            acx[next[j]] = ax[p];
            ++next[j];
        }
}
constexpr const char* kNotReduced =
    "presolve found the LP infeasible or unbounded: only its ray is available";
bool reduced(const igaos_pdhg_presolved* p) {
    return p->p.unbounded_col < 0 && p->p.infeasible_row < 0 && !p->p.row_red.empty();
}

constexpr const char* kPresolvedInspect =
    "inspection entry points see the engine's LP, which a presolved handle does not share "
    "with its caller";

// A ray (xr, yr) of the ORIGINAL LP checked with the certificate test: true
// and the normalised ray in x / y (whichever are non-NULL; the other part 0)
// when it is a ray of the expected kind (1 dual, 2 primal).
bool original_ray(const igaos_pdhg_problem* p, const double* xr, const double* yr, int kind,
                  double* x, double* y) {
    const igx::Presolved& R = *p->pre;
    const igx::HostLP& L = p->orig;
    const int m0 = R.m0, n0 = R.n0;
    std::vector<double> ax(m0, 0.0), aty(n0, 0.0), xn(n0, 0.0), yn(m0, 0.0);
    for (int j = 0; j < n0; ++j)
        for (int q = R.cp0[j]; q < R.cp0[j + 1]; ++q) {
            ax[R.ci0[q]] += R.acx0[q] * xr[j];
            aty[j] += R.acx0[q] * yr[R.ci0[q]];
        }
    const int got = igx::ray_certificate(m0, n0, xr, ax.data(), yr, aty.data(), L.c.data(),
                                         L.cl.data(), L.cu.data(), L.rmin.data(), L.rmax.data(),
                                         xn.data(), yn.data());
    if (got != kind) return false;
    if (kind == 1) std::fill(xn.begin(), xn.end(), 0.0);
    else std::fill(yn.begin(), yn.end(), 0.0);
    if (x) std::memcpy(x, xn.data(), sizeof(double) * n0);
    if (y) std::memcpy(y, yn.data(), sizeof(double) * m0);
    return true;
}

// igaos_pdhg_solve of a handle made with pdhg_presolve: the engine solves the
// reduced LP, postsolve maps the pair back, and the metrics are taken again
// on the original LP (other norms than the reduced LP's). When the reduced
// LP converged but the original misses the tolerance, the reduced LP is
// solved again at a tenth of the tolerance, at most twice.
int solve_presolved(igaos_pdhg_problem* p, const igaos_pdhg_options& o, igaos_pdhg_result* res,
                    double* x, double* y) {
    const igx::Presolved& R = *p->pre;
    const int m0 = R.m0, n0 = R.n0;
    std::memset(res, 0, sizeof(*res));
    res->setup_time_ms = p->presolve_ms;
    if (p->pre_outcome != igx::kPresolveReduced) {
        const bool inf = p->pre_outcome == igx::kPresolveInfeasible;
        res->status = p->pre_outcome;
        res->objective = res->pinf = res->dinf = res->rel_gap = res->prow = std::nan("");
        std::snprintf(res->message, sizeof(res->message), "%s",
                      inf ? "presolve: the LP is infeasible; y = a dual ray"
                          : "presolve: a column's cost runs to an infinite bound (unbounded if "
                            "feasible); x = its ray");
        std::vector<double> xr(n0, 0.0), yr(m0, 0.0);
        const bool have = inf ? igx::infeasible_ray(R, yr.data()) : igx::unbounded_ray(R, xr.data());
        if (!have || !original_ray(p, xr.data(), yr.data(), inf ? 1 : 2, x, y)) {
            if (x) std::fill(x, x + n0, 0.0);
            if (y) std::fill(y, y + m0, 0.0);
            std::snprintf(res->message, sizeof(res->message), "%s",
                          inf ? "presolve: the LP is infeasible"
                              : "presolve: a column's cost runs to an infinite bound "
                                "(unbounded if feasible)");
        }
        return ok();
    }
    std::vector<double> xr(R.n), yr(R.m), xo(n0), yo(m0), ax(m0), d(n0);
    igaos_pdhg_options oo = o;
    const bool timed = o.time_limit_s > 0.0 && o.time_limit_s < 1e6;
    igaos_pdhg_result rr;
    igx::HostMetrics mt{};
    bool pass = false;
    for (int round = 0;; ++round) {
        if (p->eng) {
            const int rc = guarded([&] { p->eng->solve(oo, rr, xr.data(), yr.data()); });
            if (rc != IGAOS_PDHG_OK) {
                std::memset(res, 0, sizeof(*res));
                res->status = IGAOS_STATUS_ERROR;
                res->error_code = rc;
                std::snprintf(res->message, sizeof(res->message), "%.159s", g_msg);
                return rc;
            }
            if (rr.error_code != IGAOS_PDHG_OK) {
                *res = rr;
                return fail(rr.error_code, rr.message);
            }
        } else {  // presolve removed every row and column
            std::memset(&rr, 0, sizeof(rr));
            rr.status = IGAOS_STATUS_NEAR_OPTIMAL;
            std::snprintf(rr.message, sizeof(rr.message), "solved by presolve");
        }
        res->iterations += rr.iterations;
        res->attempts += rr.attempts;
        res->kkt_checks += rr.kkt_checks;
        res->restarts += rr.restarts;
        res->kkt_passes += rr.kkt_passes;
        res->refinements += rr.refinements;
        res->solve_time_ms += rr.solve_time_ms;
        res->device_time_ms += rr.device_time_ms;
        res->attempt_time_ms += rr.attempt_time_ms;
        res->launches += rr.launches;
        res->rollbacks += rr.rollbacks;
        if (round == 0) res->setup_time_ms += rr.setup_time_ms;
        if (rr.status == IGAOS_STATUS_INFEASIBLE || rr.status == IGAOS_STATUS_UNBOUNDED) {
            // a ray of the reduced LP: mapped to the original and checked there
            res->status = rr.status;
            res->objective = rr.objective;
            res->pinf = rr.pinf;
            res->dinf = rr.dinf;
            res->rel_gap = rr.rel_gap;
            res->prow = rr.prow;
            const bool dual = rr.status == IGAOS_STATUS_INFEASIBLE;
            if (dual) std::fill(xr.begin(), xr.end(), 0.0);
            else std::fill(yr.begin(), yr.end(), 0.0);
            igx::postsolve_ray(R, xr.data(), yr.data(), xo.data(), yo.data());
            if (original_ray(p, xo.data(), yo.data(), dual ? 1 : 2, x, y)) {
                std::snprintf(res->message, sizeof(res->message), "%.159s", rr.message);
            } else {
                std::snprintf(res->message, sizeof(res->message),
                              "%.120s (reduced LP's ray)", rr.message);
                for (int j = 0; j < n0 && x; ++j)
                    x[j] = R.col_red[j] >= 0 ? xr[R.col_red[j]] : 0.0;
                for (int i = 0; i < m0 && y; ++i)
                    y[i] = R.row_red[i] >= 0 ? yr[R.row_red[i]] : 0.0;
            }
            return ok();
        }
        igx::postsolve(R, xr.data(), yr.data(), xo.data(), yo.data());
        std::fill(ax.begin(), ax.end(), 0.0);
        for (int j = 0; j < n0; ++j) {
            double dj = R.c0[j];
            for (int q = R.cp0[j]; q < R.cp0[j + 1]; ++q) {
                ax[R.ci0[q]] += R.acx0[q] * xo[j];
                dj += R.acx0[q] * yo[R.ci0[q]];
            }
            d[j] = dj;
        }
        mt = igx::host_evaluate(p->orig, xo.data(), yo.data(), ax.data(), d.data());
        pass = mt.pinf <= o.tolerance && mt.dinf <= o.tolerance && mt.prow <= o.tolerance &&
               std::isfinite(mt.gap) && mt.gap <= o.tolerance;
        if (pass || rr.status != IGAOS_STATUS_NEAR_OPTIMAL || !p->eng || round == 2) break;
        oo.tolerance *= 0.1;
        if (timed) {
            oo.time_limit_s = o.time_limit_s - res->solve_time_ms / 1000.0;
            if (oo.time_limit_s <= 0.0) break;
        }
    }
    if (pass) res->status = IGAOS_STATUS_NEAR_OPTIMAL;
    else if (rr.status != IGAOS_STATUS_NEAR_OPTIMAL) res->status = rr.status;
    else res->status = mt.pinf <= o.tolerance && mt.prow <= o.tolerance ? IGAOS_STATUS_FEASIBLE
                                                                         : IGAOS_STATUS_ITERATION_LIMIT;
    res->objective = mt.op + p->obj_const;
    res->pinf = mt.pinf;
    res->dinf = mt.dinf;
    res->rel_gap = mt.gap;
    res->prow = mt.prow;
    std::snprintf(res->message, sizeof(res->message), "%.100s; presolve %d->%d rows, %d->%d cols",
                  pass || rr.status != IGAOS_STATUS_NEAR_OPTIMAL
                      ? rr.message
                      : "converged on the reduced LP, original-LP metrics above tolerance",
                  m0, R.m, n0, R.n);
    if (x) std::memcpy(x, xo.data(), sizeof(double) * n0);
    if (y) std::memcpy(y, yo.data(), sizeof(double) * m0);
    return ok();
}
// Crossover after a solve (crossover option): from the answer's x to a
// vertex of the original LP; the vertex replaces the answer (status
// IGAOS_STATUS_OPTIMAL) when crossover ends at an optimal basis whose pair
// passes the tolerance on the original LP. Rays and errors are left alone.
void run_crossover(igaos_pdhg_problem* p, const igaos_pdhg_options& o, igaos_pdhg_result* res,
                   double* x, double* y) {
    const int st = res->status;
    if (st == IGAOS_STATUS_ERROR || st == IGAOS_STATUS_INFEASIBLE ||
        st == IGAOS_STATUS_UNBOUNDED)
        return;
    const igx::HostLP& L = p->orig;
    std::vector<double> xv(L.n), yv(L.m), ax(L.m), d(L.n);
    igx::CrossoverInfo info;
    igx::crossover(L.m, L.n, L.cp.data(), L.ci.data(), L.acx.data(), L.c.data(), L.cl.data(),
                   L.cu.data(), L.rmin.data(), L.rmax.data(), x, xv.data(), yv.data(), nullptr,
                   info);
    res->solve_time_ms += info.time_ms;
    bool taken = false;
    if (info.status == igx::kXoOptimal) {
        for (int j = 0; j < L.n; ++j) {
            double dj = L.c[j];
            for (int q = L.cp[j]; q < L.cp[j + 1]; ++q) {
                ax[L.ci[q]] += L.acx[q] * xv[j];
                dj += L.acx[q] * yv[L.ci[q]];
            }
            d[j] = dj;
        }
        const igx::HostMetrics mt = igx::host_evaluate(L, xv.data(), yv.data(), ax.data(), d.data());
        if (mt.pinf <= o.tolerance && mt.dinf <= o.tolerance && mt.prow <= o.tolerance &&
            std::isfinite(mt.gap) && mt.gap <= o.tolerance) {
            taken = true;
            res->status = IGAOS_STATUS_OPTIMAL;
            res->objective = mt.op + p->obj_const;
            res->pinf = mt.pinf;
            res->dinf = mt.dinf;
            res->rel_gap = mt.gap;
            res->prow = mt.prow;
            std::memcpy(x, xv.data(), sizeof(double) * L.n);
            std::memcpy(y, yv.data(), sizeof(double) * L.m);
        }
    }
    static const char* kNames[] = {"optimal", "pivot cap", "singular basis", "unbounded edge",
                                   "infeasible", "too large"};
    char note[96];
    std::snprintf(note, sizeof(note), "crossover: %s, %lld pivots, %.0f ms",
                  taken ? "optimal vertex" : kNames[info.status], (long long)info.pivots,
                  info.time_ms);
    char msg[sizeof(res->message)];
    std::snprintf(msg, sizeof(msg), "%.*s; %s", (int)(sizeof(msg) - std::strlen(note) - 3),
                  res->message, note);
    std::memcpy(res->message, msg, sizeof(msg));
}
}  // namespace

int igx::igx_set_error(int code, const char* msg) {
    if (code == IGAOS_PDHG_OK) return ok();
    return fail(code, msg);
}

extern "C" {

int igaos_pdhg_abi_version(void) { return IGAOS_PDHG_ABI_VERSION; }

int igaos_pdhg_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

void igaos_pdhg_default_options(igaos_pdhg_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->time_limit_s = 120.0;
    o->tolerance = 1e-4;
    o->max_iterations = 500000;
    o->seed = 0;
    o->presolve = 1;
    o->restarts = 0;
    o->verbosity = 0;
    o->precision = IGAOS_PDHG_FP64;
    o->check_period = 64;
    o->inner_tolerance = 1e-4;
    o->max_refinements = 12;
    o->use_graphs = 1;
    o->device = -1;
}

int igaos_pdhg_last_error(char* buf, size_t len) {
    if (buf && len > 0) {
        std::strncpy(buf, g_msg, len - 1);
        buf[len - 1] = 0;
    }
    return g_code;
}

int igaos_pdhg_create(igaos_pdhg_problem** out, int m, int n, int64_t nnz, const int* ap,
                      const int* ai, const double* ax, const int* cp, const int* ci,
                      const double* acx, const double* c, const double* cl, const double* cu,
                      const double* rmin, const double* rmax, double obj_const,
                      const igaos_pdhg_options* opt) {
    if (!out) return fail(IGAOS_PDHG_ERR_INVALID, "out handle pointer is NULL");
    *out = nullptr;
    return guarded([&] {
        validate(m, n, nnz, ap, ai, ax, cp, ci, acx, c, cl, cu, rmin, rmax);
        if (opt && opt->scaling != IGAOS_PDHG_SCALING_RUIZ &&
            opt->scaling != IGAOS_PDHG_SCALING_RUIZ_PC)
            throw igx::CudaError(IGAOS_PDHG_ERR_INVALID, "unknown scaling");
        if (igaos_pdhg_device_count() == 0)
            throw igx::CudaError(IGAOS_PDHG_ERR_NODEVICE,
                                 "no CUDA device: PDHG engine unavailable");
        const int dev = opt ? opt->device : -1;
        std::unique_ptr<igaos_pdhg_problem, void (*)(igaos_pdhg_problem*)> p(
            new igaos_pdhg_problem, igaos_pdhg_destroy);
        std::vector<int> tcp, tci;
        std::vector<double> tacx;
        if (opt && opt->pdhg_presolve) {
            const auto t0 = std::chrono::steady_clock::now();
            p->pre = new igx::Presolved;
            p->pre_outcome = igx::presolve(m, n, ap, ai, ax, c, cl, cu, rmin, rmax, obj_const,
                                           *p->pre);
            igx::HostLP& o = p->orig;
            o.m = m;
            o.n = n;
            o.c.assign(c, c + n);
            o.cl.assign(cl, cl + n);
            o.cu.assign(cu, cu + n);
            o.rmin.assign(rmin, rmin + m);
            o.rmax.assign(rmax, rmax + m);
            p->obj_const = obj_const;
            const igx::Presolved& R = *p->pre;
            if (p->pre_outcome == igx::kPresolveReduced && R.m > 0)
                transpose_host(R.m, R.n, R.ap.data(), R.ai.data(), R.ax.data(), tcp, tci, tacx);
            p->presolve_ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                    .count();
            if (p->pre_outcome == igx::kPresolveReduced && R.m > 0)
                p->eng = new igx::Engine(R.m, R.n, (int64_t)R.ai.size(), R.ap.data(),
                                         R.ai.data(), R.ax.data(), tcp.data(), tci.data(),
                                         tacx.data(), R.c.data(), R.cl.data(), R.cu.data(),
                                         R.rmin.data(), R.rmax.data(), R.obj_const, dev,
                                         opt->scaling);
        } else {
            if (!cp) {
                transpose_host(m, n, ap, ai, ax, tcp, tci, tacx);
                cp = tcp.data();
                ci = tci.data();
                acx = tacx.data();
            }
            p->eng = new igx::Engine(m, n, nnz, ap, ai, ax, cp, ci, acx, c, cl, cu, rmin, rmax,
                                     obj_const, dev, opt ? opt->scaling : IGAOS_PDHG_SCALING_RUIZ);
        }
        if (opt && opt->crossover && m <= igx::kCrossoverMaxRows) {
            p->xo = true;
            igx::HostLP& o = p->orig;
            o.m = m;
            o.n = n;
            o.c.assign(c, c + n);
            o.cl.assign(cl, cl + n);
            o.cu.assign(cu, cu + n);
            o.rmin.assign(rmin, rmin + m);
            o.rmax.assign(rmax, rmax + m);
            transpose_host(m, n, ap, ai, ax, o.cp, o.ci, o.acx);
            p->obj_const = obj_const;
        }
        *out = p.release();
    });
}

int igaos_pdhg_solve(igaos_pdhg_problem* p, const igaos_pdhg_options* opt,
                     igaos_pdhg_result* res, double* x, double* y) {
    if (!p || (!p->eng && !p->pre)) return fail(IGAOS_PDHG_ERR_INVALID, "problem handle is NULL");
    if (!res) return fail(IGAOS_PDHG_ERR_INVALID, "result pointer is NULL");
    igaos_pdhg_options o;
    if (opt) o = *opt;
    else igaos_pdhg_default_options(&o);
    if (!(o.tolerance > 0)) return fail(IGAOS_PDHG_ERR_INVALID, "tolerance must be positive");
    if (o.precision < 0 || o.precision > 2) return fail(IGAOS_PDHG_ERR_INVALID, "unknown precision");
    if (o.schedule != IGAOS_PDHG_SCHEDULE_FIXED && o.schedule != IGAOS_PDHG_SCHEDULE_AUTOTUNE)
        return fail(IGAOS_PDHG_ERR_INVALID, "unknown schedule");
    std::vector<double> xb, yb;  // the answer, when crossover needs it and the caller does not
    if (p->xo && !x) {
        xb.resize(p->orig.n);
        x = xb.data();
    }
    if (p->xo && !y) {
        yb.resize(p->orig.m);
        y = yb.data();
    }
    int rc;
    if (p->pre) {
        rc = solve_presolved(p, o, res, x, y);
    } else {
        rc = guarded([&] { p->eng->solve(o, *res, x, y); });
        if (rc != IGAOS_PDHG_OK) {
            std::memset(res, 0, sizeof(*res));
            res->status = IGAOS_STATUS_ERROR;
            res->error_code = rc;
            std::snprintf(res->message, sizeof(res->message), "%.159s", g_msg);
            return rc;
        }
        if (res->error_code != IGAOS_PDHG_OK) return fail(res->error_code, res->message);
    }
    if (rc == IGAOS_PDHG_OK && p->xo) rc = guarded([&] { run_crossover(p, o, res, x, y); });
    return rc;
}

void igaos_pdhg_destroy(igaos_pdhg_problem* p) {
    if (!p) return;
    delete p->eng;
    delete p->pre;
    delete p;
}

int igaos_pdhg_solve_csr(int m, int n, int64_t nnz, const int* ap, const int* ai,
                         const double* ax, const int* cp, const int* ci, const double* acx,
                         const double* c, const double* cl, const double* cu,
                         const double* rmin, const double* rmax, double obj_const,
                         const igaos_pdhg_options* opt, igaos_pdhg_result* res, double* x,
                         double* y) {
    if (!res) return fail(IGAOS_PDHG_ERR_INVALID, "result pointer is NULL");
    igaos_pdhg_problem* p = nullptr;
    int rc = igaos_pdhg_create(&p, m, n, nnz, ap, ai, ax, cp, ci, acx, c, cl, cu, rmin, rmax,
                               obj_const, opt);
    if (rc != IGAOS_PDHG_OK) {
        std::memset(res, 0, sizeof(*res));
        res->status = IGAOS_STATUS_ERROR;
        res->error_code = rc;
        std::snprintf(res->message, sizeof(res->message), "%.159s", g_msg);
        return rc;
    }
    rc = igaos_pdhg_solve(p, opt, res, x, y);
    igaos_pdhg_destroy(p);
    return rc;
}

int igaos_pdhg_get_scaling(const igaos_pdhg_problem* p, double* dr, double* dc) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng || !dr || !dc) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    std::memcpy(dr, p->eng->h_dr.data(), sizeof(double) * p->eng->m);
    std::memcpy(dc, p->eng->h_dc.data(), sizeof(double) * p->eng->n);
    return ok();
}

int igaos_pdhg_get_step_init(const igaos_pdhg_problem* p, double* lambda, double* eta0,
                             double* omega0) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (lambda) *lambda = p->eng->lam2;
    if (eta0) *eta0 = p->eng->eta0;
    if (omega0) *omega0 = p->eng->omega0;
    return ok();
}

int igaos_pdhg_get_transpose(const igaos_pdhg_problem* p, int* cp, int* ci, double* acx) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng || !cp || !ci || !acx) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    return guarded([&] { p->eng->get_transpose(cp, ci, acx); });
}

int igaos_pdhg_iterate(igaos_pdhg_problem* p, int precision, int64_t iters, double* x, double* y,
                       double* xavg, double* yavg, double* axcur, double* state6) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng || !x || !y || !xavg || !yavg || !axcur || !state6)
        return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (iters < 0) return fail(IGAOS_PDHG_ERR_INVALID, "iters must be >= 0");
    if (precision != IGAOS_PDHG_FP64 && precision != IGAOS_PDHG_FP32)
        return fail(IGAOS_PDHG_ERR_INVALID, "precision must be FP64 or FP32");
    return guarded([&] { p->eng->iterate(precision, iters, x, y, xavg, yavg, axcur, state6); });
}

int igaos_pdhg_set_start(igaos_pdhg_problem* p, const double* x0, const double* y0) {
    if (p && p->pre)
        return fail(IGAOS_PDHG_ERR_INVALID, "a start point is not available on a presolved handle");
    if (!p || !p->eng) return fail(IGAOS_PDHG_ERR_INVALID, "problem handle is NULL");
    if (!x0 != !y0) return fail(IGAOS_PDHG_ERR_INVALID, "x0 and y0 are both given or both NULL");
    return guarded([&] { p->eng->set_start(x0, y0); });
}

int igaos_pdhg_evaluate(igaos_pdhg_problem* p, const double* x, const double* y, double* out6) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng || !x || !y || !out6) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    return guarded([&] { p->eng->evaluate(x, y, out6); });
}

int igaos_pdhg_dual_repair_device(igaos_pdhg_problem* p, const double* x, const double* y_it,
                                  double col_tol, double tol, double* y, int* certified,
                                  double* metrics6) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng || !x || !y_it || !y || !certified)
        return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (!(col_tol >= 0.0)) return fail(IGAOS_PDHG_ERR_INVALID, "col_tol must be >= 0");
    if (!(tol > 0.0)) return fail(IGAOS_PDHG_ERR_INVALID, "tol must be > 0");
    return guarded([&] {
        double m6[6];
        *certified = p->eng->repair_device(x, y_it, col_tol, tol, y, m6) ? 1 : 0;
        if (metrics6) std::memcpy(metrics6, m6, sizeof(m6));
    });
}

int igaos_pdhg_ray_certificate(int m, int n, const double* x, const double* ax, const double* y,
                               const double* aty, const double* c, const double* cl,
                               const double* cu, const double* rmin, const double* rmax,
                               double* xray, double* yray, int* kind) {
    if (m < 0 || n < 0) return fail(IGAOS_PDHG_ERR_INVALID, "negative size");
    if (!kind || (m > 0 && (!ax || !y || !rmin || !rmax)) ||
        (n > 0 && (!x || !aty || !c || !cl || !cu)))
        return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    return guarded([&] {
        *kind = igx::ray_certificate(m, n, x, ax, y, aty, c, cl, cu, rmin, rmax, xray, yray);
    });
}

int igaos_pdhg_spmv(igaos_pdhg_problem* p, int transpose, int precision, const double* x,
                    double* y) {
    if (p && p->pre) return fail(IGAOS_PDHG_ERR_INVALID, kPresolvedInspect);
    if (!p || !p->eng || !x || !y) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (precision != IGAOS_PDHG_FP64 && precision != IGAOS_PDHG_FP32)
        return fail(IGAOS_PDHG_ERR_INVALID, "precision must be FP64 or FP32");
    return guarded([&] { p->eng->spmv(transpose, precision, x, y); });
}

int igaos_pdhg_presolve(int m, int n, int64_t nnz, const int* ap, const int* ai,
                        const double* ax, const double* c, const double* cl, const double* cu,
                        const double* rmin, const double* rmax, double obj_const,
                        igaos_pdhg_presolved** out, int* outcome) {
    if (!out || !outcome) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    *out = nullptr;
    *outcome = 0;
    return guarded([&] {
        validate(m, n, nnz, ap, ai, ax, nullptr, nullptr, nullptr, c, cl, cu, rmin, rmax);
        std::unique_ptr<igaos_pdhg_presolved> h(new igaos_pdhg_presolved);
        *outcome = igx::presolve(m, n, ap, ai, ax, c, cl, cu, rmin, rmax, obj_const, h->p);
        *out = h.release();
    });
}

int igaos_pdhg_presolved_info(const igaos_pdhg_presolved* p, int* m, int* n, int64_t* nnz,
                              double* obj_const, int64_t* counts6) {
    if (!p) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (!reduced(p)) return fail(IGAOS_PDHG_ERR_INVALID, kNotReduced);
    const igx::Presolved& R = p->p;
    if (m) *m = R.m;
    if (n) *n = R.n;
    if (nnz) *nnz = (int64_t)R.ai.size();
    if (obj_const) *obj_const = R.obj_const;
    if (counts6) {
        const igx::PresolveCounts& k = R.counts;
        const int64_t v[6] = {k.empty_rows, k.singleton_rows, k.redundant_rows,
                              k.fixed_cols, k.empty_cols,     k.free_singletons};
        std::memcpy(counts6, v, sizeof(v));
    }
    return ok();
}

int igaos_pdhg_presolved_lp(const igaos_pdhg_presolved* p, int* ap, int* ai, double* ax,
                            double* c, double* cl, double* cu, double* rmin, double* rmax) {
    if (!p || !ap || !c || !cl || !cu || !rmin || !rmax ||
        (!p->p.ai.empty() && (!ai || !ax)))
        return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (!reduced(p)) return fail(IGAOS_PDHG_ERR_INVALID, kNotReduced);
    const igx::Presolved& R = p->p;
    std::copy(R.ap.begin(), R.ap.end(), ap);
    std::copy(R.ai.begin(), R.ai.end(), ai);
    std::copy(R.ax.begin(), R.ax.end(), ax);
    std::copy(R.c.begin(), R.c.end(), c);
    std::copy(R.cl.begin(), R.cl.end(), cl);
    std::copy(R.cu.begin(), R.cu.end(), cu);
    std::copy(R.rmin.begin(), R.rmin.end(), rmin);
    std::copy(R.rmax.begin(), R.rmax.end(), rmax);
    return ok();
}

int igaos_pdhg_postsolve(const igaos_pdhg_presolved* p, const double* x_red,
                         const double* y_red, double* x, double* y) {
    if (!p || !x || !y || (p->p.n > 0 && !x_red) || (p->p.m > 0 && !y_red))
        return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (!reduced(p)) return fail(IGAOS_PDHG_ERR_INVALID, kNotReduced);
    igx::postsolve(p->p, x_red, y_red, x, y);
    return ok();
}

int igaos_pdhg_postsolve_ray(const igaos_pdhg_presolved* p, const double* x_red,
                             const double* y_red, double* x, double* y) {
    if (!p || !x || !y || (p->p.n > 0 && !x_red) || (p->p.m > 0 && !y_red))
        return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    if (!reduced(p)) return fail(IGAOS_PDHG_ERR_INVALID, kNotReduced);
    igx::postsolve_ray(p->p, x_red, y_red, x, y);
    return ok();
}

int igaos_pdhg_presolved_ray(const igaos_pdhg_presolved* p, double* x, double* y) {
    if (!p || !x || !y) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    std::fill(x, x + p->p.n0, 0.0);
    std::fill(y, y + p->p.m0, 0.0);
    if (!igx::unbounded_ray(p->p, x) && !igx::infeasible_ray(p->p, y))
        return fail(IGAOS_PDHG_ERR_INVALID, "presolve found no ray for this LP");
    return ok();
}

void igaos_pdhg_presolved_destroy(igaos_pdhg_presolved* p) { delete p; }

int igaos_pdhg_crossover(int m, int n, int64_t nnz, const int* ap, const int* ai,
                         const double* ax, const double* c, const double* cl, const double* cu,
                         const double* rmin, const double* rmax, const double* x0, double* x,
                         double* y, signed char* basis, igaos_pdhg_crossover_info* info) {
    if (!x0 || !x || !y || !info) return fail(IGAOS_PDHG_ERR_INVALID, "NULL argument");
    return guarded([&] {
        validate(m, n, nnz, ap, ai, ax, nullptr, nullptr, nullptr, c, cl, cu, rmin, rmax);
        for (int j = 0; j < n; ++j)
            if (!std::isfinite(x0[j])) throw std::invalid_argument("x0 must be finite");
        if (m > igx::kCrossoverMaxRows)
            throw std::invalid_argument("crossover needs m <= 2048 (dense basis inverse)");
        std::vector<int> cp, ci;
        std::vector<double> acx;
        transpose_host(m, n, ap, ai, ax, cp, ci, acx);
        igx::CrossoverInfo ci_;
        igx::crossover(m, n, cp.data(), ci.data(), acx.data(), c, cl, cu, rmin, rmax, x0, x, y,
                       basis, ci_);
        std::memset(info, 0, sizeof(*info));
        info->status = ci_.status;
        info->pushes = ci_.pushes;
        info->pivots = ci_.pivots;
        info->bound_flips = ci_.bound_flips;
        info->phase1_iterations = ci_.phase1_iters;
        info->refactorizations = ci_.refactors;
        info->basis_repairs = ci_.basis_repairs;
        info->superbasic_left = ci_.superbasic_left;
        info->time_ms = ci_.time_ms;
    });
}

}  // extern "C"
