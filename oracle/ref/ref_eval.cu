// Exposes helpers of the reference PDHG engine through a C ABI so the oracle
// can be pinned against them. The reference translation unit is compiled
// as-is (it is included, not copied): its internal evaluate() sits in an
// anonymous namespace and is only reachable from inside the same unit.
// Built by oracle/Makefile into oracle/_ref/; test infrastructure only.
#include "pdhg.cu"  // reference src/pdhg/pdhg.cu (include path set by the Makefile)

#include <chrono>
#include <cstring>
#include <exception>
#include <string>
#include <tuple>
#include <vector>

extern "C" {

void ref_evaluate(int m, int n, const double* rmin, const double* rmax,
                  const double* cl, const double* cu, const double* c,
                  const double* x, const double* y, const double* Ax,
                  const double* d, double* out6) {
    std::vector<double> vrmin(rmin, rmin + m), vrmax(rmax, rmax + m),
        vcl(cl, cl + n), vcu(cu, cu + n), vc(c, c + n), vx(x, x + n),
        vy(y, y + m), vAx(Ax, Ax + m), vd(d, d + n);
    auto mt = igaos::pdhg::evaluate(m, n, vrmin, vrmax, vcl, vcu, vc, vx, vy,
                                    vAx, vd);
    out6[0] = mt.pinf;
    out6[1] = mt.dinf;
    out6[2] = mt.gap;
    out6[3] = mt.op;
    out6[4] = mt.od;
    out6[5] = mt.prow;
}

void ref_counting_sort(long nt, const int* ti, const int* tj, const double* tv,
                       int rows, int cols, int* ap, int* ai, double* ax,
                       int* cp, int* ci, double* acx) {
    std::vector<std::tuple<int, int, double>> trips;
    trips.reserve(nt);
    for (long t = 0; t < nt; ++t) trips.emplace_back(ti[t], tj[t], tv[t]);
    std::vector<int> vap, vai, vcp, vci;
    std::vector<double> vax, vacx;
    igaos::io::counting_sort(trips, rows, cols, vap, vai, vax, vcp, vci, vacx);
    std::memcpy(ap, vap.data(), sizeof(int) * vap.size());
    std::memcpy(cp, vcp.data(), sizeof(int) * vcp.size());
    if (nt > 0) {
        std::memcpy(ai, vai.data(), sizeof(int) * nt);
        std::memcpy(ax, vax.data(), sizeof(double) * nt);
        std::memcpy(ci, vci.data(), sizeof(int) * nt);
        std::memcpy(acx, vacx.data(), sizeof(double) * nt);
    }
}

// MPS reader: parse into a static model, then fetch arrays.
static igaos::io::Model g_model;

int ref_parse_mps(const char* path, int* m, int* n, long* nnz,
                  double* obj_const) {
    g_model = igaos::io::Model();
    try {
        igaos::io::parse_mps(path, g_model);
    } catch (...) {
        return 1;
    }
    *m = g_model.m;
    *n = g_model.n;
    *nnz = g_model.nnz();
    *obj_const = g_model.obj_const;
    return 0;
}

// integer flag of each column of the last parsed model (1: integer)
void ref_fetch_integ(unsigned char* out) {
    for (size_t j = 0; j < g_model.integ.size(); ++j) out[j] = g_model.integ[j] ? 1 : 0;
}

void ref_fetch_model(int* ap, int* ai, double* ax, int* cp, int* ci,
                     double* acx, double* c, double* cl, double* cu,
                     double* rmin, double* rmax) {
    const auto& M = g_model;
    std::memcpy(ap, M.ap.data(), sizeof(int) * M.ap.size());
    std::memcpy(cp, M.cp.data(), sizeof(int) * M.cp.size());
    std::memcpy(ai, M.ai.data(), sizeof(int) * M.ai.size());
    std::memcpy(ax, M.ax.data(), sizeof(double) * M.ax.size());
    std::memcpy(ci, M.ci.data(), sizeof(int) * M.ci.size());
    std::memcpy(acx, M.acx.data(), sizeof(double) * M.acx.size());
    std::memcpy(c, M.c.data(), sizeof(double) * M.c.size());
    std::memcpy(cl, M.cl.data(), sizeof(double) * M.cl.size());
    std::memcpy(cu, M.cu.data(), sizeof(double) * M.cu.size());
    std::memcpy(rmin, M.rmin.data(), sizeof(double) * M.rmin.size());
    std::memcpy(rmax, M.rmax.data(), sizeof(double) * M.rmax.size());
}

// The reference's dual_repair (internal to the pdhg.cu unit) on a model
// given by arrays; returns its certified flag, y receives its output.
int ref_dual_repair(int m, int n, const int* ap, const int* ai, const double* ax,
                    const int* cp, const int* ci, const double* acx, const double* c,
                    const double* cl, const double* cu, const double* rmin,
                    const double* rmax, const double* x, const double* Ax,
                    const double* y_it, double col_tol, double* y) {
    igaos::io::Model M;
    M.m = m;
    M.n = n;
    const int nnz = ap[m];
    M.ap.assign(ap, ap + m + 1);
    M.ai.assign(ai, ai + nnz);
    M.ax.assign(ax, ax + nnz);
    M.cp.assign(cp, cp + n + 1);
    M.ci.assign(ci, ci + nnz);
    M.acx.assign(acx, acx + nnz);
    M.c.assign(c, c + n);
    M.cl.assign(cl, cl + n);
    M.cu.assign(cu, cu + n);
    M.rmin.assign(rmin, rmin + m);
    M.rmax.assign(rmax, rmax + m);
    std::vector<double> vx(x, x + n), vAx(Ax, Ax + m), vy(y_it, y_it + m), out;
    const bool ok = igaos::pdhg::dual_repair(M, vx, vAx, vy, col_tol, out);
    // the reference leaves its output untouched when the factorisation fails
    if ((int)out.size() == m) std::memcpy(y, out.data(), sizeof(double) * m);
    else for (int i = 0; i < m; ++i) y[i] = std::numeric_limits<double>::quiet_NaN();
    return ok ? 1 : 0;
}

// The reference's GPU PDHG solve (src/pdhg/pdhg.cu:457-1156, cuSPARSE and
// cuBLAS on the legacy default stream) on a model given by arrays. Options
// follow igaos::Options (include/igaos/options.h): max_iterations binds only
// when time_limit is not in (0, 1e6) (pdhg.cu:669-671).
// out[0..6] = objective, pinf, dinf, rel_gap, iterations, solve_time_ms
// (the reference's own loop timer), wall_ms (the whole call: handles, Ruiz,
// upload, power iteration, loop, download, frees). Returns the Status value,
// or -1 when the call threw (the message says what).
int ref_pdhg_solve(int m, int n, const int* ap, const int* ai, const double* ax,
                   const int* cp, const int* ci, const double* acx, const double* c,
                   const double* cl, const double* cu, const double* rmin,
                   const double* rmax, double obj_const, double tolerance,
                   double time_limit, long max_iterations, int verbosity,
                   double* out, double* x, double* y, char* msg, int msglen) {
    igaos::io::Model M;
    M.m = m;
    M.n = n;
    const int nnz = ap[m];
    M.ap.assign(ap, ap + m + 1);
    M.ai.assign(ai, ai + nnz);
    M.ax.assign(ax, ax + nnz);
    M.cp.assign(cp, cp + n + 1);
    M.ci.assign(ci, ci + nnz);
    M.acx.assign(acx, acx + nnz);
    M.c.assign(c, c + n);
    M.cl.assign(cl, cl + n);
    M.cu.assign(cu, cu + n);
    M.rmin.assign(rmin, rmin + m);
    M.rmax.assign(rmax, rmax + m);
    M.integ.assign(n, 0);
    M.obj_const = obj_const;
    igaos::Options o;
    o.tolerance = tolerance;
    o.time_limit_s = time_limit;
    o.max_iterations = max_iterations;
    o.verbosity = verbosity;
    int rc = -1;
    std::string text;
    auto t0 = std::chrono::steady_clock::now();
    try {
        igaos::Solution s = igaos::pdhg::solve(M, o);
        cudaDeviceSynchronize();
        auto t1 = std::chrono::steady_clock::now();
        out[0] = s.objective;
        out[1] = s.pinf;
        out[2] = s.dinf;
        out[3] = s.rel_gap;
        out[4] = (double)s.iterations;
        out[5] = s.solve_time_ms;
        out[6] = std::chrono::duration<double, std::milli>(t1 - t0).count();
        if ((int)s.x.size() == n) std::memcpy(x, s.x.data(), sizeof(double) * n);
        if ((int)s.y.size() == m) std::memcpy(y, s.y.data(), sizeof(double) * m);
        rc = (int)s.status;
        text = s.message;
    } catch (const std::exception& e) {
        text = std::string("exception: ") + e.what();
    } catch (...) {
        text = "exception";
    }
    if (msg && msglen > 0) {
        std::strncpy(msg, text.c_str(), (size_t)msglen - 1);
        msg[msglen - 1] = 0;
    }
    return rc;
}

}  // extern "C"
