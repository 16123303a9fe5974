// C ABI over the reference CPU simplex (src/simplex/simplex.hpp:24-28), the
// exact-optimum oracle for LPs given as CSR + CSC arrays. Compiled together
// with the reference's simplex.cpp by oracle/Makefile into oracle/_ref/.
// Test infrastructure only.
#include <cstring>
#include <string>

#include "model.hpp"
#include "simplex.hpp"

extern "C" int ref_simplex_solve(int m, int n, long nnz, const int* ap,
                                 const int* ai, const double* ax,
                                 const int* cp, const int* ci,
                                 const double* acx, const double* c,
                                 const double* cl, const double* cu,
                                 const double* rmin, const double* rmax,
                                 double obj_const, double time_limit,
                                 double* objective, long* iterations,
                                 double* x, double* y, char* msg, int msglen) {
    igaos::io::Model M;
    M.m = m;
    M.n = n;
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
    o.time_limit_s = time_limit;
    igaos::Solution s = igaos::simplex::solve(M, o);
    *objective = s.objective;
    *iterations = s.iterations;
    if (x && (int)s.x.size() == n) std::memcpy(x, s.x.data(), sizeof(double) * n);
    if (y && (int)s.y.size() == m) std::memcpy(y, s.y.data(), sizeof(double) * m);
    if (msg && msglen > 0) {
        std::string t = std::string(igaos::status_name(s.status)) + ": " + s.message;
        std::strncpy(msg, t.c_str(), msglen - 1);
        msg[msglen - 1] = 0;
    }
    return (int)s.status;
}
