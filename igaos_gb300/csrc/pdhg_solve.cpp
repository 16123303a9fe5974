// igaos::pdhg::solve over the C ABI (see pdhg.hpp).
#include <cstring>

#include "igaos_pdhg.h"
#include "pdhg.hpp"

namespace igaos::pdhg {

Solution solve_ex(const io::Model& lp, const Options& opt, const void* engine_opts) {
    Solution sol;
    igaos_pdhg_options o;
    if (engine_opts) std::memcpy(&o, engine_opts, sizeof(o));
    else igaos_pdhg_default_options(&o);
    o.time_limit_s = opt.time_limit_s;
    o.tolerance = opt.tolerance;
    o.max_iterations = opt.max_iterations;
    o.seed = opt.seed;
    o.presolve = opt.presolve ? 1 : 0;
    o.restarts = opt.restarts ? 1 : 0;
    o.verbosity = opt.verbosity;
    igaos_pdhg_result r;
    sol.x.assign(lp.n, 0.0);
    sol.y.assign(lp.m, 0.0);
    const bool have_t = !lp.cp.empty();
    igaos_pdhg_solve_csr(lp.m, lp.n, lp.nnz(), lp.ap.data(), lp.ai.data(), lp.ax.data(),
                         have_t ? lp.cp.data() : nullptr, have_t ? lp.ci.data() : nullptr,
                         have_t ? lp.acx.data() : nullptr, lp.c.data(), lp.cl.data(),
                         lp.cu.data(), lp.rmin.data(), lp.rmax.data(), lp.obj_const, &o, &r,
                         sol.x.data(), sol.y.data());
    sol.status = static_cast<Status>(r.status);
    sol.message = r.message;
    if (sol.status == Status::Error) {
        sol.x.clear();
        sol.y.clear();
        return sol;
    }
    sol.objective = r.objective;
    sol.pinf = r.pinf;
    sol.dinf = r.dinf;
    sol.rel_gap = r.rel_gap;
    sol.iterations = (long)r.iterations;
    sol.solve_time_ms = r.solve_time_ms;
    return sol;
}

Solution solve(const io::Model& lp, const Options& opt) { return solve_ex(lp, opt, nullptr); }

}  // namespace igaos::pdhg
