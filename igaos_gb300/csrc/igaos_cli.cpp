// `igaos` command line, the surface of the reference CLI
// (src/api/igaos_cli.cpp): `igaos info <model.mps>` and
// `igaos solve <model.mps> [flags] --engine pdhg`, same flags and the same
// JSON solution record. Added flag: --precision fp64|fp32-refine|fp32.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <string>

#include "engine_dispatch.hpp"
#include "igaos/status.h"
#include "igaos_pdhg.h"
#include "model.hpp"

namespace {

void usage() {
    std::printf(
        "igaos -- GB300 PDHG LP engine\n\n"
        "USAGE:\n"
        "  igaos info   <model.mps>\n"
        "  igaos solve  <model.mps> [flags]\n\n"
        "FLAGS (solve):\n"
        "  --time-limit <sec>      wall-clock budget (default 120)\n"
        "  --tol <float>           relative KKT tolerance (default 1e-4)\n"
        "  --max-iter <int>        iteration cap (default 500000)\n"
        "  --presolve on|off       accepted, ignored by the PDHG engine\n"
        "  --seed <int>            accepted, ignored by the PDHG engine\n"
        "  --out <file.json>       write solution JSON here (else stdout)\n"
        "  --engine <name>         auto|simplex|pdhg|milp|qp (this build: pdhg)\n"
        "  --precision <p>         fp64|fp32-refine|fp32 (default fp64)\n"
        "  --verbose               engine progress to stderr (repeat for more)\n"
        "  --detect-infeasibility  stop with infeasible/unbounded on a ray certificate\n"
        "  --pdhg-presolve         reduce the LP on the host first (exact dual postsolve)\n"
        "  --crossover             finish at an optimal vertex (host simplex, m <= 2048)\n"
        "  --scaling <s>           ruiz|ruiz-pc (default ruiz; ruiz-pc adds a Pock-Chambolle pass)\n");
}

struct Args {
    std::string cmd, path, out, engine = "auto";
    igaos::Options opts;
    int precision = IGAOS_PDHG_FP64;
    bool detect = false;
    bool reduce = false;
    bool xo = false;
    int scaling = IGAOS_PDHG_SCALING_RUIZ;
    bool ok = true;
};

Args parse(int argc, char** argv) {
    Args a;
    if (argc < 3) {
        a.ok = false;
        return a;
    }
    a.cmd = argv[1];
    a.path = argv[2];
    if (a.cmd != "info" && a.cmd != "solve") a.ok = false;
    for (int i = 3; i < argc && a.ok; ++i) {
        const std::string f = argv[i];
        const bool has = i + 1 < argc;
        if (f == "--time-limit" && has) a.opts.time_limit_s = std::atof(argv[++i]);
        else if (f == "--tol" && has) a.opts.tolerance = std::atof(argv[++i]);
        else if (f == "--max-iter" && has) a.opts.max_iterations = std::atol(argv[++i]);
        else if (f == "--seed" && has) a.opts.seed = std::atoi(argv[++i]);
        else if (f == "--presolve" && has) a.opts.presolve = std::string(argv[++i]) == "on";
        else if (f == "--verbose") ++a.opts.verbosity;
        else if (f == "--detect-infeasibility") a.detect = true;
        else if (f == "--pdhg-presolve") a.reduce = true;
        else if (f == "--crossover") a.xo = true;
        else if (f == "--scaling" && has) {
            const std::string s = argv[++i];
            if (s == "ruiz") a.scaling = IGAOS_PDHG_SCALING_RUIZ;
            else if (s == "ruiz-pc") a.scaling = IGAOS_PDHG_SCALING_RUIZ_PC;
            else a.ok = false;
        }
        else if (f == "--out" && has) a.out = argv[++i];
        else if (f == "--engine" && has) {
            a.engine = argv[++i];
            if (a.engine != "auto" && a.engine != "simplex" && a.engine != "pdhg" &&
                a.engine != "milp" && a.engine != "qp")
                a.ok = false;
        } else if (f == "--precision" && has) {
            const std::string p = argv[++i];
            if (p == "fp64") a.precision = IGAOS_PDHG_FP64;
            else if (p == "fp32-refine") a.precision = IGAOS_PDHG_FP32_REFINE;
            else if (p == "fp32") a.precision = IGAOS_PDHG_FP32;
            else a.ok = false;
        } else {
            a.ok = false;
        }
    }
    return a;
}

std::string fmt(const char* f, double v) {
    if (!std::isfinite(v)) return "null";
    char b[64];
    std::snprintf(b, sizeof(b), f, v);
    return b;
}

std::string esc(const std::string& s) {
    std::string r;
    for (char ch : s) {
        if (ch == '"' || ch == '\\') r += '\\';
        r += ch;
    }
    return r;
}

// The reference's JSON record (src/api/igaos_cli.cpp:115-150).
void emit(const igaos::io::Model& M, const igaos::Solution& s, const Args& a) {
    std::string j = "{\n";
    j += "  \"instance\": \"" + esc(a.path) + "\",\n";
    j += "  \"m\": " + std::to_string(M.m) + ",\n";
    j += "  \"n\": " + std::to_string(M.n) + ",\n";
    j += "  \"nnz\": " + std::to_string(M.nnz()) + ",\n";
    j += std::string("  \"status\": \"") + igaos::status_name(s.status) + "\",\n";
    j += "  \"objective\": " + fmt("%.10g", s.objective) + ",\n";
    j += "  \"pinf\": " + fmt("%.3e", s.pinf) + ",\n";
    j += "  \"dinf\": " + fmt("%.3e", s.dinf) + ",\n";
    j += "  \"rel_gap\": " + fmt("%.3e", s.rel_gap) + ",\n";
    j += "  \"iterations\": " + std::to_string(s.iterations) + ",\n";
    char tb[64];
    std::snprintf(tb, sizeof(tb), "%.1f", s.solve_time_ms);
    j += "  \"solve_time_ms\": " + std::string(tb) + ",\n";
    j += "  \"engine\": \"" + esc(a.engine) + "\",\n";
    j += "  \"x\": [";
    for (size_t k = 0; k < s.x.size(); ++k) {
        char xb[64];
        std::snprintf(xb, sizeof(xb), "%.10g", s.x[k]);
        j += xb;
        if (k + 1 < s.x.size()) j += ",";
    }
    j += "],\n";
    j += "  \"message\": \"" + esc(s.message) + "\"\n";
    j += "}\n";
    if (a.out.empty()) std::fputs(j.c_str(), stdout);
    else std::ofstream(a.out) << j;
}

int info(const igaos::io::Model& M) {
    int nE = 0, nL = 0, nG = 0, nR = 0;
    for (int i = 0; i < M.m; ++i) {
        if (M.rmin[i] == M.rmax[i]) {
            ++nE;
            continue;
        }
        const bool fl = std::isfinite(M.rmin[i]), fu = std::isfinite(M.rmax[i]);
        nG += fl;
        nL += fu;
        nR += fl && fu;
    }
    int fr = 0, fx = 0, bx = 0, one = 0;
    for (int j = 0; j < M.n; ++j) {
        const bool fl = std::isfinite(M.cl[j]), fu = std::isfinite(M.cu[j]);
        if (!fl && !fu) ++fr;
        else if (fl && fu && M.cl[j] == M.cu[j]) ++fx;
        else if (fl && fu) ++bx;
        else ++one;
    }
    double cmax = 0;
    for (double v : M.c) cmax = std::fmax(cmax, std::fabs(v));
    std::printf("rows           %d\n", M.m);
    std::printf("cols           %d\n", M.n);
    std::printf("nnz            %d\n", M.nnz());
    std::printf("row types      E=%d L=%d G=%d ranged=%d\n", nE, nL - nR > 0 ? nL - nR : 0, nG, nR);
    std::printf("col bounds     free=%d fixed=%d boxed=%d one-sided=%d\n", fr, fx, bx, one);
    std::printf("objective      |c|max=%.6g\n", cmax);
    std::printf("parsed         FR=%d RANGES=%d obj_const=%.6g\n", M.n_fr_parsed,
                M.n_ranges_parsed, M.obj_const);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        usage();
        return 2;
    }
    if (!std::strcmp(argv[1], "--help") || !std::strcmp(argv[1], "-h")) {
        usage();
        return 0;
    }
    Args a = parse(argc, argv);
    if (!a.ok) {
        usage();
        return 2;
    }
    igaos::io::Model M;
    try {
        igaos::io::parse_mps(a.path, M);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 3;
    }
    if (a.cmd == "info") return info(M);
    igaos::Solution s;
    if (a.engine == "pdhg" && (a.precision != IGAOS_PDHG_FP64 || a.detect || a.reduce || a.xo ||
                               a.scaling != IGAOS_PDHG_SCALING_RUIZ)) {
        igaos_pdhg_options o;
        igaos_pdhg_default_options(&o);
        o.precision = a.precision;
        o.detect_infeasibility = a.detect ? 1 : 0;
        o.pdhg_presolve = a.reduce ? 1 : 0;
        o.crossover = a.xo ? 1 : 0;
        o.scaling = a.scaling;
        s = igaos::pdhg::solve_ex(M, a.opts, &o);
    } else {
        s = igaos::solve_with_engine(M, a.opts, a.engine);
    }
    emit(M, s, a);
    return 0;
}
