// pybind11 module `igaos_gb300._core`: the surface of the reference's
// `igaos._core` (python/igaos_bindings.cpp): solve(path, ...), read_mps,
// Model, Solution, Status, has_pdhg. Built against the pybind11 headers that
// ship with PyTorch; no torch type crosses this module.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>

#include "engine_dispatch.hpp"
#include "igaos/status.h"
#include "igaos_pdhg.h"
#include "model.hpp"

namespace py = pybind11;
using igaos::Options;
using igaos::Solution;
using igaos::io::Model;

namespace {

Solution py_solve(const std::string& path, double time_limit, double tolerance,
                  long max_iterations, bool presolve, long seed, const std::string& engine,
                  const std::string& precision, bool detect_infeasibility,
                  bool pdhg_presolve, bool crossover) {
    static const char* kEngines[] = {"auto", "simplex", "pdhg", "milp", "qp"};
    bool valid = false;
    for (const char* e : kEngines) valid |= engine == e;
    if (!valid)
        throw std::invalid_argument("engine must be one of auto|simplex|pdhg|milp|qp, got '" +
                                    engine + "'");
    int prec;
    if (precision == "fp64") prec = IGAOS_PDHG_FP64;
    else if (precision == "fp32-refine") prec = IGAOS_PDHG_FP32_REFINE;
    else if (precision == "fp32") prec = IGAOS_PDHG_FP32;
    else throw std::invalid_argument("precision must be one of fp64|fp32-refine|fp32");
    Model mdl;
    igaos::io::parse_mps(path, mdl);
    Options o;
    o.time_limit_s = time_limit;
    o.tolerance = tolerance;
    o.max_iterations = max_iterations;
    o.presolve = presolve;
    o.seed = static_cast<int>(seed);
    py::gil_scoped_release nogil;
    if (engine == "pdhg" && (prec != IGAOS_PDHG_FP64 || detect_infeasibility || pdhg_presolve ||
                             crossover)) {
        igaos_pdhg_options eo;
        igaos_pdhg_default_options(&eo);
        eo.precision = prec;
        eo.detect_infeasibility = detect_infeasibility ? 1 : 0;
        eo.pdhg_presolve = pdhg_presolve ? 1 : 0;
        eo.crossover = crossover ? 1 : 0;
        return igaos::pdhg::solve_ex(mdl, o, &eo);
    }
    return igaos::solve_with_engine(mdl, o, engine);
}

// Counting rules of `igaos info` (same as the reference's Model.stats).
py::dict model_stats(const Model& m) {
    int e = 0, l = 0, g = 0, ranged = 0;
    for (int i = 0; i < m.m; ++i) {
        if (m.rmin[i] == m.rmax[i]) {
            ++e;
            continue;
        }
        const bool fl = std::isfinite(m.rmin[i]), fu = std::isfinite(m.rmax[i]);
        g += fl;
        l += fu;
        ranged += fl && fu;
    }
    int nfree = 0, nfixed = 0, nboxed = 0, nonesided = 0, n_int = 0;
    for (int j = 0; j < m.n; ++j) {
        const bool fl = std::isfinite(m.cl[j]), fu = std::isfinite(m.cu[j]);
        if (!fl && !fu) ++nfree;
        else if (fl && fu && m.cl[j] == m.cu[j]) ++nfixed;
        else if (fl && fu) ++nboxed;
        else ++nonesided;
    }
    for (unsigned char v : m.integ) n_int += v != 0;
    py::dict d;
    d["rows_e"] = e;
    d["rows_l"] = l - ranged > 0 ? l - ranged : 0;
    d["rows_g"] = g;
    d["rows_ranged"] = ranged;
    d["cols_free"] = nfree;
    d["cols_fixed"] = nfixed;
    d["cols_boxed"] = nboxed;
    d["cols_one_sided"] = nonesided;
    d["n_int"] = n_int;
    d["n_fr_parsed"] = m.n_fr_parsed;
    d["n_ranges_parsed"] = m.n_ranges_parsed;
    d["obj_const"] = m.obj_const;
    return d;
}

}  // namespace

PYBIND11_MODULE(_core, m) {
    m.doc() = "GB300 PDHG LP engine core (igaos-compatible surface)";

    py::class_<Model>(m, "Model")
        .def_readonly("m", &Model::m)
        .def_readonly("n", &Model::n)
        .def_readonly("obj_const", &Model::obj_const)
        .def_readonly("n_fr_parsed", &Model::n_fr_parsed)
        .def_readonly("n_ranges_parsed", &Model::n_ranges_parsed)
        .def_readonly("ap", &Model::ap)
        .def_readonly("ai", &Model::ai)
        .def_readonly("ax", &Model::ax)
        .def_readonly("cp", &Model::cp)
        .def_readonly("ci", &Model::ci)
        .def_readonly("acx", &Model::acx)
        .def_readonly("c", &Model::c)
        .def_readonly("cl", &Model::cl)
        .def_readonly("cu", &Model::cu)
        .def_readonly("rmin", &Model::rmin)
        .def_readonly("rmax", &Model::rmax)
        .def_readonly("integ", &Model::integ)
        .def("nnz", &Model::nnz)
        .def_property_readonly("stats", &model_stats)
        .def("__repr__", [](const Model& mm) {
            return "<igaos.Model m=" + std::to_string(mm.m) + " n=" + std::to_string(mm.n) +
                   " nnz=" + std::to_string(mm.nnz()) + ">";
        });

    py::class_<Solution>(m, "Solution")
        .def_property_readonly("status",
                               [](const Solution& s) { return igaos::status_name(s.status); })
        .def_property_readonly("status_enum", [](const Solution& s) { return s.status; })
        .def_readonly("objective", &Solution::objective)
        .def_readonly("x", &Solution::x)
        .def_readonly("y", &Solution::y)
        .def_readonly("row_activity", &Solution::row_activity)
        .def_readonly("pinf", &Solution::pinf)
        .def_readonly("dinf", &Solution::dinf)
        .def_readonly("rel_gap", &Solution::rel_gap)
        .def_readonly("iterations", &Solution::iterations)
        .def_readonly("solve_time_ms", &Solution::solve_time_ms)
        .def_readonly("message", &Solution::message)
        .def("__repr__", [](const Solution& s) {
            return "<igaos.Solution status='" + std::string(igaos::status_name(s.status)) +
                   "' objective=" + std::to_string(s.objective) + ">";
        });

    py::enum_<igaos::Status>(m, "Status")
        .value("Optimal", igaos::Status::Optimal)
        .value("NearOptimal", igaos::Status::NearOptimal)
        .value("Feasible", igaos::Status::Feasible)
        .value("Infeasible", igaos::Status::Infeasible)
        .value("Unbounded", igaos::Status::Unbounded)
        .value("IterationLimit", igaos::Status::IterationLimit)
        .value("TimeLimit", igaos::Status::TimeLimit)
        .value("Error", igaos::Status::Error);

    m.attr("has_pdhg") = true;

    m.def("solve", &py_solve, py::arg("path"), py::arg("time_limit") = 120.0,
          py::arg("tolerance") = 1e-4, py::arg("max_iterations") = 500000L,
          py::arg("presolve") = true, py::arg("seed") = 0L, py::arg("engine") = "auto",
          py::arg("precision") = "fp64", py::arg("detect_infeasibility") = false,
          py::arg("pdhg_presolve") = false, py::arg("crossover") = false);

    m.def(
        "read_mps",
        [](const std::string& path) {
            auto mdl = std::make_unique<Model>();
            igaos::io::parse_mps(path, *mdl);
            return mdl;
        },
        py::arg("path"), py::return_value_policy::move);
}
