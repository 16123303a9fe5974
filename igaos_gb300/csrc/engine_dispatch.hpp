// Engine dispatch shared by the CLI and the Python module, shape of the
// reference's igaos::solve_with_engine (src/api/engine.hpp:22-45). This build
// carries the PDHG engine only; the reference's CPU engines (simplex, milp,
// qp and the "auto" choice that routes to simplex) report an honest error.
#pragma once

#include <string>

#include "igaos/options.h"
#include "igaos/solution.h"
#include "model.hpp"
#include "pdhg.hpp"

namespace igaos {

inline Solution solve_with_engine(const io::Model& model, const Options& opts,
                                  const std::string& engine) {
    if (engine == "pdhg") return pdhg::solve(model, opts);
    Solution sol;
    sol.status = Status::Error;
    sol.message = "engine '" + engine + "' is not part of the GB300 build (PDHG engine only)";
    return sol;
}

}  // namespace igaos
