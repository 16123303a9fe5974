// igaos::pdhg::solve -- the C++ entry point of the reference engine
// (src/pdhg/pdhg.hpp:9), implemented over the C ABI in include/igaos_pdhg.h.
#pragma once

#include "igaos/options.h"
#include "igaos/solution.h"
#include "model.hpp"

namespace igaos::pdhg {

// Same signature and contract as the reference: never throws; failures come
// back as Status::Error with a message; success is Status::NearOptimal.
Solution solve(const io::Model& model, const Options& options);

// GB300 extension: the same call with the engine's own options
// (precision, check period, refinement rounds ...). `engine_opts` points to
// an igaos_pdhg_options; its first seven fields are overwritten from
// `options`.
Solution solve_ex(const io::Model& model, const Options& options, const void* engine_opts);

}  // namespace igaos::pdhg
