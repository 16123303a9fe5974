#pragma once
// Solver options shared by every engine surface (C++ solve, CLI, Python).
// Field names, types and defaults mirror include/igaos/options.h:5-13 of the
// reference so that code written against it compiles unchanged.

namespace igaos {

struct Options {
    double time_limit_s = 120.0;
    double tolerance = 1e-4;
    long max_iterations = 500000;
    int seed = 0;
    bool presolve = true;
    bool restarts = false;
    int verbosity = 0;
};

}  // namespace igaos
