// LP model and free-format MPS reader of the engine's C++ surface.
// Same type name, fields and conventions as the reference's io::Model
// (src/io/model.hpp:16-37) so that callers of igaos::pdhg::solve(Model,
// Options) are unchanged: rows rmin <= A x <= rmax, columns cl <= x <= cu,
// A held as CSR (ap, ai, ax) and CSC (cp, ci, acx) with identical values.
#pragma once

#include <string>
#include <vector>

namespace igaos::io {

struct Model {
    int m = 0, n = 0;
    std::vector<double> rmin, rmax;
    std::vector<double> cl, cu;
    std::vector<double> c;
    std::vector<int> ap, ai;
    std::vector<double> ax;
    std::vector<int> cp, ci;
    std::vector<double> acx;
    std::vector<unsigned char> integ;
    double obj_const = 0.0;   // constant of the objective (negated objective RHS)
    int n_fr_parsed = 0;      // FR bounds read
    int n_ranges_parsed = 0;  // RANGES entries applied
    // 0.5 x'Px, upper-triangular COO (read, not used by the PDHG engine)
    std::vector<int> q_i, q_j;
    std::vector<double> q_v;

    bool has_quadratic() const { return !q_v.empty(); }
    int nnz() const { return static_cast<int>(ax.size()); }
};

// Builds CSR and CSC from (row, col, value) entries in the given order: each
// row of the CSR and each column of the CSC keeps the entries' input order
// (a stable counting sort, as src/io/model.hpp:39-67).
void build_csr_csc(int rows, int cols, const std::vector<int>& ti, const std::vector<int>& tj,
                   const std::vector<double>& tv, Model& out);

// Reads a free-format MPS file (ROWS, COLUMNS with integer MARKERs, RHS,
// RANGES, BOUNDS, QUADOBJ/QSECTION/QMATRIX). Throws std::runtime_error if the
// file cannot be opened. Semantics follow src/io/model.hpp:69-218.
void parse_mps(const std::string& path, Model& model);

}  // namespace igaos::io
