// MPS reader and CSR/CSC builder (see model.hpp).
#include "model.hpp"

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <stdexcept>
#include <string_view>
#include <unordered_map>

namespace igaos::io {

void build_csr_csc(int rows, int cols, const std::vector<int>& ti, const std::vector<int>& tj,
                   const std::vector<double>& tv, Model& out) {
    const size_t nt = tv.size();
    out.ap.assign(rows + 1, 0);
    out.cp.assign(cols + 1, 0);
    for (size_t t = 0; t < nt; ++t) {
        ++out.ap[ti[t] + 1];
        ++out.cp[tj[t] + 1];
    }
    for (int i = 0; i < rows; ++i) out.ap[i + 1] += out.ap[i];
    for (int j = 0; j < cols; ++j) out.cp[j + 1] += out.cp[j];
    std::vector<int> rnext(out.ap.begin(), out.ap.end() - 1);
    std::vector<int> cnext(out.cp.begin(), out.cp.end() - 1);
    out.ai.resize(nt);
    out.ax.resize(nt);
    out.ci.resize(nt);
    out.acx.resize(nt);
    for (size_t t = 0; t < nt; ++t) {
        const int r = ti[t], c = tj[t];
        const int pr = rnext[r]++, pc = cnext[c]++;
        out.ai[pr] = c;
        out.ax[pr] = tv[t];
        out.ci[pc] = r;
        out.acx[pc] = tv[t];
    }
}

namespace {

// Whitespace tokenizer over one line (views into the line buffer).
void split(std::string_view s, std::vector<std::string_view>& tok) {
    tok.clear();
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r')) ++i;
        if (i >= s.size()) break;
        size_t j = i;
        while (j < s.size() && s[j] != ' ' && s[j] != '\t' && s[j] != '\r') ++j;
        tok.push_back(s.substr(i, j - i));
        i = j;
    }
}

double num(std::string_view v) {
    // std::stod semantics (leading number, throws if none)
    std::string s(v);
    return std::stod(s);
}

struct Reader {
    static constexpr double INF = std::numeric_limits<double>::infinity();
    std::unordered_map<std::string, int> rows;  // -1: objective / free row
    std::unordered_map<std::string, int> cols;
    std::string obj;
    std::vector<char> sense;
    std::vector<double> rhs;
    std::vector<int> ti, tj;
    std::vector<double> tv;
    std::vector<std::pair<int, double>> ranges;
    bool in_int = false;

    int row_of(std::string_view name) const {
        auto it = rows.find(std::string(name));
        return it == rows.end() ? -1 : it->second;
    }
};

}  // namespace

void parse_mps(const std::string& path, Model& M) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open " + path);
    Reader R;
    std::string line, section;
    std::vector<std::string_view> t;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '*') continue;
        const bool header = line[0] != ' ' && line[0] != '\t';
        split(line, t);
        if (t.empty()) continue;
        if (header) {
            section.assign(t[0]);
            continue;
        }
        if (section == "ROWS") {
            if (t.size() < 2) continue;
            const std::string name(t[1]);
            if (t[0][0] == 'N') {
                if (R.obj.empty()) R.obj = name;
                R.rows[name] = -1;
            } else {
                R.rows[name] = (int)R.sense.size();
                R.sense.push_back(t[0][0]);
                R.rhs.push_back(0.0);
            }
        } else if (section == "COLUMNS") {
            if (line.find("'MARKER'") != std::string::npos) {
                R.in_int = line.find("INTORG") != std::string::npos;
                continue;
            }
            const std::string cname(t[0]);
            auto it = R.cols.find(cname);
            int j;
            if (it == R.cols.end()) {
                j = (int)R.cols.size();
                R.cols.emplace(cname, j);
                M.c.push_back(0.0);
                M.cl.push_back(0.0);
                M.cu.push_back(Reader::INF);
                M.integ.push_back(R.in_int ? 1 : 0);
            } else {
                j = it->second;
            }
            for (size_t k = 1; k + 1 < t.size(); k += 2) {
                const double v = num(t[k + 1]);
                if (t[k] == R.obj) {
                    M.c[j] += v;
                    continue;
                }
                const int r = R.row_of(t[k]);
                if (r < 0) continue;
                R.ti.push_back(r);
                R.tj.push_back(j);
                R.tv.push_back(v);
            }
        } else if (section == "RHS") {
            for (size_t k = 1; k + 1 < t.size(); k += 2) {
                if (t[k] == R.obj) {
                    M.obj_const -= num(t[k + 1]);
                    continue;
                }
                const int r = R.row_of(t[k]);
                if (r < 0) continue;
                R.rhs[r] = num(t[k + 1]);
            }
        } else if (section == "RANGES") {
            for (size_t k = 1; k + 1 < t.size(); k += 2) {
                const int r = R.row_of(t[k]);
                if (r < 0) continue;
                R.ranges.emplace_back(r, num(t[k + 1]));
                ++M.n_ranges_parsed;
            }
        } else if (section == "QUADOBJ" || section == "QSECTION" || section == "QMATRIX") {
            for (size_t k = 0; k + 2 < t.size(); k += 3) {
                auto a = R.cols.find(std::string(t[k]));
                auto b = R.cols.find(std::string(t[k + 1]));
                if (a == R.cols.end() || b == R.cols.end()) continue;
                M.q_i.push_back(a->second);
                M.q_j.push_back(b->second);
                M.q_v.push_back(num(t[k + 2]));
            }
        } else if (section == "BOUNDS") {
            if (t.size() < 3) continue;
            auto it = R.cols.find(std::string(t[2]));
            if (it == R.cols.end()) throw std::out_of_range("BOUNDS names an unknown column");
            const int j = it->second;
            const double v = t.size() > 3 ? num(t[3]) : 0.0;
            const std::string_view ty = t[0];
            if (ty == "UP") {
                M.cu[j] = v;
                if (v < 0 && M.cl[j] == 0.0) M.cl[j] = -Reader::INF;
            } else if (ty == "LO") {
                M.cl[j] = v;
            } else if (ty == "FX") {
                M.cl[j] = M.cu[j] = v;
            } else if (ty == "FR") {
                M.cl[j] = -Reader::INF;
                M.cu[j] = Reader::INF;
                ++M.n_fr_parsed;
            } else if (ty == "MI") {
                M.cl[j] = -Reader::INF;
            } else if (ty == "PL") {
                M.cu[j] = Reader::INF;
            } else if (ty == "BV") {
                M.cl[j] = 0.0;
                M.cu[j] = 1.0;
                M.integ[j] = 1;
            } else if (ty == "LI") {
                M.cl[j] = v;
                M.integ[j] = 1;
            } else if (ty == "UI") {
                M.cu[j] = v;
                M.integ[j] = 1;
            }
        }
    }
    M.m = (int)R.sense.size();
    M.n = (int)R.cols.size();
    M.rmin.assign(M.m, -Reader::INF);
    M.rmax.assign(M.m, Reader::INF);
    for (int i = 0; i < M.m; ++i) {
        if (R.sense[i] == 'E') M.rmin[i] = M.rmax[i] = R.rhs[i];
        else if (R.sense[i] == 'L') M.rmax[i] = R.rhs[i];
        else M.rmin[i] = R.rhs[i];
    }
    for (const auto& [i, r] : R.ranges) {
        const double b = R.rhs[i];
        if (R.sense[i] == 'E') {
            if (r >= 0) { M.rmin[i] = b; M.rmax[i] = b + r; }
            else { M.rmin[i] = b + r; M.rmax[i] = b; }
        } else if (R.sense[i] == 'G') {
            M.rmin[i] = b;
            M.rmax[i] = b + std::fabs(r);
        } else {
            M.rmin[i] = b - std::fabs(r);
            M.rmax[i] = b;
        }
    }
    build_csr_csc(M.m, M.n, R.ti, R.tj, R.tv, M);
}

}  // namespace igaos::io
