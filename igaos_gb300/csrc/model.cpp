// MPS reader and CSR/CSC builder (see model.hpp).
#include "model.hpp"

#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string_view>
#include <system_error>

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

// std::stod semantics (leading number; std::invalid_argument if none,
// std::out_of_range if it does not fit), on the fast path of std::from_chars
// (correctly rounded, as strtod): plain decimal tokens, an optional leading
// '+'; anything from_chars does not take whole goes to std::stod itself.
double num(std::string_view v) {
    const char* b = v.data();
    const char* e = b + v.size();
    if (e - b > 1 && *b == '+' && (std::isdigit((unsigned char)b[1]) || b[1] == '.')) ++b;
    double out = 0.0;
    const auto r = std::from_chars(b, e, out, std::chars_format::general);
    // normal finite values taken whole; zeros only when spelled with zero
    // digits (underflow and subnormals are std::stod's range errors)
    const bool whole = r.ec == std::errc() && r.ptr == e;
    if (whole && std::isfinite(out) &&
        (out == 0.0 ? v.find_first_of("123456789") == std::string_view::npos
                    : std::fabs(out) >= std::numeric_limits<double>::min()))
        return out;
    return std::stod(std::string(v));
}

// Names -> indices over views into the file buffer: open addressing,
// FNV-1a hashing, power-of-two capacity kept under half full.
class NameTable {
   public:
    explicit NameTable(size_t expect = 1024) { rehash(expect * 2); }
    // index of `key`, or -2 if absent
    int find(std::string_view key) const {
        size_t h = hash(key) & mask_;
        while (slots_[h].used) {
            if (slots_[h].key == key) return slots_[h].val;
            h = (h + 1) & mask_;
        }
        return -2;
    }
    void assign(std::string_view key, int val) { *slot(key) = val; }
    // existing index of `key`, or `fresh` after inserting it (inserted = true)
    int find_or_insert(std::string_view key, int fresh, bool& inserted) {
        int* v = slot(key, &inserted);
        if (inserted) *v = fresh;
        return *v;
    }
    size_t size() const { return count_; }

   private:
    struct Slot {
        std::string_view key;
        int val = 0;
        bool used = false;
    };
    std::vector<Slot> slots_;
    size_t mask_ = 0, count_ = 0;
    static size_t hash(std::string_view k) {
        uint64_t h = 1469598103934665603ull;
        for (unsigned char ch : k) h = (h ^ ch) * 1099511628211ull;
        return (size_t)(h ^ (h >> 29));
    }
    void rehash(size_t want) {
        size_t cap = 16;
        while (cap < want) cap <<= 1;
        std::vector<Slot> old;
        old.swap(slots_);
        slots_.assign(cap, Slot{});
        mask_ = cap - 1;
        for (const Slot& s : old)
            if (s.used) {
                size_t h = hash(s.key) & mask_;
                while (slots_[h].used) h = (h + 1) & mask_;
                slots_[h] = s;
            }
    }
    int* slot(std::string_view key, bool* inserted = nullptr) {
        if (2 * (count_ + 1) > slots_.size()) rehash(slots_.size() * 4);
        size_t h = hash(key) & mask_;
        while (slots_[h].used) {
            if (slots_[h].key == key) {
                if (inserted) *inserted = false;
                return &slots_[h].val;
            }
            h = (h + 1) & mask_;
        }
        slots_[h].used = true;
        slots_[h].key = key;
        ++count_;
        if (inserted) *inserted = true;
        return &slots_[h].val;
    }
};

struct Reader {
    static constexpr double INF = std::numeric_limits<double>::infinity();
    NameTable rows;  // -1: objective / free row
    NameTable cols;
    std::string_view obj;
    bool have_obj = false;
    std::vector<char> sense;
    std::vector<double> rhs;
    std::vector<int> ti, tj;
    std::vector<double> tv;
    std::vector<std::pair<int, double>> ranges;
    bool in_int = false;
    std::string_view last_col;  // COLUMNS lines come grouped by column
    int last_j = -1;

    int row_of(std::string_view name) const {
        const int r = rows.find(name);
        return r == -2 ? -1 : r;
    }
};

}  // namespace

void parse_mps(const std::string& path, Model& M) {
    // the whole file in memory; names stay views into it while parsing
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open " + path);
    std::string buf;
    {
        std::fseek(f, 0, SEEK_END);
        const long size = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (size > 0) {
            buf.resize((size_t)size);
            buf.resize(std::fread(&buf[0], 1, (size_t)size, f));
        }
        char chunk[1 << 16];  // anything beyond the size seen (growing files)
        size_t got;
        while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.append(chunk, got);
        std::fclose(f);
    }
    Reader R;
    {
        // one entry per line at most: reserve the triplets once
        size_t lines = 0;
        for (const char* q = buf.data(); (q = static_cast<const char*>(std::memchr(
                                              q, '\n', (size_t)(buf.data() + buf.size() - q))));
             ++q)
            ++lines;
        R.ti.reserve(lines);
        R.tj.reserve(lines);
        R.tv.reserve(lines);
    }
    std::string section;
    std::vector<std::string_view> t;
    const char* p = buf.data();
    const char* const end = p + buf.size();
    while (p < end) {
        const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        if (!eol) eol = end;
        const std::string_view line(p, (size_t)(eol - p));
        p = eol + 1;
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
            const std::string_view name = t[1];
            if (t[0][0] == 'N') {
                if (!R.have_obj) {
                    R.obj = name;
                    R.have_obj = true;
                }
                R.rows.assign(name, -1);
            } else {
                R.rows.assign(name, (int)R.sense.size());
                R.sense.push_back(t[0][0]);
                R.rhs.push_back(0.0);
            }
        } else if (section == "COLUMNS") {
            if (line.find("'MARKER'") != std::string_view::npos) {
                R.in_int = line.find("INTORG") != std::string_view::npos;
                continue;
            }
            int j;
            if (R.last_j >= 0 && t[0] == R.last_col) {
                j = R.last_j;
            } else {
                bool inserted = false;
                j = R.cols.find_or_insert(t[0], (int)R.cols.size(), inserted);
                if (inserted) {
                    M.c.push_back(0.0);
                    M.cl.push_back(0.0);
                    M.cu.push_back(Reader::INF);
                    M.integ.push_back(R.in_int ? 1 : 0);
                }
                R.last_col = t[0];
                R.last_j = j;
            }
            for (size_t k = 1; k + 1 < t.size(); k += 2) {
                const double v = num(t[k + 1]);
                if (R.have_obj && t[k] == R.obj) {
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
                if (R.have_obj && t[k] == R.obj) {
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
                const int a = R.cols.find(t[k]), b = R.cols.find(t[k + 1]);
                if (a == -2 || b == -2) continue;
                M.q_i.push_back(a);
                M.q_j.push_back(b);
                M.q_v.push_back(num(t[k + 2]));
            }
        } else if (section == "BOUNDS") {
            if (t.size() < 3) continue;
            const int j = R.cols.find(t[2]);
            if (j == -2) throw std::out_of_range("BOUNDS names an unknown column");
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
