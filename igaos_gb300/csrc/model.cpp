// MPS reader and CSR/CSC builder (see model.hpp).
#include "model.hpp"

#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <limits>
#include <stdexcept>
#include <string_view>
#include <system_error>
#include <thread>

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
// FNV-1a hashing, power-of-two capacity kept under half full. Each slot keeps
// 32 bits of the hash, so probes and rehashes touch the names only on a match.
class NameTable {
   public:
    explicit NameTable(size_t expect = 1024) { rehash(expect * 2); }
    // index of `key`, or -2 if absent
    int find(std::string_view key) const {
        const uint64_t h = hash(key);
        const uint32_t tg = tag(h);
        for (size_t i = h & mask_; slots_[i].tag; i = (i + 1) & mask_)
            if (slots_[i].tag == tg && slots_[i].len == key.size() &&
                std::memcmp(slots_[i].ptr, key.data(), key.size()) == 0)
                return slots_[i].val;
        return -2;
    }
    // maps `key` to `val`; returns the index it replaced, or -2 if it was new
    int assign(std::string_view key, int val) {
        bool inserted = false;
        int* v = slot(key, &inserted);
        const int prev = inserted ? -2 : *v;
        *v = val;
        return prev;
    }
    // existing index of `key`, or `fresh` after inserting it (inserted = true)
    int find_or_insert(std::string_view key, int fresh, bool& inserted) {
        int* v = slot(key, &inserted);
        if (inserted) *v = fresh;
        return *v;
    }
    // room for `n` names without growing
    void reserve(size_t n) {
        if (2 * n > slots_.size()) rehash(2 * n);
    }
    size_t size() const { return count_; }

   private:
    struct Slot {
        const char* ptr = nullptr;
        uint32_t len = 0;
        uint32_t tag = 0;  // 0: empty
        int val = 0;
    };
    std::vector<Slot> slots_;
    size_t mask_ = 0, count_ = 0;
    static uint64_t hash(std::string_view k) {
        uint64_t h = 1469598103934665603ull;
        for (unsigned char ch : k) h = (h ^ ch) * 1099511628211ull;
        return h ^ (h >> 29);
    }
    static uint32_t tag(uint64_t h) { return (uint32_t)(h >> 32) | 1u; }
    void rehash(size_t want) {
        size_t cap = 16;
        while (cap < want) cap <<= 1;
        std::vector<Slot> old;
        old.swap(slots_);
        slots_.assign(cap, Slot{});
        mask_ = cap - 1;
        for (const Slot& s : old)
            if (s.tag) {
                size_t i = hash(std::string_view(s.ptr, s.len)) & mask_;
                while (slots_[i].tag) i = (i + 1) & mask_;
                slots_[i] = s;
            }
    }
    int* slot(std::string_view key, bool* inserted = nullptr) {
        if (2 * (count_ + 1) > slots_.size()) rehash(slots_.size() * 4);
        const uint64_t h = hash(key);
        const uint32_t tg = tag(h);
        size_t i = h & mask_;
        for (; slots_[i].tag; i = (i + 1) & mask_)
            if (slots_[i].tag == tg && slots_[i].len == key.size() &&
                std::memcmp(slots_[i].ptr, key.data(), key.size()) == 0) {
                if (inserted) *inserted = false;
                return &slots_[i].val;
            }
        slots_[i].ptr = key.data();
        slots_[i].len = (uint32_t)key.size();
        slots_[i].tag = tg;
        ++count_;
        if (inserted) *inserted = true;
        return &slots_[i].val;
    }
};

struct Reader {
    static constexpr double INF = std::numeric_limits<double>::infinity();
    NameTable rows;  // -1: objective / free row
    NameTable cols;
    // name of each row / column index (empty once a later ROWS line takes the
    // name away): lookups try the index after the previous one first
    std::vector<std::string_view> row_names, col_names;
    std::string_view obj;
    bool have_obj = false;
    std::vector<char> sense;
    std::vector<double> rhs;
    std::vector<int> ti, tj;
    std::vector<double> tv;
    std::vector<std::pair<int, double>> ranges;
    bool in_int = false;

    int row_of(std::string_view name) const {
        const int r = rows.find(name);
        return r == -2 ? -1 : r;
    }
    // row_of / column index (-2 if absent) of a name, trying `hint` + 1 and
    // `hint` before the table: RHS and BOUNDS entries mostly follow the order
    // of ROWS and COLUMNS
    int row_near(std::string_view name, int hint) const {
        for (int c = hint + 1; c >= hint && c >= 0; --c)
            if ((size_t)c < row_names.size() && row_names[c] == name) return c;
        return row_of(name);
    }
    int col_near(std::string_view name, int hint) const {
        for (int c = hint + 1; c >= hint && c >= 0; --c)
            if ((size_t)c < col_names.size() && col_names[c] == name) return c;
        return cols.find(name);
    }
};

// Next line of [p, end): the view without its '\n', and p moved past it.
std::string_view next_line(const char*& p, const char* end) {
    const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!eol) eol = end;
    const std::string_view line(p, (size_t)(eol - p));
    p = eol + 1;
    return line;
}

// A section header: a non-blank, non-comment line starting in column 1.
bool is_header(std::string_view line) {
    if (line.empty() || line[0] == '*' || line[0] == ' ' || line[0] == '\t') return false;
    for (char ch : line)
        if (ch != ' ' && ch != '\t' && ch != '\r') return true;
    return false;
}

// End of the section whose body starts at p (the next header line, or end),
// and its line count.
const char* section_end(const char* p, const char* end, size_t* lines = nullptr) {
    size_t k = 0;
    while (p < end) {
        const char* at = p;
        if (is_header(next_line(p, end))) return at;
        ++k;
        if (lines) *lines = k;
    }
    return end;
}

// One slice of a COLUMNS section parsed on its own: columns numbered locally
// in order of first appearance, with the integer-marker state at that point
// (-1: no marker yet in this slice, the state entering it applies).
struct ColumnSlice {
    NameTable local{64};
    std::vector<std::string_view> names;
    std::vector<signed char> integ;
    signed char end_state = -1;
    std::vector<int> ti, tj;
    std::vector<double> tv;
    std::vector<std::pair<int, double>> obj;  // (local column, value), file order
    std::exception_ptr err;

    void parse(const Reader& R, const char* p, const char* end) {
        std::vector<std::string_view> t;
        std::string_view last;
        int last_j = -1;
        signed char state = -1;
        try {
            while (p < end) {
                const std::string_view line = next_line(p, end);
                if (line.empty() || line[0] == '*') continue;
                split(line, t);
                if (t.empty()) continue;
                if (line.find("'MARKER'") != std::string_view::npos) {
                    state = line.find("INTORG") != std::string_view::npos ? 1 : 0;
                    continue;
                }
                int j;
                if (last_j >= 0 && t[0] == last) {
                    j = last_j;
                } else {
                    bool inserted = false;
                    j = local.find_or_insert(t[0], (int)names.size(), inserted);
                    if (inserted) {
                        names.push_back(t[0]);
                        integ.push_back(state);
                    }
                    last = t[0];
                    last_j = j;
                }
                for (size_t k = 1; k + 1 < t.size(); k += 2) {
                    const double v = num(t[k + 1]);
                    if (R.have_obj && t[k] == R.obj) {
                        obj.emplace_back(j, v);
                        continue;
                    }
                    const int r = R.row_of(t[k]);
                    if (r < 0) continue;
                    ti.push_back(r);
                    tj.push_back(j);
                    tv.push_back(v);
                }
            }
        } catch (...) {
            err = std::current_exception();
        }
        end_state = state;
    }
};

// The COLUMNS section starting at p, on the host's threads: slices at line
// boundaries parsed independently (row names are only read), then merged in
// file order, so column numbering, integer flags, objective sums and the
// triplet order are those of a sequential pass; the first error in file
// order is the one raised. Returns the start of the next section.
const char* parse_columns_parallel(Reader& R, Model& M, const char* p, const char* end) {
    const char* sec_end = section_end(p, end);
    const size_t bytes = (size_t)(sec_end - p);
    const int nt = bytes < (8u << 20)
                       ? 1
                       : (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<const char*> cut(nt + 1, p);
    cut[nt] = sec_end;
    for (int s = 1; s < nt; ++s) {
        const char* c = p + bytes * s / nt;
        c = std::max(c, cut[s - 1]);
        const char* nl = static_cast<const char*>(std::memchr(c, '\n', (size_t)(sec_end - c)));
        cut[s] = nl ? nl + 1 : sec_end;
    }
    std::vector<ColumnSlice> sl(nt);
    if (nt == 1) {
        sl[0].parse(R, cut[0], cut[1]);
    } else {
        std::vector<std::thread> pool;
        for (int s = 0; s < nt; ++s) pool.emplace_back([&, s] { sl[s].parse(R, cut[s], cut[s + 1]); });
        for (auto& th : pool) th.join();
    }
    size_t names = R.cols.size(), trip = R.tv.size();
    std::vector<size_t> at(nt + 1, trip);
    for (int k = 0; k < nt; ++k) {
        if (sl[k].err) std::rethrow_exception(sl[k].err);
        names += sl[k].names.size();
        at[k + 1] = at[k] + sl[k].tv.size();
    }
    R.cols.reserve(names);
    R.col_names.reserve(names);
    M.c.reserve(names);
    M.cl.reserve(names);
    M.cu.reserve(names);
    M.integ.reserve(names);
    // global numbering in file order
    std::vector<std::vector<int>> gj(nt);
    bool in_int = R.in_int;
    for (int k = 0; k < nt; ++k) {
        ColumnSlice& s = sl[k];
        gj[k].resize(s.names.size());
        for (size_t q = 0; q < s.names.size(); ++q) {
            bool inserted = false;
            gj[k][q] = R.cols.find_or_insert(s.names[q], (int)R.cols.size(), inserted);
            if (inserted) {
                const bool flag = s.integ[q] < 0 ? in_int : s.integ[q] == 1;
                R.col_names.push_back(s.names[q]);
                M.c.push_back(0.0);
                M.cl.push_back(0.0);
                M.cu.push_back(Reader::INF);
                M.integ.push_back(flag ? 1 : 0);
            }
        }
        for (const auto& [lj, v] : s.obj) M.c[gj[k][lj]] += v;
        if (s.end_state >= 0) in_int = s.end_state == 1;
    }
    R.in_int = in_int;
    // triplets at their file-order offsets
    R.ti.resize(at[nt]);
    R.tj.resize(at[nt]);
    R.tv.resize(at[nt]);
    auto place = [&](int k) {
        const ColumnSlice& s = sl[k];
        const std::vector<int>& g = gj[k];
        for (size_t e = 0; e < s.tv.size(); ++e) {
            R.ti[at[k] + e] = s.ti[e];
            R.tj[at[k] + e] = g[s.tj[e]];
            R.tv[at[k] + e] = s.tv[e];
        }
    };
    if (nt == 1) {
        place(0);
    } else {
        std::vector<std::thread> pool;
        for (int k = 0; k < nt; ++k) pool.emplace_back(place, k);
        for (auto& th : pool) th.join();
    }
    return sec_end;
}

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
    int hint_r = -1, hint_j = -1;  // last row of RHS, last column of BOUNDS
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
            if (section == "COLUMNS") {
                p = parse_columns_parallel(R, M, p, end);
            } else if (section == "ROWS") {
                size_t lines = 0;
                section_end(p, end, &lines);
                R.rows.reserve(R.rows.size() + lines);
                R.row_names.reserve(R.row_names.size() + lines);
            }
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
                const int prev = R.rows.assign(name, -1);
                if (prev >= 0) R.row_names[prev] = {};
            } else {
                const int prev = R.rows.assign(name, (int)R.sense.size());
                if (prev >= 0) R.row_names[prev] = {};
                R.row_names.push_back(name);
                R.sense.push_back(t[0][0]);
                R.rhs.push_back(0.0);
            }
        } else if (section == "RHS") {
            for (size_t k = 1; k + 1 < t.size(); k += 2) {
                if (R.have_obj && t[k] == R.obj) {
                    M.obj_const -= num(t[k + 1]);
                    continue;
                }
                const int r = R.row_near(t[k], hint_r);
                if (r < 0) continue;
                hint_r = r;
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
            const int j = R.col_near(t[2], hint_j);
            if (j == -2) throw std::out_of_range("BOUNDS names an unknown column");
            hint_j = j;
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
