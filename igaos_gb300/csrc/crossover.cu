// Crossover (host code; see crossover.hpp).
#include "crossover.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <exception>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace igx {
namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr double kZeroAlpha = 1e-11;  // |alpha_r| at or below: the basic does not move
constexpr double kPivTol = 1e-7;     // pivots at least this large are preferred
constexpr double kSnap = 1e-9;       // start values this close to a bound sit on it
constexpr int kDegenerateRun = 100;  // degenerate steps before Bland's rule
constexpr double kDevexReset = 1e6;  // reference weights reset above this
constexpr double kCrashRoom = 1e-6;  // a row this close to a bound (relative) is active

// Host threads for the dense O(m^2) loops: run(count, f) calls f(begin, end)
// on contiguous slices of [0, count), one per thread, the caller's included.
class Pool {
public:
    explicit Pool(int threads) : nthreads_(std::max(1, threads)) {
        for (int t = 1; t < nthreads_; ++t) workers_.emplace_back([this, t] { loop(t); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& w : workers_) w.join();
    }
    void run(int count, const std::function<void(int, int)>& f) {
        if (nthreads_ == 1 || count < 2 * nthreads_) {
            f(0, count);
            return;
        }
        {
            std::lock_guard<std::mutex> g(mu_);
            job_ = &f;
            count_ = count;
            pending_ = nthreads_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        std::exception_ptr own;
        try {
            slice(0, f);
        } catch (...) {
            own = std::current_exception();
        }
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return pending_ == 0; });
        // a worker's exception (e.g. bad_alloc) surfaces on the calling
        // thread, where the C ABI turns it into an error code
        std::exception_ptr err = own ? own : error_;
        error_ = nullptr;
        lk.unlock();
        if (err) std::rethrow_exception(err);
    }

private:
    void slice(int t, const std::function<void(int, int)>& f) const {
        const int b = (int)((int64_t)count_ * t / nthreads_);
        const int e = (int)((int64_t)count_ * (t + 1) / nthreads_);
        if (b < e) f(b, e);
    }
    void loop(int t) {
        uint64_t seen = 0;
        for (;;) {
            const std::function<void(int, int)>* f;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
                f = job_;
            }
            std::exception_ptr e;
            try {
                slice(t, *f);
            } catch (...) {
                e = std::current_exception();
            }
            std::lock_guard<std::mutex> g(mu_);
            if (e && !error_) error_ = e;
            if (--pending_ == 0) done_.notify_one();
        }
    }
    const int nthreads_;
    std::vector<std::thread> workers_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int, int)>* job_ = nullptr;
    int count_ = 0, pending_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
    std::exception_ptr error_;  // first worker exception of the current job
};

// Up to 16 host threads from m = 768 on (below, the hand-offs cost more than
// they save); IGAOS_PDHG_HOST_THREADS caps the count. Every thread owns whole
// columns or rows of the dense loops, so the results do not depend on it.
int pool_threads(int m) {
    if (m < 768) return 1;
    unsigned t = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    if (const char* e = std::getenv("IGAOS_PDHG_HOST_THREADS")) {
        const int v = std::atoi(e);
        if (v >= 1) t = std::min(t, (unsigned)v);
    }
    return (int)t;
}

class Simplex {
public:
    Simplex(int m, int n, const int* cp, const int* ci, const double* acx, CrossoverInfo& info)
        : m_(m), n_(n), nt_(n + m), cp_(cp), ci_(ci), acx_(acx), I_(info),
          pool_(new Pool(pool_threads(m))) {}

    std::vector<double> lb, ub, cost, val;
    std::vector<signed char> st;

    int run(const double* x0, bool use_crash);
    void duals(double* y) const {
        for (int i = 0; i < m_; ++i) y[i] = -pi_[i];
    }

private:
    const int m_, n_, nt_;
    const int *cp_, *ci_;
    const double* acx_;
    CrossoverInfo& I_;
    std::unique_ptr<Pool> pool_;
    std::vector<int> head_;
    std::vector<double> devex_;  // reference weights of the nonbasic variables
    std::vector<double> prow_;   // row r of B^-1 before a basis change
    std::vector<double> binv_;  // B^-1, column-major m x m
    std::vector<double> alpha_, pi_, work_a_, work_b_;
    std::vector<char> rejected_;  // candidates whose best pivot was below kPivTol
    int since_ = 0, every_ = 64;
    bool bland_ = false;
    int degen_ = 0;

    double ftol(int j) const {
        double b = 0.0;
        if (std::isfinite(lb[j])) b = std::fabs(lb[j]);
        if (std::isfinite(ub[j])) b = std::max(b, std::fabs(ub[j]));
        return 1e-9 * (1.0 + b);
    }
    double dtol(int j) const { return 1e-9 * (1.0 + std::fabs(cost[j])); }
    bool infeasible(int j) const {
        const double t = ftol(j);
        return val[j] < lb[j] - t || val[j] > ub[j] + t;
    }
    // v^T a_j, a_j the column of [A -I]
    double dot_col(int j, const double* v) const {
        if (j >= n_) return -v[j - n_];
        double s = 0.0;
        for (int p = cp_[j]; p < cp_[j + 1]; ++p) s += acx_[p] * v[ci_[p]];
        return s;
    }
    // alpha = B^-1 a_j
    void ftran(int j) {
        std::fill(alpha_.begin(), alpha_.end(), 0.0);
        auto axpy = [&](double a, int k) {
            const double* col = &binv_[(size_t)k * m_];
            for (int i = 0; i < m_; ++i) alpha_[i] += a * col[i];
        };
        if (j >= n_) {
            axpy(-1.0, j - n_);
            return;
        }
        for (int p = cp_[j]; p < cp_[j + 1]; ++p) axpy(acx_[p], ci_[p]);
    }
    // pi = c_B^T B^-1 with the phase's basic costs
    void compute_pi(bool phase1) {
        std::vector<double>& cb = work_a_;
        cb.assign(m_, 0.0);
        for (int r = 0; r < m_; ++r) {
            const int h = head_[r];
            if (!phase1) cb[r] = cost[h];
            else if (val[h] < lb[h] - ftol(h)) cb[r] = -1.0;
            else if (val[h] > ub[h] + ftol(h)) cb[r] = 1.0;
        }
        pool_->run(m_, [&](int k0, int k1) {
            for (int k = k0; k < k1; ++k) {
                const double* col = &binv_[(size_t)k * m_];
                double s = 0.0;
                for (int r = 0; r < m_; ++r) s += cb[r] * col[r];
                pi_[k] = s;
            }
        });
    }
    // basis position r takes the column whose B^-1 a_q is alpha
    void update_binv(int r) {
        const double ar = alpha_[r];
        pool_->run(m_, [&](int k0, int k1) {
            for (int k = k0; k < k1; ++k) {
                double* col = &binv_[(size_t)k * m_];
                const double t = col[r] / ar;
                if (t == 0.0) continue;
                for (int i = 0; i < m_; ++i) col[i] -= t * alpha_[i];
                col[r] = t;
            }
        });
    }
    // B^-1 of the basic columns by Gauss-Jordan with partial pivoting. A basis
    // column without a pivot (dependent on the others to within 1e-11) is
    // replaced by the slack of a row no pivot used, and its variable leaves
    // the basis where it stands; then the factorisation starts again.
    bool refactor() {
        ++I_.refactors;
        since_ = 0;
        for (int attempt = 0; attempt < 2; ++attempt) {
            std::vector<int> dep, spare;
            if (factor(dep, spare)) return true;
            if (attempt == 1) return false;
            for (size_t t = 0; t < dep.size(); ++t) {
                const int j = head_[dep[t]];
                head_[dep[t]] = n_ + spare[t];
                st[n_ + spare[t]] = kBasic;
                st[j] = at_bound(j);
                ++I_.basis_repairs;
            }
        }
        return false;
    }
    signed char at_bound(int j) {
        if (std::isfinite(lb[j]) && val[j] - lb[j] <= kSnap * (1.0 + std::fabs(lb[j]))) {
            val[j] = lb[j];
            return kAtLower;
        }
        if (std::isfinite(ub[j]) && ub[j] - val[j] <= kSnap * (1.0 + std::fabs(ub[j]))) {
            val[j] = ub[j];
            return kAtUpper;
        }
        return kSuperbasic;
    }
    // true: binv_ = B^-1. false: dep lists the basis positions without a
    // pivot and spare as many rows no pivot used.
    bool factor(std::vector<int>& dep, std::vector<int>& spare) {
        std::vector<double>& M = work_a_;
        std::vector<double>& R = work_b_;
        const size_t mm = (size_t)m_ * m_;
        M.assign(mm, 0.0);
        R.assign(mm, 0.0);
        std::vector<int> rowid(m_);
        for (int r = 0; r < m_; ++r) {
            const int j = head_[r];
            if (j >= n_) M[(size_t)(j - n_) * m_ + r] = -1.0;
            else  // repeated (row, column) entries add up
                for (int p = cp_[j]; p < cp_[j + 1]; ++p) M[(size_t)ci_[p] * m_ + r] += acx_[p];
            R[(size_t)r * m_ + r] = 1.0;
            rowid[r] = r;
        }
        int prow = 0;  // next pivot row
        for (int k = 0; k < m_; ++k) {
            int piv = -1;
            double best = 1e-11;
            for (int i = prow; i < m_; ++i) {
                const double v = std::fabs(M[(size_t)i * m_ + k]);
                if (v > best) {
                    best = v;
                    piv = i;
                }
            }
            if (piv < 0) {
                dep.push_back(k);
                continue;
            }
            double* mk = &M[(size_t)prow * m_];
            double* rk = &R[(size_t)prow * m_];
            if (piv != prow) {
                std::swap_ranges(mk, mk + m_, &M[(size_t)piv * m_]);
                std::swap_ranges(rk, rk + m_, &R[(size_t)piv * m_]);
                std::swap(rowid[prow], rowid[piv]);
            }
            const double inv = 1.0 / mk[k];
            for (int j = k; j < m_; ++j) mk[j] *= inv;
            for (int j = 0; j < m_; ++j) rk[j] *= inv;
            pool_->run(m_, [&](int i0, int i1) {
                for (int i = i0; i < i1; ++i) {
                    if (i == prow) continue;
                    double* mi = &M[(size_t)i * m_];
                    const double f = mi[k];
                    if (f == 0.0) continue;
                    double* ri = &R[(size_t)i * m_];
                    for (int j = k; j < m_; ++j) mi[j] -= f * mk[j];
                    for (int j = 0; j < m_; ++j) ri[j] -= f * rk[j];
                }
            });
            ++prow;
        }
        if (!dep.empty()) {
            for (int i = prow; i < m_; ++i) spare.push_back(rowid[i]);
            return false;
        }
        for (int i = 0; i < m_; ++i)
            for (int k = 0; k < m_; ++k) binv_[(size_t)k * m_ + i] = R[(size_t)i * m_ + k];
        return true;
    }
    // basic values from the nonbasic ones, B x_B = -N x_N, then two steps of
    // iterative refinement on the residual [A -I] (x, s)
    void recompute_basics() {
        std::vector<double>& rhs = work_a_;
        for (int round = 0; round < 3; ++round) {
            rhs.assign(m_, 0.0);  // -[A -I] v over the variables counted
            for (int j = 0; j < nt_; ++j) {
                if ((round == 0 && st[j] == kBasic) || val[j] == 0.0) continue;
                if (j >= n_) rhs[j - n_] += val[j];
                else
                    for (int p = cp_[j]; p < cp_[j + 1]; ++p) rhs[ci_[p]] -= acx_[p] * val[j];
            }
            if (round == 0)
                for (int r = 0; r < m_; ++r) val[head_[r]] = 0.0;
            for (int k = 0; k < m_; ++k) {
                if (rhs[k] == 0.0) continue;
                const double* col = &binv_[(size_t)k * m_];
                for (int r = 0; r < m_; ++r) val[head_[r]] += rhs[k] * col[r];
            }
        }
    }
    bool maybe_refactor(bool& pi_valid) {
        if (since_ < every_) return true;
        if (!refactor()) return false;
        recompute_basics();
        pi_valid = false;
        return true;
    }
    int ratio(int q, int dir, double& theta, bool& leave_upper);
    void move(int q, int dir, double theta) {
        if (theta == 0.0) return;
        val[q] += dir * theta;
        for (int i = 0; i < m_; ++i)
            if (alpha_[i] != 0.0) val[head_[i]] -= dir * theta * alpha_[i];
    }
    // q enters at position r; the leaving variable lands on its bound; pi
    // follows in phase 2 (dq = q's phase-2 reduced cost)
    void enter(int q, int r, bool leave_upper, bool phase2, double dq) {
        const int l = head_[r];
        const double ar = alpha_[r];
        for (int k = 0; k < m_; ++k) prow_[k] = binv_[(size_t)k * m_ + r];
        if (phase2) {
            const double f = dq / ar;
            for (int k = 0; k < m_; ++k) pi_[k] += f * prow_[k];
        }
        // Devex reference weights from the pivot row alpha_rj = rho_r^T a_j
        const double wq = devex_[q];
        double wmax = 0.0;
        for (int j = 0; j < nt_; ++j) {
            if (st[j] == kBasic || j == q) continue;
            const double arj = dot_col(j, prow_.data());
            if (arj != 0.0) devex_[j] = std::max(devex_[j], (arj / ar) * (arj / ar) * wq);
            wmax = std::max(wmax, devex_[j]);
        }
        devex_[l] = std::max(wq / (ar * ar), 1.0);
        if (std::max(wmax, devex_[l]) > kDevexReset) std::fill(devex_.begin(), devex_.end(), 1.0);
        val[l] = leave_upper ? ub[l] : lb[l];
        st[l] = leave_upper ? kAtUpper : kAtLower;
        head_[r] = q;
        st[q] = kBasic;
        update_binv(r);
        ++since_;
        ++I_.pivots;
    }
    bool push(int j, bool& pi_valid, bool zero_cost_only);
    bool crash();
    int simplex(int64_t& it, int64_t cap, bool& pi_valid);
    int n_rejected_ = 0;
    bool retried_ = false;
    void clear_rejected() {
        std::fill(rejected_.begin(), rejected_.end(), 0);
        n_rejected_ = 0;
    }
    void price(bool phase1, int& q, int& dir, double& dq) const;
    bool clean() const;
};

// Entering q moves by theta * dir (dir = +1 up, -1 down). Returns the basis
// position of the blocking variable, -1 when q reaches its own bound first,
// -2 when nothing blocks. A basic variable inside its bounds (within its
// tolerance) blocks at the bound it moves toward; one outside them blocks
// when it comes back to the violated bound, never while it moves away. Pass
// 1 finds the largest step with every block relaxed by its tolerance; pass 2
// takes, among the blocks within that step, the largest |alpha| (Bland's
// rule: the smallest variable index).
int Simplex::ratio(int q, int dir, double& theta, bool& leave_upper) {
    const double own = dir > 0 ? ub[q] - val[q] : val[q] - lb[q];
    auto block = [&](int i, double relax, double& lim, bool& upper) -> bool {
        const double a = alpha_[i];
        if (std::fabs(a) <= kZeroAlpha) return false;
        const double rate = -dir * a;  // change of the basic value per unit step
        const int h = head_[i];
        const double v = val[h], t = ftol(h), s = relax * t;
        if (rate < 0.0) {
            if (v > ub[h] + t) {
                lim = (v - ub[h] + s) / -rate;
                upper = true;
                return true;
            }
            if (v < lb[h] - t || !std::isfinite(lb[h])) return false;
            lim = (v - lb[h] + s) / -rate;
            upper = false;
            return true;
        }
        if (v < lb[h] - t) {
            lim = (lb[h] - v + s) / rate;
            upper = false;
            return true;
        }
        if (v > ub[h] + t || !std::isfinite(ub[h])) return false;
        lim = (ub[h] - v + s) / rate;
        upper = true;
        return true;
    };
    double tmax = kInf, lim = 0.0;
    bool up = false;
    for (int i = 0; i < m_; ++i)
        if (block(i, 1.0, lim, up)) tmax = std::min(tmax, lim);
    if (!std::isfinite(tmax)) {
        if (!std::isfinite(own)) return -2;
        theta = std::max(own, 0.0);
        return -1;
    }
    if (own <= tmax) {
        theta = std::max(own, 0.0);
        return -1;
    }
    int best = -1;
    double best_abs = -1.0;
    for (int i = 0; i < m_; ++i) {
        if (!block(i, 0.0, lim, up) || lim > tmax) continue;
        const double a = std::fabs(alpha_[i]);
        const bool take =
            bland_ ? (best < 0 || (a >= kPivTol && (best_abs < kPivTol || head_[i] < head_[best])))
                   : a > best_abs;
        if (!take) continue;
        best = i;
        best_abs = std::fabs(alpha_[i]);
        theta = std::max(lim, 0.0);
        leave_upper = up;
    }
    return best;
}

// Moves variable j (nonbasic, inside its bounds) to a bound or into the
// basis along the edge its phase-2 reduced cost does not worsen; either way
// (nearer bound first) when that cost is within tolerance of 0. With
// zero_cost_only, j moves only in that last case. False: j did not move.
bool Simplex::push(int j, bool& pi_valid, bool zero_cost_only) {
    if (!pi_valid) {
        compute_pi(false);
        pi_valid = true;
    }
    const double d = cost[j] - dot_col(j, pi_.data());
    int dirs[2] = {0, 0}, nd = 0;
    if (d < -dtol(j) || d > dtol(j)) {
        if (zero_cost_only) return false;
        dirs[nd++] = d < 0.0 ? 1 : -1;
    } else {
        dirs[0] = ub[j] - val[j] < val[j] - lb[j] ? 1 : -1;
        dirs[1] = -dirs[0];
        nd = 2;
    }
    ftran(j);
    for (int k = 0; k < nd; ++k) {
        double theta = 0.0;
        bool up = false;
        const int r = ratio(j, dirs[k], theta, up);
        if (r == -2) continue;
        ++I_.pushes;
        move(j, dirs[k], theta);
        if (r == -1) {
            val[j] = dirs[k] > 0 ? ub[j] : lb[j];
            st[j] = dirs[k] > 0 ? kAtUpper : kAtLower;
            ++I_.bound_flips;
        } else {
            enter(j, r, up, true, d);
        }
        return true;
    }
    return false;
}

// Composite primal simplex from the current basis until no candidate prices
// out (kXoOptimal) or an outcome ends it; it counts pivots against cap.
int Simplex::simplex(int64_t& it, int64_t cap, bool& pi_valid) {
    for (;; ++it) {
        if (it >= cap) return kXoIterLimit;
        if (!maybe_refactor(pi_valid)) return kXoSingular;
        bool phase1 = false;
        for (int r = 0; r < m_ && !phase1; ++r) phase1 = infeasible(head_[r]);
        if (phase1) {
            compute_pi(true);
            pi_valid = false;
            ++I_.phase1_iters;
        } else if (!pi_valid) {
            compute_pi(false);
            pi_valid = true;
        }
        int q = -1, dir = 0;
        double dq = 0.0;
        price(phase1, q, dir, dq);
        if (q < 0) {
            // phase 1 stuck: confirm on a fresh factorisation before ending
            if (phase1 && n_rejected_ == 0 && since_ > 0) {
                since_ = every_;
                continue;
            }
            if (n_rejected_ == 0) return phase1 ? kXoInfeasible : kXoOptimal;
            // only candidates with pivots below kPivTol are left: refactor
            // and give them one more chance before ending
            if (retried_) return phase1 ? kXoSingular : kXoOptimal;
            retried_ = true;
            clear_rejected();
            since_ = every_;
            continue;
        }
        ftran(q);
        double theta = 0.0;
        bool up = false;
        const int r = ratio(q, dir, theta, up);
        // a phase-1 candidate always meets a violated basic on its way back,
        // unless rounding hid it: a numerical failure, not an unbounded edge
        if (r == -2) {
            if (since_ > 0) {  // confirm on a fresh factorisation first
                since_ = every_;
                continue;
            }
            return phase1 ? kXoSingular : kXoUnbounded;
        }
        if (r >= 0 && std::fabs(alpha_[r]) < kPivTol && !retried_) {
            rejected_[q] = 1;  // a poor pivot: try the other candidates first
            ++n_rejected_;
            continue;
        }
        if (theta <= 1e-12) {
            if (++degen_ > kDegenerateRun) bland_ = true;
        } else {
            degen_ = 0;
            bland_ = false;
        }
        move(q, dir, theta);
        if (r == -1) {
            val[q] = dir > 0 ? ub[q] : lb[q];
            st[q] = dir > 0 ? kAtUpper : kAtLower;
            ++I_.bound_flips;
        } else {
            enter(q, r, up, !phase1 && pi_valid, dq);
            if (std::fabs(alpha_[r]) >= kPivTol) {
                retried_ = false;
                if (n_rejected_) clear_rejected();
            }
        }
        if (phase1) pi_valid = false;
    }
}

// Devex pricing (largest d_j^2 / w_j; Bland's rule: the first candidate) of
// the nonbasic variables with the phase's costs: q = -1 when none improves.
void Simplex::price(bool phase1, int& q, int& dir, double& dq) const {
    double best = 0.0;
    for (int j = 0; j < nt_; ++j) {
        if (st[j] == kBasic || (st[j] != kSuperbasic && lb[j] == ub[j])) continue;
        if (rejected_[j]) continue;
        const double d = (phase1 ? 0.0 : cost[j]) - dot_col(j, pi_.data());
        const double t = phase1 ? 1e-9 : dtol(j);
        int dj = 0;
        if (st[j] == kAtLower) dj = d < -t ? 1 : 0;
        else if (st[j] == kAtUpper) dj = d > t ? -1 : 0;
        else dj = d < -t ? 1 : (d > t ? -1 : 0);
        if (!dj) continue;
        if (bland_) {
            q = j;
            dir = dj;
            dq = d;
            return;
        }
        const double score = d * d / devex_[j];
        if (score > best) {
            best = score;
            q = j;
            dir = dj;
            dq = d;
        }
    }
}

// every basic value within its bounds and no nonbasic variable pricing out
bool Simplex::clean() const {
    for (int r = 0; r < m_; ++r)
        if (infeasible(head_[r])) return false;
    int q = -1, dir = 0;
    double dq = 0.0;
    price(false, q, dir, dq);
    return q < 0;
}

// Crash basis: the structurals strictly inside their bounds (most interior
// first) enter at once in place of the slacks of the rows with the least
// room, whose activities go to their nearest bound; one factorisation
// (dependent columns go back out) replaces that many one-pivot pushes, and
// the basic values follow from the nonbasic ones. False: the slack basis
// stays (no structural inside its bounds, or the factorisation failed).
bool Simplex::crash() {
    std::vector<std::pair<double, int>> inner, room;
    for (int j = 0; j < n_; ++j) {
        if (st[j] != kSuperbasic) continue;
        const double d = std::min(val[j] - lb[j], ub[j] - val[j]);  // inf when free
        inner.push_back({-d / (1.0 + std::fabs(val[j])), j});
    }
    for (int i = 0; i < m_; ++i) {
        const int s = n_ + i;
        const double d = std::min(val[s] - lb[s], ub[s] - val[s]);
        const double r = d / (1.0 + std::fabs(val[s]));
        if (r <= kCrashRoom) room.push_back({r, i});  // only rows at a bound swap their slack
    }
    const int out = (int)std::min(inner.size(), room.size());
    if (out == 0) return false;
    std::sort(inner.begin(), inner.end());
    std::sort(room.begin(), room.end());  // least room first: these slacks leave
    const std::vector<double> val0 = val;
    const std::vector<signed char> st0 = st;
    for (int t = 0; t < out; ++t) {
        const int i = room[t].second, s = n_ + i, j = inner[t].second;
        const bool up = ub[s] - val[s] < val[s] - lb[s];
        val[s] = up ? ub[s] : lb[s];
        st[s] = up ? kAtUpper : kAtLower;
        head_[i] = j;
        st[j] = kBasic;
    }
    if (refactor()) {
        recompute_basics();
        return true;
    }
    val = val0;  // back to the slack basis
    st = st0;
    std::fill(binv_.begin(), binv_.end(), 0.0);
    for (int i = 0; i < m_; ++i) {
        head_[i] = n_ + i;
        binv_[(size_t)i * m_ + i] = -1.0;
    }
    return false;
}

int Simplex::run(const double* x0, bool use_crash) {
    val.assign(nt_, 0.0);
    st.assign(nt_, kBasic);
    head_.resize(m_);
    alpha_.assign(m_, 0.0);
    pi_.assign(m_, 0.0);
    binv_.assign((size_t)m_ * m_, 0.0);
    rejected_.assign(nt_, 0);
    every_ = m_ <= 256 ? 64 : m_;
    devex_.assign(nt_, 1.0);
    prow_.assign(m_, 0.0);
    for (int j = 0; j < n_; ++j) {
        double v = std::min(std::max(x0[j], lb[j]), ub[j]);
        if (!std::isfinite(v)) v = 0.0;
        if (lb[j] == ub[j] || (std::isfinite(lb[j]) && v - lb[j] <= kSnap * (1.0 + std::fabs(lb[j])))) {
            v = lb[j];
            st[j] = kAtLower;
        } else if (std::isfinite(ub[j]) && ub[j] - v <= kSnap * (1.0 + std::fabs(ub[j]))) {
            v = ub[j];
            st[j] = kAtUpper;
        } else {
            st[j] = kSuperbasic;
        }
        val[j] = v;
    }
    for (int i = 0; i < m_; ++i) {  // slack basis: B = -I, row activities A x
        head_[i] = n_ + i;
        binv_[(size_t)i * m_ + i] = -1.0;
    }
    for (int j = 0; j < n_; ++j)
        for (int p = cp_[j]; p < cp_[j + 1]; ++p) val[n_ + ci_[p]] += acx_[p] * val[j];
    bool pi_valid = true;  // slack costs are 0, so pi = 0
    if (use_crash && crash()) pi_valid = false;

    for (int j = 0; j < nt_; ++j) {  // 1. primal push
        if (st[j] != kSuperbasic) continue;
        push(j, pi_valid, false);
        if (!maybe_refactor(pi_valid)) return kXoSingular;
    }
    // 2. composite primal simplex, 3. last push; repeated when the values
    // and duals of a fresh factorisation are not clean
    const int64_t cap = 20LL * nt_ + 10000;
    int64_t it = 0;
    for (int pass = 0;; ++pass) {
        const int rc = simplex(it, cap, pi_valid);
        if (rc != kXoOptimal) return rc;
        clear_rejected();
        retried_ = false;
        for (int j = 0; j < nt_; ++j) {  // a basis repair can leave a slack inside
            if (st[j] != kSuperbasic) continue;
            push(j, pi_valid, true);
            if (!maybe_refactor(pi_valid)) return kXoSingular;
        }
        if (!refactor()) return kXoSingular;
        recompute_basics();
        compute_pi(false);
        pi_valid = true;
        if (clean() || pass == 3) break;
    }
    for (int j = 0; j < nt_; ++j) I_.superbasic_left += st[j] == kSuperbasic;
    return kXoOptimal;
}

}  // namespace

int crossover(int m, int n, const int* cp, const int* ci, const double* acx, const double* c,
              const double* cl, const double* cu, const double* rmin, const double* rmax,
              const double* x0, double* x, double* y, signed char* basis, CrossoverInfo& info) {
    const auto t0 = std::chrono::steady_clock::now();
    info = CrossoverInfo();
    if (m > kCrossoverMaxRows) {
        info.status = kXoTooLarge;
        return kXoTooLarge;
    }
    // with the crash basis first; a start it does not suit is run again
    // from the slack basis
    int rc = kXoSingular;
    for (int attempt = 0; attempt < 2 && rc != kXoOptimal; ++attempt) {
        if (attempt == 1) info = CrossoverInfo();
        Simplex S(m, n, cp, ci, acx, info);
        S.lb.assign(cl, cl + n);
        S.lb.insert(S.lb.end(), rmin, rmin + m);
        S.ub.assign(cu, cu + n);
        S.ub.insert(S.ub.end(), rmax, rmax + m);
        S.cost.assign(c, c + n);
        S.cost.resize(n + m, 0.0);
        rc = S.run(x0, attempt == 0);
        std::copy(S.val.begin(), S.val.begin() + n, x);
        S.duals(y);
        if (basis) std::copy(S.st.begin(), S.st.end(), basis);
    }
    info.status = rc;
    info.time_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

}  // namespace igx
