// Host side of the GB300 PDHG engine: owns the device copy of one LP and
// drives the iteration loop. Only the C ABI (capi.cu) is exported.
#pragma once

#include <chrono>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "igaos_pdhg.h"
#include "device.cuh"
#include "host_kkt.hpp"

#include <memory>

namespace igx {

struct CudaError : std::runtime_error {
    int code;
    CudaError(int c, const std::string& s) : std::runtime_error(s), code(c) {}
};

void cuda_check(cudaError_t e, const char* what, int line);

// Records the calling thread's last error (igaos_pdhg_last_error) and returns
// `code`; IGAOS_PDHG_OK clears it.
int igx_set_error(int code, const char* msg);
#define CU(x) ::igx::cuda_check((x), #x, __LINE__)

// Every device allocation of a problem, freed together.
class Arena {
   public:
    ~Arena();
    void* raw(size_t bytes);
    template <typename T>
    T* alloc(size_t n) { return static_cast<T*>(raw(sizeof(T) * (n ? n : 1))); }
    size_t bytes() const { return total_; }

   private:
    std::vector<void*> ptrs_;
    size_t total_ = 0;
};

struct Sched {
    int* row = nullptr;
    unsigned char* lg = nullptr;
    int nwarps = 0;
    int ctas = 0;  // kWarps warps per CTA
    int ctas64 = 0;  // launch width of the FP64 attempt kernels (3 CTAs per SM)
    int ctas64w = 0; // the same at 4 CTAs per SM
    int entries = 0; // entries per lane the schedule was built for
    WarpSched view() const { return WarpSched{row, lg, nwarps}; }
};

// Host-side warp schedule of a (length-sorted) CSR row pointer: consecutive
// rows dealt to warps, G lanes per row from the first row's length.
void build_warps(const int* ptr, int rows, std::vector<int>& wrow, std::vector<unsigned char>& wlg,
                 int entries = kLaneEntries);

// Entries per lane of the schedules the autotuner chooses from (the first
// value that is not the default is tried first; kLaneEntries is the default).
constexpr int kTuneCount = 5;
constexpr int kTuneEntries[kTuneCount] = {2, 4, 8, 16, 32};

// Permutation sorting rows by decreasing length (stable): new -> old index.
std::vector<int> length_order(const int* ptr, int rows);

// Vectors defining one LP over the engine's shared matrix: original units
// (FP64, for the KKT pass) and scaled units (FP64 and FP32, for iterating).
struct Vecs {
    double *c, *cl, *cu, *rmin, *rmax;      // original
    double *lob, *hib;                      // at-bound bands of cl, cu (k_bands)
    double *sc, *scl, *scu, *srmin, *srmax; // scaled FP64
    float *fc, *fcl, *fcu, *frmin, *frmax;  // scaled FP32
    double cmax;
    float* fyhat = nullptr;                 // anchored FP32 iterations: rounded y anchor
};

// FP64 anchor state of the FP32 + FP64-refinement mode (scaled units):
// iterates are x = xh + dx, y = yh + dy with FP32 deltas in Work<float>.
struct Anchor {
    double *xh, *yh;       // anchor
    double *xf[2], *yf[2]; // full current / averaged iterate at a check
    double *xb, *yb;       // incumbent
    double *pesx, *pesy;   // previous epoch start (= previous anchor)
    double *aty, *ax;      // A~^T yh, A~ xh
};

template <typename T>
struct Work {
    T *x[2], *y[2], *xavg[2], *yavg[2], *axc[2];
    T *xbar, *xb, *yb, *pesx, *pesy;
    double *part_p, *part_d;
};

template <typename T> struct PrimalArgs;  // kernels.cuh
template <typename T> struct DualArgs;

struct GraphKey {
    int prec, count;
    uintptr_t vecs;
    int sched;  // schedules in use (kTuneCount * index of A's + index of A^T's)
    bool operator<(const GraphKey& o) const {
        if (prec != o.prec) return prec < o.prec;
        if (count != o.count) return count < o.count;
        if (sched != o.sched) return sched < o.sched;
        return vecs < o.vecs;
    }
};

struct LoopOpts {
    double tol = 1e-4;
    double deadline = 1e300; // seconds since solve start, checked at each KKT check
    long long maxit = 500000;
    int check = 64;
    int verbosity = 0;
    bool graphs = true;
    bool detect_inf = false;  // infeasibility certificates at restarts
    double eta_init = 1, omega_init = 1, eta0 = 1;
    // testing knob (IGAOS_PDHG_PERTURB_AT): at the first KKT check at or after
    // this iteration, 1e6 is added to every entry of the current x before its
    // metrics are taken, a blown-up state that exercises the rollback to the
    // incumbent (src/pdhg/pdhg.cu:965-988). 0: never.
    long long perturb_at = 0;
};

struct LoopOut {
    int status = IGAOS_STATUS_ERROR;
    DevMetrics last{};
    bool last_is_avg = false, use_inc = false;
    long long iters = 0, attempts = 0, checks = 0, restarts = 0, spmvs = 0, anchors = 0;
    long long rollbacks = 0;
    double eta = 0, omega = 0;
    int parity = 0;
    bool numeric_failure = false;
    bool repaired = false;            // certified by dual repair: answer in rx, ry
    int ray = 0;                      // 1: dual ray in ry (infeasible); 2: primal ray in rx
    std::vector<double> rx, ry;       // original units, caller's numbering
};

class Engine {
   public:
    Engine(int m, int n, long long nnz, const int* ap, const int* ai, const double* ax,
           const int* cp, const int* ci, const double* acx, const double* c,
           const double* cl, const double* cu, const double* rmin, const double* rmax,
           double obj_const, int device, int scaling = IGAOS_PDHG_SCALING_RUIZ);
    ~Engine();

    void solve(const igaos_pdhg_options& o, igaos_pdhg_result& r, double* x, double* y);

    // inspection / parity entry points
    int m, n;
    long long nnz;
    double obj_const;
    std::vector<double> h_dr, h_dc;
    double lam2 = 1, eta0 = 1, omega0 = 1;
    double setup_ms = 0;
    void get_transpose(int* cp, int* ci, double* acx);
    void iterate(int precision, long long iters, double* x, double* y, double* xavg,
                 double* yavg, double* axc, double* st6);
    void evaluate(const double* x, const double* y, double* out6);
    // start point of the following solves (original units, caller's
    // numbering; NULLs clear it)
    void set_start(const double* x0, const double* y0);
    void fetch_host_data();
    void spmv(int transpose, int precision, const double* x, double* y);
    // matrix-free dual repair on the device (any m): original units, caller's
    // numbering; certified when pinf, prow and a finite gap are <= tol.
    // out6 = pinf, dinf, gap, op, od, prow of (x, y).
    bool repair_device(const double* x, const double* y_it, double col_tol, double tol, double* y,
                       double* out6);

   private:
    int device_ = 0;
    cudaStream_t st_ = nullptr;
    Arena ar_;
    // matrix (scaled in place at setup)
    int *ap_, *ai_, *cp_, *ci_;
    double *ax_, *acx_;
    float *ax32_, *acx32_;
    int *ap4_ = nullptr, *ai4_ = nullptr;  // A padded to rows of 4k entries (FP32 copy)
    float* ax4_ = nullptr;
    Sched sA_, sAT_;
    Sched sRA_, sRAT_;  // default schedules (setup passes, cluster path)
    // warp schedules of A and A^T for every kTuneEntries value; sA_ / sAT_
    // are one of them (kLaneEntries unless the autotuner chose otherwise)
    Sched candA_[kTuneCount], candAT_[kTuneCount];
    int cap_ctas_A_ = 0, cap_ctas_AT_ = 0;  // largest launch width of the candidates
    int ia_ = 2, iat_ = 2;                  // candidates in use as sA_ / sAT_ (8 entries)
    int occ_[2] = {3, 3};                   // FP64 attempts: CTAs per SM of k_dual (A), k_primal (A^T)
    int choice_[2][2] = {{-1, -1}, {-1, -1}};  // autotuned (A, A^T) per FP32 / FP64
    int choice_occ_[2] = {3, 3};            // autotuned FP64 occupancy (A, A^T)
    float tune_us_[2][2][kTuneCount][2] = {};  // per attempt-kernel launch, us (occupancy 3, 4)
    void use_sched(int ia, int iat);
    template <typename T> void tune();
    template <typename T> void attempt_args(const Vecs& v, PrimalArgs<T>& pa, DualArgs<T>& da);
    double *dr_, *dc_;
    double* idr_;  // 1 / dr, for the KKT kernels
    double* idc_;  // 1 / dc, for the KKT kernels
    Vecs base_{};
    // device numbering: new index -> original (pr_, pc_) and inverses
    std::vector<int> pr_, pc_, ipr_, ipc_;
    std::vector<double> hp_dr_, hp_dc_;  // scaling in device numbering
    std::vector<double> start_x_, start_y_;  // scaled start point, device numbering (or empty)
    void to_dev_order(const double* in, double* out, bool rows) const;
    void to_user_order(const double* in, double* out, bool rows) const;
    // workspace
    Work<double> w64_{};
    Work<float> w32_{};
    bool have64_ = false, have32_ = false;
    DevCtl* ctl_ = nullptr;
    DevCtl* h_ctl_ = nullptr;      // pinned mirror
    DevMetrics* met_ = nullptr;    // device [2]
    DevMetrics* h_met_ = nullptr;  // pinned mirror [2]
    double* kkt_part_ = nullptr;
    double* kkt_ax_ = nullptr;     // device [2m]: A~ x~ of the KKT candidates
    double* kkt_aty_ = nullptr;    // device [2n]: A~^T y~ of the KKT candidates
    double* red_part_ = nullptr;
    double* scal_ = nullptr;       // device scalars
    double* h_scal_ = nullptr;     // pinned
    unsigned int* ticket_ = nullptr;
    int* flag_ = nullptr;
    double* tmp_n_ = nullptr;      // FP64 scratch vectors
    double* tmp_n2_ = nullptr;
    double* tmp_m_ = nullptr;
    double* tmp_m2_ = nullptr;
    int red_blocks_ = 0;
    std::map<GraphKey, cudaGraphExec_t> graphs_;
    std::chrono::steady_clock::time_point t0_;
    cudaEvent_t ev_[4] = {nullptr, nullptr, nullptr, nullptr};
    double attempt_ms_ = 0;   // accumulated time of attempt launches
    static constexpr int kFac = 512;  // step-factor table entries
    double* fac_ = nullptr;   // device (1 - k^-0.3, 1 + k^-0.6) table
    double* h_fac_ = nullptr; // pinned staging
    void* h_pin_ = nullptr;   // the pinned block holding every host mirror
    double* h_rep_ = nullptr; // pinned mirror of the dual repair's scalars
    long long fac_base_ = 0;  // iteration index of table entry 0 (0: empty)
    long long launches_ = 0;  // kernel launches of the current solve

    template <typename T> Work<T>& work();
    template <typename T> Csr<T> csrA() const;
    template <typename T> Csr<T> csrAT() const;
    template <typename T> void ensure_work();
    template <typename T> void launch_attempts(int count, const Vecs& v, bool graphs);
    // launch widths of the attempt kernels and one attempt's two launches at
    // the occupancies in use
    template <typename T> int grid_primal() const;
    template <typename T> int grid_dual() const;
    template <typename T> void launch_primal(const PrimalArgs<T>& pa);
    template <typename T> void launch_dual(const DualArgs<T>& da);
    template <typename T> void enqueue_attempt(const PrimalArgs<T>& pa, const DualArgs<T>& da) {
        launch_primal<T>(pa);
        launch_dual<T>(da);
    }
    template <typename T> void run_until_stop(const Vecs& v, bool graphs, LoopOut& out);
    template <typename T> void kkt(const Vecs& v, const T* x0, const T* y0, const T* x1,
                                   const T* y1, int ncand);
    template <typename T> void spmv_dev(bool transpose, const T* x, T* y);
    template <typename T> LoopOut loop(const Vecs& v, const LoopOpts& o);
    template <typename T> void fetch_scaled(const T* src, int len, double* dst);
    template <typename T> void unscale_cols(const T* xs, const Vecs& v, double* host_out);
    // anchored (FP32 + FP64 refinement) iterations
    void emit_repaired(const LoopOut& out, igaos_pdhg_result& r, double* x, double* y);
    // infeasibility certificates from the change between restart points
    // (0: none, 1: dual ray, 2: primal ray; the ray in out.ry / out.rx)
    template <typename T> int ray_check(bool anch, int p, LoopOut& out);
    std::vector<double> h_c_, h_cl_, h_cu_, h_rmin_, h_rmax_;  // original units, device order
    template <typename T>
    bool try_repair(const Vecs& v, int p, bool anch, const DevMetrics& ma, const DevMetrics* inc,
                    double tol, int verbosity, long long k, LoopOut& out);
    // matrix-free dual repair (device path; csrc/repair_dev.cuh)
    struct RepBufs {
        double *d, *r, *q, *step, *nrm2, *xs;  // n
        signed char* sgn;
        unsigned char *inj, *rm;  // inner columns (n), movable rows (m)
        double *y, *z, *t, *p, *ybest, *ys;    // m
        double* s;                             // CGLS scalars (16)
        double* h;                             // pinned mirror of s
    };
    RepBufs rep_{};
    bool have_rep_ = false;
    // dynamic shared memory of the cluster attempt kernel for FP32 / FP64
    // (0: that precision uses the grid-wide kernels)
    int small_bytes_[2] = {0, 0};
    void ensure_rep();
    void rep_sum(const double* v, const double* w, const unsigned char* mask, int len, double* out);
    void rep_cgls(int iters, double rtol);
    bool repair_dev(const double* xs, const double* ys_it, double col_tol, double tol,
                    int verbosity, DevMetrics& mt);
    Anchor anc_{};
    Vecs av_{};
    bool have_anchor_ = false;
    void ensure_anchor();
    void anchor_data();                                // av_ from (xh, yh)
    void anchor_zero(int p);                           // deltas of slot p := 0
    void anchor_full(int p);                           // xf/yf := anchor + deltas
    void anchor_to(const double* x, const double* y);  // new anchor + its data
    void upload_ctl();
    void download_ctl();
    double elapsed() const;
    void setup_scaling();
    int scaling_ = IGAOS_PDHG_SCALING_RUIZ;  // igaos_pdhg_options.scaling
    // FP32 / FP64 products stream the matrix with an L2 evict-first policy
    // (Csr::stream): set when that precision's attempt working set exceeds L2
    int stream_[2] = {0, 0};
    void power_iteration();
    void solve_refine(const igaos_pdhg_options& o, igaos_pdhg_result& r, double* x, double* y);
};

}  // namespace igx
