// Host engine of the GB300 PDHG LP solver. Mirrors the control flow of the
// reference engine (IGAOS src/pdhg/pdhg.cu:457-1156) with the per-iteration
// work moved onto the device (kernels.cuh) and replayed from CUDA graphs.
#include "engine.hpp"
#include "kernels.cuh"
#include "repair_dev.cuh"
#include "cluster.cuh"
#include "certificate.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>
#include <type_traits>

namespace igx {

static const double kInf = std::numeric_limits<double>::infinity();

void cuda_check(cudaError_t e, const char* what, int line) {
    if (e == cudaSuccess) return;
    char buf[400];
    std::snprintf(buf, sizeof(buf), "CUDA error in PDHG engine: %s (%s, line %d)",
                  cudaGetErrorString(e), what, line);
    throw CudaError(e == cudaErrorMemoryAllocation ? IGAOS_PDHG_ERR_NOMEM : IGAOS_PDHG_ERR_CUDA,
                    buf);
}

Arena::~Arena() {
    for (void* p : ptrs_) cudaFree(p);
}

void* Arena::raw(size_t bytes) {
    void* p = nullptr;
    bytes = (bytes + 255) & ~size_t(255);
    CU(cudaMalloc(&p, bytes));
    ptrs_.push_back(p);
    total_ += bytes;
    return p;
}

// ------------------------------------------------- permutation + schedule
std::vector<int> length_order(const int* ptr, int rows) {
    // counting sort by decreasing length, stable within a length
    int maxlen = 0;
    for (int r = 0; r < rows; ++r) maxlen = std::max(maxlen, ptr[r + 1] - ptr[r]);
    std::vector<int> start(maxlen + 2, 0);
    for (int r = 0; r < rows; ++r) ++start[maxlen - (ptr[r + 1] - ptr[r]) + 1];
    for (int k = 0; k <= maxlen; ++k) start[k + 1] += start[k];
    std::vector<int> ord(rows);
    for (int r = 0; r < rows; ++r) ord[start[maxlen - (ptr[r + 1] - ptr[r])]++] = r;
    return ord;
}

void build_warps(const int* ptr, int rows, std::vector<int>& wrow, std::vector<unsigned char>& wlg,
                 int entries) {
    wrow.assign(1, 0);
    wlg.clear();
    int r = 0;
    while (r < rows) {
        const int len = ptr[r + 1] - ptr[r];
        int lg = 0;
        while (lg < 5 && (1 << lg) * entries < len) ++lg;
        r = std::min(rows, r + (32 >> lg));
        wrow.push_back(r);
        wlg.push_back((unsigned char)lg);
    }
}

// Whether one cluster of the attempt kernel with `bytes` of dynamic shared
// memory can be resident on this device (else the grid-wide kernels serve).
static bool cluster_fits(bool f64, int bytes) {
    const void* fn = f64 ? (const void*)k_attempts_cluster<double> : (const void*)k_attempts_cluster<float>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kSmallCluster);
    cfg.blockDim = dim3(kSmallThreads);
    cfg.dynamicSmemBytes = bytes;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return clusters > 0;
}

// Per-rank staged entries and row-pointer slots of a schedule for the cluster
// attempt kernel (rank r's warps take items r * kSmallWarps + wi + k *
// kSmallCluster * kSmallWarps); false when a warp would hold more than
// kSmallItems items.
static bool small_share(const int* ptr, int rows, std::vector<long long>& ent,
                        std::vector<long long>& slots) {
    // a warp item holds at most 32 rows: more rows than that many items hold
    // cannot fit (no need to build the schedule to know)
    if ((long long)rows > 32LL * kSmallCluster * kSmallWarps * kSmallItems) return false;
    std::vector<int> wr;
    std::vector<unsigned char> wl;
    build_warps(ptr, rows, wr, wl);
    const int nw = (int)wl.size(), stride = kSmallCluster * kSmallWarps;
    if (nw > stride * kSmallItems) return false;
    ent.assign(kSmallCluster, 0);
    slots.assign(kSmallCluster, 0);
    for (int w = 0; w < nw; ++w) {
        const int r = (w % stride) / kSmallWarps;
        ent[r] += ptr[wr[w + 1]] - ptr[wr[w]];
        slots[r] += wr[w + 1] - wr[w] + 1;
    }
    return true;
}

// Launch width: enough CTAs for every warp item, capped at what stays
// resident (6 CTAs of 256 threads per SM at <= 40 registers); the kernels
// grid-stride over the items.
static Sched upload_sched(Arena& ar, const int* ptr, int rows, int resident_ctas,
                          int entries) {
    std::vector<int> wr;
    std::vector<unsigned char> wl;
    build_warps(ptr, rows, wr, wl, entries);
    Sched s;
    s.entries = entries;
    s.nwarps = (int)wl.size();
    s.ctas = std::max(1, std::min(resident_ctas, (s.nwarps + kWarps - 1) / kWarps));
    s.ctas64 = std::max(1, std::min(s.ctas, resident_ctas / kHotCtasPerSm * HotCtas<double>::value));
    s.ctas64w = std::max(1, std::min(s.ctas, resident_ctas / kHotCtasPerSm * 4));
    s.row = ar.alloc<int>(wr.size());
    s.lg = ar.alloc<unsigned char>(wl.size());
    CU(cudaMemcpy(s.row, wr.data(), sizeof(int) * wr.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(s.lg, wl.data(), wl.size(), cudaMemcpyHostToDevice));
    return s;
}

// CSR of the row-permuted matrix with renumbered indices; each row keeps its
// entries in their original order (the same summation order).
// The entries are gathered by the host's threads over row ranges of equal
// size (the output does not depend on the split).
// Row pointers of a CSR structure padded for 16-byte loads: row r gets
// [P4[r], P4[r+1]), its length rounded up to a multiple of 4 (k_pad4 fills
// the slots on the device). Left empty when the pads would exceed max_extra
// entries.
static void pad4_layout(const int* P, int rows, long long max_extra, std::vector<int>& P4) {
    P4.assign(rows + 1, 0);
    for (int r = 0; r < rows; ++r) P4[r + 1] = P4[r] + ((P[r + 1] - P[r] + 3) & ~3);
    if ((long long)P4[rows] - P[rows] > max_extra) P4.clear();
}

static void permute_csr(int rows, const int* ptr, const int* idx, const double* val,
                        const std::vector<int>& rnew2old, const std::vector<int>& iold2new,
                        std::vector<int>& P, std::unique_ptr<int[]>& I,
                        std::unique_ptr<double[]>& V) {
    P.assign(rows + 1, 0);
    for (int r = 0; r < rows; ++r) {
        const int o = rnew2old[r];
        P[r + 1] = P[r] + (ptr[o + 1] - ptr[o]);
    }
    const long long nnz = P[rows];
    I.reset(new int[std::max<long long>(1, nnz)]);
    V.reset(new double[std::max<long long>(1, nnz)]);
    auto fill = [&](int r0, int r1) {
        for (int r = r0; r < r1; ++r) {
            const int o = rnew2old[r];
            int q = P[r];
            for (int p = ptr[o]; p < ptr[o + 1]; ++p, ++q) {
                I[q] = iold2new[idx[p]];
                V[q] = val[p];
            }
        }
    };
    const int nt = nnz < (1 << 20) ? 1
                                   : (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    if (nt == 1) {
        fill(0, rows);
        return;
    }
    std::vector<std::thread> pool;
    int r0 = 0;
    for (int t = 1; t <= nt; ++t) {
        const long long target = nnz * t / nt;
        const int r1 = t == nt ? rows
                               : (int)(std::lower_bound(P.begin(), P.end(), (int)target) - P.begin());
        const int hi = std::max(r0, std::min(rows, r1));
        pool.emplace_back(fill, r0, hi);
        r0 = hi;
    }
    for (auto& th : pool) th.join();
}

static std::vector<int> inverse(const std::vector<int>& p) {
    std::vector<int> q(p.size());
    for (size_t i = 0; i < p.size(); ++i) q[p[i]] = (int)i;
    return q;
}

#ifndef IGX_SETUP_TIMES
#define IGX_SETUP_TIMES 0
#endif
// IGX_PAD4=0 compiles out the padded FP32 copy of A (16-byte loads).
// A^T is not padded: on the multicommodity LP (3-entry columns) the third
// more bytes cost more than the fewer loads saved (FP32 attempt 67.6 ->
// 69.3 us; 200k x 500k LP 53.9 -> 54.2 us).
#ifndef IGX_PAD4
#define IGX_PAD4 1
#endif

static int grid_for(long long n, int per_block = kThreads, int cap = 152 * 16) {
    long long g = (n + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// ------------------------------------------------------------------ setup
Engine::Engine(int m_, int n_, long long nnz_, const int* ap, const int* ai, const double* ax,
               const int* cp, const int* ci, const double* acx, const double* c,
               const double* cl, const double* cu, const double* rmin, const double* rmax,
               double obj_const_, int device, int scaling)
    : m(m_), n(n_), nnz(nnz_), obj_const(obj_const_), scaling_(scaling) {
    auto t_setup = std::chrono::steady_clock::now();
    auto t_mark = t_setup;
    // IGX_SETUP_TIMES=1 builds print the setup's phases (stream synchronised)
    auto mark = [&](const char* what) {
#if IGX_SETUP_TIMES
        CU(cudaStreamSynchronize(st_));
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[pdhg-gb300 setup] %-28s %8.2f ms\n", what,
                     std::chrono::duration<double, std::milli>(now - t_mark).count());
        t_mark = now;
#else
        (void)what;
        (void)t_mark;
#endif
    };
    if (device >= 0) CU(cudaSetDevice(device));
    CU(cudaGetDevice(&device_));
    CU(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    for (auto& e : ev_) CU(cudaEventCreate(&e));
    // Length-sorted numbering of rows and columns (the warp schedule needs
    // rows of similar length next to each other). Everything on the device
    // lives in this numbering; the API permutes at its edges.
    pr_ = length_order(ap, m);
    pc_ = length_order(cp, n);
    ipr_ = inverse(pr_);
    ipc_ = inverse(pc_);
    mark("stream, orderings");
    {
        std::vector<int> P;
        std::unique_ptr<int[]> I;
        std::unique_ptr<double[]> V;
        ap_ = ar_.alloc<int>(m + 1);
        ai_ = ar_.alloc<int>(nnz);
        ax_ = ar_.alloc<double>(nnz);
        cp_ = ar_.alloc<int>(n + 1);
        ci_ = ar_.alloc<int>(nnz);
        acx_ = ar_.alloc<double>(nnz);
        ax32_ = ar_.alloc<float>(nnz);
        acx32_ = ar_.alloc<float>(nnz);
        permute_csr(m, ap, ai, ax, pr_, ipc_, P, I, V);
        CU(cudaMemcpy(ap_, P.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(ai_, I.get(), sizeof(int) * nnz, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(ax_, V.get(), sizeof(double) * nnz, cudaMemcpyHostToDevice));
        int sms = 0;
        CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
        const int resident = std::max(1, sms) * kHotCtasPerSm;
        sRA_ = upload_sched(ar_, P.data(), m, resident, kLaneEntries);
        for (int c = 0; c < kTuneCount; ++c) {
            candA_[c] = upload_sched(ar_, P.data(), m, resident, kTuneEntries[c]);
            if (kTuneEntries[c] == kLaneEntries) sA_ = candA_[c];
            cap_ctas_A_ = std::max(cap_ctas_A_, candA_[c].ctas);
        }
        std::vector<long long> ent_a, slot_a, ent_at, slot_at;
        bool fit = small_share(P.data(), m, ent_a, slot_a);
        // FP32 copy of A with every row padded to a multiple of 4 entries
        // (16-byte aligned rows, pads: value 0 and the row's first index) for
        // 16-byte vector loads (lane_products); built below when the LP runs
        // on the grid-wide kernels and the pads add at most nnz / 8 entries
        std::vector<int> P4;
        if (IGX_PAD4) pad4_layout(P.data(), m, nnz / 8, P4);
        mark("A: permute, upload, schedules");
        permute_csr(n, cp, ci, acx, pc_, ipr_, P, I, V);
        CU(cudaMemcpy(cp_, P.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(ci_, I.get(), sizeof(int) * nnz, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(acx_, V.get(), sizeof(double) * nnz, cudaMemcpyHostToDevice));
        sRAT_ = upload_sched(ar_, P.data(), n, resident, kLaneEntries);
        for (int c = 0; c < kTuneCount; ++c) {
            candAT_[c] = upload_sched(ar_, P.data(), n, resident, kTuneEntries[c]);
            if (kTuneEntries[c] == kLaneEntries) sAT_ = candAT_[c];
            cap_ctas_AT_ = std::max(cap_ctas_AT_, candAT_[c].ctas);
        }
        fit = small_share(P.data(), n, ent_at, slot_at) && fit;
        // small LPs: the attempts of a chunk in one thread-block cluster with
        // the LP staged in its shared memory (cluster.cuh) when the largest
        // rank's share fits. FP32 only by default: on the 2,000 x 5,000 LP an
        // FP32 attempt takes 7.9 us there against 12.1 us on the grid-wide
        // kernels, an FP64 attempt 17.9 us against 17.3 us (FP64 arithmetic
        // on 8 SMs). IGAOS_PDHG_CLUSTER=0: never; =all: FP64 too.
        const char* e = std::getenv("IGAOS_PDHG_CLUSTER");
        const bool allow = !(e && std::strcmp(e, "0") == 0);
        const bool with64 = e && std::strcmp(e, "all") == 0;
        if (allow && fit) {
            for (int k = 0; k < (with64 ? 2 : 1); ++k) {
                const int sz = k ? 8 : 4;
                size_t worst = 0;
                for (int r = 0; r < kSmallCluster; ++r)
                    worst = std::max(worst, small_smem_bytes(m, n,
                                                             SmallLayout{ent_at[r], slot_at[r], ent_a[r],
                                                                         slot_a[r]},
                                                             sz));
                if (worst <= kSmallSmemMax && cluster_fits(k == 1, (int)worst))
                    small_bytes_[k] = (int)worst;
            }
        }
        // the cluster path stages A by its unpadded row pointers: no padded
        // copy for LPs it runs
        if (!P4.empty() && small_bytes_[0] == 0) {
            ap4_ = ar_.alloc<int>(m + 1);
            ai4_ = ar_.alloc<int>((size_t)P4[m]);
            ax4_ = ar_.alloc<float>((size_t)P4[m]);
            CU(cudaMemcpy(ap4_, P4.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice));
        }
        mark("A^T: permute, upload, sched.");
    }
    // vectors
    auto vec = [&](const double* h, const std::vector<int>& perm) {
        std::vector<double> t(perm.size());
        for (size_t i = 0; i < perm.size(); ++i) t[i] = h[perm[i]];
        double* d = ar_.alloc<double>(t.size());
        CU(cudaMemcpy(d, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice));
        return d;
    };
    base_.c = vec(c, pc_);
    base_.cl = vec(cl, pc_);
    base_.cu = vec(cu, pc_);
    base_.rmin = vec(rmin, pr_);
    base_.rmax = vec(rmax, pr_);
    base_.cmax = 0.0;
    for (int j = 0; j < n; ++j) base_.cmax = std::max(base_.cmax, std::fabs(c[j]));
    base_.lob = ar_.alloc<double>(n);
    base_.hib = ar_.alloc<double>(n);
    k_bands<<<grid_for(n), kThreads, 0, st_>>>(n, base_.cl, base_.cu, base_.lob, base_.hib);
    CU(cudaGetLastError());
    base_.sc = ar_.alloc<double>(n);
    base_.scl = ar_.alloc<double>(n);
    base_.scu = ar_.alloc<double>(n);
    base_.srmin = ar_.alloc<double>(m);
    base_.srmax = ar_.alloc<double>(m);
    base_.fc = ar_.alloc<float>(n);
    base_.fcl = ar_.alloc<float>(n);
    base_.fcu = ar_.alloc<float>(n);
    base_.frmin = ar_.alloc<float>(m);
    base_.frmax = ar_.alloc<float>(m);
    dr_ = ar_.alloc<double>(m);
    dc_ = ar_.alloc<double>(n);
    idr_ = ar_.alloc<double>(m);
    idc_ = ar_.alloc<double>(n);
    // control + scratch
    ctl_ = ar_.alloc<DevCtl>(1);
    met_ = ar_.alloc<DevMetrics>(2);
    CU(cudaMemsetAsync(ctl_, 0, sizeof(DevCtl), st_));
    {  // one pinned block for every host mirror (a pinned allocation costs ~1 ms)
        const size_t o_met = (sizeof(DevCtl) + 63) & ~(size_t)63;
        const size_t o_scal = o_met + ((2 * sizeof(DevMetrics) + 63) & ~(size_t)63);
        const size_t o_fac = o_scal + 16 * sizeof(double);
        const size_t o_rep = o_fac + 2 * kFac * sizeof(double);
        CU(cudaMallocHost(&h_pin_, o_rep + 16 * sizeof(double)));
        char* b = static_cast<char*>(h_pin_);
        h_ctl_ = reinterpret_cast<DevCtl*>(b);
        h_met_ = reinterpret_cast<DevMetrics*>(b + o_met);
        h_scal_ = reinterpret_cast<double*>(b + o_scal);
        h_fac_ = reinterpret_cast<double*>(b + o_fac);
        h_rep_ = reinterpret_cast<double*>(b + o_rep);
    }
    fac_ = ar_.alloc<double>(2 * kFac);
    std::memset(h_ctl_, 0, sizeof(DevCtl));
    red_blocks_ = grid_for(std::max(m, n), kThreads, 152 * 4);
    const int kkt_blocks = std::max(std::max(cap_ctas_A_, cap_ctas_AT_), red_blocks_);
    kkt_part_ = ar_.alloc<double>((size_t)2 * kkt_blocks * 8);
    kkt_ax_ = ar_.alloc<double>((size_t)2 * m);
    kkt_aty_ = ar_.alloc<double>((size_t)2 * n);
    red_part_ = ar_.alloc<double>((size_t)2 * red_blocks_ + 8);
    scal_ = ar_.alloc<double>(16);
    ticket_ = ar_.alloc<unsigned int>(4);
    flag_ = ar_.alloc<int>(4);
    CU(cudaMemsetAsync(ticket_, 0, 4 * sizeof(unsigned int), st_));
    tmp_n_ = ar_.alloc<double>(n);
    tmp_n2_ = ar_.alloc<double>(n);
    tmp_m_ = ar_.alloc<double>(m);
    tmp_m2_ = ar_.alloc<double>(m);

    // matrices streamed with an L2 evict-first policy when the attempt's
    // working set (matrix in both orientations, pointers, nine vectors per
    // side) exceeds L2; IGAOS_PDHG_L2_STREAM=0/1 overrides (measurement)
    {
        int l2 = 0;
        CU(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device_));
        for (int k = 0; k < 2; ++k) {
            const long long s = k ? 8 : 4;
            const long long ws = 2 * nnz * (s + 4) + 4LL * (m + n + 2) + 9 * s * (m + n);
            stream_[k] = ws > (long long)l2 ? 1 : 0;
        }
        if (const char* e = std::getenv("IGAOS_PDHG_L2_STREAM")) stream_[0] = stream_[1] = std::atoi(e) ? 1 : 0;
    }
    mark("vectors, scratch");
    setup_scaling();
    mark("scaling");
    power_iteration();
    mark("power iteration");
    // eta0, omega0 (src/pdhg/pdhg.cu:642-663), from the scaled cost and
    // row bounds, in the reference's summation order.
    eta0 = 1.2 / std::sqrt(lam2);
    omega0 = 1.0;
    {
        double cn = 0.0, qn = 0.0;
        for (int j = 0; j < n; ++j) {
            const double s = c[j] * h_dc[j] / 1.0;
            cn += s * s;
        }
        for (int i = 0; i < m; ++i) {
            const double hi = rmax[i] / h_dr[i], lo = rmin[i] / h_dr[i];
            const double q = std::isfinite(hi) ? hi : (std::isfinite(lo) ? lo : 0.0);
            qn += q * q;
        }
        if (cn > 1e-24 && qn > 1e-24) omega0 = std::clamp(std::sqrt(cn / qn), 0.3, 3.0);
    }
    CU(cudaStreamSynchronize(st_));
    setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                         t_setup).count();
}

Engine::~Engine() {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    for (auto& e : ev_)
        if (e) cudaEventDestroy(e);
    if (h_pin_) cudaFreeHost(h_pin_);
    if (st_) cudaStreamDestroy(st_);
}

// Ruiz equilibration (src/pdhg/pdhg.cu:472-492) and the scaled problem
// (:499-513), all on the device, bit-identical to the host loops.
void Engine::setup_scaling() {
    const int gr = grid_for((long long)m * 32), gc = grid_for((long long)n * 32);
    const int gr_full = (int)(((long long)m * 32 + kThreads - 1) / kThreads);
    const int gc_full = (int)(((long long)n * 32 + kThreads - 1) / kThreads);
    (void)gr;
    (void)gc;
    k_fill<<<grid_for(m), kThreads, 0, st_>>>(m, 1.0, dr_);
    k_fill<<<grid_for(n), kThreads, 0, st_>>>(n, 1.0, dc_);
    for (int sweep = 0; sweep < 10; ++sweep) {
        k_ruiz_rows<<<sRA_.ctas, kThreads, 0, st_>>>(sRA_.view(), ap_, ai_, ax_, dc_, dr_);
        k_ruiz_cols<<<sRAT_.ctas, kThreads, 0, st_>>>(sRAT_.view(), cp_, ci_, acx_, dr_, dc_);
    }
    if (scaling_ == IGAOS_PDHG_SCALING_RUIZ_PC) {
        k_pc_sums<<<sRA_.ctas, kThreads, 0, st_>>>(sRA_.view(), ap_, ai_, ax_, dr_, dc_, 1, tmp_m_);
        k_pc_sums<<<sRAT_.ctas, kThreads, 0, st_>>>(sRAT_.view(), cp_, ci_, acx_, dr_, dc_, 0,
                                                   tmp_n_);
        k_pc_apply<<<grid_for(m), kThreads, 0, st_>>>(m, tmp_m_, 1, dr_);
        k_pc_apply<<<grid_for(n), kThreads, 0, st_>>>(n, tmp_n_, 0, dc_);
    }
    k_fix_scale<<<grid_for(m), kThreads, 0, st_>>>(m, dr_);
    k_fix_scale<<<grid_for(n), kThreads, 0, st_>>>(n, dc_);
    k_scale_matrix<<<gr_full, kThreads, 0, st_>>>(m, ap_, ai_, ax_, ax32_, dr_, dc_, 1);
    if (ax4_) k_pad4<<<grid_for(m), kThreads, 0, st_>>>(m, ap_, ai_, ax32_, ap4_, ai4_, ax4_);
    k_scale_matrix<<<gc_full, kThreads, 0, st_>>>(n, cp_, ci_, acx_, acx32_, dr_, dc_, 0);
    k_scale_vec<<<grid_for(m), kThreads, 0, st_>>>(m, base_.rmin, dr_, 0, base_.srmin, base_.frmin);
    k_scale_vec<<<grid_for(m), kThreads, 0, st_>>>(m, base_.rmax, dr_, 0, base_.srmax, base_.frmax);
    k_scale_vec<<<grid_for(n), kThreads, 0, st_>>>(n, base_.c, dc_, 1, base_.sc, base_.fc);
    k_scale_vec<<<grid_for(n), kThreads, 0, st_>>>(n, base_.cl, dc_, 0, base_.scl, base_.fcl);
    k_scale_vec<<<grid_for(n), kThreads, 0, st_>>>(n, base_.cu, dc_, 0, base_.scu, base_.fcu);
    k_recip<<<grid_for(m), kThreads, 0, st_>>>(m, dr_, idr_);
    k_recip<<<grid_for(n), kThreads, 0, st_>>>(n, dc_, idc_);
    CU(cudaGetLastError());
    hp_dr_.resize(m);
    hp_dc_.resize(n);
    CU(cudaMemcpyAsync(hp_dr_.data(), dr_, sizeof(double) * m, cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(hp_dc_.data(), dc_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
    h_dr.resize(m);
    h_dc.resize(n);
    to_user_order(hp_dr_.data(), h_dr.data(), true);
    to_user_order(hp_dc_.data(), h_dc.data(), false);
    CU(cudaStreamSynchronize(st_));
}

template <> Csr<double> Engine::csrA<double>() const { return Csr<double>{ap_, ai_, ax_, m, stream_[1]}; }
template <> Csr<double> Engine::csrAT<double>() const { return Csr<double>{cp_, ci_, acx_, n, stream_[1]}; }
template <> Csr<float> Engine::csrA<float>() const {
    return ax4_ ? Csr<float>{ap4_, ai4_, ax4_, m, stream_[0], 1} : Csr<float>{ap_, ai_, ax32_, m, stream_[0]};
}
template <> Csr<float> Engine::csrAT<float>() const { return Csr<float>{cp_, ci_, acx32_, n, stream_[0]}; }

template <typename T>
void Engine::spmv_dev(bool transpose, const T* x, T* y) {
    ++launches_;
    if (transpose)
        k_spmv<T, T><<<sAT_.ctas, kThreads, 0, st_>>>(sAT_.view(), csrAT<T>(), x, y);
    else
        k_spmv<T, T><<<sA_.ctas, kThreads, 0, st_>>>(sA_.view(), csrA<T>(), x, y);
    CU(cudaGetLastError());
}

// lambda ~ ||A~||_2^2 by 30 power iterations (src/pdhg/pdhg.cu:605-631),
// norms and normalisation kept on the device.
void Engine::power_iteration() {
    double* v = tmp_n_;
    double* w = tmp_n2_;
    double* tm = tmp_m_;
    k_fill<<<grid_for(n), kThreads, 0, st_>>>(n, 1.0 / std::sqrt((double)n), v);
    CU(cudaMemsetAsync(flag_, 0, sizeof(int), st_));
    for (int it = 0; it < 30; ++it) {
        spmv_dev<double>(false, v, tm);
        spmv_dev<double>(true, tm, w);
        k_sumsq<<<red_blocks_, kThreads, 0, st_>>>(NormArgs{w, n, red_part_, scal_, ticket_ + 1}, 1);
        k_power_normalise<<<grid_for(n), kThreads, 0, st_>>>(n, w, v, scal_, flag_);
    }
    spmv_dev<double>(false, v, tm);
    k_sumsq<<<red_blocks_, kThreads, 0, st_>>>(NormArgs{tm, m, red_part_, scal_ + 1, ticket_ + 1}, 1);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(h_scal_, scal_, 2 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
    const double na = h_scal_[1];
    lam2 = na * na;
    if (!(lam2 > 0) || !std::isfinite(lam2)) lam2 = 1.0;
}

// -------------------------------------------------------------- workspace
template <> Work<double>& Engine::work<double>() { return w64_; }
template <> Work<float>& Engine::work<float>() { return w32_; }

template <typename T>
void Engine::ensure_work() {
    bool& have = std::is_same<T, double>::value ? have64_ : have32_;
    if (have) return;
    Work<T>& w = work<T>();
    for (int s = 0; s < 2; ++s) {
        w.x[s] = ar_.alloc<T>(n);
        w.xavg[s] = ar_.alloc<T>(n);
        w.y[s] = ar_.alloc<T>(m);
        w.yavg[s] = ar_.alloc<T>(m);
        w.axc[s] = ar_.alloc<T>(m);
    }
    w.xbar = ar_.alloc<T>(n);
    w.xb = ar_.alloc<T>(n);
    w.pesx = ar_.alloc<T>(n);
    w.yb = ar_.alloc<T>(m);
    w.pesy = ar_.alloc<T>(m);
    w.part_p = ar_.alloc<double>(std::max(cap_ctas_AT_, kSmallCluster));
    w.part_d = ar_.alloc<double>(2 * (size_t)std::max(cap_ctas_A_, kSmallCluster));
    have = true;
}

template <typename T> struct VecSel;
template <> struct VecSel<double> {
    static const double* c(const Vecs& v) { return v.sc; }
    static const double* l(const Vecs& v) { return v.scl; }
    static const double* u(const Vecs& v) { return v.scu; }
    static const double* rl(const Vecs& v) { return v.srmin; }
    static const double* ru(const Vecs& v) { return v.srmax; }
    static const double* yh(const Vecs&) { return nullptr; }
};
template <> struct VecSel<float> {
    static const float* c(const Vecs& v) { return v.fc; }
    static const float* l(const Vecs& v) { return v.fcl; }
    static const float* u(const Vecs& v) { return v.fcu; }
    static const float* rl(const Vecs& v) { return v.frmin; }
    static const float* ru(const Vecs& v) { return v.frmax; }
    static const float* yh(const Vecs& v) { return v.fyhat; }
};

// Arguments of the two attempt kernels on the current schedules.
template <typename T>
void Engine::attempt_args(const Vecs& v, PrimalArgs<T>& pa, DualArgs<T>& da) {
    Work<T>& w = work<T>();
    pa.ws = sAT_.view();
    pa.AT = csrAT<T>();
    pa.y[0] = w.y[0];
    pa.y[1] = w.y[1];
    pa.c = VecSel<T>::c(v);
    pa.lo = VecSel<T>::l(v);
    pa.hi = VecSel<T>::u(v);
    for (int s = 0; s < 2; ++s) {
        pa.x[s] = w.x[s];
        pa.xavg[s] = w.xavg[s];
    }
    pa.xbar = w.xbar;
    pa.part = reinterpret_cast<Acc<T>*>(w.part_p);
    pa.ctl = ctl_;
    da.ws = sA_.view();
    da.A = csrA<T>();
    da.xbar = w.xbar;
    da.rmin = VecSel<T>::rl(v);
    da.rmax = VecSel<T>::ru(v);
    for (int s = 0; s < 2; ++s) {
        da.y[s] = w.y[s];
        da.axc[s] = w.axc[s];
        da.yavg[s] = w.yavg[s];
    }
    da.part = reinterpret_cast<Acc<T>*>(w.part_d);
    da.part_primal = reinterpret_cast<const Acc<T>*>(w.part_p);
    da.n_primal = grid_primal<T>();
    da.yhat = VecSel<T>::yh(v);
    da.fac = fac_;
    da.n_fac = kFac;
    da.ctl = ctl_;
}

template <typename T>
int Engine::grid_primal() const {
    if constexpr (std::is_same<T, double>::value) return occ_[1] == 4 ? sAT_.ctas64w : sAT_.ctas64;
    return sAT_.ctas;
}
template <typename T>
int Engine::grid_dual() const {
    if constexpr (std::is_same<T, double>::value) return occ_[0] == 4 ? sA_.ctas64w : sA_.ctas64;
    return sA_.ctas;
}
template <typename T>
void Engine::launch_primal(const PrimalArgs<T>& pa) {
    const int gp = grid_primal<T>();
    if constexpr (std::is_same<T, double>::value) {
        if (occ_[1] == 4) k_primal<double, 4><<<gp, kThreads, 0, st_>>>(pa);
        else k_primal<double, 3><<<gp, kThreads, 0, st_>>>(pa);
    } else {
        k_primal<T><<<gp, kThreads, 0, st_>>>(pa);
    }
}
template <typename T>
void Engine::launch_dual(const DualArgs<T>& da) {
    const int gd = grid_dual<T>();
    if constexpr (std::is_same<T, double>::value) {
        if (occ_[0] == 4) k_dual<double, 4><<<gd, kThreads, 0, st_>>>(da);
        else k_dual<double, 3><<<gd, kThreads, 0, st_>>>(da);
    } else {
        k_dual<T><<<gd, kThreads, 0, st_>>>(da);
    }
}

// Enqueues `count` line-search attempts (2 launches each). With graphs the
// sequence is captured once per (precision, count, vector set, schedules and
// occupancies in use) and replayed.
template <typename T>
void Engine::launch_attempts(int count, const Vecs& v, bool graphs) {
    PrimalArgs<T> pa;
    DualArgs<T> da;
    attempt_args<T>(v, pa, da);
    if (const int sb = small_bytes_[std::is_same<T, double>::value ? 1 : 0]) {
        // one cluster runs the whole chunk with the LP in shared memory (it
        // stages the default schedule)
        pa.ws = sRAT_.view();
        da.ws = sRA_.view();
        ++launches_;
        CU(cudaFuncSetAttribute(k_attempts_cluster<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb));
        k_attempts_cluster<T><<<kSmallCluster, kSmallThreads, sb, st_>>>(pa, da, m, n, count);
        CU(cudaGetLastError());
        return;
    }
    launches_ += 2LL * count;
    auto enqueue = [&](int cnt) {
        for (int a = 0; a < cnt; ++a) enqueue_attempt<T>(pa, da);
    };
    if (!graphs) {
        enqueue(count);
        CU(cudaGetLastError());
        return;
    }
    // key: precision, attempt count, vector set
    const GraphKey key{std::is_same<T, double>::value ? 1 : 2, count,
                       (uintptr_t)VecSel<T>::c(v),
                       4 * (kTuneCount * ia_ + iat_) + 2 * (occ_[0] == 4) + (occ_[1] == 4)};
    auto it = graphs_.find(key);
    if (it == graphs_.end()) {
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        enqueue(count);
        CU(cudaStreamEndCapture(st_, &g));
        cudaGraphExec_t ge;
        CU(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
        it = graphs_.emplace(key, ge).first;
    }
    CU(cudaGraphLaunch(it->second, st_));
}

void Engine::use_sched(int ia, int iat) {
    ia_ = ia;
    iat_ = iat;
    sA_ = candA_[ia];
    sAT_ = candAT_[iat];
}

// Autotuner (igaos_pdhg_options.schedule = IGAOS_PDHG_SCHEDULE_AUTOTUNE).
// For each orientation the attempt kernel of precision T is timed on every
// candidate warp schedule -- kTuneEntries entries per lane, which sets how
// many lanes share a row of each length and how many rows a warp item holds
// -- with CUDA events over kReps launches after a warming one, and the
// fastest is kept for this problem and precision (later solves reuse it).
// The probe runs on zero iterates under a control block that never stops;
// the solve loop resets both afterwards. Small LPs that run on the
// thread-block cluster path keep their staged layout.
template <typename T>
void Engine::tune() {
    const int pi = std::is_same<T, double>::value ? 1 : 0;
    if (choice_[pi][0] >= 0) return;
    int def = 0;
    for (int c = 0; c < kTuneCount; ++c)
        if (kTuneEntries[c] == kLaneEntries) def = c;
    if (small_bytes_[pi]) {
        choice_[pi][0] = choice_[pi][1] = def;
        return;
    }
    ensure_work<T>();
    Work<T>& w = work<T>();
    for (int s = 0; s < 2; ++s) {
        CU(cudaMemsetAsync(w.x[s], 0, sizeof(T) * n, st_));
        CU(cudaMemsetAsync(w.xavg[s], 0, sizeof(T) * n, st_));
        CU(cudaMemsetAsync(w.y[s], 0, sizeof(T) * m, st_));
        CU(cudaMemsetAsync(w.yavg[s], 0, sizeof(T) * m, st_));
        CU(cudaMemsetAsync(w.axc[s], 0, sizeof(T) * m, st_));
    }
    CU(cudaMemsetAsync(w.xbar, 0, sizeof(T) * n, st_));
    std::memset(h_ctl_, 0, sizeof(DevCtl));
    h_ctl_->eta = eta0;
    h_ctl_->omega = omega0;
    h_ctl_->k = 1;
    h_ctl_->k_stop = std::numeric_limits<long long>::max() / 2;
    upload_ctl();
    constexpr int kReps = 8;  // launches per timing (after a warming one)
    cudaEvent_t e[3];
    for (auto& ev : e) CU(cudaEventCreate(&ev));
    // FP64 attempts are also timed at 4 resident CTAs per SM (their 64
    // registers hold without spills): more warps hide more gather latency on
    // some LPs (multicommodity LP: 140 -> 134 us), fewer cost the FP64-pipe
    // bound ones less (200k x 500k LP: 89 against 91 us)
    const int nocc = pi == 1 ? 2 : 1;
    for (int c = 0; c < kTuneCount; ++c)
        for (int oi = 0; oi < nocc; ++oi) {
            use_sched(c, c);
            occ_[0] = occ_[1] = oi ? 4 : 3;
            PrimalArgs<T> pa;
            DualArgs<T> da;
            attempt_args<T>(base_, pa, da);
            enqueue_attempt<T>(pa, da);
            CU(cudaEventRecord(e[0], st_));
            for (int r = 0; r < kReps; ++r) launch_primal<T>(pa);
            CU(cudaEventRecord(e[1], st_));
            for (int r = 0; r < kReps; ++r) launch_dual<T>(da);
            CU(cudaEventRecord(e[2], st_));
            CU(cudaGetLastError());
            CU(cudaEventSynchronize(e[2]));
            float tp = 0.f, td = 0.f;
            CU(cudaEventElapsedTime(&tp, e[0], e[1]));
            CU(cudaEventElapsedTime(&td, e[1], e[2]));
            tune_us_[pi][1][c][oi] = 1e3f * tp / kReps;
            tune_us_[pi][0][c][oi] = 1e3f * td / kReps;
            launches_ += 2 * (kReps + 1);
        }
    for (auto& ev : e) cudaEventDestroy(ev);
    occ_[0] = occ_[1] = 3;
    for (int o = 0; o < 2; ++o) {
        int best = def, bo = 0;
        for (int c = 0; c < kTuneCount; ++c)
            for (int oi = 0; oi < nocc; ++oi)
                if (tune_us_[pi][o][c][oi] < tune_us_[pi][o][best][bo]) {
                    best = c;
                    bo = oi;
                }
        choice_[pi][o] = best;
        if (pi == 1) choice_occ_[o] = bo ? 4 : 3;
    }
}

void Engine::upload_ctl() {
    // Step-growth factors 1 - k^-0.3 and 1 + k^-0.6 for the iterations the
    // next launches can reach, computed with std::pow exactly as the
    // reference does on the host (src/pdhg/pdhg.cu:778-782).
    const long long k = h_ctl_->k;
    if (fac_base_ < 1 || k < fac_base_ || h_ctl_->k_stop >= fac_base_ + kFac) {
        fac_base_ = std::max(1LL, k);
        for (int i = 0; i < kFac; ++i) {
            const double kk = (double)(fac_base_ + i);
            h_fac_[2 * i] = 1.0 - std::pow(kk, -0.3);
            h_fac_[2 * i + 1] = 1.0 + std::pow(kk, -0.6);
        }
        CU(cudaMemcpyAsync(fac_, h_fac_, sizeof(double) * 2 * kFac, cudaMemcpyHostToDevice, st_));
    }
    h_ctl_->fac_base = fac_base_;
    ctl_derive(h_ctl_);
    CU(cudaMemcpyAsync(ctl_, h_ctl_, sizeof(DevCtl), cudaMemcpyHostToDevice, st_));
}
void Engine::download_ctl() {
    CU(cudaMemcpyAsync(h_ctl_, ctl_, sizeof(DevCtl), cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
}
double Engine::elapsed() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

// Launch attempts until the device raises `stop` (iteration k_stop accepted
// or NaN). The first batch covers the accepted iterations still needed plus
// the rejections the history predicts; the rest are topped up in small
// batches (a stopped launch is a no-op).
template <typename T>
void Engine::run_until_stop(const Vecs& v, bool graphs, LoopOut& out) {
    for (;;) {
        const long long need = h_ctl_->k_stop - (h_ctl_->k - 1);
        const double rej = h_ctl_->accepted > 0
                               ? (double)(h_ctl_->attempts - h_ctl_->accepted) / h_ctl_->attempts
                               : 0.0;
        long long want = (long long)std::ceil((double)need * (1.0 + 1.2 * rej)) + (rej > 0 ? 1 : 0);
        int cnt = want <= 1 ? 1 : want <= 4 ? 4 : want <= 8 ? 8 : want <= 16 ? 16
                  : want <= 32 ? 32 : want <= 64 ? 64 : want <= 72 ? 72 : want <= 80 ? 80 : 96;
        CU(cudaEventRecord(ev_[2], st_));
        launch_attempts<T>(cnt, v, graphs);
        CU(cudaEventRecord(ev_[3], st_));
        download_ctl();
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, ev_[2], ev_[3]));
        attempt_ms_ += ms;
        if (h_ctl_->stop) break;
    }
    out.attempts = h_ctl_->attempts;
}

template <typename T>
void Engine::kkt(const Vecs& v, const T* x0, const T* y0, const T* x1, const T* y1, int ncand) {
    KktArgs<T> ka;
    ka.x[0] = x0;
    ka.y[0] = y0;
    ka.x[1] = x1;
    ka.y[1] = y1;
    ka.ax[0] = kkt_ax_;
    ka.ax[1] = kkt_ax_ + m;
    ka.aty[0] = kkt_aty_;
    ka.aty[1] = kkt_aty_ + n;
    ka.dr = dr_;
    ka.dc = dc_;
    ka.idr = idr_;
    ka.idc = idc_;
    ka.lob = v.lob;
    ka.hib = v.hib;
    ka.c = v.c;
    ka.cl = v.cl;
    ka.cu = v.cu;
    ka.rmin = v.rmin;
    ka.rmax = v.rmax;
    ka.slo = VecSel<T>::l(v);
    ka.shi = VecSel<T>::u(v);
    ka.cmax = v.cmax;
    ka.part = kkt_part_;
    ka.out = met_;
    ka.ticket = ticket_ + 2;
    launches_ += 4;
    k_kkt_prod<T><<<dim3(sA_.ctas, ncand), kThreads, 0, st_>>>(sA_.view(), csrA<T>(), x0, x1,
                                                              kkt_ax_, kkt_ax_ + m);
    k_kkt_prod<T><<<dim3(sAT_.ctas, ncand), kThreads, 0, st_>>>(sAT_.view(), csrAT<T>(), y0, y1,
                                                               kkt_aty_, kkt_aty_ + n);
    // about four rows (columns) per thread, at most 2 CTAs per SM per candidate
    k_kkt_rows<T><<<dim3(grid_for(m, 4 * kThreads, 152 * 2), ncand), kThreads, 0, st_>>>(ka, m);
    k_kkt_cols<T><<<dim3(grid_for(n, 4 * kThreads, 152 * 2), ncand), kThreads, 0, st_>>>(ka, n, m);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(h_met_, met_, ncand * sizeof(DevMetrics), cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
}

// The reference iteration loop with its 64-iteration checks: termination,
// Dual repair from the solve loop (src/pdhg/pdhg.cu:854-931): candidates are
// the averaged iterate (its x and y) and the incumbent (its x with the
// current y, as the reference takes them), tried when they pass pinf and
// prow, have dinf <= 10 tol and no certified gap; col_tol tiers 1e-6 then
// 1e-1; a repaired pair is accepted on pinf, prow and a finite gap <= tol.
template <typename T>
bool Engine::try_repair(const Vecs& v, int p, bool anch, const DevMetrics& ma,
                        const DevMetrics* inc, double tol, int verbosity, long long k,
                        LoopOut& out) {
    Work<T>& w = work<T>();
    for (int cnd = 1; cnd <= 2; ++cnd) {
        const DevMetrics* t = cnd == 1 ? &ma : inc;
        if (!t) break;
        if (!(t->pinf <= tol && t->prow <= tol && t->dinf <= 10.0 * tol &&
              !(std::isfinite(t->gap) && t->gap <= tol)))
            continue;
        if (verbosity > 1)
            std::fprintf(stderr, "[pdhg-gb300] dual repair @k=%lld candidate %d (pinf %.2e prow %.2e "
                                 "dinf %.2e)\n", k, cnd, t->pinf, t->prow, t->dinf);
        ensure_rep();
        const double *xs, *ys;
        if (anch) {
            xs = cnd == 1 ? anc_.xf[1] : anc_.xb;
            ys = cnd == 1 ? anc_.yf[1] : anc_.yf[0];
        } else if constexpr (std::is_same<T, double>::value) {
            xs = cnd == 1 ? w.xavg[p] : w.xb;
            ys = cnd == 1 ? w.yavg[p] : w.y[p];
        } else {
            k_convert<T, double><<<grid_for(n), kThreads, 0, st_>>>(n, cnd == 1 ? w.xavg[p] : w.xb,
                                                                   rep_.xs);
            k_convert<T, double><<<grid_for(m), kThreads, 0, st_>>>(m, cnd == 1 ? w.yavg[p] : w.y[p],
                                                                   rep_.ys);
            CU(cudaGetLastError());
            xs = rep_.xs;
            ys = rep_.ys;
        }
        for (const double col_tol : {1e-6, 1e-1}) {
            DevMetrics mt{};
            const bool ok = repair_dev(xs, ys, col_tol, tol, verbosity, mt);
            if (verbosity > 1)
                std::fprintf(stderr, "[pdhg-gb300] device dual repair col_tol %.0e: gap %.3e\n",
                             col_tol, ok ? mt.gap : std::numeric_limits<double>::infinity());
            if (!ok) continue;
            std::vector<double> hx(n), hy(m);
            CU(cudaMemcpyAsync(hx.data(), xs, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
            CU(cudaMemcpyAsync(hy.data(), rep_.ybest, sizeof(double) * m, cudaMemcpyDeviceToHost,
                               st_));
            CU(cudaStreamSynchronize(st_));
            out.rx.assign(n, 0.0);
            out.ry.assign(m, 0.0);
            for (int j = 0; j < n; ++j) out.rx[pc_[j]] = hx[j] * hp_dc_[j];
            for (int i = 0; i < m; ++i) out.ry[pr_[i]] = hy[i] / hp_dr_[i];
            out.last = mt;
            out.last_is_avg = cnd == 1;
            out.use_inc = false;
            out.repaired = true;
            out.status = IGAOS_STATUS_NEAR_OPTIMAL;
            return true;
        }
    }
    return false;
}

void Engine::ensure_rep() {
    if (have_rep_) return;
    rep_.d = ar_.alloc<double>(n);
    rep_.r = ar_.alloc<double>(n);
    rep_.q = ar_.alloc<double>(n);
    rep_.step = ar_.alloc<double>(n);
    rep_.nrm2 = ar_.alloc<double>(n);
    rep_.xs = ar_.alloc<double>(n);
    rep_.sgn = ar_.alloc<signed char>(n);
    rep_.inj = ar_.alloc<unsigned char>(n);
    rep_.rm = ar_.alloc<unsigned char>(m);
    rep_.y = ar_.alloc<double>(m);
    rep_.z = ar_.alloc<double>(m);
    rep_.t = ar_.alloc<double>(m);
    rep_.p = ar_.alloc<double>(m);
    rep_.ybest = ar_.alloc<double>(m);
    rep_.ys = ar_.alloc<double>(m);
    rep_.s = ar_.alloc<double>(16);
    rep_.h = h_rep_;
    have_rep_ = true;
}

void Engine::rep_sum(const double* v, const double* w, const unsigned char* mask, int len,
                     double* out) {
    ++launches_;
    k_rep_sum<<<red_blocks_, kThreads, 0, st_>>>(
        RepSum{v, w, mask, len, red_part_, out, ticket_ + 1});
    CU(cudaGetLastError());
}

// CGLS for min ||(A~^T z)_J + d_J||^2 + ridge ||z||^2 from z = 0 over the
// rows k_rep_rowmask frees at the current dual, with r = -d_J already in
// rep_.r and the ridge in s[6]; scalars stay on the device (a converged or
// broken-down iteration turns the rest into no-ops).
void Engine::rep_cgls(int iters, double rtol) {
    RepBufs& b = rep_;
    const int gm = grid_for(m), gn = grid_for(n), gmn = grid_for(std::max(m, n));
    CU(cudaMemsetAsync(b.z, 0, sizeof(double) * m, st_));
    k_rep_rowmask<<<gm, kThreads, 0, st_>>>(m, b.y, base_.rmin, base_.rmax, b.rm);
    spmv_dev<double>(false, b.r, b.t);            // t = P A~ r (r is 0 off J)
    k_rep_grad<<<gm, kThreads, 0, st_>>>(m, b.s, b.z, b.rm, b.t);
    k_rep_dir<<<gm, kThreads, 0, st_>>>(m, b.s, b.t, b.p, 1);
    rep_sum(b.t, b.t, nullptr, m, b.s + 0);        // gamma
    k_rep_cg_init<<<1, 1, 0, st_>>>(b.s);
    for (int k = 0; k < iters; ++k) {
        spmv_dev<double>(true, b.p, b.q);         // q = (A~^T p)_J
        k_rep_mask<<<gn, kThreads, 0, st_>>>(n, b.inj, b.q);
        rep_sum(b.q, b.q, nullptr, n, b.s + 9);    // ||q||^2
        rep_sum(b.p, b.p, nullptr, m, b.s + 11);   // ||p||^2
        k_rep_cg_alpha<<<1, 1, 0, st_>>>(b.s, rtol * rtol);
        k_rep_zr<<<gmn, kThreads, 0, st_>>>(m, n, b.s, b.p, b.z, b.q, b.r);
        spmv_dev<double>(false, b.r, b.t);        // t = A~ r - ridge z
        k_rep_grad<<<gm, kThreads, 0, st_>>>(m, b.s, b.z, b.rm, b.t);
        rep_sum(b.t, b.t, nullptr, m, b.s + 13);   // gamma'
        k_rep_cg_beta<<<1, 1, 0, st_>>>(b.s);
        k_rep_dir<<<gm, kThreads, 0, st_>>>(m, b.s, b.t, b.p, 0);
        launches_ += 7;
    }
    CU(cudaGetLastError());
}

// Matrix-free dual repair (see repair_dev.cuh) of the candidate (xs, ys_it),
// scaled FP64 device vectors in device numbering. On success the certified
// scaled dual is in rep_.ybest and mt holds its metrics.
bool Engine::repair_dev(const double* xs, const double* ys_it, double col_tol, double tol,
                        int verbosity, DevMetrics& mt) {
    ensure_rep();
    RepBufs& b = rep_;
    const int gm = grid_for(m), gn = grid_for(n);
    constexpr int kRounds = 150;  // per anchor
    constexpr int kStall = 40;
    constexpr int kCg = 40;
    constexpr double kCgTol = 1e-10;
    k_rep_cols<<<gn, kThreads, 0, st_>>>(n, cp_, acx_, xs, dc_, base_.cl, base_.cu, col_tol, b.sgn,
                                         b.inj, b.nrm2);
    rep_sum(b.nrm2, nullptr, b.inj, n, b.s + 9);  // trace of A~_J A~_J^T, |J|
    CU(cudaMemcpyAsync(b.h, b.s, 16 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
    const double trace = b.h[9];
    const long long nj = (long long)b.h[10];
    b.h[6] = trace > 0 ? 1e-10 * trace / m : 1e-14;  // ridge (src/pdhg/pdhg.cu:335-337)
    CU(cudaMemcpyAsync(b.s + 6, b.h + 6, sizeof(double), cudaMemcpyHostToDevice, st_));
    double best_gap = std::numeric_limits<double>::infinity();
    bool certified = false;
    for (int anchor = 0; anchor < 2 && !certified; ++anchor) {
        k_rep_start<<<gm, kThreads, 0, st_>>>(m, anchor == 0 ? ys_it : nullptr, base_.rmin,
                                              base_.rmax, b.y);
        bool finite_seen = false;
        for (int it = 0; it < kRounds; ++it) {
            // an anchor whose duals stay uncertifiable (infinite gap) for
            // kStall rounds is abandoned
            if (it == kStall && !finite_seen) break;
            if (nj > 0) {  // onto d_J = 0
                spmv_dev<double>(true, b.y, b.d);
                k_rep_rinit<<<gn, kThreads, 0, st_>>>(n, base_.sc, b.d, b.inj, b.r);
                rep_cgls(kCg, kCgTol);
                k_rep_addz<<<gm, kThreads, 0, st_>>>(m, b.z, b.y);
            }
            // onto the violated sign half-spaces, then the row cone
            spmv_dev<double>(true, b.y, b.d);
            k_rep_sign<<<gn, kThreads, 0, st_>>>(n, base_.sc, b.d, b.sgn, b.nrm2, b.step);
            k_rep_rows<<<gm, kThreads, 0, st_>>>(m, ap_, ai_, ax_, b.step, base_.rmin, base_.rmax,
                                                 b.y);
            launches_ += 5;
            CU(cudaGetLastError());
            kkt<double>(base_, xs, b.y, xs, b.y, 1);
            const DevMetrics t = h_met_[0];
            if (verbosity > 2 && it % 25 == 0)
                std::fprintf(stderr, "[pdhg-gb300] device repair anchor %d round %d: gap %.3e "
                                     "dinf %.3e\n", anchor, it, t.gap, t.dinf);
            finite_seen = finite_seen || std::isfinite(t.gap);
            if (std::isfinite(t.gap) && t.gap < best_gap) {
                best_gap = t.gap;
                mt = t;
                CU(cudaMemcpyAsync(b.ybest, b.y, sizeof(double) * m, cudaMemcpyDeviceToDevice, st_));
                if (t.pinf <= tol && t.prow <= tol && t.gap <= tol) {
                    certified = true;
                    break;
                }
            }
        }
    }
    if (!std::isfinite(best_gap))
        CU(cudaMemcpyAsync(b.ybest, b.y, sizeof(double) * m, cudaMemcpyDeviceToDevice, st_));
    CU(cudaStreamSynchronize(st_));
    return certified;
}

bool Engine::repair_device(const double* x, const double* y_it, double col_tol, double tol,
                           double* y, double* out6) {
    ensure_rep();
    std::vector<double> xs(n), ys(m);
    for (int j = 0; j < n; ++j) xs[j] = x[pc_[j]] / hp_dc_[j];
    for (int i = 0; i < m; ++i) ys[i] = y_it[pr_[i]] * hp_dr_[i];
    CU(cudaMemcpyAsync(rep_.xs, xs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st_));
    CU(cudaMemcpyAsync(rep_.ys, ys.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st_));
    DevMetrics mt{};
    mt.gap = std::numeric_limits<double>::infinity();
    const bool ok = repair_dev(rep_.xs, rep_.ys, col_tol, tol, 0, mt);
    CU(cudaMemcpyAsync(ys.data(), rep_.ybest, sizeof(double) * m, cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
    for (int i = 0; i < m; ++i) y[pr_[i]] = ys[i] / hp_dr_[i];
    kkt<double>(base_, rep_.xs, rep_.ybest, rep_.xs, rep_.ybest, 1);
    const DevMetrics& t = h_met_[0];
    out6[0] = t.pinf;
    out6[1] = t.dinf;
    out6[2] = t.gap;
    out6[3] = t.op;
    out6[4] = t.od;
    out6[5] = t.prow;
    return ok;
}


// Infeasibility certificates (no counterpart in the reference engine): the
// change between consecutive restart points of an LP without a solution
// tends to a ray (the iterates diverge along it), as in PDLP's test on
// iterate differences. The difference and its products are formed on the
// device in FP64; the test itself (certificate.hpp) runs on the host in
// original units.
template <typename T>
int Engine::ray_check(bool anch, int p, LoopOut& out) {
    Work<T>& w = work<T>();
    const int gn = grid_for(n), gm = grid_for(m);
    if (anch) {
        k_ray_diff<double><<<gn, kThreads, 0, st_>>>(n, anc_.xh, anc_.pesx, tmp_n_);
        k_ray_diff<double><<<gm, kThreads, 0, st_>>>(m, anc_.yh, anc_.pesy, tmp_m_);
    } else {
        k_ray_diff<T><<<gn, kThreads, 0, st_>>>(n, w.x[p], w.pesx, tmp_n_);
        k_ray_diff<T><<<gm, kThreads, 0, st_>>>(m, w.y[p], w.pesy, tmp_m_);
    }
    launches_ += 2;
    CU(cudaGetLastError());
    spmv_dev<double>(true, tmp_m_, tmp_n2_);   // A~^T dy~
    spmv_dev<double>(false, tmp_n_, tmp_m2_);  // A~ dx~
    out.spmvs += 2;
    std::vector<double> dx(n), dy(m), aty(n), ax(m);
    CU(cudaMemcpyAsync(dx.data(), tmp_n_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(dy.data(), tmp_m_, sizeof(double) * m, cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(aty.data(), tmp_n2_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(ax.data(), tmp_m2_, sizeof(double) * m, cudaMemcpyDeviceToHost, st_));
    fetch_host_data();
    CU(cudaStreamSynchronize(st_));
    // original units: x = dc x~, y = y~ / dr, A^T y = (A~^T y~) / dc, A x = dr (A~ x~)
    for (int i = 0; i < m; ++i) {
        dy[i] /= hp_dr_[i];
        ax[i] *= hp_dr_[i];
    }
    for (int j = 0; j < n; ++j) {
        dx[j] *= hp_dc_[j];
        aty[j] /= hp_dc_[j];
    }
    std::vector<double> xr(n), yr(m);
    const int kind = ray_certificate(m, n, dx.data(), ax.data(), dy.data(), aty.data(), h_c_.data(),
                                     h_cl_.data(), h_cu_.data(), h_rmin_.data(), h_rmax_.data(),
                                     xr.data(), yr.data());
    if (kind == 1) {
        out.ry.assign(m, 0.0);
        for (int i = 0; i < m; ++i) out.ry[pr_[i]] = yr[i];
    } else if (kind == 2) {
        out.rx.assign(n, 0.0);
        for (int j = 0; j < n; ++j) out.rx[pc_[j]] = xr[j];
    }
    return kind;
}

// incumbent, rollback, restart and primal weight (src/pdhg/pdhg.cu:665-1085).
template <typename T>
LoopOut Engine::loop(const Vecs& v, const LoopOpts& o) {
    ensure_work<T>();
    Work<T>& w = work<T>();
    LoopOut out;
    const size_t nb = sizeof(T) * n, mb = sizeof(T) * m;
    CU(cudaMemsetAsync(w.x[0], 0, nb, st_));
    CU(cudaMemsetAsync(w.xavg[0], 0, nb, st_));
    CU(cudaMemsetAsync(w.y[0], 0, mb, st_));
    CU(cudaMemsetAsync(w.yavg[0], 0, mb, st_));
    CU(cudaMemsetAsync(w.axc[0], 0, mb, st_));
    // anchored FP32 iterations (FP32 + FP64 refinement): start at anchor 0
    const bool anch = v.fyhat != nullptr;
    const bool warm = !start_x_.empty();
    if (anch) {  // the first anchor: the start point, else 0
        if (warm) {
            CU(cudaMemcpyAsync(anc_.xh, start_x_.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st_));
            CU(cudaMemcpyAsync(anc_.yh, start_y_.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st_));
        } else {
            CU(cudaMemsetAsync(anc_.xh, 0, sizeof(double) * n, st_));
            CU(cudaMemsetAsync(anc_.yh, 0, sizeof(double) * m, st_));
        }
        anchor_data();
        out.spmvs += 2;
    } else if (warm) {  // x = xavg = x0, y = yavg = y0, A x committed
        std::vector<T> sx(start_x_.begin(), start_x_.end()), sy(start_y_.begin(), start_y_.end());
        CU(cudaMemcpyAsync(w.x[0], sx.data(), nb, cudaMemcpyHostToDevice, st_));
        CU(cudaMemcpyAsync(w.xavg[0], sx.data(), nb, cudaMemcpyHostToDevice, st_));
        CU(cudaMemcpyAsync(w.y[0], sy.data(), mb, cudaMemcpyHostToDevice, st_));
        CU(cudaMemcpyAsync(w.yavg[0], sy.data(), mb, cudaMemcpyHostToDevice, st_));
        spmv_dev<T>(false, w.x[0], w.axc[0]);
        CU(cudaStreamSynchronize(st_));  // the host vectors go out of scope
        out.spmvs += 1;
    }
    std::memset(h_ctl_, 0, sizeof(DevCtl));
    h_ctl_->eta = o.eta_init;
    h_ctl_->omega = o.omega_init;
    h_ctl_->k = 1;
    const int CHECK = o.check > 0 ? o.check : 64;
    const long long MAXIT = o.maxit;
    h_ctl_->k_stop = std::min<long long>(CHECK, MAXIT);
    upload_ctl();

    double epoch_kkt = -1.0, prev_cand = kInf;
    long long epoch_start = 0, last_rollback = 0;
    long long next_repair = 5000, repair_spacing = 2000;  // src/pdhg/pdhg.cu:741-743
    bool have_pe = false, have_last = false, have_inc = false, perturbed = false;
    int ray_prev = 0;  // certificate kind found at the previous restart
    double inc_op = 0.0;
    DevMetrics inc{};
    out.status = IGAOS_STATUS_ITERATION_LIMIT;
    long long k_done = 0;
    auto passes = [&](const DevMetrics& t) {
        return t.pinf <= o.tol && t.dinf <= o.tol && t.prow <= o.tol && std::isfinite(t.gap) &&
               t.gap <= o.tol;
    };
    while (k_done < MAXIT) {
        run_until_stop<T>(v, o.graphs, out);
        k_done = h_ctl_->k - 1;
        out.spmvs = 2 * h_ctl_->attempts;
        if (h_ctl_->nan_flag) {
            out.numeric_failure = true;
            out.status = IGAOS_STATUS_ERROR;
            break;
        }
        if (k_done % CHECK == 0) {
            ++out.checks;
            const int p = h_ctl_->parity;
            if (o.perturb_at > 0 && k_done >= o.perturb_at && !perturbed) {
                k_add_const<T><<<grid_for(n), kThreads, 0, st_>>>(n, (T)1e6, w.x[p]);
                CU(cudaGetLastError());
                perturbed = true;
            }
            if (anch) {  // FP64 metrics of the full iterates anchor + delta
                anchor_full(p);
                kkt<double>(base_, anc_.xf[0], anc_.yf[0], anc_.xf[1], anc_.yf[1], 2);
            } else {
                kkt<T>(v, w.x[p], w.y[p], w.xavg[p], w.yavg[p], 2);
            }
            const DevMetrics mc = h_met_[0], ma = h_met_[1];
            const double ec = mc.finite ? mc.err : kInf;
            const double ea = ma.finite ? ma.err : kInf;
            out.last = (ec <= ea) ? mc : ma;
            out.last_is_avg = (ea < ec);
            have_last = true;
            if (o.verbosity > 0 && k_done % (CHECK * 40) == 0)
                std::fprintf(stderr, "[pdhg-gb300] k=%lld pinf=%.3e dinf=%.3e gap=%.3e\n", k_done,
                             out.last.pinf, out.last.dinf, out.last.gap);
            if (passes(mc)) { out.last = mc; out.last_is_avg = false; out.status = IGAOS_STATUS_NEAR_OPTIMAL; break; }
            if (passes(ma)) { out.last = ma; out.last_is_avg = true; out.status = IGAOS_STATUS_NEAR_OPTIMAL; break; }
            // dual repair of a converged candidate whose dual bound is not
            // certified (src/pdhg/pdhg.cu:854-931), on the reference's schedule
            if (k_done >= 5000 && k_done >= next_repair) {
                next_repair = k_done + repair_spacing;
                repair_spacing = std::min(repair_spacing * 3, 30000LL);
                if (try_repair<T>(v, p, anch, ma, have_inc ? &inc : nullptr, o.tol, o.verbosity,
                                  k_done, out))
                    break;
            }
            // incumbent (src/pdhg/pdhg.cu:937-958)
            int inc_src = -1;
            for (int cnd = 0; cnd < 2; ++cnd) {
                const DevMetrics& t = cnd ? ma : mc;
                if (t.pinf <= 1e-4 && std::isfinite(t.op) && (!have_inc || t.op < inc_op)) {
                    have_inc = true;
                    inc_op = t.op;
                    inc = t;
                    inc_src = cnd;
                }
            }
            if (inc_src >= 0 && anch) {
                CU(cudaMemcpyAsync(anc_.xb, anc_.xf[inc_src], sizeof(double) * n, cudaMemcpyDeviceToDevice, st_));
                CU(cudaMemcpyAsync(anc_.yb, anc_.yf[inc_src], sizeof(double) * m, cudaMemcpyDeviceToDevice, st_));
            } else if (inc_src >= 0) {
                CU(cudaMemcpyAsync(w.xb, inc_src ? w.xavg[p] : w.x[p], nb, cudaMemcpyDeviceToDevice, st_));
                CU(cudaMemcpyAsync(w.yb, inc_src ? w.yavg[p] : w.y[p], mb, cudaMemcpyDeviceToDevice, st_));
            }
            // rollback (src/pdhg/pdhg.cu:965-988)
            if (mc.pinf >= 0.5 && have_inc && k_done - last_rollback > 2000) {
                if (anch) {
                    anchor_to(anc_.xb, anc_.yb);
                    anchor_zero(p);
                    ++out.anchors;
                    out.spmvs += 2;
                } else {
                    CU(cudaMemcpyAsync(w.x[p], w.xb, nb, cudaMemcpyDeviceToDevice, st_));
                    CU(cudaMemcpyAsync(w.y[p], w.yb, mb, cudaMemcpyDeviceToDevice, st_));
                    CU(cudaMemcpyAsync(w.xavg[p], w.xb, nb, cudaMemcpyDeviceToDevice, st_));
                    CU(cudaMemcpyAsync(w.yavg[p], w.yb, mb, cudaMemcpyDeviceToDevice, st_));
                    spmv_dev<T>(false, w.x[p], w.axc[p]);
                    ++out.spmvs;
                }
                h_ctl_->eta = std::min(h_ctl_->eta, 0.5 * o.eta0);
                h_ctl_->hn = 0;
                epoch_start = k_done;
                epoch_kkt = -1.0;
                prev_cand = kInf;
                last_rollback = k_done;
                ++out.rollbacks;
                if (o.verbosity > 1)
                    std::fprintf(stderr, "[pdhg-gb300] rollback @k=%lld to the incumbent, eta %.17g\n",
                                 k_done, h_ctl_->eta);
            }
            // restart + primal weight (src/pdhg/pdhg.cu:1001-1075)
            const double cand = std::min(ec, ea);
            if (epoch_kkt < 0.0) {
                epoch_kkt = cand;
                prev_cand = cand;
            }
            const long long t_epoch = k_done - epoch_start;
            const bool restart_now =
                (std::isfinite(cand) && std::isfinite(epoch_kkt) && epoch_kkt > 0.0 &&
                 (cand <= 0.2 * epoch_kkt ||
                  (cand <= 0.8 * epoch_kkt && std::isfinite(prev_cand) && cand > prev_cand))) ||
                (double)t_epoch >= 0.36 * (double)k_done;
            prev_cand = cand;
            if (restart_now) {
                ++out.restarts;
                if (anch) {
                    // the restart point becomes the new FP64 anchor (A x and
                    // the deltas restart from zero, residual data refreshed)
                    anchor_to(anc_.xf[ea < ec ? 1 : 0], anc_.yf[ea < ec ? 1 : 0]);
                    anchor_zero(p);
                    ++out.anchors;
                    out.spmvs += 2;
                } else {
                    if (ea < ec) {
                        CU(cudaMemcpyAsync(w.x[p], w.xavg[p], nb, cudaMemcpyDeviceToDevice, st_));
                        CU(cudaMemcpyAsync(w.y[p], w.yavg[p], mb, cudaMemcpyDeviceToDevice, st_));
                    }
                    CU(cudaMemcpyAsync(w.xavg[p], w.x[p], nb, cudaMemcpyDeviceToDevice, st_));
                    CU(cudaMemcpyAsync(w.yavg[p], w.y[p], mb, cudaMemcpyDeviceToDevice, st_));
                    spmv_dev<T>(false, w.x[p], w.axc[p]);
                    ++out.spmvs;
                }
                h_ctl_->hn = 0;
                epoch_start = k_done;
                epoch_kkt = cand;
                prev_cand = kInf;
                if (have_pe) {
                    ++launches_;
                    if (anch)
                        k_diffnorms<double><<<red_blocks_, kThreads, 0, st_>>>(
                            n, anc_.xh, anc_.pesx, m, anc_.yh, anc_.pesy, red_part_, scal_, ticket_ + 1);
                    else
                        k_diffnorms<T><<<red_blocks_, kThreads, 0, st_>>>(
                            n, w.x[p], w.pesx, m, w.y[p], w.pesy, red_part_, scal_, ticket_ + 1);
                    CU(cudaGetLastError());
                    CU(cudaMemcpyAsync(h_scal_, scal_, 2 * sizeof(double), cudaMemcpyDeviceToHost, st_));
                    CU(cudaStreamSynchronize(st_));
                    const double dxn = h_scal_[0], dyn = h_scal_[1];
                    if (dxn > 1e-24 && dyn > 1e-24) {
                        const double om = std::sqrt(h_ctl_->omega * std::sqrt(dyn / dxn));
                        if (std::isfinite(om) && om > 0.0)
                            h_ctl_->omega = std::clamp(om, 1e-6, 1e6);
                    }
                    if (o.detect_inf) {
                        // the same kind of certificate at two consecutive restarts
                        const int kind = ray_check<T>(anch, p, out);
                        if (kind != 0 && kind == ray_prev) {
                            out.ray = kind;
                            out.status = kind == 1 ? IGAOS_STATUS_INFEASIBLE : IGAOS_STATUS_UNBOUNDED;
                            if (o.verbosity > 0)
                                std::fprintf(stderr, "[pdhg-gb300] %s certificate @k=%lld\n",
                                             kind == 1 ? "dual-ray (infeasible)" : "primal-ray (unbounded)",
                                             k_done);
                            break;
                        }
                        ray_prev = kind;
                    }
                }
                have_pe = true;
                if (anch) {
                    CU(cudaMemcpyAsync(anc_.pesx, anc_.xh, sizeof(double) * n, cudaMemcpyDeviceToDevice, st_));
                    CU(cudaMemcpyAsync(anc_.pesy, anc_.yh, sizeof(double) * m, cudaMemcpyDeviceToDevice, st_));
                } else {
                    CU(cudaMemcpyAsync(w.pesx, w.x[p], nb, cudaMemcpyDeviceToDevice, st_));
                    CU(cudaMemcpyAsync(w.pesy, w.y[p], mb, cudaMemcpyDeviceToDevice, st_));
                }
                if (o.verbosity > 1)
                    std::fprintf(stderr, "[pdhg-gb300] restart @k=%lld t=%lld r=%.3e eta=%.3e om=%.3e\n",
                                 k_done, t_epoch, cand, h_ctl_->eta, h_ctl_->omega);
            }
            out.spmvs += 4;
            if (elapsed() > o.deadline) {
                out.status = IGAOS_STATUS_TIME_LIMIT;
                break;
            }
        }
        if (k_done >= MAXIT) break;
        h_ctl_->k_stop = std::min<long long>((k_done / CHECK + 1) * CHECK, MAXIT);
        h_ctl_->stop = 0;
        upload_ctl();
    }
    out.iters = k_done;
    out.attempts = h_ctl_->attempts;
    out.eta = h_ctl_->eta;
    out.omega = h_ctl_->omega;
    out.parity = h_ctl_->parity;
    if (!have_last && !out.numeric_failure) {
        // no check ran (fewer than CHECK iterations): evaluate the last iterate
        const int p = h_ctl_->parity;
        if (anch) {
            anchor_full(p);
            kkt<double>(base_, anc_.xf[0], anc_.yf[0], anc_.xf[0], anc_.yf[0], 1);
        } else {
            kkt<T>(v, w.x[p], w.y[p], w.x[p], w.y[p], 1);
        }
        out.last = h_met_[0];
        out.last_is_avg = false;
        out.spmvs += 2;
    }
    auto certified = [&](const DevMetrics& t) {
        return t.pinf <= o.tol && t.prow <= o.tol && std::isfinite(t.gap) && t.gap <= o.tol;
    };
    if (out.status == IGAOS_STATUS_ITERATION_LIMIT && certified(out.last))
        out.status = IGAOS_STATUS_NEAR_OPTIMAL;
    if (!certified(out.last) && have_inc && inc.pinf <= o.tol && std::isfinite(inc.op) &&
        (inc.op < out.last.op || out.last.pinf > o.tol)) {
        out.last = inc;
        out.use_inc = true;
        out.last_is_avg = false;
    }
    return out;
}

template <typename T>
void Engine::fetch_scaled(const T* src, int len, double* dst) {
    if (std::is_same<T, double>::value) {
        CU(cudaMemcpyAsync(dst, src, sizeof(double) * len, cudaMemcpyDeviceToHost, st_));
    } else {
        double* staging = (len == n) ? tmp_n_ : tmp_m_;
        k_convert<T, double><<<grid_for(len), kThreads, 0, st_>>>(len, src, staging);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(dst, staging, sizeof(double) * len, cudaMemcpyDeviceToHost, st_));
    }
    CU(cudaStreamSynchronize(st_));
}

// Original-unit x (device numbering) of a scaled iterate, with the FP32
// at-bound rule of unscale_x.
template <typename T>
void Engine::unscale_cols(const T* xs, const Vecs& v, double* host_out) {
    k_unscale_cols<T><<<grid_for(n), kThreads, 0, st_>>>(n, xs, VecSel<T>::l(v), VecSel<T>::u(v),
                                                          dc_, v.cl, v.cu, tmp_n_);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(host_out, tmp_n_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
}

// -------------------------------------------------------------------- solve
static void fill_message(igaos_pdhg_result& r, const char* s) {
    std::snprintf(r.message, sizeof(r.message), "%s", s);
}

void Engine::solve(const igaos_pdhg_options& o, igaos_pdhg_result& r, double* x, double* y) {
    std::memset(&r, 0, sizeof(r));
    r.status = IGAOS_STATUS_ERROR;
    r.setup_time_ms = setup_ms;
    // warp schedules: the fixed default, or the autotuner's choice for the
    // attempt kernels' precision (timed once per handle and precision)
    const int pi = o.precision == IGAOS_PDHG_FP64 ? 1 : 0;
    int def = 0;
    for (int c = 0; c < kTuneCount; ++c)
        if (kTuneEntries[c] == kLaneEntries) def = c;
    if (o.schedule == IGAOS_PDHG_SCHEDULE_AUTOTUNE) {
        if (pi) tune<double>();
        else tune<float>();
        use_sched(choice_[pi][0], choice_[pi][1]);
        occ_[0] = pi ? choice_occ_[0] : 3;
        occ_[1] = pi ? choice_occ_[1] : 3;
        if (o.verbosity > 0) {
            const char* name[2] = {"A", "A^T"};
            const int chosen[2] = {sA_.entries, sAT_.entries};
            for (int q = 0; q < 2; ++q) {
                std::fprintf(stderr, "[pdhg-gb300] autotuned %s (us per launch at 2/4/8/16/32 entries "
                                     "per lane):", name[q]);
                for (int oi = 0; oi < (pi ? 2 : 1); ++oi) {
                    std::fprintf(stderr, " %d CTAs/SM", oi ? 4 : (pi ? 3 : kHotCtasPerSm));
                    for (int c = 0; c < kTuneCount; ++c)
                        std::fprintf(stderr, "%s%.1f", c ? "/" : " ", tune_us_[pi][q][c][oi]);
                }
                std::fprintf(stderr, " -> %d entries, %d CTAs/SM\n", chosen[q],
                             pi ? occ_[q] : kHotCtasPerSm);
            }
        }
    } else {
        use_sched(def, def);
        occ_[0] = occ_[1] = 3;
    }
    if (o.precision == IGAOS_PDHG_FP32_REFINE) {
        solve_refine(o, r, x, y);
        return;
    }
    t0_ = std::chrono::steady_clock::now();
    attempt_ms_ = 0;
    launches_ = 0;
    CU(cudaEventRecord(ev_[0], st_));
    LoopOpts lo;
    lo.tol = o.tolerance;
    const bool finite_tl = o.time_limit_s > 0 && o.time_limit_s < 1e6;
    lo.deadline = o.time_limit_s;  // checked at every KKT check, as the reference (:1077-1083)
    lo.maxit = finite_tl ? 20000000LL : (long long)o.max_iterations;
    lo.check = o.check_period > 0 ? o.check_period : 64;
    lo.verbosity = o.verbosity;
    lo.graphs = o.use_graphs != 0;
    lo.detect_inf = o.detect_infeasibility != 0;
    lo.eta_init = eta0;
    lo.eta0 = eta0;
    lo.omega_init = omega0;
    if (const char* e = std::getenv("IGAOS_PDHG_PERTURB_AT")) lo.perturb_at = std::atoll(e);
    LoopOut out;
    std::vector<double> hx(n), hy(m);
    if (o.precision == IGAOS_PDHG_FP32) {
        out = loop<float>(base_, lo);
        Work<float>& w = w32_;
        const int p = out.parity;
        const float* fx = out.use_inc ? w.xb : (out.last_is_avg ? w.xavg[p] : w.x[p]);
        const float* fy = out.use_inc ? w.yb : (out.last_is_avg ? w.yavg[p] : w.y[p]);
        unscale_cols<float>(fx, base_, hx.data());
        fetch_scaled<float>(fy, m, hy.data());
    } else {
        out = loop<double>(base_, lo);
        Work<double>& w = w64_;
        const int p = out.parity;
        const double* fx = out.use_inc ? w.xb : (out.last_is_avg ? w.xavg[p] : w.x[p]);
        const double* fy = out.use_inc ? w.yb : (out.last_is_avg ? w.yavg[p] : w.y[p]);
        unscale_cols<double>(fx, base_, hx.data());
        fetch_scaled<double>(fy, m, hy.data());
    }
    const double secs = elapsed();
    CU(cudaEventRecord(ev_[1], st_));
    CU(cudaEventSynchronize(ev_[1]));
    {
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
        r.device_time_ms = ms;
        r.attempt_time_ms = attempt_ms_;
        r.launches = launches_;
    }
    r.status = out.status;
    r.objective = out.last.op + obj_const;
    r.pinf = out.last.pinf;
    r.dinf = out.last.dinf;
    r.rel_gap = out.last.gap;
    r.prow = out.last.prow;
    r.iterations = out.iters;
    r.attempts = out.attempts;
    r.kkt_checks = out.checks;
    r.restarts = out.restarts;
    r.rollbacks = out.rollbacks;
    r.entries_a = sA_.entries;
    r.entries_at = sAT_.entries;
    r.kkt_passes = out.spmvs / 2;
    r.solve_time_ms = secs * 1000.0;
    if (out.numeric_failure) {
        r.error_code = IGAOS_PDHG_ERR_NUMERIC;
        fill_message(r, "numerical failure: NaN/Inf in the PDHG iterates");
    } else if (out.status == IGAOS_STATUS_NEAR_OPTIMAL) {
        fill_message(r, "converged: residuals + duality gap @tol");
    } else if (out.status == IGAOS_STATUS_TIME_LIMIT) {
        fill_message(r, "wall-clock budget exhausted");
    } else {
        fill_message(r, out.last.pinf <= o.tolerance && out.last.dinf <= o.tolerance
                            ? "iteration cap: residuals @tol but gap not certified (dual bound "
                              "-inf or > tol)"
                            : "iteration cap reached before tolerance");
    }
    // unscale (x = dc x~, y = y~/dr) and return to the caller's numbering
    if (x)
        for (int j = 0; j < n; ++j) x[pc_[j]] = hx[j];  // already in original units
    if (y)
        for (int i = 0; i < m; ++i) y[pr_[i]] = 1.0 * hy[i] / hp_dr_[i];
    emit_repaired(out, r, x, y);
}

// A pair certified by dual repair is the answer as the repair produced it;
// an infeasibility certificate replaces y (dual ray) or x (primal ray).
void Engine::emit_repaired(const LoopOut& out, igaos_pdhg_result& r, double* x, double* y) {
    if (out.ray == 1) {
        fill_message(r, "primal infeasible: a dual ray (change between restart points) certifies it; "
                        "y holds the ray");
        if (y) std::memcpy(y, out.ry.data(), sizeof(double) * m);
        return;
    }
    if (out.ray == 2) {
        fill_message(r, "dual infeasible (unbounded if feasible): a primal ray certifies it; x holds "
                        "the ray");
        if (x) std::memcpy(x, out.rx.data(), sizeof(double) * n);
        return;
    }
    if (!out.repaired) return;
    fill_message(r, "converged: residuals @tol, duality gap certified by dual repair");
    if (x) std::memcpy(x, out.rx.data(), sizeof(double) * n);
    if (y) std::memcpy(y, out.ry.data(), sizeof(double) * m);
}

// ------------------------------------------------------- numbering helpers
void Engine::to_dev_order(const double* in, double* out, bool rows) const {
    const std::vector<int>& p = rows ? pr_ : pc_;
    for (size_t i = 0; i < p.size(); ++i) out[i] = in[p[i]];
}
void Engine::to_user_order(const double* in, double* out, bool rows) const {
    const std::vector<int>& p = rows ? pr_ : pc_;
    for (size_t i = 0; i < p.size(); ++i) out[p[i]] = in[i];
}

// --------------------------------------------------------- inspection API
// The device CSC is in device numbering; map it back: column j of the
// caller is device column ipc_[j], row indices through pr_, entries of a
// column keep their order.
void Engine::get_transpose(int* cp, int* ci, double* acx) {
    std::vector<int> dcp(n + 1), dci(nnz);
    std::vector<double> dacx(nnz);
    CU(cudaMemcpyAsync(dcp.data(), cp_, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(dci.data(), ci_, sizeof(int) * nnz, cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(dacx.data(), acx_, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st_));
    CU(cudaStreamSynchronize(st_));
    cp[0] = 0;
    for (int j = 0; j < n; ++j) {
        const int d = ipc_[j];
        const int len = dcp[d + 1] - dcp[d];
        for (int k = 0; k < len; ++k) {
            ci[cp[j] + k] = pr_[dci[dcp[d] + k]];
            acx[cp[j] + k] = dacx[dcp[d] + k];
        }
        cp[j + 1] = cp[j] + len;
    }
}

template <typename T>
static void upload_as(cudaStream_t st, T* dst, const double* src, int len, double* staging) {
    if (std::is_same<T, double>::value) {
        CU(cudaMemcpyAsync(dst, src, sizeof(double) * len, cudaMemcpyHostToDevice, st));
    } else {
        CU(cudaMemcpyAsync(staging, src, sizeof(double) * len, cudaMemcpyHostToDevice, st));
        k_convert<double, T><<<grid_for(len), kThreads, 0, st>>>(len, staging, dst);
        CU(cudaGetLastError());
    }
    CU(cudaStreamSynchronize(st));
}

void Engine::iterate(int precision, long long iters, double* x, double* y, double* xavg,
                     double* yavg, double* axc, double* st6) {
    std::vector<double> bn(n), bm(m);
    auto up = [&](auto* dst, const double* src, bool rows) {
        using T = std::remove_pointer_t<decltype(dst)>;
        double* b = rows ? bm.data() : bn.data();
        to_dev_order(src, b, rows);
        upload_as<T>(st_, dst, b, rows ? m : n, rows ? tmp_m_ : tmp_n_);
    };
    auto down = [&](const auto* src, double* dst, bool rows) {
        using T = std::remove_const_t<std::remove_pointer_t<decltype(src)>>;
        double* b = rows ? bm.data() : bn.data();
        fetch_scaled<T>(src, rows ? m : n, b);
        to_user_order(b, dst, rows);
    };
    auto run = [&](auto tag) {
        using T = decltype(tag);
        ensure_work<T>();
        Work<T>& w = work<T>();
        up(w.x[0], x, false);
        up(w.xavg[0], xavg, false);
        up(w.y[0], y, true);
        up(w.yavg[0], yavg, true);
        up(w.axc[0], axc, true);
        std::memset(h_ctl_, 0, sizeof(DevCtl));
        h_ctl_->eta = st6[0];
        h_ctl_->omega = st6[1];
        h_ctl_->k = (long long)st6[2];
        h_ctl_->hn = (long long)st6[3];
        h_ctl_->k_stop = h_ctl_->k + iters - 1;
        upload_ctl();
        LoopOut out;
        if (iters > 0) run_until_stop<T>(base_, false, out);
        else download_ctl();
        const int p = h_ctl_->parity;
        down(w.x[p], x, false);
        down(w.xavg[p], xavg, false);
        down(w.y[p], y, true);
        down(w.yavg[p], yavg, true);
        down(w.axc[p], axc, true);
        st6[0] = h_ctl_->eta;
        st6[1] = h_ctl_->omega;
        st6[2] = (double)h_ctl_->k;
        st6[3] = (double)h_ctl_->hn;
        st6[4] = (double)h_ctl_->attempts;
        st6[5] = (double)p;
    };
    if (precision == IGAOS_PDHG_FP64) run(double());
    else run(float());
}

// Host copies of c, cl, cu, rmin, rmax (original units, device order), once.
void Engine::fetch_host_data() {
    if (!h_c_.empty()) return;
    auto get = [&](const double* d, int len, std::vector<double>& h) {
        h.resize(len);
        CU(cudaMemcpyAsync(h.data(), d, sizeof(double) * len, cudaMemcpyDeviceToHost, st_));
    };
    get(base_.c, n, h_c_);
    get(base_.cl, n, h_cl_);
    get(base_.cu, n, h_cu_);
    get(base_.rmin, m, h_rmin_);
    get(base_.rmax, m, h_rmax_);
}

void Engine::set_start(const double* x0, const double* y0) {
    if (!x0 || !y0) {
        start_x_.clear();
        start_y_.clear();
        return;
    }
    fetch_host_data();
    CU(cudaStreamSynchronize(st_));
    // x~ = clamp(x, cl, cu) / dc, y~ = y dr; non-finite entries start at 0
    start_x_.assign(n, 0.0);
    start_y_.assign(m, 0.0);
    for (int j = 0; j < n; ++j) {
        const double v = std::min(std::max(x0[pc_[j]], h_cl_[j]), h_cu_[j]) / hp_dc_[j];
        start_x_[j] = std::isfinite(v) ? v : 0.0;
    }
    for (int i = 0; i < m; ++i) {
        const double v = y0[pr_[i]] * hp_dr_[i];
        start_y_[i] = std::isfinite(v) ? v : 0.0;
    }
}

void Engine::evaluate(const double* x, const double* y, double* out6) {
    // scaled copies: x~ = x / dc, y~ = y * dr
    std::vector<double> xs(n), ys(m);
    for (int j = 0; j < n; ++j) xs[j] = x[pc_[j]] / hp_dc_[j];
    for (int i = 0; i < m; ++i) ys[i] = y[pr_[i]] * hp_dr_[i];
    CU(cudaMemcpyAsync(tmp_n2_, xs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st_));
    CU(cudaMemcpyAsync(tmp_m2_, ys.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st_));
    kkt<double>(base_, tmp_n2_, tmp_m2_, tmp_n2_, tmp_m2_, 1);
    const DevMetrics& t = h_met_[0];
    out6[0] = t.pinf;
    out6[1] = t.dinf;
    out6[2] = t.gap;
    out6[3] = t.op;
    out6[4] = t.od;
    out6[5] = t.prow;
}

void Engine::spmv(int transpose, int precision, const double* x_user, double* y_user) {
    const int lin = transpose ? m : n, lout = transpose ? n : m;
    std::vector<double> xin(lin), yout(lout);
    to_dev_order(x_user, xin.data(), transpose != 0);
    const double* x = xin.data();
    double* y = yout.data();
    struct Back {
        const Engine* e;
        double* y;
        double* u;
        bool rows;
        ~Back() { e->to_user_order(y, u, rows); }
    } back{this, y, y_user, transpose == 0};
    if (precision == IGAOS_PDHG_FP64) {
        double* dx = transpose ? tmp_m_ : tmp_n_;
        double* dy = transpose ? tmp_n2_ : tmp_m2_;
        CU(cudaMemcpyAsync(dx, x, sizeof(double) * lin, cudaMemcpyHostToDevice, st_));
        spmv_dev<double>(transpose != 0, dx, dy);
        CU(cudaMemcpyAsync(y, dy, sizeof(double) * lout, cudaMemcpyDeviceToHost, st_));
        CU(cudaStreamSynchronize(st_));
    } else {
        ensure_work<float>();
        float* fx = transpose ? w32_.y[0] : w32_.x[0];
        float* fy = transpose ? w32_.x[1] : w32_.y[1];
        upload_as<float>(st_, fx, x, lin, transpose ? tmp_m_ : tmp_n_);
        spmv_dev<float>(transpose != 0, fx, fy);
        k_convert<float, double><<<grid_for(lout), kThreads, 0, st_>>>(lout, fy, transpose ? tmp_n2_ : tmp_m2_);
        CU(cudaMemcpyAsync(y, transpose ? tmp_n2_ : tmp_m2_, sizeof(double) * lout,
                           cudaMemcpyDeviceToHost, st_));
        CU(cudaStreamSynchronize(st_));
    }
}

}  // namespace igx

namespace igx {
// ------------------------------------ FP32 iterations with FP64 refinement
// The reference iteration (line search, averaging, checks, restarts, primal
// weight) on FP32 deltas from an FP64 anchor: every restart (and rollback)
// makes the restart point the new anchor, i.e. restarts PDHG on the residual
// problem seen from it, whose data -- reduced costs c~ + A~^T yh, row bounds
// minus A~ xh, the shifted box -- are formed in FP64 and rounded once. The
// KKT checks, the incumbent and the answer are FP64 on anchor + delta, so the
// attainable accuracy is set by FP64, while every attempt streams FP32.
void Engine::ensure_anchor() {
    if (have_anchor_) return;
    anc_.xh = ar_.alloc<double>(n);
    anc_.yh = ar_.alloc<double>(m);
    for (int s = 0; s < 2; ++s) {
        anc_.xf[s] = ar_.alloc<double>(n);
        anc_.yf[s] = ar_.alloc<double>(m);
    }
    anc_.xb = ar_.alloc<double>(n);
    anc_.yb = ar_.alloc<double>(m);
    anc_.pesx = ar_.alloc<double>(n);
    anc_.pesy = ar_.alloc<double>(m);
    anc_.aty = ar_.alloc<double>(n);
    anc_.ax = ar_.alloc<double>(m);
    av_ = base_;  // original-unit vectors are the base LP's
    av_.fc = ar_.alloc<float>(n);
    av_.fcl = ar_.alloc<float>(n);
    av_.fcu = ar_.alloc<float>(n);
    av_.frmin = ar_.alloc<float>(m);
    av_.frmax = ar_.alloc<float>(m);
    av_.fyhat = ar_.alloc<float>(m);
    have_anchor_ = true;
}

void Engine::anchor_data() {
    spmv_dev<double>(false, anc_.xh, anc_.ax);
    spmv_dev<double>(true, anc_.yh, anc_.aty);
    k_anchor_cols<<<grid_for(n), kThreads, 0, st_>>>(n, base_.sc, base_.scl, base_.scu, anc_.aty,
                                                     anc_.xh, av_.fc, av_.fcl, av_.fcu);
    k_anchor_rows<<<grid_for(m), kThreads, 0, st_>>>(m, base_.srmin, base_.srmax, anc_.ax,
                                                     anc_.yh, av_.frmin, av_.frmax, av_.fyhat);
    launches_ += 2;
    CU(cudaGetLastError());
}

void Engine::anchor_zero(int p) {
    Work<float>& w = w32_;
    CU(cudaMemsetAsync(w.x[p], 0, sizeof(float) * n, st_));
    CU(cudaMemsetAsync(w.xavg[p], 0, sizeof(float) * n, st_));
    CU(cudaMemsetAsync(w.y[p], 0, sizeof(float) * m, st_));
    CU(cudaMemsetAsync(w.yavg[p], 0, sizeof(float) * m, st_));
    CU(cudaMemsetAsync(w.axc[p], 0, sizeof(float) * m, st_));
}

void Engine::anchor_full(int p) {
    Work<float>& w = w32_;
    const int gn = grid_for(n), gm = grid_for(m);
    k_anchor_full_cols<<<gn, kThreads, 0, st_>>>(n, anc_.xh, w.x[p], av_.fcl, av_.fcu, base_.scl,
                                                 base_.scu, anc_.xf[0]);
    k_anchor_full_cols<<<gn, kThreads, 0, st_>>>(n, anc_.xh, w.xavg[p], av_.fcl, av_.fcu,
                                                 base_.scl, base_.scu, anc_.xf[1]);
    k_anchor_full_rows<<<gm, kThreads, 0, st_>>>(m, anc_.yh, w.y[p], anc_.yf[0]);
    k_anchor_full_rows<<<gm, kThreads, 0, st_>>>(m, anc_.yh, w.yavg[p], anc_.yf[1]);
    launches_ += 4;
    CU(cudaGetLastError());
}

void Engine::anchor_to(const double* x, const double* y) {
    if (x != anc_.xh)
        CU(cudaMemcpyAsync(anc_.xh, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st_));
    if (y != anc_.yh)
        CU(cudaMemcpyAsync(anc_.yh, y, sizeof(double) * m, cudaMemcpyDeviceToDevice, st_));
    anchor_data();
}

void Engine::solve_refine(const igaos_pdhg_options& o, igaos_pdhg_result& r, double* x, double* y) {
    t0_ = std::chrono::steady_clock::now();
    attempt_ms_ = 0;
    launches_ = 0;
    CU(cudaEventRecord(ev_[0], st_));
    ensure_work<float>();
    ensure_anchor();
    LoopOpts lo;
    lo.tol = o.tolerance;
    const bool finite_tl = o.time_limit_s > 0 && o.time_limit_s < 1e6;
    lo.deadline = o.time_limit_s;
    lo.maxit = finite_tl ? 20000000LL : (long long)o.max_iterations;
    lo.check = o.check_period > 0 ? o.check_period : 64;
    lo.verbosity = o.verbosity;
    lo.graphs = o.use_graphs != 0;
    lo.detect_inf = o.detect_infeasibility != 0;
    lo.eta_init = eta0;
    lo.eta0 = eta0;
    lo.omega_init = omega0;
    if (const char* e = std::getenv("IGAOS_PDHG_PERTURB_AT")) lo.perturb_at = std::atoll(e);
    LoopOut out = loop<float>(av_, lo);
    // the answer: incumbent, or anchor + delta of the current / averaged iterate
    const double *fx, *fy;
    if (out.use_inc) {
        fx = anc_.xb;
        fy = anc_.yb;
    } else {
        anchor_full(out.parity);
        fx = anc_.xf[out.last_is_avg ? 1 : 0];
        fy = anc_.yf[out.last_is_avg ? 1 : 0];
    }
    std::vector<double> hx(n), hy(m);
    CU(cudaMemcpyAsync(hx.data(), fx, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
    CU(cudaMemcpyAsync(hy.data(), fy, sizeof(double) * m, cudaMemcpyDeviceToHost, st_));
    CU(cudaEventRecord(ev_[1], st_));
    CU(cudaEventSynchronize(ev_[1]));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
    r.device_time_ms = ms;
    r.attempt_time_ms = attempt_ms_;
    r.launches = launches_;
    r.solve_time_ms = elapsed() * 1000.0;
    r.status = out.status;
    r.objective = out.last.op + obj_const;
    r.pinf = out.last.pinf;
    r.dinf = out.last.dinf;
    r.rel_gap = out.last.gap;
    r.prow = out.last.prow;
    r.iterations = out.iters;
    r.attempts = out.attempts;
    r.kkt_checks = out.checks;
    r.restarts = out.restarts;
    r.rollbacks = out.rollbacks;
    r.entries_a = sA_.entries;
    r.entries_at = sAT_.entries;
    r.kkt_passes = out.spmvs / 2;
    r.refinements = (int)out.anchors;
    if (out.numeric_failure) {
        r.error_code = IGAOS_PDHG_ERR_NUMERIC;
        fill_message(r, "numerical failure: NaN/Inf in the PDHG iterates");
    } else if (out.status == IGAOS_STATUS_NEAR_OPTIMAL) {
        fill_message(r, "converged: residuals + duality gap @tol (FP32 iterates, FP64 refinement)");
    } else if (out.status == IGAOS_STATUS_TIME_LIMIT) {
        fill_message(r, "wall-clock budget exhausted");
    } else {
        fill_message(r, "iteration cap reached before tolerance");
    }
    if (x)
        for (int j = 0; j < n; ++j) x[pc_[j]] = hx[j] * hp_dc_[j];
    if (y)
        for (int i = 0; i < m; ++i) y[pr_[i]] = 1.0 * hy[i] / hp_dr_[i];
    emit_repaired(out, r, x, y);
}
}  // namespace igx
