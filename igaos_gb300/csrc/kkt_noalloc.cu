// Allocation-free FP64 KKT evaluation (igaos_pdhg_evaluate_noalloc).
//
// For callers that cannot call cudaMalloc: code whose device memory is owned
// by a framework allocator or a fixed pool sized up front, or that runs where
// an allocation (which can synchronise the device) is not acceptable, such
// as a latency-bound serving loop. They pass every input and the output as
// device buffers they already own; the kernels' scratch (per-CTA partials,
// the metric accumulators, the last-CTA counters) lives in one file-scope
// __device__ array that every GPU loading this library holds until the
// process exits.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "device.cuh"
#include "engine.hpp"

namespace igx {
namespace {

constexpr int kNaRowsPerCta = 256;  // one CTA per 256 rows or columns
constexpr int kNaMaxCtas = 16384;   // => m, n <= 4,194,304
constexpr int kNaMaxDim = kNaRowsPerCta * kNaMaxCtas;

struct NaScratch {
    double part[kNaMaxCtas * 8];  // per-CTA partials of the current pass
    DevMetrics met;               // accumulated metrics
    double cmax;                  // max |c_j|
    unsigned int ticket[4];       // last-CTA counters (must start at zero)
};

// 1 MiB + a few bytes of device memory, per device that loads the library.
static __device__ __align__(256) NaScratch g_na_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_na_mu;
NaScratch* g_na_ptr[kMaxDevices] = {};

// Row pass: A x in original units -> pinf numerator/normaliser, prow,
// max |y|; also max |c| (grid-stride over columns). A warp per row.
__global__ void __launch_bounds__(kThreads) na_rows(int m, int n, const int* __restrict__ ap,
                                                    const int* __restrict__ ai,
                                                    const double* __restrict__ ax,
                                                    const double* __restrict__ x,
                                                    const double* __restrict__ y,
                                                    const double* __restrict__ c,
                                                    const double* __restrict__ rmin,
                                                    const double* __restrict__ rmax,
                                                    NaScratch* s) {
    __shared__ double red[kWarps * 8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double pv = 0.0, pa = 0.0, prow = 0.0, ymax = 0.0, cmax = 0.0;
    for (int k = 0; k < 32; ++k) {
        const int i = blockIdx.x * kNaRowsPerCta + warp * 32 + k;
        if (i >= m) break;
        double acc = 0.0;
        for (int p = ap[i] + lane; p < ap[i + 1]; p += 32) acc = fma(ax[p], x[ai[p]], acc);
        acc = warp_sum(acc);
        if (lane == 0) {
            const double Ax = acc, lo = rmin[i], hi = rmax[i];
            const double vi = smax(lo - Ax, Ax - hi);
            pv = smax(pv, vi);
            pa = smax(pa, fabs(smin(smax(Ax, lo), hi)));
            double sc = fabs(Ax);
            if (isfinite(lo)) sc = smax(sc, fabs(lo));
            if (isfinite(hi)) sc = smax(sc, fabs(hi));
            prow = smax(prow, smax(0.0, vi) / (1.0 + sc));
            ymax = smax(ymax, fabs(y[i]));
        }
    }
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        cmax = smax(cmax, fabs(c[j]));
    double r[5] = {pv, pa, prow, ymax, cmax};
    block_max<5>(r, red);
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; ++q) s->part[blockIdx.x * 8 + q] = r[q];
    if (!last_cta(&s->ticket[0])) return;
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads)
        for (int q = 0; q < 5; ++q) t[q] = smax(t[q], s->part[b * 8 + q]);
    block_max<5>(t, red);
    if (threadIdx.x == 0) {
        s->met.pv = t[0];
        s->met.pa = t[1];
        s->met.pinf = smax(t[0], 0.0) / (1.0 + t[1]);
        s->met.prow = t[2];
        s->met.ymax = t[3];
        s->cmax = t[4];
    }
}

// Column pass: d = c + A^T y -> dinf, c^T x, column part of the dual bound.
__global__ void __launch_bounds__(kThreads) na_cols(int n, const int* __restrict__ cp,
                                                    const int* __restrict__ ci,
                                                    const double* __restrict__ acx,
                                                    const double* __restrict__ x,
                                                    const double* __restrict__ y,
                                                    const double* __restrict__ c,
                                                    const double* __restrict__ cl,
                                                    const double* __restrict__ cu, NaScratch* s) {
    __shared__ double red[kWarps * 8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double dz = 1e-8 * (1.0 + s->cmax);
    double dv = 0.0, op = 0.0, od = 0.0, unb = 0.0;
    for (int k = 0; k < 32; ++k) {
        const int j = blockIdx.x * kNaRowsPerCta + warp * 32 + k;
        if (j >= n) break;
        double acc = 0.0;
        for (int p = cp[j] + lane; p < cp[j + 1]; p += 32) acc = fma(acx[p], y[ci[p]], acc);
        acc = warp_sum(acc);
        if (lane == 0) {
            const double d = c[j] + acc, xj = x[j], lo = cl[j], hi = cu[j];
            const double bnd = fabs(isfinite(hi) ? hi : lo);
            const double tol = 1e-9 * (1.0 + bnd);
            double e;
            if (xj <= lo + tol && d > 0) e = 0.0;
            else if (xj >= hi - tol && d < 0) e = 0.0;
            else e = fabs(d);
            dv = smax(dv, e);
            op += c[j] * xj;
            if (d >= 0) {
                if (isfinite(lo)) od += d * lo;
                else if (d > dz) unb = 1.0;
            } else {
                if (isfinite(hi)) od += d * hi;
                else if (-d > dz) unb = 1.0;
            }
        }
    }
    double mx[2] = {dv, unb};
    block_max<2>(mx, red);
    double sm[2] = {op, od};
    block_sum<2>(sm, red);
    if (threadIdx.x == 0) {
        double* P = s->part + blockIdx.x * 8;
        P[0] = mx[0];
        P[1] = mx[1];
        P[2] = sm[0];
        P[3] = sm[1];
    }
    if (!last_cta(&s->ticket[1])) return;
    double tm[2] = {0.0, 0.0}, ts[2] = {0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) {
        tm[0] = smax(tm[0], s->part[b * 8]);
        tm[1] = smax(tm[1], s->part[b * 8 + 1]);
        ts[0] += s->part[b * 8 + 2];
        ts[1] += s->part[b * 8 + 3];
    }
    block_max<2>(tm, red);
    block_sum<2>(ts, red);
    if (threadIdx.x == 0) {
        s->met.dv = tm[0];
        s->met.dinf = tm[0] / (1.0 + s->cmax);
        s->met.unb_col = tm[1] > 0.0;
        s->met.op = ts[0];
        s->met.od_col = ts[1];
    }
}

// Row part of the dual bound (its noise threshold needs max |y|) and the
// final metrics, written to the caller's out6.
__global__ void __launch_bounds__(kThreads) na_rowdual(int m, const double* __restrict__ y,
                                                       const double* __restrict__ rmin,
                                                       const double* __restrict__ rmax,
                                                       NaScratch* s, double* out6) {
    __shared__ double red[kWarps * 8];
    const double yz = 1e-8 * (1.0 + s->met.ymax);
    double od = 0.0, unb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double yi = y[i];
        if (yi > yz) {
            if (isfinite(rmax[i])) od -= yi * rmax[i];
            else unb = 1.0;
        } else if (yi < -yz) {
            if (isfinite(rmin[i])) od -= yi * rmin[i];
            else unb = 1.0;
        }
    }
    double sm[1] = {od};
    block_sum<1>(sm, red);
    double u[1] = {unb};
    block_max<1>(u, red);
    if (threadIdx.x == 0) {
        s->part[blockIdx.x * 8] = sm[0];
        s->part[blockIdx.x * 8 + 1] = u[0];
    }
    if (!last_cta(&s->ticket[2])) return;
    double t[1] = {0.0}, w[1] = {0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) {
        t[0] += s->part[b * 8];
        w[0] = smax(w[0], s->part[b * 8 + 1]);
    }
    block_sum<1>(t, red);
    block_max<1>(w, red);
    if (threadIdx.x == 0) {
        DevMetrics& o = s->met;
        const bool bounded = !o.unb_col && !(w[0] > 0.0);
        o.od = bounded ? o.od_col + t[0] : -CUDART_INF;
        o.gap = bounded ? smax(0.0, o.op - o.od) / (1.0 + fabs(o.op)) : CUDART_INF;
        out6[0] = o.pinf;
        out6[1] = o.dinf;
        out6[2] = o.gap;
        out6[3] = o.op;
        out6[4] = o.od;
        out6[5] = o.prow;
    }
}

// Device address of the scratch on the current device. The symbol names a
// host-side stand-in in host code; its device address is looked up once per
// device, with that device current, and cached.
int scratch_for_current_device(NaScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return igx_set_error(IGAOS_PDHG_ERR_NODEVICE, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "device ordinal beyond the scratch table");
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess || !p) {
            char buf[256];
            std::snprintf(buf, sizeof(buf), "cudaGetSymbolAddress of the evaluation scratch: %s",
                          cudaGetErrorString(e));
            return igx_set_error(IGAOS_PDHG_ERR_CUDA, buf);
        }
        g_na_ptr[dev] = static_cast<NaScratch*>(p);
    }
    *out = g_na_ptr[dev];
    return IGAOS_PDHG_OK;
}

}  // namespace
}  // namespace igx

extern "C" int igaos_pdhg_evaluate_noalloc(int m, int n, const int* ap, const int* ai,
                                           const double* ax, const int* cp, const int* ci,
                                           const double* acx, const double* c, const double* cl,
                                           const double* cu, const double* rmin,
                                           const double* rmax, const double* x, const double* y,
                                           double* out6, void* stream) {
    using namespace igx;
    if (m <= 0 || n <= 0) return igx_set_error(IGAOS_PDHG_ERR_INVALID, "m and n must be positive");
    if (m > kNaMaxDim || n > kNaMaxDim)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID,
                             "m or n above 4,194,304: beyond the fixed scratch of the "
                             "allocation-free evaluation (use igaos_pdhg_evaluate)");
    if (!ap || !ai || !ax || !cp || !ci || !acx || !c || !cl || !cu || !rmin || !rmax || !x ||
        !y || !out6)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "NULL device pointer");
    NaScratch* s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc != IGAOS_PDHG_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the last-CTA counters must start at zero (they are left at zero by a
    // completed call; cleared here in case an earlier call was interrupted)
    cudaError_t e = cudaMemsetAsync(s->ticket, 0, sizeof(s->ticket), st);
    const int gr = (m + kNaRowsPerCta - 1) / kNaRowsPerCta;
    const int gc = (n + kNaRowsPerCta - 1) / kNaRowsPerCta;
    if (e == cudaSuccess) {
        na_rows<<<gr, kThreads, 0, st>>>(m, n, ap, ai, ax, x, y, c, rmin, rmax, s);
        na_cols<<<gc, kThreads, 0, st>>>(n, cp, ci, acx, x, y, c, cl, cu, s);
        na_rowdual<<<gr, kThreads, 0, st>>>(m, y, rmin, rmax, s, out6);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "CUDA error in PDHG engine: %s", cudaGetErrorString(e));
        return igx_set_error(IGAOS_PDHG_ERR_CUDA, buf);
    }
    return igx_set_error(IGAOS_PDHG_OK, "");
}
