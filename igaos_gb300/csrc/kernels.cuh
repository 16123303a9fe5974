// Kernels of the GB300 PDHG engine. Reference algorithm: IGAOS
// src/pdhg/pdhg.cu (file:line cited per kernel).
#pragma once

#include "device.cuh"

namespace igx {

// Original-unit column value x = dc * x~ (src/pdhg/pdhg.cu:712). An FP32
// iterate projected onto its FP32-rounded bound is exactly at that bound:
// it maps to the FP64 bound itself (dc * fl32(l/dc) would sit ~6e-8 |l|
// away, outside evaluate()'s 1e-9 "at bound" band). FP64 iterates are
// unscaled as the reference does, without snapping.
__device__ __forceinline__ double unscale_x(double xs, double, double, double dc, double,
                                           double) {
    return xs * dc;
}
__device__ __forceinline__ double unscale_x(float xs, float slo, float shi, double dc, double lo,
                                           double hi) {
    if (xs == slo) return lo;
    if (xs == shi) return hi;
    return (double)xs * dc;
}

template <typename TI>
__global__ void k_unscale_cols(int n, const TI* __restrict__ xs, const TI* __restrict__ slo,
                               const TI* __restrict__ shi, const double* __restrict__ dc,
                               const double* __restrict__ lo, const double* __restrict__ hi,
                               double* __restrict__ out) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        out[j] = unscale_x(xs[j], slo[j], shi[j], dc[j], lo[j], hi[j]);
}

// ------------------------------------------------------------ attempt state
// Per-launch view of the control block, read once per CTA.
template <typename T>
struct CtlView {
    int parity, stop;
    T tau, sigma, w, isigma;
};
template <typename T>
__device__ __forceinline__ CtlView<T> read_ctl(const DevCtl* c);
template <>
__device__ __forceinline__ CtlView<double> read_ctl<double>(const DevCtl* c) {
    return CtlView<double>{c->parity, *(volatile const int*)&c->stop, c->tau, c->sigma, c->w,
                           c->isigma};
}
template <>
__device__ __forceinline__ CtlView<float> read_ctl<float>(const DevCtl* c) {
    return CtlView<float>{c->parity, *(volatile const int*)&c->stop, c->tau_f, c->sigma_f, c->w_f,
                          c->isigma_f};
}

template <typename T>
struct PrimalArgs {
    WarpSched ws;
    Csr<T> AT;              // A~^T (rows = columns of A)
    const T* y[2];          // dual iterate slots
    const T* c;             // scaled cost
    const T* lo;            // scaled column bounds
    const T* hi;
    T* x[2];
    T* xavg[2];
    T* xbar;
    Acc<T>* part;           // per-CTA ||dx||^2 (compensated in FP32 kernels)
    DevCtl* ctl;
};

// Primal half of one line-search attempt, fused into the A^T y SpMV:
//   g = c + A^T y;  x' = P_[l,u](x - tau g);  xbar = 2x' - x;  dx = x' - x
// (kern_primal, src/pdhg/pdhg.cu:33-45) plus the candidate Halpern average
// xavg' = xavg + w (x' - xavg), w = 2/(hn+2) (kern_mix2, :129-141, :795-799),
// written to the other parity slot so that a rejected attempt leaves the
// accepted state untouched.
// Hook called with each row's new gathered-vector entry (xbar_j, y'_i):
// nothing for the grid-wide kernels.
struct NoBcast {
    template <typename U>
    __device__ __forceinline__ void operator()(int, U) const {}
};

template <typename T, class B = NoBcast>
struct PrimalEpi {
    const T *c, *lo, *hi, *xc, *xa;
    T *xn_out, *xa_out, *xbar;
    T tau, w, dx2;
    B bc{};
    struct Pre {
        T c, lo, hi, x, xa;
    };
    __device__ __forceinline__ Pre load(int j) const {
        return Pre{__ldg(c + j), __ldg(lo + j), __ldg(hi + j), xc[j], xa[j]};
    }
    __device__ __forceinline__ void apply(int j, const Acc<T>& acc, const Pre& v) {
        const T g = v.c + acc.result();
        const T xn = clamp_val(fma(-tau, g, v.x), v.lo, v.hi);
        xn_out[j] = xn;
        const T xb = fma((T)2, xn, -v.x);
        xbar[j] = xb;
        bc(j, xb);
        const T dx = xn - v.x;
        dx2 = fma(dx, dx, dx2);
        xa_out[j] = fma(w, xn - v.xa, v.xa);
    }
};

// OCC: resident CTAs per SM the kernel is compiled for (its register
// budget); FP64 attempts come in two (3 and 4), chosen by the autotuner.
template <typename T, int OCC = HotCtas<T>::value>
__global__ void __launch_bounds__(kThreads, OCC) k_primal(PrimalArgs<T> a) {
    __shared__ __align__(16) double smred[kWarps * 4];
    const CtlView<T> cv = read_ctl<T>(a.ctl);
    if (cv.stop) return;
    const int p = cv.parity, q = p ^ 1;
    PrimalEpi<T> epi{a.c, a.lo, a.hi, a.x[p], a.xavg[p], a.x[q], a.xavg[q], a.xbar,
                     cv.tau, cv.w, (T)0};
    warp_rows_all<T>(a.ws, a.AT, a.y[p], epi);
    const T dx2 = epi.dx2;
    T v[1] = {dx2};
    block_sum_t<T, 1>(v, reinterpret_cast<T*>(smred));
    if (threadIdx.x == 0) {
        Acc<T> e;
        e.s = v[0];
        a.part[blockIdx.x] = e;
    }
}

template <typename T>
struct DualArgs {
    WarpSched ws;
    Csr<T> A;
    const T* xbar;
    const T* rmin;          // scaled row bounds
    const T* rmax;
    T* y[2];
    T* axc[2];              // A x of the accepted iterate
    T* yavg[2];
    Acc<T>* part;           // per-CTA (||dy||^2, dy'A dx)
    const Acc<T>* part_primal;
    const T* yhat;          // anchor of anchored iterations (rounded), or nullptr
    const double* fac;      // (1 - k^-0.3, 1 + k^-0.6) for k = ctl->fac_base + i
    int n_fac;
    int n_primal;
    DevCtl* ctl;
};

// Anchored iterations (FP32 + FP64 refinement) hold y = yhat + dy with an
// FP64 anchor yhat; the dual projection must act on the full value, so the
// clamp argument is (t + yhat)/sigma with t = dy + sigma A dxbar and the row
// bounds shifted by the anchor's activity. yhat == nullptr: plain iterates.
// The quotient u / sigma (u = t, or t + yhat) is formed from the correctly
// rounded reciprocal 1/sigma of the step decision by one remainder
// correction (Markstein): q0 = u (1/sigma), r = fma(-sigma, q0, u),
// q = fma(r, 1/sigma, q0). q is the correctly rounded quotient except in
// rare cases (where it is one ulp off); an IEEE FP64 division costs about
// ten FP64 instructions, and FP64's pipe (2 per clock per SM on this GPU)
// bounds the FP64 attempt. The rest is the reference's formula (kern_dual,
// src/pdhg/pdhg.cu:49-61), y' = fma(-sigma, clamp(q, lo, hi), t), so an
// in-range row keeps the reference's rounding residue, which the line search
// sees through dy. (An oracle run with this quotient took the same
// iterations to the same objective, bit for bit, on the 14 golden LPs, six
// Netlib LPs and a 1 x 1 LP; giving in-range rows an exact 0 instead froze
// the 1 x 1 LP's step size: with dy = 0 the line search sees no curvature.)
template <typename T, class B = NoBcast>
struct DualEpi {
    const T *rmin, *rmax, *yc, *axc, *ya, *yhat;
    T *yn_out, *axc_out, *ya_out;
    T sigma, isigma, w, dy2, cross;
    B bc{};
    struct Pre {
        T lo, hi, y, ax, ya, yh;
    };
    __device__ __forceinline__ Pre load(int i) const {
        return Pre{__ldg(rmin + i), __ldg(rmax + i), yc[i], axc[i], ya[i],
                   yhat ? __ldg(yhat + i) : T(0)};
    }
    __device__ __forceinline__ void apply(int i, const Acc<T>& acc, const Pre& v) {
        const T ab = acc.result();
        const T t = fma(sigma, ab, v.y);
        const T u = yhat ? t + v.yh : t;
        const T q0 = u * isigma;
        const T q = fma(fma(-sigma, q0, u), isigma, q0);
        const T yn = fma(-sigma, clamp_val(q, v.lo, v.hi), t);
        yn_out[i] = yn;
        bc(i, yn);
        const T dy = yn - v.y;
        const T adx = (T)0.5 * (ab - v.ax);
        axc_out[i] = v.ax + adx;
        dy2 = fma(dy, dy, dy2);
        cross = fma(dy, adx, cross);
        ya_out[i] = fma(w, yn - v.ya, v.ya);
    }
};

// Adaptive step decision (src/pdhg/pdhg.cu:770-794), one thread. Host-side
// arithmetic of the reference has no FMA contraction; the explicit _rn
// intrinsics keep it that way here.
__device__ inline void decide_step(DevCtl* c, double dx2, double dy2, double cross,
                                   const double* fac, int n_fac) {
    c->dots[0] = dx2;
    c->dots[1] = dy2;
    c->dots[2] = cross;
    if (!isfinite(dx2) || !isfinite(dy2) || !isfinite(cross)) c->nan_flag = 1;
    const double eta = c->eta, omega = c->omega;
    const double num = __dadd_rn(__dmul_rn(omega, dx2), __ddiv_rn(dy2, omega));
    const double etabar =
        (num > 0.0 && cross > 0.0) ? __ddiv_rn(num, __dmul_rn(2.0, cross)) : CUDART_INF;
    // growth/shrink factors 1 - k^-0.3 and 1 + k^-0.6, tabulated by the host
    // (std::pow, as the reference) for the iterations of this chunk
    const long long fi = c->k - c->fac_base;
    double f_lo, f_hi;
    if (fac && fi >= 0 && fi < n_fac) {
        f_lo = fac[2 * fi];
        f_hi = fac[2 * fi + 1];
    } else {
        const double kk = (double)c->k;
        f_lo = __dsub_rn(1.0, pow(kk, -0.3));
        f_hi = __dadd_rn(1.0, pow(kk, -0.6));
    }
    double eta_new = CUDART_INF;
    if (isfinite(etabar)) eta_new = smin(__dmul_rn(f_lo, etabar), __dmul_rn(f_hi, eta));
    bool accept = !(eta > etabar) || num <= 0.0 || cross <= 0.0;
    if (!accept) accept = ++c->retries > 20;
    c->attempts += 1;
    if (accept) {
        if (isfinite(eta_new) && eta_new > 1e-12) c->eta = smin(eta_new, 1e12);
        c->parity ^= 1;
        c->hn += 1;
        c->accepted += 1;
        c->retries = 0;
        if (c->k >= c->k_stop || c->nan_flag) c->stop = 1;
        c->k += 1;
    } else {
        c->eta = smax(eta_new, 1e-12);
    }
    ctl_derive(c);
}

// Dual half of one attempt, fused into the A xbar SpMV:
//   t = y + sigma A xbar;  y' = t - sigma P_[rmin,rmax](t/sigma);
//   A(x'-x) = (A xbar - A x)/2   (kern_dual, src/pdhg/pdhg.cu:49-61),
// the candidate averages/commits of kern_mix2 (:129-141), the dot partials of
// kern_dots (:67-97), and -- in the last CTA to finish -- the fixed-order
// reduction of all partials (kern_dotfin, :99-125) and the step decision that
// the reference made on the host after a blocking copy (:768-794).
template <typename T, int OCC = HotCtas<T>::value>
__global__ void __launch_bounds__(kThreads, OCC) k_dual(DualArgs<T> a) {
    __shared__ __align__(16) double smred[kWarps * 4];
    const CtlView<T> cv = read_ctl<T>(a.ctl);
    if (cv.stop) return;
    const int p = cv.parity, q = p ^ 1;
    DualEpi<T> epi{a.rmin, a.rmax, a.y[p], a.axc[p], a.yavg[p], a.yhat, a.y[q], a.axc[q], a.yavg[q],
                   cv.sigma, cv.isigma, cv.w, (T)0, (T)0};
    warp_rows_all<T>(a.ws, a.A, a.xbar, epi);
    T v[2] = {epi.dy2, epi.cross};
    block_sum_t<T, 2>(v, reinterpret_cast<T*>(smred));
    if (threadIdx.x == 0) {
        Acc<T> e0, e1;
        e0.s = v[0];
        e1.s = v[1];
        a.part[2 * blockIdx.x] = e0;
        a.part[2 * blockIdx.x + 1] = e1;
    }
    if (!last_cta(&a.ctl->ticket)) return;
    // fixed-order compensated merge of all CTA partials
    Acc<T> s[3];
    for (int i = threadIdx.x; i < a.n_primal; i += kThreads) s[0].merge(a.part_primal[i]);
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) {
        s[1].merge(a.part[2 * i]);
        s[2].merge(a.part[2 * i + 1]);
    }
    block_merge<T, 3>(s, reinterpret_cast<Acc<T>*>(smred));
    if (threadIdx.x == 0)
        decide_step(a.ctl, s[0].result_d(), s[1].result_d(), s[2].result_d(), a.fac, a.n_fac);
}

// ------------------------------------------------------------- plain SpMV
// y = A x (Spmv::mv, src/pdhg/pdhg.cu:143-157).
template <typename T, typename TO>
__global__ void __launch_bounds__(kThreads, HotCtas<T>::value)
    k_spmv(WarpSched ws, Csr<T> A, const T* __restrict__ x, TO* __restrict__ y) {
    auto f = [&](int r, const Acc<T>& acc) { y[r] = (TO)acc.result_d(); };
    PlainEpi<decltype(f)> epi{f};
    warp_rows_all<T>(ws, A, x, epi);
}

// -------------------------------------------------------- Ruiz equilibration
// src/pdhg/pdhg.cu:474-481: dr_i *= sqrt(max_j |a_ij| dc_j / dr_i), and
// :482-490: dc_j /= sqrt(max_i |a_ij| / dr_i * dc_j), over the warp schedule
// of the length-sorted matrix (G lanes per row). The max is order-free and
// the division and sqrt are IEEE, so the factors are bit-identical to the
// sequential host loops.
__global__ void __launch_bounds__(kThreads) k_ruiz_rows(WarpSched ws, const int* __restrict__ ap,
                                                          const int* __restrict__ ai,
                                                          const double* __restrict__ ax,
                                                          const double* __restrict__ dc,
                                                          double* __restrict__ dr) {
    const int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * kWarps + (threadIdx.x >> 5); w < ws.nwarps; w += gridDim.x * kWarps) {
        const int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1);
        const int lg = __ldg(ws.lg + w), G = 1 << lg, gl = lane & (G - 1);
        const int i = r0 + (lane >> lg);
        double mx = 0.0, dri = 1.0;
        if (i < r1) {
            dri = dr[i];
            for (int p = ap[i] + gl; p < ap[i + 1]; p += G)
                mx = smax(mx, __ddiv_rn(__dmul_rn(fabs(ax[p]), dc[ai[p]]), dri));
        }
        for (int o = G >> 1; o > 0; o >>= 1) mx = smax(mx, __shfl_xor_sync(0xffffffffu, mx, o, G));
        if (i < r1 && gl == 0 && (mx > 0) && isfinite(mx)) dr[i] = __dmul_rn(dri, __dsqrt_rn(mx));
    }
}

__global__ void __launch_bounds__(kThreads) k_ruiz_cols(WarpSched ws, const int* __restrict__ cp,
                                                          const int* __restrict__ ci,
                                                          const double* __restrict__ acx,
                                                          const double* __restrict__ dr,
                                                          double* __restrict__ dc) {
    const int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * kWarps + (threadIdx.x >> 5); w < ws.nwarps; w += gridDim.x * kWarps) {
        const int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1);
        const int lg = __ldg(ws.lg + w), G = 1 << lg, gl = lane & (G - 1);
        const int j = r0 + (lane >> lg);
        double mx = 0.0, dcj = 1.0;
        if (j < r1) {
            dcj = dc[j];
            for (int p = cp[j] + gl; p < cp[j + 1]; p += G)
                mx = smax(mx, __dmul_rn(__ddiv_rn(fabs(acx[p]), dr[ci[p]]), dcj));
        }
        for (int o = G >> 1; o > 0; o >>= 1) mx = smax(mx, __shfl_xor_sync(0xffffffffu, mx, o, G));
        if (j < r1 && gl == 0 && (mx > 0) && isfinite(mx)) dc[j] = __ddiv_rn(dcj, __dsqrt_rn(mx));
    }
}

// Pock-Chambolle pass (alpha = 1) after Ruiz, opt-in (no reference
// counterpart: the reference scales by Ruiz alone, src/pdhg/pdhg.cu:472-498).
// sum[r] = sum over row r of |a_rj| dc_j / dr_r for rows of A (rowmajor = 1)
// or over column r of |a_ir| dc_r / dr_i (rowmajor = 0), on the warp schedule
// of that orientation; both sums come from the same scaled matrix.
__global__ void __launch_bounds__(kThreads) k_pc_sums(WarpSched ws, const int* __restrict__ ptr,
                                                        const int* __restrict__ idx,
                                                        const double* __restrict__ val,
                                                        const double* __restrict__ dr,
                                                        const double* __restrict__ dc, int rowmajor,
                                                        double* __restrict__ sum) {
    const int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * kWarps + (threadIdx.x >> 5); w < ws.nwarps; w += gridDim.x * kWarps) {
        const int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1);
        const int lg = __ldg(ws.lg + w), G = 1 << lg, gl = lane & (G - 1);
        const int r = r0 + (lane >> lg);
        double s = 0.0;
        if (r < r1) {
            for (int p = ptr[r] + gl; p < ptr[r + 1]; p += G) {
                const int k = idx[p];
                s += rowmajor ? fabs(val[p]) * dc[k] / dr[r] : fabs(val[p]) * dc[r] / dr[k];
            }
        }
        for (int o = G >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
        if (r < r1 && gl == 0) sum[r] = s;
    }
}

// d *= sqrt(sum) (rows, mul = 1) or d /= sqrt(sum) (columns, mul = 0) where
// the sum is positive and finite (empty rows and columns keep their factor).
__global__ void k_pc_apply(int n, const double* __restrict__ sum, int mul, double* __restrict__ d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double s = sum[i];
        if (!(s > 0) || !isfinite(s)) continue;
        d[i] = mul ? d[i] * sqrt(s) : d[i] / sqrt(s);
    }
}

// evaluate()'s at-bound bands per column (src/pdhg/pdhg.cu:206-212), the
// same FP64 operations as the inline test: tol = 1e-9 (1 + |b|), b = cu if
// finite else cl; lob = cl + tol, hib = cu - tol. A free column gives
// inf - inf = NaN there, which the inline test's x <= NaN / x >= NaN never
// passes; -inf / +inf keep that outcome for the integer-pipe compares.
__global__ void k_bands(int n, const double* __restrict__ cl, const double* __restrict__ cu,
                        double* __restrict__ lob, double* __restrict__ hib) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const double l = cl[j], u = cu[j];
        const double tol = 1e-9 * (1.0 + fabs(isfinite(u) ? u : l));
        const double lb = l + tol, hb = u - tol;
        lob[j] = isnan(lb) ? -CUDART_INF : lb;
        hib[j] = isnan(hb) ? CUDART_INF : hb;
    }
}

__global__ void k_fill(int n, double v, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = v;
}

// :491-492 -- non-finite or non-positive factors fall back to 1.
__global__ void k_fix_scale(int n, double* __restrict__ d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (!(d[i] > 0) || !isfinite(d[i])) d[i] = 1.0;
}

// Scaled values a~_ij = a_ij dc_j / dr_i (src/pdhg/pdhg.cu:505,512), in
// place over the original FP64 values, with an FP32 copy. `rowmajor`
// selects which index array names the column.
__global__ void k_scale_matrix(int rows, const int* __restrict__ ptr, const int* __restrict__ idx,
                               double* __restrict__ val, float* __restrict__ val32,
                               const double* __restrict__ dr, const double* __restrict__ dc,
                               int rowmajor) {
    const int lane = threadIdx.x & 31;
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= rows) return;
    for (int p = ptr[r] + lane; p < ptr[r + 1]; p += 32) {
        double v;
        if (rowmajor) v = __ddiv_rn(__dmul_rn(val[p], dc[idx[p]]), dr[r]);
        else v = __ddiv_rn(__dmul_rn(val[p], dc[r]), dr[idx[p]]);
        val[p] = v;
        val32[p] = (float)v;
    }
}

// The FP32 copy of A into its padded layout (row r in [ptr4[r], ptr4[r+1]),
// a multiple of 4 slots; pads hold value 0 and the row's first index).
__global__ void k_pad4(int rows, const int* __restrict__ ptr, const int* __restrict__ idx,
                       const float* __restrict__ val, const int* __restrict__ ptr4,
                       int* __restrict__ idx4, float* __restrict__ val4) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        const int b = ptr[r], len = ptr[r + 1] - b, b4 = ptr4[r], len4 = ptr4[r + 1] - b4;
        for (int k = 0; k < len4; ++k) {
            idx4[b4 + k] = idx[b + (k < len ? k : 0)];
            val4[b4 + k] = k < len ? val[b + k] : 0.f;
        }
    }
}

// s = v / d (bounds) or v * d (cost), elementwise, FP64 and FP32 copies.
// out = a - b in FP64 (change between two restart points)
template <typename T>
__global__ void k_ray_diff(int n, const T* __restrict__ a, const T* __restrict__ b,
                           double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (double)a[i] - (double)b[i];
}

// out = 1 / d (IEEE quotient, as the inline 1.0 / d it replaces)
__global__ void k_recip(int n, const double* __restrict__ d, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = __ddiv_rn(1.0, d[i]);
}

__global__ void k_scale_vec(int n, const double* __restrict__ v, const double* __restrict__ d,
                            int mul, double* __restrict__ out, float* __restrict__ out32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s = mul ? __dmul_rn(v[i], d[i]) : __ddiv_rn(v[i], d[i]);
        out[i] = s;
        if (out32) out32[i] = (float)s;
    }
}

// ----------------------------------------------------- reductions / norms
// out[0] = sum v^2 (sqrt if `root`), deterministic fixed-order tree.
struct NormArgs {
    const double* v;
    int n;
    double* part;
    double* out;
    unsigned int* ticket;
};
__global__ void k_sumsq(NormArgs a, int root) {
    __shared__ double red[kWarps * 4];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
        s = fma(a.v[i], a.v[i], s);
    double v[1] = {s};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) a.part[blockIdx.x] = v[0];
    if (!last_cta(a.ticket)) return;
    double t[1] = {0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) t[0] += a.part[i];
    block_sum<1>(t, red);
    if (threadIdx.x == 0) a.out[0] = root ? sqrt(t[0]) : t[0];
}

// Power-iteration normalisation (src/pdhg/pdhg.cu:617-622): v = w / ||w||
// unless ||w|| < 1e-300, in which case the loop is over (flag latched).
__global__ void k_power_normalise(int n, const double* __restrict__ w, double* __restrict__ v,
                                  const double* nw, int* done) {
    if (*(volatile int*)done) return;
    const double nrm = *nw;
    if (nrm < 1e-300) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *done = 1;
        return;
    }
    const double inv = 1.0 / nrm;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        v[i] = w[i] * inv;
}

// sum (a-b)^2 over two vector pairs (primal-weight update,
// src/pdhg/pdhg.cu:1044-1052), FP64 accumulation.
template <typename T>
__global__ void k_diffnorms(int n, const T* __restrict__ x, const T* __restrict__ px, int m,
                            const T* __restrict__ y, const T* __restrict__ py,
                            double* part, double* out, unsigned int* ticket) {
    __shared__ double red[kWarps * 4];
    double s[2] = {0.0, 0.0};
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double d = (double)x[i] - (double)px[i];
        s[0] = fma(d, d, s[0]);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        double d = (double)y[i] - (double)py[i];
        s[1] = fma(d, d, s[1]);
    }
    block_sum<2>(s, red);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s[0];
        part[2 * blockIdx.x + 1] = s[1];
    }
    if (!last_cta(ticket)) return;
    double t[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) {
        t[0] += part[2 * i];
        t[1] += part[2 * i + 1];
    }
    block_sum<2>(t, red);
    if (threadIdx.x == 0) {
        out[0] = t[0];
        out[1] = t[1];
    }
}

template <typename T>
__global__ void k_add_const(int n, T v, T* __restrict__ x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] += v;
}

template <typename TI, typename TO>
__global__ void k_convert(int n, const TI* __restrict__ in, TO* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (TO)in[i];
}

// --------------------------------------------------------------- KKT pass
// FP64 metrics of candidate pairs (x~, y~) in ORIGINAL units, one fused
// device pass replacing metrics_of + evaluate (src/pdhg/pdhg.cu:698-733,
// 173-254). Candidate v = blockIdx.y. Four launches:
//   prod (A)  : A~ x~ over the warp schedule, stored in FP64 (scaled units)
//   prod (A^T): A~^T y~, likewise
//   rows      : one thread per row: pinf numerator/normaliser, prow, max |y|
//   cols      : one thread per column: reduced costs d, dinf, c^T x, the
//               column part of the Lagrangian bound; then one thread per row
//               for its row part (needs max |y| for its noise threshold) and
//               the final metrics.
// The metrics run with every lane of a warp busy (inside the warp schedule
// only 32/G lanes hold a row, and an FP64 instruction issued with partial
// lanes occupies GB300's narrow FP64 pipe as long as a full one), several
// rows or columns per thread, and their maxima reduce on the integer pipe:
// with a row per thread, the FP64 compares of the block reductions cost
// more of that pipe than the metrics themselves.

template <typename T>
struct KktArgs {
    const T* x[2];
    const T* y[2];
    const double* ax[2];                      // A~ x~ per candidate (scaled units)
    const double* aty[2];                     // A~^T y~ per candidate (scaled units)
    const double *dr, *dc;
    const double* idr;                        // 1 / dr (IEEE quotients)
    const double* idc;                        // 1 / dc (IEEE quotients)
    // evaluate()'s at-bound bands (src/pdhg/pdhg.cu:206-212), per column:
    // lob = cl + 1e-9 (1 + |b|), hib = cu - 1e-9 (1 + |b|), b = finite cu else cl
    const double *lob, *hib;
    const double *c, *cl, *cu, *rmin, *rmax;  // original units
    const T *slo, *shi;                       // scaled column bounds, iterate precision
    double cmax;
    double* part;   // >= 2 * blocks * 8 doubles
    DevMetrics* out;
    unsigned int* ticket;
};

// Products of both candidates: out[v] = M v_in[v] in FP64 (the same warp
// traversal and accumulator as every other product of the engine).
template <typename T>
__global__ void __launch_bounds__(kThreads, HotCtas<T>::value)
    k_kkt_prod(WarpSched ws, Csr<T> M, const T* in0, const T* in1, double* out0, double* out1) {
    const T* __restrict__ in = blockIdx.y ? in1 : in0;
    double* __restrict__ out = blockIdx.y ? out1 : out0;
    auto f = [&](int r, const Acc<T>& acc) { out[r] = acc.result_d(); };
    PlainEpi<decltype(f)> epi{f};
    warp_rows_all<T>(ws, M, in, epi);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_kkt_rows(KktArgs<T> a, int m) {
    __shared__ __align__(16) double smred[kWarps * 4];
    const int v = blockIdx.y;
    const T* __restrict__ yv = a.y[v];
    const double* __restrict__ axv = a.ax[v];
    double pv = 0.0, pa = 0.0, prow = 0.0, ymax = 0.0;
    // comparisons on the integer pipe (dmax, dmin, ...; see device.cuh)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double Ax = axv[i] * a.dr[i];
        const double lo = a.rmin[i], hi = a.rmax[i];
        const double vi = dmax(lo - Ax, Ax - hi);
        pv = dmax(pv, vi);
        pa = dmax(pa, dabs(dmin(dmax(Ax, lo), hi)));
        // vi / (1 + sc) <= vi: the FP64 division only when vi beats this
        // thread's running maximum (with prow = 0 that is vi > 0)
        if (dlt(prow, vi)) {
            double sc = dabs(Ax);
            if (dfinite(lo)) sc = dmax(sc, dabs(lo));
            if (dfinite(hi)) sc = dmax(sc, dabs(hi));
            prow = dmax(prow, vi / (1.0 + sc));
        }
        ymax = dmax(ymax, dabs((double)yv[i] * a.idr[i]));
    }
    double r[4] = {pv, pa, prow, ymax};
    block_dmax<4>(r, smred);
    const int nt = gridDim.x;
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; ++q) a.part[(v * nt + blockIdx.x) * 4 + q] = r[q];
    if (!last_cta(a.ticket)) return;
    for (int cv = 0; cv < (int)gridDim.y; ++cv) {
        double t[4] = {0.0, 0.0, 0.0, 0.0};
        for (int b = threadIdx.x; b < nt; b += kThreads)
            for (int q = 0; q < 4; ++q) t[q] = dmax(t[q], a.part[(cv * nt + b) * 4 + q]);
        block_dmax<4>(t, smred);
        if (threadIdx.x == 0) {
            DevMetrics& o = a.out[cv];
            o.pv = t[0];
            o.pa = t[1];
            o.pinf = smax(t[0], 0.0) / (1.0 + t[1]);
            o.prow = t[2];
            o.ymax = t[3];
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_kkt_cols(KktArgs<T> a, int n, int m) {
    __shared__ __align__(16) double smred[kWarps * 4];
    const int v = blockIdx.y;
    const T* __restrict__ xv = a.x[v];
    const double* __restrict__ atyv = a.aty[v];
    const double dz = 1e-8 * (1.0 + a.cmax);
    double dv = 0.0, op = 0.0, od = 0.0, unb = 0.0;
    // comparisons on the integer pipe, at-bound bands precomputed (k_bands);
    // the reduced cost multiplies by 1/dc instead of dividing by dc
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const double d = a.c[j] + atyv[j] * a.idc[j];
        const double x = unscale_x(xv[j], a.slo[j], a.shi[j], a.dc[j], a.cl[j], a.cu[j]);
        const double cl = a.cl[j], cu = a.cu[j];
        const bool pos = dgt0(d), neg = dlt0(d);
        const bool excused = (pos && !dlt(a.lob[j], x)) || (neg && !dlt(x, a.hib[j]));
        if (!excused) dv = dmax(dv, dabs(d));
        op += a.c[j] * x;
        if (!neg) {  // d >= 0
            if (dfinite(cl)) od += d * cl;
            else if (dlt(dz, d)) unb = 1.0;
        } else {
            if (dfinite(cu)) od += d * cu;
            else if (dlt(dz, -d)) unb = 1.0;
        }
    }
    // row part of the Lagrangian bound (src/pdhg/pdhg.cu:232-242)
    const T* __restrict__ yv = a.y[v];
    const double yz = 1e-8 * (1.0 + a.out[v].ymax);
    double odr = 0.0, unbr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double y = (double)yv[i] * a.idr[i];
        if (dlt(yz, y)) {
            if (dfinite(a.rmax[i])) odr -= y * a.rmax[i];
            else unbr = 1.0;
        } else if (dlt(y, -yz)) {
            if (dfinite(a.rmin[i])) odr -= y * a.rmin[i];
            else unbr = 1.0;
        }
    }
    double mx[4] = {dv, unb, unbr, 0.0};
    block_dmax<4>(mx, smred);
    double sm3[4] = {op, od, odr, 0.0};
    block_sum<4>(sm3, smred);
    const int nt = gridDim.x;
    if (threadIdx.x == 0) {
        double* P = a.part + (v * nt + blockIdx.x) * 8;
        P[0] = mx[0];
        P[1] = mx[1];
        P[2] = mx[2];
        P[3] = sm3[0];
        P[4] = sm3[1];
        P[5] = sm3[2];
    }
    if (!last_cta(a.ticket)) return;
    for (int cv = 0; cv < (int)gridDim.y; ++cv) {
        double tm[4] = {0.0, 0.0, 0.0, 0.0}, ts[4] = {0.0, 0.0, 0.0, 0.0};
        for (int b = threadIdx.x; b < nt; b += kThreads) {
            const double* P = a.part + (cv * nt + b) * 8;
            for (int q = 0; q < 3; ++q) {
                tm[q] = dmax(tm[q], P[q]);
                ts[q] += P[3 + q];
            }
        }
        block_dmax<4>(tm, smred);
        block_sum<4>(ts, smred);
        if (threadIdx.x == 0) {
            DevMetrics& o = a.out[cv];
            o.dv = tm[0];
            o.dinf = tm[0] / (1.0 + a.cmax);
            o.unb_col = tm[1] > 0.0;
            o.op = ts[0];
            o.od_col = ts[1];
            o.od_row = ts[2];
            o.unb_row = tm[2] > 0.0;
            const bool bounded = !o.unb_col && !o.unb_row;
            o.od = bounded ? o.od_col + o.od_row : -CUDART_INF;
            o.gap = bounded ? smax(0.0, o.op - o.od) / (1.0 + fabs(o.op)) : CUDART_INF;
            o.finite = isfinite(o.pinf) && isfinite(o.dinf);
            const double g = isfinite(o.gap) ? o.gap : 0.0;
            o.err = smax(o.pinf, smax(o.dinf, g));
        }
    }
}

// ------------------------------------------------------ anchored iterations
// The LP seen from an FP64 anchor (x^, y^) in scaled units, rounded to FP32
// for the FP32 iteration on the deltas (x = x^ + dx, y = y^ + dy):
//   columns: c' = c~ + A~^T y^ (the reduced cost at the anchor),
//            l' = l~ - x^, u' = u~ - x^;
//   rows:    [rmin~, rmax~] - A~ x^, and y^ itself for the dual projection.
// Each value is formed in FP64 and rounded once, so it carries FP32 relative
// error of the residual, not of the original data.
__global__ void k_anchor_cols(int n, const double* __restrict__ sc, const double* __restrict__ scl,
                              const double* __restrict__ scu, const double* __restrict__ aty,
                              const double* __restrict__ xh, float* __restrict__ fc,
                              float* __restrict__ fcl, float* __restrict__ fcu) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        fc[j] = (float)(sc[j] + aty[j]);
        fcl[j] = (float)(scl[j] - xh[j]);
        fcu[j] = (float)(scu[j] - xh[j]);
    }
}

__global__ void k_anchor_rows(int m, const double* __restrict__ srmin,
                              const double* __restrict__ srmax, const double* __restrict__ ax,
                              const double* __restrict__ yh, float* __restrict__ frmin,
                              float* __restrict__ frmax, float* __restrict__ yh32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        frmin[i] = (float)(srmin[i] - ax[i]);
        frmax[i] = (float)(srmax[i] - ax[i]);
        yh32[i] = (float)yh[i];
    }
}

// Full FP64 iterate anchor + delta. A primal delta sitting on its FP32
// shifted bound is exactly at the bound (the same rule as unscale_x).
__global__ void k_anchor_full_cols(int n, const double* __restrict__ xh, const float* __restrict__ dx,
                                   const float* __restrict__ flo, const float* __restrict__ fhi,
                                   const double* __restrict__ scl, const double* __restrict__ scu,
                                   double* __restrict__ out) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const float d = dx[j];
        out[j] = d == flo[j] ? scl[j] : (d == fhi[j] ? scu[j] : xh[j] + (double)d);
    }
}

__global__ void k_anchor_full_rows(int m, const double* __restrict__ yh, const float* __restrict__ dy,
                                   double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        out[i] = yh[i] + (double)dy[i];
}

}  // namespace igx
