// Batched PDHG: thousands of independent LPs of uneven sizes solved in one
// persistent launch (igaos_pdhg_solve_batch).
//
// Each CTA takes instances from a work queue (largest first, an atomic
// counter; no CTA waits on another) and runs one LP to the end on its own:
// deterministic CSC build, Ruiz equilibration (src/pdhg/pdhg.cu:472-492),
// power iteration (:605-631), and the reference iteration -- adaptive line
// search (:751-794), averaging (:795-799), KKT checks every `check`
// iterations with the termination test (:835-840), restarts and the
// primal-weight update (:1001-1075) -- with per-instance restart and
// termination. Attempts stream FP32 (compensated row sums); the iterates are
// FP32 deltas from an FP64 anchor that every restart re-sets, with the
// residual data (reduced costs, shifted row bounds and box) formed in FP64
// from the original FP64 values, so the termination metrics -- evaluated in
// FP64 on anchor + delta -- reach FP64-level accuracy. Incumbent/rollback and
// dual repair are not part of this path.
//
// FP32 iterates can stall where FP64 ones do not (one instance of a 4,096-LP
// set needs 255,872 FP32 + refinement iterations against 54,336 in FP64),
// and the launch lasts as long as its slowest instance. So the first
// `handoff_max` instances still running at `handoff_at` iterations stop
// there (a device counter bounds how many), and, with those the launch left
// at max_iterations, the host finishes them in FP64 with the single-LP engine,
// several at once on their own streams and threads.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "device.cuh"
#include "engine.hpp"

namespace igx {
namespace {

// threads per instance (one CTA): big instances are latency-bound per
// iteration, so the whole CTA's width goes to one LP
constexpr int kBT = 512;
constexpr int kBW = kBT / 32;

struct BatchDesc {
    int m, n, nnz, pad;
    long long ap_off, cp_off, nz_off, row_off, col_off;
};

struct BatchOut {
    int status, handed;  // handed: stopped at handoff_at for the FP64 finish
    double objective, pinf, dinf, gap, prow;
    long long iterations, attempts, restarts;
    long long ns;  // device time of the instance (global timer)
};

__device__ __forceinline__ long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int kFacTab = 1 << 16;  // tabulated 1 - k^-0.3, 1 + k^-0.6

struct BatchArgs {
    int count;
    const int* order;
    unsigned int* queue;
    const BatchDesc* desc;
    const int *ap, *ai;
    const float* ax;     // original values, FP32 (Ruiz, scaled FP32 copies)
    const double* axd;   // original values, FP64 (anchor residuals)
    const double *c, *cl, *cu, *rmin, *rmax;
    int *cp, *ci, *cnt;
    float *cax, *sax, *scax;
    double* cax64;       // original values in CSC order, FP64
    float *dr, *dc, *sc, *scl, *scu, *srmin, *srmax, *yh32;
    float *x[2], *xa[2], *xbar, *vt;
    float *y[2], *ya[2], *axc[2], *mt;
    double *xh, *yh, *pesx, *pesy, *axh, *atyh;
    const float* fac;
    double tol;
    long long maxit;
    long long handoff_at;        // iterations after which an instance may be handed off
    unsigned int* handoff_count; // instances that asked (device counter)
    int handoff_max;             // at most this many are handed off
    int check;
    double* x_out;
    double* y_out;
    BatchOut* out;
};

struct BatchShared {
    Acc<float> acc[kBW * 4];
    double dred[kBW * 8];
    float fmax_[kBW * 8];
    int part[kBT];
    int inst;
    float tau, sigma, w;
    int parity, accept;
    long long kdone;
};

// ---- block-level helpers (every thread of the CTA calls them) -----------
template <int NV>
__device__ void bmerge(BatchShared& sh, Acc<float> (&v)[NV]) {
    block_merge<float, NV, kBW>(v, sh.acc);
}

template <int NV>
__device__ void bmaxf(BatchShared& sh, float (&v)[NV]) {
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o > 0; o >>= 1) v[q] = fmaxf(v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh.fmax_[wp * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            float s = sh.fmax_[q];
            for (int k = 1; k < kBW; ++k) s = fmaxf(s, sh.fmax_[k * NV + q]);
            v[q] = s;
        }
    __syncthreads();
}

// exclusive block scan of cnt[0..len) into out[0..len], out[len] = total
__device__ void bscan(BatchShared& sh, const int* cnt, int* out, int len) {
    const int t = threadIdx.x;
    const int per = (len + kBT - 1) / kBT;
    const int b = min(len, t * per), e = min(len, b + per);
    int s = 0;
    for (int j = b; j < e; ++j) s += cnt[j];
    sh.part[t] = s;
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int k = 0; k < kBT; ++k) {
            const int v = sh.part[k];
            sh.part[k] = run;
            run += v;
        }
        out[len] = run;
    }
    __syncthreads();
    int run = sh.part[t];
    for (int j = b; j < e; ++j) {
        out[j] = run;
        run += cnt[j];
    }
    __syncthreads();
}

struct Inst {
    int m, n;
    const int *ap, *ai;
    const float* ax;
    const double* axd;
    const double *c, *cl, *cu, *rmin, *rmax;
    int *cp, *ci, *cnt;
    float *cax, *sax, *scax;
    double* cax64;
    float *dr, *dc, *sc, *scl, *scu, *srmin, *srmax, *yh32;
    float *x[2], *xa[2], *xbar, *vt;
    float *y[2], *ya[2], *axc[2], *mt;
    double *xh, *yh, *pesx, *pesy, *axh, *atyh;
};

__device__ Inst make_inst(const BatchArgs& a, const BatchDesc& d) {
    Inst I;
    I.m = d.m;
    I.n = d.n;
    I.ap = a.ap + d.ap_off;
    I.ai = a.ai + d.nz_off;
    I.ax = a.ax + d.nz_off;
    I.axd = a.axd + d.nz_off;
    I.c = a.c + d.col_off;
    I.cl = a.cl + d.col_off;
    I.cu = a.cu + d.col_off;
    I.rmin = a.rmin + d.row_off;
    I.rmax = a.rmax + d.row_off;
    I.cp = a.cp + d.cp_off;
    I.ci = a.ci + d.nz_off;
    I.cnt = a.cnt + d.col_off;
    I.cax = a.cax + d.nz_off;
    I.cax64 = a.cax64 + d.nz_off;
    I.sax = a.sax + d.nz_off;
    I.scax = a.scax + d.nz_off;
    I.dr = a.dr + d.row_off;
    I.srmin = a.srmin + d.row_off;
    I.srmax = a.srmax + d.row_off;
    I.yh32 = a.yh32 + d.row_off;
    I.dc = a.dc + d.col_off;
    I.sc = a.sc + d.col_off;
    I.scl = a.scl + d.col_off;
    I.scu = a.scu + d.col_off;
    for (int s = 0; s < 2; ++s) {
        I.x[s] = a.x[s] + d.col_off;
        I.xa[s] = a.xa[s] + d.col_off;
        I.y[s] = a.y[s] + d.row_off;
        I.ya[s] = a.ya[s] + d.row_off;
        I.axc[s] = a.axc[s] + d.row_off;
    }
    I.xbar = a.xbar + d.col_off;
    I.vt = a.vt + d.col_off;
    I.mt = a.mt + d.row_off;
    I.xh = a.xh + d.col_off;
    I.pesx = a.pesx + d.col_off;
    I.atyh = a.atyh + d.col_off;
    I.yh = a.yh + d.row_off;
    I.pesy = a.pesy + d.row_off;
    I.axh = a.axh + d.row_off;
    return I;
}

// one row of a CSR times v (thread per row, compensated FP32)
__device__ __forceinline__ Acc<float> row_dot(const int* ptr, const int* idx, const float* val,
                                              const float* v, int r) {
    Acc<float> acc;
    for (int p = ptr[r]; p < ptr[r + 1]; ++p) acc.add(val[p], v[idx[p]]);
    return acc;
}

// Full FP64 column value of delta dx (scaled units), with the at-bound rule:
// a delta on its FP32 shifted bound is exactly at the bound.
__device__ __forceinline__ double full_x(const Inst& I, int j, float dx) {
    if (dx == I.scl[j]) return I.cl[j] / (double)I.dc[j];
    if (dx == I.scu[j]) return I.cu[j] / (double)I.dc[j];
    return I.xh[j] + (double)dx;
}

// Residual data of the LP seen from the anchor (xh, yh), FP64 -> FP32:
// sc = c~ + A~^T yh, [scl, scu] = box~ - xh, [srmin, srmax] = rows~ - A~ xh,
// with A~_ij = a_ij dc_j / dr_i formed in FP64 from the FP64 values.
__device__ void anchor_data(Inst& I) {
    const int t = threadIdx.x;
    for (int i = t; i < I.m; i += kBT) {
        const double dri = I.dr[i];
        double s = 0.0;
        for (int p = I.ap[i]; p < I.ap[i + 1]; ++p) {
            const int j = I.ai[p];
            s = fma(I.axd[p] * (double)I.dc[j] / dri, I.xh[j], s);
        }
        I.axh[i] = s;
        I.srmin[i] = (float)(I.rmin[i] / dri - s);
        I.srmax[i] = (float)(I.rmax[i] / dri - s);
        I.yh32[i] = (float)I.yh[i];
    }
    for (int j = t; j < I.n; j += kBT) {
        const double dcj = I.dc[j];
        double s = 0.0;
        for (int p = I.cp[j]; p < I.cp[j + 1]; ++p) {
            const int i = I.ci[p];
            s = fma(I.cax64[p] * dcj / (double)I.dr[i], I.yh[i], s);
        }
        I.atyh[j] = s;
        I.sc[j] = (float)(I.c[j] * dcj + s);
        I.scl[j] = (float)(I.cl[j] / dcj - I.xh[j]);
        I.scu[j] = (float)(I.cu[j] / dcj - I.xh[j]);
    }
    __syncthreads();
}

// ---- setup: CSC, Ruiz, scaled data, power iteration ----------------------
__device__ void setup(BatchShared& sh, Inst& I, float& eta0, float& omega0) {
    const int t = threadIdx.x, m = I.m, n = I.n;
    // CSC by counting sort; each column's entries ordered by row afterwards
    for (int j = t; j < n; j += kBT) I.cnt[j] = 0;
    __syncthreads();
    for (int i = t; i < m; i += kBT)
        for (int p = I.ap[i]; p < I.ap[i + 1]; ++p) atomicAdd(&I.cnt[I.ai[p]], 1);
    __syncthreads();
    bscan(sh, I.cnt, I.cp, n);
    for (int j = t; j < n; j += kBT) I.cnt[j] = I.cp[j];
    __syncthreads();
    for (int i = t; i < m; i += kBT)
        for (int p = I.ap[i]; p < I.ap[i + 1]; ++p) {
            const int q = atomicAdd(&I.cnt[I.ai[p]], 1);
            I.ci[q] = i;
            I.cax64[q] = I.axd[p];
        }
    __syncthreads();
    for (int j = t; j < n; j += kBT) {  // insertion sort by row index
        const int b = I.cp[j], e = I.cp[j + 1];
        for (int q = b + 1; q < e; ++q) {
            const int r = I.ci[q];
            const double v = I.cax64[q];
            int k = q - 1;
            while (k >= b && I.ci[k] > r) {
                I.ci[k + 1] = I.ci[k];
                I.cax64[k + 1] = I.cax64[k];
                --k;
            }
            I.ci[k + 1] = r;
            I.cax64[k + 1] = v;
        }
        for (int q = b; q < e; ++q) I.cax[q] = (float)I.cax64[q];
    }
    // Ruiz, 10 sweeps (FP32 factors)
    for (int i = t; i < m; i += kBT) I.dr[i] = 1.f;
    for (int j = t; j < n; j += kBT) I.dc[j] = 1.f;
    __syncthreads();
    for (int sweep = 0; sweep < 10; ++sweep) {
        for (int i = t; i < m; i += kBT) {
            float mx = 0.f;
            for (int p = I.ap[i]; p < I.ap[i + 1]; ++p)
                mx = fmaxf(mx, fabsf(I.ax[p]) * I.dc[I.ai[p]] / I.dr[i]);
            if (mx > 0.f && isfinite(mx)) I.dr[i] *= sqrtf(mx);
        }
        __syncthreads();
        for (int j = t; j < n; j += kBT) {
            float mx = 0.f;
            for (int p = I.cp[j]; p < I.cp[j + 1]; ++p)
                mx = fmaxf(mx, fabsf(I.cax[p]) / I.dr[I.ci[p]] * I.dc[j]);
            if (mx > 0.f && isfinite(mx)) I.dc[j] /= sqrtf(mx);
        }
        __syncthreads();
    }
    // scaled FP32 matrix; initial weight from the scaled cost and row bounds
    Acc<float> nq[2];
    for (int i = t; i < m; i += kBT) {
        for (int p = I.ap[i]; p < I.ap[i + 1]; ++p) I.sax[p] = I.ax[p] * I.dc[I.ai[p]] / I.dr[i];
        const float lo = (float)I.rmin[i] / I.dr[i], hi = (float)I.rmax[i] / I.dr[i];
        const float q = isfinite(hi) ? hi : (isfinite(lo) ? lo : 0.f);
        nq[1].add(q, q);
    }
    for (int j = t; j < n; j += kBT) {
        for (int p = I.cp[j]; p < I.cp[j + 1]; ++p) I.scax[p] = I.cax[p] * I.dc[j] / I.dr[I.ci[p]];
        const float cs = (float)I.c[j] * I.dc[j];
        nq[0].add(cs, cs);
    }
    bmerge<2>(sh, nq);
    if (t == 0) {
        const double cn = nq[0].result_d(), qn = nq[1].result_d();
        omega0 = (cn > 1e-24 && qn > 1e-24) ? fminf(3.f, fmaxf(0.3f, (float)sqrt(cn / qn))) : 1.f;
    }
    // power iteration for ||A~||_2^2
    const float v0 = rsqrtf((float)n);
    for (int j = t; j < n; j += kBT) I.vt[j] = v0;
    __syncthreads();
    __shared__ float s_norm;
    for (int it = 0; it < 31; ++it) {
        for (int i = t; i < m; i += kBT) I.mt[i] = row_dot(I.ap, I.ai, I.sax, I.vt, i).result();
        __syncthreads();
        if (it == 30) break;
        Acc<float> nrm[1];
        for (int j = t; j < n; j += kBT) {
            const float wv = row_dot(I.cp, I.ci, I.scax, I.mt, j).result();
            I.xbar[j] = wv;
            nrm[0].add(wv, wv);
        }
        bmerge<1>(sh, nrm);
        if (t == 0) s_norm = sqrtf((float)nrm[0].result_d());
        __syncthreads();
        const float nw = s_norm;
        if (!(nw > 1e-30f)) break;
        for (int j = t; j < n; j += kBT) I.vt[j] = I.xbar[j] / nw;
        __syncthreads();
    }
    Acc<float> na[1];
    for (int i = t; i < m; i += kBT) na[0].add(I.mt[i], I.mt[i]);
    bmerge<1>(sh, na);
    if (t == 0) {
        double lam = na[0].result_d();
        if (!(lam > 0) || !isfinite(lam)) lam = 1.0;
        eta0 = (float)(1.2 / sqrt(lam));
    }
    __syncthreads();
}

// ---- FP64 metrics of one candidate (anchor + delta, original units) -----
struct BMetrics {
    double pinf, dinf, gap, op, od, prow, err;
    bool finite;
};

__device__ BMetrics metrics(BatchShared& sh, Inst& I, const float* xs, const float* ys,
                            double cmax) {
    const int t = threadIdx.x;
    double r4[4] = {0.0, 0.0, 0.0, 0.0};  // pv, pa, prow, ymax
    for (int i = t; i < I.m; i += kBT) {
        const double Ax = (I.axh[i] + row_dot(I.ap, I.ai, I.sax, xs, i).result_d()) * (double)I.dr[i];
        const double lo = I.rmin[i], hi = I.rmax[i];
        const double vi = smax(lo - Ax, Ax - hi);
        r4[0] = smax(r4[0], vi);
        r4[1] = smax(r4[1], fabs(smin(smax(Ax, lo), hi)));
        double scv = fabs(Ax);
        if (isfinite(lo)) scv = smax(scv, fabs(lo));
        if (isfinite(hi)) scv = smax(scv, fabs(hi));
        r4[2] = smax(r4[2], smax(0.0, vi) / (1.0 + scv));
        r4[3] = smax(r4[3], fabs((I.yh[i] + (double)ys[i]) / (double)I.dr[i]));
    }
    block_max<4, kBW>(r4, sh.dred);
    __shared__ double s_r[4];
    if (t == 0)
        for (int q = 0; q < 4; ++q) s_r[q] = r4[q];
    __syncthreads();
    const double yz = 1e-8 * (1.0 + s_r[3]);
    const double dz = 1e-8 * (1.0 + cmax);
    double mx[2] = {0.0, 0.0};  // dv, unbounded
    double sm[3] = {0.0, 0.0, 0.0};  // op, od (columns), od (rows)
    for (int j = t; j < I.n; j += kBT) {
        const double aty = I.atyh[j] + row_dot(I.cp, I.ci, I.scax, ys, j).result_d();
        const double d = I.c[j] + aty / (double)I.dc[j];
        const double lo = I.cl[j], hi = I.cu[j];
        const float xv = xs[j];
        const double x = xv == I.scl[j] ? lo : (xv == I.scu[j] ? hi : (I.xh[j] + (double)xv) * (double)I.dc[j]);
        const double bnd = fabs(isfinite(hi) ? hi : lo);
        const double tol = 1e-9 * (1.0 + bnd);
        double e;
        if (x <= lo + tol && d > 0) e = 0.0;
        else if (x >= hi - tol && d < 0) e = 0.0;
        else e = fabs(d);
        mx[0] = smax(mx[0], e);
        sm[0] += I.c[j] * x;
        if (d >= 0) {
            if (isfinite(lo)) sm[1] += d * lo;
            else if (d > dz) mx[1] = 1.0;
        } else {
            if (isfinite(hi)) sm[1] += d * hi;
            else if (-d > dz) mx[1] = 1.0;
        }
    }
    for (int i = t; i < I.m; i += kBT) {
        const double yv = (I.yh[i] + (double)ys[i]) / (double)I.dr[i];
        if (yv > yz) {
            if (isfinite(I.rmax[i])) sm[2] -= yv * I.rmax[i];
            else mx[1] = 1.0;
        } else if (yv < -yz) {
            if (isfinite(I.rmin[i])) sm[2] -= yv * I.rmin[i];
            else mx[1] = 1.0;
        }
    }
    block_max<2, kBW>(mx, sh.dred);
    block_sum<3, kBW>(sm, sh.dred);
    __shared__ BMetrics s_m;
    if (t == 0) {
        BMetrics mt;
        mt.pinf = smax(s_r[0], 0.0) / (1.0 + s_r[1]);
        mt.prow = s_r[2];
        mt.dinf = mx[0] / (1.0 + cmax);
        mt.op = sm[0];
        const bool bounded = !(mx[1] > 0.0);
        mt.od = bounded ? sm[1] + sm[2] : -CUDART_INF;
        mt.gap = bounded ? smax(0.0, mt.op - mt.od) / (1.0 + fabs(mt.op)) : CUDART_INF;
        mt.finite = isfinite(mt.pinf) && isfinite(mt.dinf);
        mt.err = smax(mt.pinf, smax(mt.dinf, isfinite(mt.gap) ? mt.gap : 0.0));
        s_m = mt;
    }
    __syncthreads();
    return s_m;
}

// ---- one LP --------------------------------------------------------------
__device__ void solve_one(const BatchArgs& a, BatchShared& sh, const BatchDesc& d, int b) {
    const long long t_begin = global_ns();
    Inst I = make_inst(a, d);
    const int t = threadIdx.x, m = I.m, n = I.n;
    __shared__ float s_eta0, s_omega0;
    __shared__ double s_cmax;
    for (int j = t; j < n; j += kBT) I.xh[j] = I.pesx[j] = 0.0;
    for (int i = t; i < m; i += kBT) I.yh[i] = I.pesy[i] = 0.0;
    setup(sh, I, s_eta0, s_omega0);
    anchor_data(I);
    {
        double cm[1] = {0.0};
        for (int j = t; j < n; j += kBT) cm[0] = smax(cm[0], fabs(I.c[j]));
        block_max<1, kBW>(cm, sh.dred);
        if (t == 0) s_cmax = cm[0];
    }
    for (int j = t; j < n; j += kBT) I.x[0][j] = I.xa[0][j] = 0.f;
    for (int i = t; i < m; i += kBT) I.y[0][i] = I.ya[0][i] = I.axc[0][i] = 0.f;
    // controller state (thread 0)
    __shared__ double s_epoch_kkt, s_prev_cand, s_omega, s_eta;
    __shared__ long long s_k, s_hn, s_epoch_start, s_attempts, s_restarts;
    __shared__ int s_retries, s_have_pe, s_done, s_status, s_use_avg, s_restart, s_avg_better;
    __shared__ int s_asked, s_handed;
    __shared__ BMetrics s_last;
    if (t == 0) {
        s_eta = s_eta0;
        s_omega = s_omega0;
        s_k = 1;
        s_hn = 0;
        s_epoch_kkt = -1.0;
        s_prev_cand = CUDART_INF;
        s_epoch_start = 0;
        s_attempts = 0;
        s_restarts = 0;
        s_retries = 0;
        s_have_pe = 0;
        s_done = 0;
        s_status = IGAOS_STATUS_ITERATION_LIMIT;
        s_use_avg = 0;
        s_asked = 0;
        s_handed = 0;
        sh.parity = 0;
        s_last.pinf = s_last.dinf = CUDART_INF;
        s_last.gap = CUDART_INF;
        s_last.op = 0.0;
        s_last.prow = CUDART_INF;
    }
    __syncthreads();
    const long long maxit = a.maxit;
    while (!s_done) {
        if (t == 0) {
            sh.tau = (float)(s_eta / s_omega);
            sh.sigma = (float)(s_eta * s_omega);
            sh.w = (float)(2.0 / ((double)s_hn + 2.0));
        }
        __syncthreads();
        const int p = sh.parity, q = p ^ 1;
        const float tau = sh.tau, sigma = sh.sigma, w = sh.w;
        Acc<float> dots[3];
        // primal step fused with A^T y (thread per column), on the deltas
        for (int j = t; j < n; j += kBT) {
            const float g = I.sc[j] + row_dot(I.cp, I.ci, I.scax, I.y[p], j).result();
            const float xv = I.x[p][j];
            const float xn = fminf(fmaxf(fmaf(-tau, g, xv), I.scl[j]), I.scu[j]);
            I.x[q][j] = xn;
            I.xbar[j] = fmaf(2.f, xn, -xv);
            const float dx = xn - xv;
            dots[0].add(dx, dx);
            const float av = I.xa[p][j];
            I.xa[q][j] = fmaf(w, xn - av, av);
        }
        __syncthreads();
        // dual step fused with A xbar (thread per row); the projection acts
        // on the full value, so the anchor enters its argument
        for (int i = t; i < m; i += kBT) {
            const float ab = row_dot(I.ap, I.ai, I.sax, I.xbar, i).result();
            const float yv = I.y[p][i];
            const float tt = fmaf(sigma, ab, yv);
            const float arg = (tt + I.yh32[i]) / sigma;
            const float yn = fmaf(-sigma, fminf(fmaxf(arg, I.srmin[i]), I.srmax[i]), tt);
            I.y[q][i] = yn;
            const float dy = yn - yv;
            const float ax = I.axc[p][i];
            const float adx = 0.5f * (ab - ax);
            I.axc[q][i] = ax + adx;
            dots[1].add(dy, dy);
            dots[2].add(dy, adx);
            const float av = I.ya[p][i];
            I.ya[q][i] = fmaf(w, yn - av, av);
        }
        bmerge<3>(sh, dots);
        // step decision (src/pdhg/pdhg.cu:770-794)
        if (t == 0) {
            ++s_attempts;
            const double dx2 = dots[0].result_d(), dy2 = dots[1].result_d(),
                         cross = dots[2].result_d();
            const double eta = s_eta, om = s_omega;
            const double num = om * dx2 + dy2 / om;
            const double etabar = (num > 0.0 && cross > 0.0) ? num / (2.0 * cross) : CUDART_INF;
            const long long k = s_k;
            const float flo = k < kFacTab ? a.fac[2 * k] : 1.f - powf((float)k, -0.3f);
            const float fhi = k < kFacTab ? a.fac[2 * k + 1] : 1.f + powf((float)k, -0.6f);
            const double eta_new =
                isfinite(etabar) ? fmin((double)flo * etabar, (double)fhi * eta) : CUDART_INF;
            bool acc_ = !(eta > etabar) || num <= 0.0 || cross <= 0.0;
            if (!acc_) acc_ = ++s_retries > 20;
            if (!isfinite(dx2) || !isfinite(dy2) || !isfinite(cross)) {
                s_done = 1;
                s_status = IGAOS_STATUS_ERROR;
            }
            if (acc_) {
                if (isfinite(eta_new) && eta_new > 1e-12) s_eta = fmin(eta_new, 1e12);
                sh.parity ^= 1;
                ++s_hn;
                s_retries = 0;
                sh.kdone = s_k;  // index of the iteration just accepted
                ++s_k;
            } else {
                s_eta = fmax(eta_new, 1e-12);
            }
            sh.accept = acc_;
        }
        __syncthreads();
        if (!sh.accept || s_done) continue;
        const long long k = sh.kdone;
        const int pc = sh.parity;
        if (k % a.check == 0 || k >= maxit) {
            const BMetrics mc = metrics(sh, I, I.x[pc], I.y[pc], s_cmax);
            const BMetrics ma = metrics(sh, I, I.xa[pc], I.ya[pc], s_cmax);
            if (t == 0) {
                auto passes = [&](const BMetrics& u) {
                    return u.pinf <= a.tol && u.dinf <= a.tol && u.prow <= a.tol &&
                           isfinite(u.gap) && u.gap <= a.tol;
                };
                const double ec = mc.finite ? mc.err : CUDART_INF;
                const double ea = ma.finite ? ma.err : CUDART_INF;
                s_last = (ec <= ea) ? mc : ma;
                s_use_avg = ea < ec;
                s_restart = 0;
                if (passes(mc)) {
                    s_last = mc;
                    s_use_avg = 0;
                    s_done = 1;
                    s_status = IGAOS_STATUS_NEAR_OPTIMAL;
                } else if (passes(ma)) {
                    s_last = ma;
                    s_use_avg = 1;
                    s_done = 1;
                    s_status = IGAOS_STATUS_NEAR_OPTIMAL;
                } else if (k >= maxit) {
                    s_done = 1;
                } else if (k >= a.handoff_at && !s_asked &&
                           (s_asked = 1, atomicAdd(a.handoff_count, 1u) < (unsigned)a.handoff_max)) {
                    s_done = 1;  // left for the FP64 finish
                    s_handed = 1;
                } else {
                    const double cand = fmin(ec, ea);
                    if (s_epoch_kkt < 0.0) {
                        s_epoch_kkt = cand;
                        s_prev_cand = cand;
                    }
                    const long long te = k - s_epoch_start;
                    s_restart = (isfinite(cand) && isfinite(s_epoch_kkt) && s_epoch_kkt > 0.0 &&
                                 (cand <= 0.2 * s_epoch_kkt ||
                                  (cand <= 0.8 * s_epoch_kkt && isfinite(s_prev_cand) &&
                                   cand > s_prev_cand))) ||
                                (double)te >= 0.36 * (double)k;
                    s_prev_cand = cand;
                    if (s_restart) {
                        s_avg_better = ea < ec;
                        s_hn = 0;
                        s_epoch_start = k;
                        s_epoch_kkt = cand;
                        s_prev_cand = CUDART_INF;
                        ++s_restarts;
                    }
                }
            }
            __syncthreads();
            if (s_restart) {
                // the restart point becomes the new FP64 anchor; deltas restart
                // at zero; primal weight from the anchors' movement
                const float* dxs = s_avg_better ? I.xa[pc] : I.x[pc];
                const float* dys = s_avg_better ? I.ya[pc] : I.y[pc];
                double dn[2] = {0.0, 0.0};
                for (int j = t; j < n; j += kBT) {
                    const double nx = full_x(I, j, dxs[j]);
                    const double dd = nx - I.pesx[j];
                    dn[0] = fma(dd, dd, dn[0]);
                    I.pesx[j] = nx;
                }
                for (int i = t; i < m; i += kBT) {
                    const double ny = I.yh[i] + (double)dys[i];
                    const double dd = ny - I.pesy[i];
                    dn[1] = fma(dd, dd, dn[1]);
                    I.pesy[i] = ny;
                }
                block_sum<2, kBW>(dn, sh.dred);
                if (t == 0 && s_have_pe) {
                    const double dxn = dn[0], dyn = dn[1];
                    if (dxn > 1e-24 && dyn > 1e-24) {
                        const double om = sqrt(s_omega * sqrt(dyn / dxn));
                        if (isfinite(om) && om > 0.0) s_omega = fmin(fmax(om, 1e-6), 1e6);
                    }
                }
                if (t == 0) s_have_pe = 1;
                // the new anchor is the restart point (held in pes)
                for (int j = t; j < n; j += kBT) {
                    I.xh[j] = I.pesx[j];
                    I.x[pc][j] = I.xa[pc][j] = 0.f;
                }
                for (int i = t; i < m; i += kBT) {
                    I.yh[i] = I.pesy[i];
                    I.y[pc][i] = I.ya[pc][i] = I.axc[pc][i] = 0.f;
                }
                __syncthreads();
                anchor_data(I);
            }
        }
    }
    // answer: anchor + delta of the chosen candidate, original units
    const int pf = sh.parity;
    const float* xs = s_use_avg ? I.xa[pf] : I.x[pf];
    const float* ys = s_use_avg ? I.ya[pf] : I.y[pf];
    double* xo = a.x_out ? a.x_out + d.col_off : nullptr;
    double* yo = a.y_out ? a.y_out + d.row_off : nullptr;
    if (xo)
        for (int j = t; j < n; j += kBT) {
            const float xv = xs[j];
            xo[j] = xv == I.scl[j] ? I.cl[j]
                                   : (xv == I.scu[j] ? I.cu[j] : (I.xh[j] + (double)xv) * (double)I.dc[j]);
        }
    if (yo)
        for (int i = t; i < m; i += kBT) yo[i] = (I.yh[i] + (double)ys[i]) / (double)I.dr[i];
    if (t == 0) {
        BatchOut o;
        o.status = s_status;
        o.handed = s_handed;
        o.objective = s_last.op;
        o.pinf = s_last.pinf;
        o.dinf = s_last.dinf;
        o.gap = s_last.gap;
        o.prow = s_last.prow;
        o.iterations = s_k - 1;
        o.attempts = s_attempts;
        o.restarts = s_restarts;
        o.ns = global_ns() - t_begin;
        a.out[b] = o;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kBT) k_batch(BatchArgs a) {
    __shared__ BatchShared sh;
    for (;;) {
        if (threadIdx.x == 0) sh.inst = (int)atomicAdd(a.queue, 1u);
        __syncthreads();
        const int qi = sh.inst;
        __syncthreads();
        if (qi >= a.count) break;
        const int b = a.order[qi];
        const BatchDesc d = a.desc[b];
        if (d.m > 0 && d.n > 0) solve_one(a, sh, d, b);
    }
}

__global__ void k_to_float(long long n, const double* __restrict__ in, float* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

}  // namespace
}  // namespace igx

// ---------------------------------------------------------------- C ABI
extern "C" int igaos_pdhg_solve_batch(int count, const int* m, const int* n, const int* ap,
                                      const int* ai, const double* ax, const double* c,
                                      const double* cl, const double* cu, const double* rmin,
                                      const double* rmax, const igaos_pdhg_options* opt,
                                      igaos_pdhg_batch_result* res, double* x, double* y) {
    using namespace igx;
    if (count <= 0 || !m || !n || !ap || !ai || !ax || !c || !cl || !cu || !rmin || !rmax || !res)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "count must be positive and arrays non-NULL");
    igaos_pdhg_options o;
    if (opt) o = *opt;
    else igaos_pdhg_default_options(&o);
    if (!(o.tolerance > 0)) return igx_set_error(IGAOS_PDHG_ERR_INVALID, "tolerance must be positive");
    try {
        auto t_start = std::chrono::steady_clock::now();
        // host descriptors, validation
        std::vector<BatchDesc> desc(count);
        long long ap_off = 0, nz = 0, rows = 0, cols = 0;
        for (int b = 0; b < count; ++b) {
            if (m[b] < 0 || n[b] < 0)
                return igx_set_error(IGAOS_PDHG_ERR_INVALID, "negative instance size");
            BatchDesc& d = desc[b];
            d.m = m[b];
            d.n = n[b];
            const int* bap = ap + ap_off;
            if (bap[0] != 0)
                return igx_set_error(IGAOS_PDHG_ERR_INVALID, "each instance's row pointer must start at 0");
            for (int i = 0; i < d.m; ++i)
                if (bap[i + 1] < bap[i])
                    return igx_set_error(IGAOS_PDHG_ERR_INVALID, "row pointer must be non-decreasing");
            d.nnz = bap[d.m];
            for (int p = 0; p < d.nnz; ++p) {
                const int j = ai[nz + p];
                if (j < 0 || j >= d.n)
                    return igx_set_error(IGAOS_PDHG_ERR_INVALID, "column index out of range");
                if (!std::isfinite(ax[nz + p]))
                    return igx_set_error(IGAOS_PDHG_ERR_INVALID, "matrix values must be finite");
            }
            d.ap_off = ap_off;
            d.cp_off = cols + b;
            d.nz_off = nz;
            d.row_off = rows;
            d.col_off = cols;
            ap_off += d.m + 1;
            nz += d.nnz;
            rows += d.m;
            cols += d.n;
        }
        for (long long j = 0; j < cols; ++j) {
            if (!std::isfinite(c[j])) return igx_set_error(IGAOS_PDHG_ERR_INVALID, "cost must be finite");
            if (std::isnan(cl[j]) || std::isnan(cu[j]) || cl[j] > cu[j])
                return igx_set_error(IGAOS_PDHG_ERR_INVALID, "bad column bounds");
        }
        for (long long i = 0; i < rows; ++i)
            if (std::isnan(rmin[i]) || std::isnan(rmax[i]) || rmin[i] > rmax[i])
                return igx_set_error(IGAOS_PDHG_ERR_INVALID, "bad row bounds");
        if (igaos_pdhg_device_count() == 0)
            return igx_set_error(IGAOS_PDHG_ERR_NODEVICE, "no CUDA device: PDHG engine unavailable");
        if (o.device >= 0) CU(cudaSetDevice(o.device));
        // largest instances first
        std::vector<int> order(count);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int p1, int p2) {
            return (long long)desc[p1].nnz + desc[p1].m + desc[p1].n >
                   (long long)desc[p2].nnz + desc[p2].m + desc[p2].n;
        });
        std::vector<float> fac(2 * kFacTab);
        for (int k = 0; k < kFacTab; ++k) {
            const double kk = k < 1 ? 1.0 : (double)k;
            fac[2 * k] = (float)(1.0 - std::pow(kk, -0.3));
            fac[2 * k + 1] = (float)(1.0 + std::pow(kk, -0.6));
        }
        cudaStream_t st;
        CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } sg{st};
        Arena ar;
        auto up = [&](const auto* h, size_t len) {
            using V = std::remove_const_t<std::remove_pointer_t<decltype(h)>>;
            V* dp = ar.alloc<V>(len);
            CU(cudaMemcpyAsync(dp, h, sizeof(V) * len, cudaMemcpyHostToDevice, st));
            return dp;
        };
        BatchArgs A{};
        A.count = count;
        A.order = up(order.data(), order.size());
        A.desc = up(desc.data(), desc.size());
        A.queue = ar.alloc<unsigned int>(1);
        CU(cudaMemsetAsync(A.queue, 0, sizeof(unsigned int), st));
        A.ap = up(ap, (size_t)ap_off);
        A.ai = up(ai, (size_t)nz);
        double* axd = up(ax, (size_t)nz);
        float* axf = ar.alloc<float>(nz);
        k_to_float<<<1216, 256, 0, st>>>(nz, axd, axf);
        A.ax = axf;
        A.axd = axd;
        A.c = up(c, cols);
        A.cl = up(cl, cols);
        A.cu = up(cu, cols);
        A.rmin = up(rmin, rows);
        A.rmax = up(rmax, rows);
        A.cp = ar.alloc<int>(cols + count);
        A.ci = ar.alloc<int>(nz);
        A.cnt = ar.alloc<int>(cols);
        A.cax = ar.alloc<float>(nz);
        A.cax64 = ar.alloc<double>(nz);
        A.sax = ar.alloc<float>(nz);
        A.scax = ar.alloc<float>(nz);
        float** colv[] = {&A.dc, &A.sc, &A.scl, &A.scu, &A.x[0], &A.x[1], &A.xa[0], &A.xa[1],
                          &A.xbar, &A.vt};
        for (float** v : colv) *v = ar.alloc<float>(cols);
        float** rowv[] = {&A.dr, &A.srmin, &A.srmax, &A.yh32, &A.y[0], &A.y[1], &A.ya[0],
                          &A.ya[1], &A.axc[0], &A.axc[1], &A.mt};
        for (float** v : rowv) *v = ar.alloc<float>(rows);
        double** col64[] = {&A.xh, &A.pesx, &A.atyh};
        for (double** v : col64) *v = ar.alloc<double>(cols);
        double** row64[] = {&A.yh, &A.pesy, &A.axh};
        for (double** v : row64) *v = ar.alloc<double>(rows);
        A.fac = up(fac.data(), fac.size());
        A.tol = o.tolerance;
        // per-instance iteration cap (the kernel has no wall clock)
        A.maxit = (long long)std::max<int64_t>(1, o.max_iterations);
        // hand-off: 100,000 iterations and 16 instances unless overridden
        // (IGAOS_PDHG_BATCH_HANDOFF=iterations, 0 = never;
        // IGAOS_PDHG_BATCH_HANDOFF_MAX=instances)
        {
            const char* e = std::getenv("IGAOS_PDHG_BATCH_HANDOFF");
            const long long h = e && *e ? std::atoll(e) : 100000;
            A.handoff_at = h > 0 ? h : A.maxit;
            const char* em = std::getenv("IGAOS_PDHG_BATCH_HANDOFF_MAX");
            A.handoff_max = em && *em ? std::max(0, std::atoi(em)) : 16;
        }
        A.handoff_count = ar.alloc<unsigned int>(1);
        CU(cudaMemsetAsync(A.handoff_count, 0, sizeof(unsigned int), st));
        A.check = o.check_period > 0 ? o.check_period : 64;
        // every instance's answer (the FP64 finish starts from it)
        A.x_out = ar.alloc<double>(cols);
        A.y_out = ar.alloc<double>(rows);
        A.out = ar.alloc<BatchOut>(count);
        int sms = 0, dev = 0, per_sm = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kBT, 0));
        const int grid = std::max(1, std::min(count, sms * std::max(1, per_sm)));
        cudaEvent_t e0, e1;
        CU(cudaEventCreate(&e0));
        CU(cudaEventCreate(&e1));
        CU(cudaEventRecord(e0, st));
        k_batch<<<grid, kBT, 0, st>>>(A);
        CU(cudaGetLastError());
        CU(cudaEventRecord(e1, st));
        std::vector<BatchOut> out(count);
        CU(cudaMemcpyAsync(out.data(), A.out, sizeof(BatchOut) * count, cudaMemcpyDeviceToHost, st));
        std::vector<double> xk, yk;  // the launch's answers when the caller wants none
        if (!x) {
            xk.resize(cols);
            x = xk.data();
        }
        if (!y) {
            yk.resize(rows);
            y = yk.data();
        }
        CU(cudaMemcpyAsync(x, A.x_out, sizeof(double) * cols, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(y, A.y_out, sizeof(double) * rows, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        float kms = 0.f;
        CU(cudaEventElapsedTime(&kms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        // Instances the launch handed off or left at the cap are solved again,
        // alone, by the single-LP engine in FP64 through the public entry
        // points, from the launch's answer (igaos_pdhg_set_start), with the
        // same tolerance and cap; up to 8 at once, each on its own host
        // thread, engine and stream.
        std::vector<igaos_pdhg_result> fin(count);
        std::vector<char> redo(count, 0);
        std::vector<double> fin_ms(count, 0.0);
        std::vector<int> todo;
        for (int b = 0; b < count; ++b)
            if (out[b].status == IGAOS_STATUS_ITERATION_LIMIT && desc[b].m > 0 && desc[b].n > 0)
                todo.push_back(b);
        std::vector<int> fin_rc(count, IGAOS_PDHG_OK);
        std::vector<std::string> fin_msg(count);
        std::atomic<size_t> next{0};
        auto finish = [&]() {
            CU(cudaSetDevice(dev));
            for (size_t t; (t = next.fetch_add(1)) < todo.size();) {
                const int b = todo[t];
                const BatchDesc& d = desc[b];
                igaos_pdhg_options o64 = o;
                o64.precision = IGAOS_PDHG_FP64;
                o64.time_limit_s = 1e9;  // the cap binds, as in the launch
                o64.pdhg_presolve = 0;
                o64.crossover = 0;
                const auto t1 = std::chrono::steady_clock::now();
                igaos_pdhg_problem* P = nullptr;
                int rc = igaos_pdhg_create(&P, d.m, d.n, d.nnz, ap + d.ap_off, ai + d.nz_off,
                                           ax + d.nz_off, nullptr, nullptr, nullptr, c + d.col_off,
                                           cl + d.col_off, cu + d.col_off, rmin + d.row_off,
                                           rmax + d.row_off, 0.0, &o64);
                if (rc == IGAOS_PDHG_OK)
                    rc = igaos_pdhg_set_start(P, x + d.col_off, y + d.row_off);
                if (rc == IGAOS_PDHG_OK)
                    rc = igaos_pdhg_solve(P, &o64, &fin[b], x + d.col_off, y + d.row_off);
                igaos_pdhg_destroy(P);
                fin_rc[b] = rc;
                if (fin_rc[b] != IGAOS_PDHG_OK) {
                    char msg[512];
                    igaos_pdhg_last_error(msg, sizeof(msg));
                    fin_msg[b] = msg;
                }
                fin_ms[b] = std::chrono::duration<double, std::milli>(
                                std::chrono::steady_clock::now() - t1).count();
                redo[b] = 1;
            }
        };
        int nthreads = 8;
        if (const char* e = std::getenv("IGAOS_PDHG_BATCH_FINISH_THREADS"))
            nthreads = std::max(1, std::atoi(e));
        nthreads = (int)std::min<size_t>((size_t)nthreads, todo.size());
        if (nthreads == 1) {
            finish();
        } else if (nthreads > 1) {
            std::vector<std::thread> pool;
            std::vector<std::exception_ptr> errs(nthreads);
            for (int i = 0; i < nthreads; ++i)
                pool.emplace_back([&, i] {
                    try {
                        finish();
                    } catch (...) {
                        errs[i] = std::current_exception();
                    }
                });
            for (auto& th : pool) th.join();
            for (auto& e : errs)
                if (e) std::rethrow_exception(e);
        }
        for (int b : todo)
            if (fin_rc[b] != IGAOS_PDHG_OK) return igx_set_error(fin_rc[b], fin_msg[b].c_str());
        const double wall = std::chrono::duration<double, std::milli>(
                                std::chrono::steady_clock::now() - t_start).count();
        for (int b = 0; b < count; ++b) {
            igaos_pdhg_batch_result& r = res[b];
            const BatchOut& q = out[b];
            r.status = (desc[b].m > 0 && desc[b].n > 0) ? q.status : IGAOS_STATUS_ERROR;
            r.finished_fp64 = 0;
            r.objective = q.objective;
            r.pinf = q.pinf;
            r.dinf = q.dinf;
            r.rel_gap = q.gap;
            r.prow = q.prow;
            r.iterations = q.iterations;
            r.attempts = q.attempts;
            r.restarts = q.restarts;
            r.kernel_time_ms = kms;
            r.total_time_ms = wall;
            r.instance_time_ms = 1e-6 * (double)q.ns;
            if (redo[b]) {
                const igaos_pdhg_result& f = fin[b];
                r.finished_fp64 = 1;
                r.status = f.status;
                r.objective = f.objective;
                r.pinf = f.pinf;
                r.dinf = f.dinf;
                r.rel_gap = f.rel_gap;
                r.prow = f.prow;
                r.iterations += f.iterations;
                r.attempts += f.attempts;
                r.restarts += f.restarts;
                r.instance_time_ms += fin_ms[b];
            }
        }
    } catch (const CudaError& e) {
        return igx_set_error(e.code, e.what());
    } catch (const std::exception& e) {
        return igx_set_error(IGAOS_PDHG_ERR_CUDA, e.what());
    }
    return igx_set_error(IGAOS_PDHG_OK, "");
}
