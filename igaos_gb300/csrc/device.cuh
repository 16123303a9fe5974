// Device-side building blocks of the GB300 PDHG engine.
//
// Layout in HBM (one LP): A~ (Ruiz-scaled) as CSR (rows of A) and as CSR of
// A~^T (rows = columns of A); int32 row pointers / column indices shared by
// both precisions, values in FP64 and FP32. Iterates live in parity pairs
// (x[2], y[2], xavg[2], yavg[2], axcur[2]): an attempt reads slot p and writes
// slot 1-p, the device-side line search flips p on acceptance, so a rejected
// attempt costs no copy and an accepted one no swap on the host.
//
// The hot SpMV is tile-scheduled: the host cuts the rows into tiles of at
// most kTileNnz nonzeros / kTileRows rows (a longer row is a tile of its own).
// A CTA streams its tile's values and column indices with coalesced loads,
// gathers x through the read-only path, stages (a_ij, x_j) pairs in shared
// memory and reduces the rows with a segmented sum balanced by nonzeros (every
// thread owns the same number of staged entries, whatever the row lengths --
// the Zipf-degree columns of the large LPs range from 1 to hundreds). The PDHG
// step for each row then runs in the same CTA with consecutive threads on
// consecutive rows, so A^T y / A xbar never round-trip through HBM.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

namespace igx {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kTileNnz = 2048;
constexpr int kTileRows = 512;
constexpr unsigned char kLongTile = 255;

struct TileSched {
    const int* tile_row;           // ntiles + 1 row boundaries
    const unsigned char* tile_lg;  // 0, or kLongTile for a single long row
    int ntiles;
};

template <typename T>
struct Csr {
    const int* __restrict__ ptr;
    const int* __restrict__ idx;
    const T* __restrict__ val;
    int rows;
};

// Device control block of the iteration loop (one per solve). Written by the
// last CTA of each dual-side launch; read by every CTA at launch start.
struct DevCtl {
    double eta, omega;
    double dots[3];      // last attempt: ||dx||^2, ||dy||^2, dy'A dx
    long long k;         // index of the iteration being attempted (1-based)
    long long hn;        // Halpern averaging counter
    long long attempts;  // total attempts
    long long accepted;  // total accepted iterations
    long long k_stop;    // raise `stop` once iteration k_stop is accepted
    long long fac_base;  // iteration index of entry 0 of the step-factor table
    int retries;
    int parity;
    int stop;
    int nan_flag;
    unsigned int ticket;  // last-CTA-done counter of the dual-side launch
    unsigned int ticket2; // counter for KKT / reduction launches
    // Step quantities derived once per decision (ctl_derive), so that no CTA
    // of the hot kernels spends FP64 divisions on them: tau = eta/omega,
    // sigma = eta*omega (src/pdhg/pdhg.cu:756) and the averaging weight
    // w = 2/(hn+2) (:795), in FP64 and rounded to FP32.
    double tau, sigma, w;
    float tau_f, sigma_f, w_f, pad_f;
};

__host__ __device__ inline void ctl_derive(DevCtl* c) {
    c->tau = c->eta / c->omega;
    c->sigma = c->eta * c->omega;
    c->w = 2.0 / ((double)c->hn + 2.0);
    c->tau_f = (float)c->tau;
    c->sigma_f = (float)c->sigma;
    c->w_f = (float)c->w;
}

// FP64 KKT metrics of one candidate (see k_kkt_* in kernels.cuh).
struct DevMetrics {
    double pinf, dinf, gap, op, od, prow;
    double err;      // max(pinf, dinf, finite gap)
    double ymax, od_col, od_row;
    double pv, pa, dv;
    int unb_col, unb_row, finite, pad;
};

// ----------------------------------------------------------- numerics
template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

// Row accumulator. FP64: a plain FMA chain. FP32: compensated dot product
// (TwoProduct by fmaf + TwoSum, Ogita-Rump-Oishi "Dot2"): the running sum and
// the exact rounding errors of every product and addition are kept apart and
// added once at the end, so the row sum is as accurate as if accumulated in
// twice the working precision.
template <typename T> struct Acc;

template <> struct Acc<double> {
    double s;
    __device__ __forceinline__ Acc() : s(0.0) {}
    __device__ __forceinline__ void add(double a, double x) { s = fma(a, x, s); }
    __device__ __forceinline__ void merge(const Acc& o) { s += o.s; }
    __device__ __forceinline__ void shfl_xor(unsigned mask, int off, int width) {
        Acc o;
        o.s = __shfl_xor_sync(mask, s, off, width);
        merge(o);
    }
    __device__ __forceinline__ double result() const { return s; }
    __device__ __forceinline__ double result_d() const { return s; }
};

template <> struct Acc<float> {
    float s, c;
    __device__ __forceinline__ Acc() : s(0.f), c(0.f) {}
    __device__ __forceinline__ void add(float a, float x) {
        float p = a * x;
        float pe = fmaf(a, x, -p);  // exact product error
        float t = s + p;
        float bp = t - s;
        float e = (s - (t - bp)) + (p - bp);  // exact addition error
        s = t;
        c += e + pe;
    }
    __device__ __forceinline__ void merge(const Acc& o) {
        float t = s + o.s;
        float bp = t - s;
        float e = (s - (t - bp)) + (o.s - bp);
        s = t;
        c += o.c + e;
    }
    __device__ __forceinline__ void shfl_xor(unsigned mask, int off, int width) {
        Acc o;
        o.s = __shfl_xor_sync(mask, s, off, width);
        o.c = __shfl_xor_sync(mask, c, off, width);
        merge(o);
    }
    __device__ __forceinline__ float result() const { return s + c; }
    __device__ __forceinline__ double result_d() const { return (double)s + (double)c; }
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = smax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of NV values; result valid in thread 0. `sh` needs
// kWarps * NV doubles. Fixed reduction tree -> deterministic.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[w * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0.0;
            for (int k = 0; k < kWarps; ++k) s += sh[k * NV + q];
            v[q] = s;
        }
    }
    __syncthreads();
}

// Same tree in the working precision (FP32 partials of FP32 kernels; the
// cross-CTA finish is FP64). `sh` needs kWarps * NV values of type T.
template <typename T, int NV>
__device__ __forceinline__ void block_sum_t(T (&v)[NV], T* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[w * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            T s = 0;
            for (int k = 0; k < kWarps; ++k) s += sh[k * NV + q];
            v[q] = s;
        }
    }
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_max(double (&v)[NV], double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = warp_max(v[q]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[w * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = sh[q];
            for (int k = 1; k < kWarps; ++k) s = smax(s, sh[k * NV + q]);
            v[q] = s;
        }
    }
    __syncthreads();
}

// Block-wide fixed-order merge of NV compensated accumulators; result in
// thread 0. `sh` needs kWarps * NV entries.
template <typename T, int NV>
__device__ __forceinline__ void block_merge(Acc<T> (&v)[NV], Acc<T>* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o > 0; o >>= 1) v[q].shfl_xor(0xffffffffu, o, 32);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[w * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            Acc<T> s = sh[q];
            for (int k = 1; k < kWarps; ++k) s.merge(sh[k * NV + q]);
            v[q] = s;
        }
    }
    __syncthreads();
}

// Last-CTA-done handshake: every CTA publishes its partials, fences, takes a
// ticket; the CTA holding the last ticket sees every partial and resets the
// counter for the next launch. No CTA waits on another.
__device__ __forceinline__ bool last_cta(unsigned int* ticket) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x * gridDim.y - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        if (threadIdx.x == 0) *ticket = 0u;
    }
    return is_last;
}

// --------------------------------------------------- tiled row reduction
// Shared staging area of one tile: (a_ij, x_j) pairs, the tile's row
// pointers and reduction scratch. 32 KB (FP64) / 16 KB (FP32) + 2.3 KB.
template <typename T>
struct TileSmem {
    typename Vec2<T>::type stage[kTileNnz];
    alignas(16) unsigned char rsum_raw[kTileRows * sizeof(Acc<T>)];   // row sums
    alignas(16) unsigned char carry_raw[kThreads * sizeof(Acc<T>)];   // per-chunk carry-out
    __device__ __forceinline__ Acc<T>* rsum() { return reinterpret_cast<Acc<T>*>(rsum_raw); }
    __device__ __forceinline__ Acc<T>* carry() { return reinterpret_cast<Acc<T>*>(carry_raw); }
    int rowptr[kTileRows + 1];
    double red[kWarps * 4];
};

template <typename T>
__device__ __forceinline__ typename Vec2<T>::type mk2(T a, T b);
template <>
__device__ __forceinline__ double2 mk2<double>(double a, double b) { return make_double2(a, b); }
template <>
__device__ __forceinline__ float2 mk2<float>(float a, float b) { return make_float2(a, b); }

// Computes every row sum of tile `t` of A (times x) and calls
// f(row, acc) once per row (acc: the row's Acc<T>) from exactly one lane. Rows of a tile are
// consecutive, so consecutive f calls touch consecutive vector entries.
template <typename T, class F>
__device__ __forceinline__ void tile_rows(TileSmem<T>& sm, const TileSched& ts, const Csr<T>& A,
                                          const T* __restrict__ x, int t, F& f) {
    const int r0 = ts.tile_row[t], r1 = ts.tile_row[t + 1];
    const int p0 = A.ptr[r0], p1 = A.ptr[r1];
    const int cnt = p1 - p0;
    const unsigned char lg = ts.tile_lg[t];
    if (lg == kLongTile) {  // one row, longer than a tile: whole CTA on it
        Acc<T> acc;
        for (int q = p0 + threadIdx.x; q < p1; q += kThreads)
            acc.add(__ldg(A.val + q), __ldg(x + __ldg(A.idx + q)));
        for (int o = 16; o > 0; o >>= 1) acc.shfl_xor(0xffffffffu, o, 32);
        __shared__ __align__(16) unsigned char wacc_raw[kWarps * sizeof(Acc<T>)];
        Acc<T>* wacc = reinterpret_cast<Acc<T>*>(wacc_raw);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) wacc[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            Acc<T> tot = wacc[0];
            for (int w = 1; w < kWarps; ++w) tot.merge(wacc[w]);
            f(r0, tot);
        }
        return;
    }
    auto* st = sm.stage;
    const int nrows = r1 - r0;
    for (int r = threadIdx.x; r <= nrows; r += kThreads) sm.rowptr[r] = A.ptr[r0 + r] - p0;
    // stage (a_ij, x_j): 4 independent loads in flight per thread
    int q = threadIdx.x;
    for (; q + 3 * kThreads < cnt; q += 4 * kThreads) {
        T a0 = __ldg(A.val + p0 + q), a1 = __ldg(A.val + p0 + q + kThreads);
        T a2 = __ldg(A.val + p0 + q + 2 * kThreads), a3 = __ldg(A.val + p0 + q + 3 * kThreads);
        int j0 = __ldg(A.idx + p0 + q), j1 = __ldg(A.idx + p0 + q + kThreads);
        int j2 = __ldg(A.idx + p0 + q + 2 * kThreads), j3 = __ldg(A.idx + p0 + q + 3 * kThreads);
        T x0 = __ldg(x + j0), x1 = __ldg(x + j1), x2 = __ldg(x + j2), x3 = __ldg(x + j3);
        st[q] = mk2<T>(a0, x0);
        st[q + kThreads] = mk2<T>(a1, x1);
        st[q + 2 * kThreads] = mk2<T>(a2, x2);
        st[q + 3 * kThreads] = mk2<T>(a3, x3);
    }
    for (; q < cnt; q += kThreads) st[q] = mk2<T>(__ldg(A.val + p0 + q), __ldg(x + __ldg(A.idx + p0 + q)));
    __syncthreads();
    // Segmented reduction, balanced by nonzeros: thread t owns the staged
    // elements [t*E, t*E+E) whatever the row lengths. A row that closes inside
    // its chunk is written directly; a row spanning chunks is summed by the
    // thread that closes it, over the spanning threads' carry-out pieces in
    // increasing order (deterministic).
    const int* rp = sm.rowptr;
    Acc<T>* rsum = sm.rsum();
    Acc<T>* carry = sm.carry();
    for (int rr = threadIdx.x; rr < nrows; rr += kThreads)
        if (rp[rr] == rp[rr + 1]) rsum[rr] = Acc<T>();  // empty row
    const int E = (cnt + kThreads - 1) / kThreads;
    const int q0 = min((int)threadIdx.x * E, cnt), q1 = min(q0 + E, cnt);
    Acc<T> head;
    int head_row = -1;
    Acc<T> acc;
    if (q0 < q1) {
        int lo = 0, hi = nrows - 1;  // first row with rp[i+1] > q0
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (rp[mid + 1] > q0) hi = mid;
            else lo = mid + 1;
        }
        int i = lo;
        bool started_here = rp[i] == q0;
        int end = rp[i + 1];
        for (int k = q0; k < q1; ++k) {
            const auto v = st[k];
            acc.add(v.x, v.y);
            if (k + 1 == end) {
                if (started_here) {
                    rsum[i] = acc;
                } else {
                    head = acc;
                    head_row = i;
                }
                acc = Acc<T>();
                ++i;
                while (i < nrows && rp[i + 1] == rp[i]) ++i;
                started_here = true;
                end = i < nrows ? rp[i + 1] : cnt + 1;
            }
        }
    }
    carry[threadIdx.x] = acc;  // piece of a row that continues past the chunk
    __syncthreads();
    if (head_row >= 0) {
        Acc<T> tot;
        for (int s = rp[head_row] / E; s < (int)threadIdx.x; ++s) tot.merge(carry[s]);
        tot.merge(head);
        rsum[head_row] = tot;
    }
    __syncthreads();
    // epilogue: consecutive threads on consecutive rows (coalesced vectors)
    for (int rr = threadIdx.x; rr < nrows; rr += kThreads) f(r0 + rr, sm.rsum()[rr]);
}

}  // namespace igx
