// Device-side building blocks of the GB300 PDHG engine.
//
// Layout in HBM (one LP): A~ (Ruiz-scaled) as CSR (rows of A) and as CSR of
// A~^T (rows = columns of A); int32 row pointers / column indices shared by
// both precisions, values in FP64 and FP32. Iterates live in parity pairs
// (x[2], y[2], xavg[2], yavg[2], axcur[2]): an attempt reads slot p and writes
// slot 1-p, the device-side line search flips p on acceptance, so a rejected
// attempt costs no copy and an accepted one no swap on the host.
//
// The hot SpMV is warp-scheduled over a length-sorted permutation of the LP
// (see WarpSched below): rows of similar length share a warp, G lanes per
// row, coalesced streaming of values and indices, x gathered through the
// read-only path, warp-shuffle reductions. The PDHG step for each row runs
// right after its sum, with consecutive lanes on consecutive rows, so
// A^T y / A xbar never round-trip through HBM.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

namespace igx {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// Resident CTAs per SM the hot kernels are compiled for; launch widths use
// the same figure. Measured on the 200k x 500k LP (FP32 attempt): 6 CTAs
// (<= 40 registers, no spills) 59 us, 7 or 8 CTAs (forced to 32-36
// registers, with spills) 70 us.
#ifndef IGX_HOT_CTAS
#define IGX_HOT_CTAS 6
#endif
constexpr int kHotCtasPerSm = IGX_HOT_CTAS;
// FP64 attempt kernels: their own residency. At 6 CTAs/SM they spill under
// 40 registers; measured on the 200k x 500k LP: 6 CTAs 173 us per FP64
// attempt, 4 CTAs (64 registers) 165 us, 3 CTAs (<= 85 registers) 160 us.
#ifndef IGX_HOT_CTAS_F64
#define IGX_HOT_CTAS_F64 3
#endif
// Entries per lane the warp schedule aims at (G = smallest power of two with
// G * kLaneEntries >= row length), and the batch of entries a lane loads
// before its gathers. Measured on the 200k x 500k LP (FP32 attempt, 6 CTAs
// per SM): 4 entries per lane 60.2 us, 8 entries 55.8 us, 16 entries 59.2 us;
// batches of 8 (5 CTAs per SM) 55.6 us.
#ifndef IGX_LANE_ENTRIES
#define IGX_LANE_ENTRIES 8
#endif
#ifndef IGX_LANE_BATCH
#define IGX_LANE_BATCH 4
#endif
constexpr int kLaneEntries = IGX_LANE_ENTRIES;
constexpr int kLaneBatch = IGX_LANE_BATCH;
template <typename T> struct HotCtas { static constexpr int value = kHotCtasPerSm; };
template <> struct HotCtas<double> { static constexpr int value = IGX_HOT_CTAS_F64; };

template <typename T>
struct Csr {
    const int* __restrict__ ptr;
    const int* __restrict__ idx;
    const T* __restrict__ val;
    int rows;
    // 1: values and indices are read with an L2 evict-first policy, so that a
    // matrix streamed once per product does not push the iterate vectors
    // (reused by the next launch) out of L2 (FP32 products of LPs whose
    // attempt working set exceeds L2; multicommodity LP: 72.5 -> 70.1 us per
    // attempt); 0: plain read-only loads
    int stream = 0;
    // 1: every row's entries start at a multiple of 4 and fill a multiple of
    // 4 slots (pads: value 0, a valid index), so lanes read 4 entries with
    // one 16-byte load of values and one of indices
    int vec4 = 0;
};

// Read-only loads with an L2 evict-first cache policy (PTX createpolicy +
// ld.global.nc.L2::cache_hint). IGX_L2_STREAM=0 compiles the products
// without the option.
#ifndef IGX_L2_STREAM
#define IGX_L2_STREAM 1
#endif
__device__ __forceinline__ unsigned long long l2_evict_first() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float ld_first(const float* a, unsigned long long pol) {
    float v;
    asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ double ld_first(const double* a, unsigned long long pol) {
    double v;
    asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ int ld_first(const int* a, unsigned long long pol) {
    int v;
    asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ float4 ld_first4(const float* a, unsigned long long pol) {
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ int4 ld_first4(const int* a, unsigned long long pol) {
    int4 v;
    asm("ld.global.nc.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(a), "l"(pol));
    return v;
}

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
    float tau_f, sigma_f, w_f, isigma_f;
    // correctly rounded 1/sigma in each precision (the dual step's quotient,
    // see DualEpi in kernels.cuh)
    double isigma;
};

__host__ __device__ inline void ctl_derive(DevCtl* c) {
    c->tau = c->eta / c->omega;
    c->sigma = c->eta * c->omega;
    c->w = 2.0 / ((double)c->hn + 2.0);
    c->tau_f = (float)c->tau;
    c->sigma_f = (float)c->sigma;
    c->w_f = (float)c->w;
    c->isigma = 1.0 / c->sigma;
    c->isigma_f = 1.0f / c->sigma_f;
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

// FP64 comparisons on the integer pipe. This GPU's FP64 pipe does about 2
// operations per clock per SM, and the FP64 attempt and KKT kernels are bound
// by it; compare, min/max and sign tests of doubles are done instead on
// order-preserving keys of the bit patterns (negative values with every bit
// flipped, non-negative ones with the sign bit set), for operands that are not
// NaN (the attempt kernels flag NaN/Inf dot products before any KKT pass).
// dlt(a, b) = a < b; dmax / dmin = smax / smin (std::max / std::min order);
// dabs = fabs; dfinite = isfinite; dgt0 = a > 0; dlt0 = a < 0.
// IGX_INT_CLAMP=0 keeps the FP64 instructions in the attempt kernels.
#ifndef IGX_INT_CLAMP
#define IGX_INT_CLAMP 1
#endif
__device__ __forceinline__ unsigned long long order_key(double a) {
    const long long b = __double_as_longlong(a);
    return (unsigned long long)b ^ ((unsigned long long)(b >> 63) | 0x8000000000000000ULL);
}
__device__ __forceinline__ bool dlt(double a, double b) { return order_key(a) < order_key(b); }
__device__ __forceinline__ double dmax(double a, double b) { return dlt(a, b) ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return dlt(b, a) ? b : a; }
__device__ __forceinline__ double dabs(double a) {
    return __longlong_as_double(__double_as_longlong(a) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool dfinite(double a) {
    return (__double_as_longlong(a) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool dgt0(double a) { return __double_as_longlong(a) > 0; }
__device__ __forceinline__ bool dlt0(double a) {
    const long long b = __double_as_longlong(a);
    return b < 0 && (b << 1) != 0;  // negative, not -0
}
// a < b and clamp(v, lo, hi) = min(max(v, lo), hi) (lo <= hi) in the
// iterate's precision: FP32 on its own pipe, FP64 on the integer pipe (the
// result is one of the three operands, bit for bit).
__device__ __forceinline__ bool less(float a, float b) { return a < b; }
__device__ __forceinline__ bool less(double a, double b) {
#if IGX_INT_CLAMP
    return dlt(a, b);
#else
    return a < b;
#endif
}
__device__ __forceinline__ float clamp_val(float v, float lo, float hi) {
    return fminf(fmaxf(v, lo), hi);
}
__device__ __forceinline__ double clamp_val(double v, double lo, double hi) {
#if IGX_INT_CLAMP
    return dlt(v, lo) ? lo : (dlt(hi, v) ? hi : v);
#else
    return fmin(fmax(v, lo), hi);
#endif
}

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
    __device__ __forceinline__ Acc shfl_from(unsigned mask, int src) const {
        Acc o;
        o.s = __shfl_sync(mask, s, src);
        return o;
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
    __device__ __forceinline__ Acc shfl_from(unsigned mask, int src) const {
        Acc o;
        o.s = __shfl_sync(mask, s, src);
        o.c = __shfl_sync(mask, c, src);
        return o;
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

// Block-wide sum of NV values over NW warps (blockDim.x = 32 NW); result valid
// in thread 0. `sh` needs NW * NV doubles. Fixed reduction tree -> deterministic.
template <int NV, int NW = kWarps>
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
            for (int k = 0; k < NW; ++k) s += sh[k * NV + q];
            v[q] = s;
        }
    }
    __syncthreads();
}

// Same tree in the working precision (FP32 partials of FP32 kernels; the
// cross-CTA finish is FP64). `sh` needs NW * NV values of type T.
template <typename T, int NV, int NW = kWarps>
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
            for (int k = 0; k < NW; ++k) s += sh[k * NV + q];
            v[q] = s;
        }
    }
    __syncthreads();
}

template <int NV, int NW = kWarps>
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
            for (int k = 1; k < NW; ++k) s = smax(s, sh[k * NV + q]);
            v[q] = s;
        }
    }
    __syncthreads();
}

// block_max on the integer pipe (order-preserving keys): the same maxima,
// without the FP64 compares that otherwise dominate a short streaming pass
// on this GPU's narrow FP64 pipe (a positive NaN wins, as the largest key).
template <int NV, int NW = kWarps>
__device__ __forceinline__ void block_dmax(double (&v)[NV], double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o > 0; o >>= 1) v[q] = dmax(v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[w * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = sh[q];
            for (int k = 1; k < NW; ++k) s = dmax(s, sh[k * NV + q]);
            v[q] = s;
        }
    }
    __syncthreads();
}

// Block-wide fixed-order merge of NV compensated accumulators; result in
// thread 0. `sh` needs kWarps * NV entries.
template <typename T, int NV, int NW = kWarps>
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
            for (int k = 1; k < NW; ++k) s.merge(sh[k * NV + q]);
            v[q] = s;
        }
    }
    __syncthreads();
}

// Last-CTA-done handshake: every CTA publishes its partials, fences, takes a
// ticket; the CTA holding the last ticket sees every partial and resets the
// counter for the next launch. No CTA waits on another.
// The partials are written by thread 0, so only thread 0 fences before its
// ticket; the winner fences again (all threads) before reading them.
__device__ __forceinline__ bool last_cta(unsigned int* ticket) {
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
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

// ------------------------------------------------------ warp row schedule
// Rows are processed by warps. The host permutes the LP so that rows (and
// columns) appear in decreasing nonzero count, then deals consecutive rows to
// warps: a warp owns 32/G consecutive rows of similar length with G lanes per
// row (G = 1..32, about kLaneEntries entries per lane). No shared memory and no
// block-wide barrier on the hot path. (Items of 32 rows taken in G passes, so
// that the per-row step runs with all lanes busy, left 4x fewer items than
// resident warps on the 200k x 500k LP and doubled its attempt time.)
struct WarpSched {
    const int* row;           // nwarps + 1 row boundaries
    const unsigned char* lg;  // log2(G) of each warp
    int nwarps;
};


// Epilogue adapter for kernels whose row step needs no prefetch.
struct NoPre {};
template <class F>
struct PlainEpi {
    F& f;
    using Pre = NoPre;
    __device__ __forceinline__ NoPre load(int) const { return NoPre{}; }
    template <class A>
    __device__ __forceinline__ void apply(int r, const A& acc, const NoPre&) { f(r, acc); }
};

// The row sums of one warp item with 2^lg lanes per row: the lane's row
// has entries [b, e) (empty for lanes without a row), taken in predicated
// batches of kLaneBatch per lane (all value and index loads of a batch, then
// its gathers in flight); then the G-lane shuffle reduction, and the sum of
// the item's i-th row handed to lane i, so consecutive lanes touch
// consecutive vector entries.
template <typename T>
__device__ __forceinline__ Acc<T> lane_products(const Csr<T>& A, const T* __restrict__ x, int b,
                                                int e, int lg) {
    const int G = 1 << lg;
    const int gl = (threadIdx.x & 31) & (G - 1);
    Acc<T> acc;
    if constexpr (sizeof(T) == 4) {
        if (A.vec4) {
            // chunks of 4 entries dealt to the G lanes in turn: one 16-byte
            // load of values and one of indices, then 4 gathers in flight
            const unsigned long long pol = A.stream ? l2_evict_first() : 0ull;
            for (int p = b + 4 * gl; p < e; p += 4 * G) {
                float4 a4;
                int4 j4;
                if (A.stream) {
                    a4 = ld_first4(A.val + p, pol);
                    j4 = ld_first4(A.idx + p, pol);
                } else {
                    a4 = __ldg(reinterpret_cast<const float4*>(A.val + p));
                    j4 = __ldg(reinterpret_cast<const int4*>(A.idx + p));
                }
                const float x0 = __ldg(x + j4.x), x1 = __ldg(x + j4.y), x2 = __ldg(x + j4.z),
                            x3 = __ldg(x + j4.w);
                acc.add(a4.x, x0);
                acc.add(a4.y, x1);
                acc.add(a4.z, x2);
                acc.add(a4.w, x3);
            }
            return acc;
        }
    }
    for (int p = b + gl; p < e; p += kLaneBatch * G) {
        T a[kLaneBatch];
        int j[kLaneBatch];
#if IGX_L2_STREAM
        // FP32 products only: in the FP64 ones the branch alone cost 3-5 %
        // and streaming gained nothing (they are FP64-pipe bound)
        if (sizeof(T) == 4 && A.stream) {  // uniform branch: one policy per batch
            const unsigned long long pol = l2_evict_first();
#pragma unroll
            for (int u = 0; u < kLaneBatch; ++u) {
                const int q = p + u * G;
                const bool ok = q < e;
                a[u] = ok ? ld_first(A.val + q, pol) : T(0);
                j[u] = ok ? ld_first(A.idx + q, pol) : 0;
            }
        } else
#endif
        {
#pragma unroll
            for (int u = 0; u < kLaneBatch; ++u) {
                const int q = p + u * G;
                const bool ok = q < e;
                a[u] = ok ? __ldg(A.val + q) : T(0);
                j[u] = ok ? __ldg(A.idx + q) : 0;
            }
        }
        T xv[kLaneBatch];
#pragma unroll
        for (int u = 0; u < kLaneBatch; ++u) xv[u] = __ldg(x + j[u]);
#pragma unroll
        for (int u = 0; u < kLaneBatch; ++u) acc.add(a[u], xv[u]);  // masked: 0 * x[0] adds 0
    }
    return acc;
}

template <typename T>
__device__ __forceinline__ Acc<T> reduce_rows(Acc<T> acc, int lg) {
    const int G = 1 << lg;
    for (int o = G >> 1; o > 0; o >>= 1) acc.shfl_xor(0xffffffffu, o, G);
    return acc.shfl_from(0xffffffffu, ((threadIdx.x & 31) << lg) & 31);
}

// The row sums of the item holding rows [r0, r1).
template <typename T>
__device__ __forceinline__ Acc<T> item_sums(const Csr<T>& A, const T* __restrict__ x, int r0,
                                            int r1, int lg) {
    const int r = r0 + ((threadIdx.x & 31) >> lg);
    int b = 0, e = 0;
    if (r < r1) {
        b = __ldg(A.ptr + r);
        e = __ldg(A.ptr + r + 1);
    }
    return reduce_rows<T>(lane_products<T>(A, x, b, e, lg), lg);
}

// One warp item with its row steps in place: the epilogue's vector entries
// for the lane's row are loaded first (epi.load), then the row sums, then
// the row step (epi.apply) on the 32/G lanes that hold a row.
template <typename T, class E>
__device__ __forceinline__ void warp_item(const WarpSched& ws, const Csr<T>& A,
                                          const T* __restrict__ x, int w, E& epi) {
    const int lane = threadIdx.x & 31;
    const int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1);
    const int lg = __ldg(ws.lg + w);
    const int er = r0 + lane;
    const bool has_epi = lane < (32 >> lg) && er < r1;
    typename E::Pre pre{};
    if (has_epi) pre = epi.load(er);
    const Acc<T> mine = item_sums<T>(A, x, r0, r1, lg);
    if (has_epi) epi.apply(er, mine, pre);
}

// All warp items of the schedule, grid-stride over the launched warps
// (CTAs are sized to stay resident, so per-CTA costs are paid once).
// IGX_ITEM_PREFETCH=0 compiles the plain loop (one dependent load chain
// per item: schedule -> row pointers -> entries -> gathers). Pipelined,
// FP32 attempts took 70.0 -> 67.9 us on the multicommodity LP and
// 56.6 -> 55.1 us on the 200k x 500k LP, FP64 89.3 -> 87.7 us on the latter.
#ifndef IGX_ITEM_PREFETCH
#define IGX_ITEM_PREFETCH 1
#endif
template <typename T, class E>
__device__ __forceinline__ void warp_rows_all(const WarpSched& ws, const Csr<T>& A,
                                              const T* __restrict__ x, E& epi) {
    const int stride = gridDim.x * kWarps;
#if IGX_ITEM_PREFETCH
    // software-pipelined: the next item's schedule entries are loaded when
    // this item starts, and its row pointers between this item's products
    // and its reduction, so each item starts with [b, e) in registers
    const int lane = threadIdx.x & 31;
    int w = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (w >= ws.nwarps) return;
    int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1), lg = __ldg(ws.lg + w);
    int b = 0, e = 0;
    {
        const int r = r0 + (lane >> lg);
        if (r < r1) {
            b = __ldg(A.ptr + r);
            e = __ldg(A.ptr + r + 1);
        }
    }
    for (;;) {
        const int wn = w + stride;
        const bool more = wn < ws.nwarps;
        int n0 = 0, n1 = 0, nlg = 0;
        if (more) {
            n0 = __ldg(ws.row + wn);
            n1 = __ldg(ws.row + wn + 1);
            nlg = __ldg(ws.lg + wn);
        }
        const int er = r0 + lane;
        const bool has_epi = lane < (32 >> lg) && er < r1;
        typename E::Pre pre{};
        if (has_epi) pre = epi.load(er);
        const Acc<T> acc = lane_products<T>(A, x, b, e, lg);
        int nb = 0, ne = 0;
        if (more) {
            const int nr = n0 + (lane >> nlg);
            if (nr < n1) {
                nb = __ldg(A.ptr + nr);
                ne = __ldg(A.ptr + nr + 1);
            }
        }
        const Acc<T> mine = reduce_rows<T>(acc, lg);
        if (has_epi) epi.apply(er, mine, pre);
        if (!more) break;
        w = wn;
        r0 = n0;
        r1 = n1;
        lg = nlg;
        b = nb;
        e = ne;
    }
#else
    for (int w = blockIdx.x * kWarps + (threadIdx.x >> 5); w < ws.nwarps; w += stride)
        warp_item<T>(ws, A, x, w, epi);
#endif
}

}  // namespace igx
