// Small LPs: the line-search attempts of a chunk in one thread-block cluster.
//
// For an LP whose warp schedules give each warp of one cluster a few items,
// an attempt is a few microseconds of work and the grid-wide kernels spend
// it on launch latency and chains of dependent L2 loads (schedule -> row
// pointer -> entries -> gathers). One cluster of kSmallCluster CTAs instead
// runs the whole chunk in one launch, with the LP held on chip:
//   * each CTA stages its warps' rows of A~ and A~^T (row pointers, indices,
//     values) in shared memory once per launch;
//   * every CTA keeps a replica of the two gathered vectors (xbar and both
//     parity slots of y) in its shared memory; the PDHG step of a row writes
//     its new entry to every CTA's replica through distributed shared memory
//     (and to global memory for the host-side KKT checks);
//   * per attempt: primal half, cluster barrier, dual half, cluster barrier,
//     step decision by rank 0 (fixed-order merge of the per-CTA partials, the
//     same decide_step), cluster barrier.
// The control block, its step-factor table and the per-CTA partials stay in
// rank 0's shared memory for the launch (rank 0 writes the block back at the
// end). A warp keeps the same items for the whole launch, so its epilogue
// reads of its own rows see its own earlier global writes.
#pragma once

#include <cooperative_groups.h>

#include <type_traits>

#include "kernels.cuh"

namespace igx {

constexpr int kSmallCluster = 8;
constexpr int kSmallThreads = 512;
constexpr int kSmallWarps = kSmallThreads / 32;
constexpr int kSmallItems = 8;  // warp items per warp at most
constexpr size_t kSmallSmemMax = 200 * 1024;  // dynamic shared memory per CTA
constexpr int kFacEntries = 512;                // step-factor table entries staged

// Dynamic shared memory of one CTA (bytes) for a rank's staged rows.
struct SmallLayout {
    long long ent_at, rows_at, ent_a, rows_a;  // staged entries / row pointers
};
__host__ __device__ inline size_t small_smem_bytes(int m, int n, const SmallLayout& L, int s) {
    size_t b = (size_t)(n + 2 * (size_t)m) * s;                  // replicas
    b = (b + 15) & ~(size_t)15;
    b += (size_t)(L.ent_at + L.ent_a) * s;                       // values
    b = (b + 15) & ~(size_t)15;
    b += (size_t)(L.ent_at + L.ent_a) * 4 + (size_t)(L.rows_at + L.rows_a) * 4;
    return b + 64;
}

__device__ __forceinline__ int cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return (int)r;
}
__device__ __forceinline__ int cluster_count() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return (int)r;
}
// all threads of every CTA of the cluster; release/acquire at cluster scope
// (global and distributed shared memory)
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// One schedule's rows as staged by a CTA: entries and row pointers in
// shared memory (row pointers are local entry offsets), the warp's item
// descriptors {first row, end row, log2 G, first local row pointer}.
template <typename T>
struct Staged {
    const int* ptr;
    const int* idx;
    const T* val;
};

// Writes a row's new entry into the same slot of every CTA's replica.
template <typename T>
struct ClusterBcast {
    T* base;  // this CTA's replica
    int nr;
    __device__ __forceinline__ void operator()(int i, T v) const {
        cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        for (int r = 0; r < nr; ++r) *cl.map_shared_rank(base + i, r) = v;
    }
};

// Entries and row-pointer slots of the items w0, w0 + stride, ... of a
// schedule (one warp's share), counted the same way by the host to size the
// shared memory.
template <typename T>
__device__ __forceinline__ int2 stage_count(const WarpSched& ws, const Csr<T>& A, int w0,
                                            int stride) {
    int2 c{0, 0};
    for (int w = w0; w < ws.nwarps; w += stride) {
        const int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1);
        c.x += __ldg(A.ptr + r1) - __ldg(A.ptr + r0);
        c.y += r1 - r0 + 1;
    }
    return c;
}

// The warp copies its items' row pointers (rebased to its local entry
// offsets), indices and values into shared memory and records one
// descriptor {r0, r1, log2 G, first row-pointer slot} per item.
template <typename T>
__device__ __forceinline__ int stage_rows(const WarpSched& ws, const Csr<T>& A, int w0, int stride,
                                          int ent0, int row0, int* sptr, int* sidx, T* sval,
                                          int4* desc) {
    const int lane = threadIdx.x & 31;
    int k = 0, ce = ent0, cp = row0;
    for (int w = w0; w < ws.nwarps; w += stride, ++k) {
        const int r0 = __ldg(ws.row + w), r1 = __ldg(ws.row + w + 1);
        const int e0 = __ldg(A.ptr + r0), e1 = __ldg(A.ptr + r1);
        for (int t = lane; t <= r1 - r0; t += 32) sptr[cp + t] = __ldg(A.ptr + r0 + t) - e0 + ce;
        for (int q = lane; q < e1 - e0; q += 32) {
            sidx[ce + q] = __ldg(A.idx + e0 + q);
            sval[ce + q] = __ldg(A.val + e0 + q);
        }
        if (lane == 0) desc[k] = make_int4(r0, r1, __ldg(ws.lg + w), cp);
        cp += r1 - r0 + 1;
        ce += e1 - e0;
    }
    return k;
}

// warp_item on staged rows, x gathered from a shared-memory replica.
template <typename T, class E>
__device__ __forceinline__ void warp_item_staged(const int4 d, const Staged<T>& S,
                                                 const T* __restrict__ sx, E& epi) {
    const int lane = threadIdx.x & 31;
    const int r0 = d.x, nr = d.y - d.x, lg = d.z, pb = d.w;
    const int G = 1 << lg;
    const int g = lane >> lg, gl = lane & (G - 1);
    const bool has_epi = lane < (32 >> lg) && lane < nr;
    typename E::Pre pre{};
    if (has_epi) pre = epi.load(r0 + lane);
    Acc<T> acc;
    if (g < nr) {
        const int b = S.ptr[pb + g], e = S.ptr[pb + g + 1];
        for (int p = b + gl; p < e; p += kLaneBatch * G) {
            T a[kLaneBatch];
            int j[kLaneBatch];
#pragma unroll
            for (int u = 0; u < kLaneBatch; ++u) {
                const int q = p + u * G;
                const bool ok = q < e;
                a[u] = ok ? S.val[q] : T(0);
                j[u] = ok ? S.idx[q] : 0;
            }
#pragma unroll
            for (int u = 0; u < kLaneBatch; ++u) acc.add(a[u], sx[j[u]]);
        }
    }
    for (int o = G >> 1; o > 0; o >>= 1) acc.shfl_xor(0xffffffffu, o, G);
    const Acc<T> mine = acc.shfl_from(0xffffffffu, (lane << lg) & 31);
    if (has_epi) epi.apply(r0 + lane, mine, pre);
}

// The attempts of one chunk (up to max_attempts, until the control block's
// stop flag), one cluster of kSmallCluster CTAs. Dynamic shared memory:
// replicas xbar (n), y slot 0 (m), y slot 1 (m); then the staged values,
// indices and row pointers of A~^T (primal half) and A~ (dual half).
template <typename T>
__global__ void __cluster_dims__(kSmallCluster, 1, 1) __launch_bounds__(kSmallThreads, 1)
    k_attempts_cluster(PrimalArgs<T> pa, DualArgs<T> da, int m, int n, int max_attempts) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(16) double smred[kSmallWarps * 4];
    __shared__ int4 sdesc[2][kSmallWarps][kSmallItems];
    __shared__ int scnt[2][kSmallWarps + 1][2];
    __shared__ int snit[2][kSmallWarps];
    // control block, step-factor table and partials live in rank 0's shared
    // memory for the whole launch; every CTA holds the view of the step
    // being attempted, written by rank 0 through distributed shared memory
    __shared__ DevCtl sctl;
    __shared__ double sfac[2 * kFacEntries];
    __shared__ Acc<T> spart[3][kSmallCluster];
    __shared__ CtlView<T> sview;
    const int rank = cluster_rank(), nr = cluster_count();
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    // rank 0 thread 0: the view of the next attempt into every CTA
    auto publish = [&]() {
        CtlView<T> v;
        v.parity = sctl.parity;
        v.stop = sctl.stop;
        if constexpr (std::is_same<T, double>::value) {
            v.tau = sctl.tau;
            v.sigma = sctl.sigma;
            v.w = sctl.w;
            v.isigma = sctl.isigma;
        } else {
            v.tau = sctl.tau_f;
            v.sigma = sctl.sigma_f;
            v.w = sctl.w_f;
            v.isigma = sctl.isigma_f;
        }
        for (int r = 0; r < nr; ++r) *cl.map_shared_rank(&sview, r) = v;
    };
    const int wi = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
    const int w0 = rank * kSmallWarps + wi, stride = nr * kSmallWarps;

    // ---- layout: each warp's share of both schedules, prefix over warps
    {
        const int2 ca = stage_count<T>(pa.ws, pa.AT, w0, stride);
        const int2 cd = stage_count<T>(da.ws, da.A, w0, stride);
        if (lane == 0) {
            scnt[0][wi + 1][0] = ca.x;
            scnt[0][wi + 1][1] = ca.y;
            scnt[1][wi + 1][0] = cd.x;
            scnt[1][wi + 1][1] = cd.y;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; ++s) {
            scnt[s][0][0] = 0;
            scnt[s][0][1] = 0;
            for (int k = 1; k <= kSmallWarps; ++k) {
                scnt[s][k][0] += scnt[s][k - 1][0];
                scnt[s][k][1] += scnt[s][k - 1][1];
            }
        }
    }
    __syncthreads();
    const int ent_at = scnt[0][kSmallWarps][0], ent_a = scnt[1][kSmallWarps][0];
    const int rows_at = scnt[0][kSmallWarps][1];
    T* sxbar = reinterpret_cast<T*>(smem);
    T* sy[2] = {sxbar + n, sxbar + n + m};
    size_t off = ((size_t)(n + 2 * (size_t)m) * sizeof(T) + 15) & ~(size_t)15;
    T* val_at = reinterpret_cast<T*>(smem + off);
    T* val_a = val_at + ent_at;
    off = (off + (size_t)(ent_at + ent_a) * sizeof(T) + 15) & ~(size_t)15;
    int* idx_at = reinterpret_cast<int*>(smem + off);
    int* idx_a = idx_at + ent_at;
    int* ptr_at = idx_a + ent_a;
    int* ptr_a = ptr_at + rows_at;
    const int nit_at = stage_rows<T>(pa.ws, pa.AT, w0, stride, scnt[0][wi][0], scnt[0][wi][1],
                                     ptr_at, idx_at, val_at, sdesc[0][wi]);
    const int nit_a = stage_rows<T>(da.ws, da.A, w0, stride, scnt[1][wi][0], scnt[1][wi][1], ptr_a,
                                    idx_a, val_a, sdesc[1][wi]);
    if (lane == 0) {
        snit[0][wi] = nit_at;
        snit[1][wi] = nit_a;
    }
    if (rank == 0) {
        for (int i = threadIdx.x; i < 2 * da.n_fac && i < 2 * kFacEntries; i += kSmallThreads)
            sfac[i] = da.fac[i];
        if (threadIdx.x == 0) sctl = *pa.ctl;
    }
    {  // replica of the current dual slot
        const int p0 = __ldcg(&pa.ctl->parity);
        const T* yg = pa.y[p0];
        for (int i = threadIdx.x; i < m; i += kSmallThreads) sy[p0][i] = yg[i];
    }
    __syncthreads();
    cluster_barrier();  // every CTA running and staged before any remote write
    if (rank == 0 && threadIdx.x == 0) publish();
    cluster_barrier();
    const Staged<T> st_at{ptr_at, idx_at, val_at}, st_a{ptr_a, idx_a, val_a};

    for (int att = 0; att < max_attempts; ++att) {
        const CtlView<T> cv = sview;
        if (cv.stop) break;  // the same value in every CTA: published before the same barrier
        const int p = cv.parity, q = p ^ 1;
        {
            PrimalEpi<T, ClusterBcast<T>> epi{pa.c,    pa.lo,   pa.hi,  pa.x[p], pa.xavg[p],
                                              pa.x[q], pa.xavg[q], pa.xbar, cv.tau, cv.w,
                                              (T)0,    ClusterBcast<T>{sxbar, nr}};
            for (int k = 0; k < snit[0][wi]; ++k) warp_item_staged<T>(sdesc[0][wi][k], st_at, sy[p], epi);
            T v[1] = {epi.dx2};
            block_sum_t<T, 1, kSmallWarps>(v, reinterpret_cast<T*>(smred));
            if (threadIdx.x == 0) {
                Acc<T> e;
                e.s = v[0];
                *cl.map_shared_rank(&spart[0][rank], 0) = e;
            }
        }
        cluster_barrier();
        {
            DualEpi<T, ClusterBcast<T>> epi{da.rmin,    da.rmax, da.y[p],  da.axc[p], da.yavg[p],
                                            da.yhat,    da.y[q], da.axc[q], da.yavg[q], cv.sigma,
                                            cv.isigma,  cv.w,    (T)0,     (T)0,
                                            ClusterBcast<T>{sy[q], nr}};
            for (int k = 0; k < snit[1][wi]; ++k) warp_item_staged<T>(sdesc[1][wi][k], st_a, sxbar, epi);
            T v[2] = {epi.dy2, epi.cross};
            block_sum_t<T, 2, kSmallWarps>(v, reinterpret_cast<T*>(smred));
            if (threadIdx.x == 0) {
                Acc<T> e0, e1;
                e0.s = v[0];
                e1.s = v[1];
                *cl.map_shared_rank(&spart[1][rank], 0) = e0;
                *cl.map_shared_rank(&spart[2][rank], 0) = e1;
            }
        }
        cluster_barrier();
        if (rank == 0 && threadIdx.x == 0) {
            Acc<T> s0, s1, s2;
            for (int i = 0; i < nr; ++i) {
                s0.merge(spart[0][i]);
                s1.merge(spart[1][i]);
                s2.merge(spart[2][i]);
            }
            decide_step(&sctl, s0.result_d(), s1.result_d(), s2.result_d(), sfac,
                        da.n_fac < kFacEntries ? da.n_fac : kFacEntries);
            publish();
        }
        cluster_barrier();
    }
    if (rank == 0 && threadIdx.x == 0) *pa.ctl = sctl;  // the host reads it after the launch
}

}  // namespace igx
