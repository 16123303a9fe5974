// Differentiable LP layer: K unrolled PDHG iterations with fixed steps and
// their exact reverse mode (igaos_pdhg_unrolled_*).
//
// One CTA of 512 threads per instance; a thread owns fixed columns and rows.
// Every per-instance vector (iterates, adjoints, gradient accumulators) lives
// in shared memory. When the instance's matrix fits beside them it is staged
// into shared memory too -- values in both orientations (the CSC values
// gathered once through each entry's CSR position) with 16-bit indices -- so
// an iteration touches global memory only for checkpoints; otherwise the
// matrix is read from global memory (L2-resident for small batches).
//
// The forward stores (x_k, y_k) every `checkpoint` iterations. The backward
// walks the segments last to first: it replays a segment from its
// checkpoint, keeping each step's extrapolated primal x_bar, the dual y_k
// and the clamp outcome of every coordinate, then runs the segment's adjoint
// steps in reverse. The gradient of A's values is accumulated by the row
// pass alone (row i owns its nonzeros), in the CSR order of the input.
//
// Iteration (reference sign convention, d = c + A^T y; kern_primal /
// kern_dual in src/pdhg/pdhg.cu:33-58; ridge term in the primal prox):
//   g = c + A^T y;  v = (x - tau g) kappa, kappa = 1 / (1 + 2 ridge tau)
//   x+ = clamp(v, cl, cu);  xb = 2 x+ - x
//   t = y + sigma A xb;  y+ = t - sigma clamp(t / sigma, rmin, rmax)
// Clamps are differentiated almost everywhere: the gradient passes to the
// argument where it lies inside the bounds (ties included), to the bound
// where it lies strictly outside.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "device.cuh"
#include "engine.hpp"

namespace igx {
namespace {

constexpr int kLT = 512;  // threads per CTA of the forward and backward
constexpr int kLW = kLT / 32;

template <typename T>
struct UArgs {
    int K, ck;
    T ridge;
    const int *row_off, *col_off, *nz_off, *ap, *ai, *cp, *ci, *cperm;
    const T *c, *cl, *cu, *rmin, *rmax, *ax, *tau, *sigma;
    T *x, *y, *obj, *ckpt;
    long long nck;
    // backward
    const T *xK, *gx, *gy, *gobj;
    T *gc, *gcl, *gcu, *grmin, *grmax, *gax;
    T* seg;
    unsigned char* segf;
    // steps
    T omega;
    T *tau_o, *sigma_o;
};

struct UInst {
    int m, n, nnz, nz0;
    long long r0, c0;
};

template <typename T>
__device__ __forceinline__ UInst uinst(const UArgs<T>& a, int b) {
    UInst I;
    I.r0 = a.row_off[b];
    I.c0 = a.col_off[b];
    I.m = a.row_off[b + 1] - (int)I.r0;
    I.n = a.col_off[b + 1] - (int)I.c0;
    I.nz0 = a.nz_off[b];
    I.nnz = a.nz_off[b + 1] - I.nz0;
    return I;
}

// The instance's matrix: CSR (A x) and CSC values (A^T y), shared memory
// with 16-bit indices when resident, else global with 32-bit indices.
template <typename T, bool RES>
struct Mat {
    using Idx = typename std::conditional<RES, uint16_t, int>::type;
    const int* ap;
    const Idx* ai;
    const T* ax;
    const int* cp;
    const Idx* ci;
    const T* acx;       // resident: CSC values
    const int* cperm;   // global: CSR position of each CSC entry
    __device__ __forceinline__ T cval(int q) const {
        if constexpr (RES) return acx[q];
        else return ax[cperm[q]];
    }
};

// bytes of the staged matrix (T values first, then ints, then 16-bit indices)
__host__ __device__ inline size_t mat_bytes(int m, int n, long long nnz, size_t es) {
    return 2 * (size_t)nnz * es + (size_t)(m + 1 + n + 1) * 4 + 2 * (size_t)nnz * 2;
}

template <typename T, bool RES>
__device__ Mat<T, RES> load_mat(const UArgs<T>& a, const UInst& I, int b, unsigned char* base) {
    Mat<T, RES> M;
    const int* gap = a.ap + I.r0 + b;
    const int* gcp = a.cp + I.c0 + b;
    const int* gai = a.ai + I.nz0;
    const int* gci = a.ci + I.nz0;
    const int* gperm = a.cperm + I.nz0;
    const T* gax = a.ax + I.nz0;
    if constexpr (RES) {
        T* sax = reinterpret_cast<T*>(base);
        T* sacx = sax + I.nnz;
        int* sap = reinterpret_cast<int*>(sacx + I.nnz);
        int* scp = sap + I.m + 1;
        uint16_t* sai = reinterpret_cast<uint16_t*>(scp + I.n + 1);
        uint16_t* sci = sai + I.nnz;
        for (int p = threadIdx.x; p < I.nnz; p += kLT) {
            sax[p] = gax[p];
            sai[p] = (uint16_t)gai[p];
            sacx[p] = gax[gperm[p]];
            sci[p] = (uint16_t)gci[p];
        }
        for (int i = threadIdx.x; i <= I.m; i += kLT) sap[i] = gap[i];
        for (int j = threadIdx.x; j <= I.n; j += kLT) scp[j] = gcp[j];
        M.ap = sap;
        M.ai = sai;
        M.ax = sax;
        M.cp = scp;
        M.ci = sci;
        M.acx = sacx;
        M.cperm = nullptr;
    } else {
        M.ap = gap;
        M.ai = gai;
        M.ax = gax;
        M.cp = gcp;
        M.ci = gci;
        M.acx = nullptr;
        M.cperm = gperm;
    }
    return M;
}

// clamp with its outcome: 0 inside (ties included), 1 below lo, 2 above hi
template <typename T>
__device__ __forceinline__ T clampf(T v, T lo, T hi, int& f) {
    if (v < lo) {
        f = 1;
        return lo;
    }
    if (v > hi) {
        f = 2;
        return hi;
    }
    f = 0;
    return v;
}

// column pass of one forward step for column j; returns the clamp outcome
template <typename T, bool RES>
__device__ __forceinline__ int fwd_col(const UArgs<T>& a, const UInst& I, const Mat<T, RES>& M,
                                       int j, T* sx, T* sxb, const T* sy, T tau, T kappa) {
    const long long gj = I.c0 + j;
    T g = a.c[gj];
    for (int q = M.cp[j]; q < M.cp[j + 1]; ++q) g = fma(M.cval(q), sy[M.ci[q]], g);
    const T xv = sx[j];
    const T v = (xv - tau * g) * kappa;
    int f;
    const T xn = clampf(v, a.cl[gj], a.cu[gj], f);
    sxb[j] = T(2) * xn - xv;
    sx[j] = xn;
    return f;
}

// row pass of one forward step for row i; returns the clamp outcome
template <typename T, bool RES>
__device__ __forceinline__ int fwd_row(const UArgs<T>& a, const UInst& I, const Mat<T, RES>& M,
                                       int i, const T* sxb, T* sy, T sigma) {
    const long long gi = I.r0 + i;
    T z = T(0);
    for (int p = M.ap[i]; p < M.ap[i + 1]; ++p) z = fma(M.ax[p], sxb[M.ai[p]], z);
    const T t = fma(sigma, z, sy[i]);
    int f;
    const T pr = clampf(t / sigma, a.rmin[gi], a.rmax[gi], f);
    sy[i] = fma(-sigma, pr, t);
    return f;
}

template <typename T, bool RES>
__global__ void __launch_bounds__(kLT) k_unroll_fwd(UArgs<T> a) {
    extern __shared__ __align__(16) unsigned char u_smem[];
    __shared__ double red[kLW];
    const int b = blockIdx.x, t = threadIdx.x;
    const UInst I = uinst(a, b);
    const int m = I.m, n = I.n;
    T* sx = reinterpret_cast<T*>(u_smem);
    T* sxb = sx + n;
    T* sy = sxb + n;
    const Mat<T, RES> M = load_mat<T, RES>(a, I, b, reinterpret_cast<unsigned char*>(sy + m));
    const T tau = a.tau[b], sigma = a.sigma[b];
    const T kappa = T(1) / (T(1) + T(2) * a.ridge * tau);
    for (int j = t; j < n; j += kLT) {
        int f;
        sx[j] = clampf(T(0), a.cl[I.c0 + j], a.cu[I.c0 + j], f);
    }
    for (int i = t; i < m; i += kLT) sy[i] = T(0);
    T* ck = a.ckpt + a.nck * (I.c0 + I.r0);
    __syncthreads();
    for (int k = 0; k < a.K; ++k) {
        if (k % a.ck == 0) {
            T* slot = ck + (long long)(k / a.ck) * (n + m);
            for (int j = t; j < n; j += kLT) slot[j] = sx[j];
            for (int i = t; i < m; i += kLT) slot[n + i] = sy[i];
        }
        for (int j = t; j < n; j += kLT) fwd_col(a, I, M, j, sx, sxb, sy, tau, kappa);
        __syncthreads();
        for (int i = t; i < m; i += kLT) fwd_row(a, I, M, i, sxb, sy, sigma);
        __syncthreads();
    }
    double o = 0.0;
    for (int j = t; j < n; j += kLT) {
        const T xv = sx[j];
        a.x[I.c0 + j] = xv;
        o += (double)a.c[I.c0 + j] * (double)xv + (double)a.ridge * (double)xv * (double)xv;
    }
    for (int i = t; i < m; i += kLT) a.y[I.r0 + i] = sy[i];
    o = warp_sum(o);
    if ((t & 31) == 0) red[t >> 5] = o;
    __syncthreads();
    if (t == 0) {
        double s = 0.0;
        for (int w = 0; w < kLW; ++w) s += red[w];
        a.obj[b] = (T)s;
    }
}

template <typename T, bool RES>
__global__ void __launch_bounds__(kLT) k_unroll_bwd(UArgs<T> a) {
    extern __shared__ __align__(16) unsigned char u_smem[];
    const int b = blockIdx.x, t = threadIdx.x;
    const UInst I = uinst(a, b);
    const int m = I.m, n = I.n, nnz = I.nnz;
    // column vectors, row vectors, then (resident) A's gradient and matrix
    T* sx = reinterpret_cast<T*>(u_smem);
    T* sxb = sx + n;
    T* xh = sxb + n;
    T* gh = xh + n;
    T* gcs = gh + n;
    T* gcls = gcs + n;
    T* gcus = gcls + n;
    T* sy = gcus + n;
    T* yh = sy + m;
    T* zh = yh + m;
    T* th = zh + m;
    T* grl = th + m;
    T* grh = grl + m;
    T* gaxs = grh + m;  // resident: nnz values; global: unused
    T* gax = RES ? gaxs : a.gax + I.nz0;
    const Mat<T, RES> M =
        load_mat<T, RES>(a, I, b, reinterpret_cast<unsigned char*>(RES ? gaxs + nnz : gaxs));
    const T tau = a.tau[b], sigma = a.sigma[b];
    const T kappa = T(1) / (T(1) + T(2) * a.ridge * tau);
    const T go = a.gobj ? a.gobj[b] : T(0);
    // adjoints of the outputs; the objective adds c + 2 ridge x_K to x's
    // adjoint and x_K to c's gradient
    for (int j = t; j < n; j += kLT) {
        const long long gj = I.c0 + j;
        const T xk = a.xK[gj];
        xh[j] = (a.gx ? a.gx[gj] : T(0)) + go * (a.c[gj] + T(2) * a.ridge * xk);
        gcs[j] = go * xk;
        gcls[j] = T(0);
        gcus[j] = T(0);
    }
    for (int i = t; i < m; i += kLT) {
        yh[i] = a.gy ? a.gy[I.r0 + i] : T(0);
        grl[i] = T(0);
        grh[i] = T(0);
    }
    for (int p = t; p < nnz; p += kLT) gax[p] = T(0);
    const T* ck = a.ckpt + a.nck * (I.c0 + I.r0);
    T* seg = a.seg + (long long)a.ck * (I.c0 + I.r0);
    unsigned char* segf = a.segf + (long long)a.ck * (I.c0 + I.r0);
    const int nseg = (a.K + a.ck - 1) / a.ck;
    __syncthreads();
    for (int s = nseg - 1; s >= 0; --s) {
        const int k0 = s * a.ck, k1 = min(a.K, k0 + a.ck);
        const T* slot = ck + (long long)s * (n + m);
        for (int j = t; j < n; j += kLT) sx[j] = slot[j];
        for (int i = t; i < m; i += kLT) sy[i] = slot[n + i];
        __syncthreads();
        // replay: keep x_bar_k, y_k and the clamp outcomes of every step
        for (int k = k0; k < k1; ++k) {
            T* sk = seg + (long long)(k - k0) * (n + m);
            unsigned char* fk = segf + (long long)(k - k0) * (n + m);
            for (int j = t; j < n; j += kLT) {
                fk[j] = (unsigned char)fwd_col(a, I, M, j, sx, sxb, sy, tau, kappa);
                sk[j] = sxb[j];
            }
            __syncthreads();
            for (int i = t; i < m; i += kLT) {
                sk[n + i] = sy[i];
                fk[n + i] = (unsigned char)fwd_row(a, I, M, i, sxb, sy, sigma);
            }
            __syncthreads();
        }
        // reverse steps k1-1 .. k0
        for (int k = k1 - 1; k >= k0; --k) {
            const T* sk = seg + (long long)(k - k0) * (n + m);
            const unsigned char* fk = segf + (long long)(k - k0) * (n + m);
            // dual prox y+ = t - sigma clamp(t / sigma): dy+/dt = 1 where the
            // clamp is active, 0 inside; -sigma to the active bound
            for (int i = t; i < m; i += kLT) {
                const int f = fk[n + i];
                const T yv = yh[i];
                const T tv = f ? yv : T(0);
                if (f == 1) grl[i] -= sigma * yv;
                if (f == 2) grh[i] -= sigma * yv;
                th[i] = tv;
                zh[i] = sigma * tv;
            }
            __syncthreads();
            // A^T of the dual adjoint; primal prox and the extrapolation
            for (int j = t; j < n; j += kLT) {
                const T xb = sk[j];
                const int f = fk[j];
                T d = T(0);
                for (int q = M.cp[j]; q < M.cp[j + 1]; ++q) d = fma(M.cval(q), zh[M.ci[q]], d);
                sxb[j] = xb;
                const T xt = fma(T(2), d, xh[j]);
                const T vh = f ? T(0) : xt;
                if (f == 1) gcls[j] += xt;
                if (f == 2) gcus[j] += xt;
                const T g = -kappa * tau * vh;
                xh[j] = fma(kappa, vh, -d);
                gh[j] = g;
                gcs[j] += g;
            }
            __syncthreads();
            // A of the cost adjoint -> adjoint of y_k; A's value gradient
            // (from A x_bar and from A^T y) by the row that owns the entry
            for (int i = t; i < m; i += kLT) {
                const T yk = sk[n + i];
                const T zi = zh[i];
                T s2 = T(0);
                for (int p = M.ap[i]; p < M.ap[i + 1]; ++p) {
                    const int j = M.ai[p];
                    const T gj = gh[j];
                    s2 = fma(M.ax[p], gj, s2);
                    gax[p] = fma(yk, gj, fma(zi, sxb[j], gax[p]));
                }
                yh[i] = th[i] + s2;
            }
            // the next step's dual pass reads and writes only its own rows;
            // the column pass after it is behind a barrier
        }
        __syncthreads();
    }
    // x0 = clamp(0, cl, cu)
    for (int j = t; j < n; j += kLT) {
        const long long gj = I.c0 + j;
        T l = gcls[j], u = gcus[j];
        if (T(0) < a.cl[gj]) l += xh[j];
        else if (T(0) > a.cu[gj]) u += xh[j];
        a.gc[gj] = gcs[j];
        a.gcl[gj] = l;
        a.gcu[gj] = u;
    }
    for (int i = t; i < m; i += kLT) {
        a.grmin[I.r0 + i] = grl[i];
        a.grmax[I.r0 + i] = grh[i];
    }
    if constexpr (RES) {
        T* out = a.gax + I.nz0;
        for (int p = t; p < nnz; p += kLT) out[p] = gax[p];
    }
}

// eta = 0.9 / ||A||_2 by power iteration on A^T A from the uniform vector
template <typename T>
__global__ void __launch_bounds__(kThreads) k_unroll_steps(UArgs<T> a) {
    extern __shared__ __align__(16) unsigned char u_smem[];
    __shared__ double red[kWarps * 2];
    __shared__ double s_nrm;
    const int b = blockIdx.x, t = threadIdx.x;
    const UInst I = uinst(a, b);
    const int m = I.m, n = I.n;
    const int* ap = a.ap + I.r0 + b;
    const int* cp = a.cp + I.c0 + b;
    const int* ai = a.ai + I.nz0;
    const int* ci = a.ci + I.nz0;
    const int* cperm = a.cperm + I.nz0;
    const T* ax = a.ax + I.nz0;
    double* v = reinterpret_cast<double*>(u_smem);
    double* u = v + n;
    double* w = u + n;
    for (int j = t; j < n; j += kThreads) v[j] = 1.0 / sqrt((double)n);
    __syncthreads();
    double lam = 0.0;
    for (int it = 0; it < 100; ++it) {
        for (int i = t; i < m; i += kThreads) {
            double s = 0.0;
            for (int p = ap[i]; p < ap[i + 1]; ++p) s = fma((double)ax[p], v[ai[p]], s);
            w[i] = s;
        }
        __syncthreads();
        double nr[1] = {0.0};
        for (int j = t; j < n; j += kThreads) {
            double s = 0.0;
            for (int q = cp[j]; q < cp[j + 1]; ++q) s = fma((double)ax[cperm[q]], w[ci[q]], s);
            u[j] = s;
            nr[0] = fma(s, s, nr[0]);
        }
        block_sum<1>(nr, red);
        if (t == 0) s_nrm = sqrt(nr[0]);
        __syncthreads();
        lam = s_nrm;
        if (!(lam > 0.0)) break;
        for (int j = t; j < n; j += kThreads) v[j] = u[j] / lam;
        __syncthreads();
    }
    if (t == 0) {
        const double eta = (lam > 0.0 && isfinite(lam)) ? 0.9 / sqrt(lam) : 1.0;
        a.tau_o[b] = (T)(eta / (double)a.omega);
        a.sigma_o[b] = (T)(eta * (double)a.omega);
    }
}

int fail_cuda(cudaError_t e) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "CUDA error in PDHG unrolled layer: %s", cudaGetErrorString(e));
    return igx_set_error(IGAOS_PDHG_ERR_CUDA, buf);
}

int check_layout(const igaos_pdhg_unrolled_layout* L) {
    if (!L) return igx_set_error(IGAOS_PDHG_ERR_INVALID, "NULL layout");
    if (L->count <= 0) return igx_set_error(IGAOS_PDHG_ERR_INVALID, "count must be positive");
    if (L->precision != IGAOS_PDHG_FP32 && L->precision != IGAOS_PDHG_FP64)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "precision must be IGAOS_PDHG_FP32 or IGAOS_PDHG_FP64");
    if (L->iterations < 1 || L->checkpoint < 1)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "iterations and checkpoint must be >= 1");
    if (!(L->ridge >= 0.0) || !std::isfinite(L->ridge))
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "ridge must be finite and >= 0");
    if (L->max_m < 1 || L->max_n < 1 || L->total_m < L->max_m || L->total_n < L->max_n ||
        L->max_nnz < 0 || L->total_nnz < L->max_nnz)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "inconsistent layout sizes");
    if (!L->row_off || !L->col_off || !L->nz_off || !L->ap || !L->ai || !L->cp || !L->ci ||
        !L->cperm)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "NULL layout array");
    return IGAOS_PDHG_OK;
}

size_t elem_size(const igaos_pdhg_unrolled_layout* L) {
    return L->precision == IGAOS_PDHG_FP64 ? sizeof(double) : sizeof(float);
}

// shared memory of each kernel for the largest instance
size_t vec_fwd(const igaos_pdhg_unrolled_layout* L) {
    return (size_t)(2 * (size_t)L->max_n + L->max_m) * elem_size(L);
}
size_t vec_bwd(const igaos_pdhg_unrolled_layout* L) {
    return (size_t)(7 * (size_t)L->max_n + 6 * (size_t)L->max_m) * elem_size(L);
}
size_t mat_res(const igaos_pdhg_unrolled_layout* L) {
    return mat_bytes(L->max_m, L->max_n, L->max_nnz, elem_size(L));
}

int smem_optin(int* optin) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return e == cudaSuccess ? IGAOS_PDHG_OK : fail_cuda(e);
}

template <typename T>
UArgs<T> base_args(const igaos_pdhg_unrolled_layout* L) {
    UArgs<T> a{};
    a.K = L->iterations;
    a.ck = L->checkpoint;
    a.ridge = (T)L->ridge;
    a.row_off = L->row_off;
    a.col_off = L->col_off;
    a.nz_off = L->nz_off;
    a.ap = L->ap;
    a.ai = L->ai;
    a.cp = L->cp;
    a.ci = L->ci;
    a.cperm = L->cperm;
    a.nck = (L->iterations + L->checkpoint - 1) / L->checkpoint;
    return a;
}

template <typename K>
cudaError_t set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int too_large(size_t need, int optin) {
    char buf[192];
    std::snprintf(buf, sizeof(buf),
                  "instance too large for the unrolled layer: needs %zu bytes of shared memory "
                  "per CTA, device allows %d", need, optin);
    return igx_set_error(IGAOS_PDHG_ERR_INVALID, buf);
}

// static shared memory of the layer kernels stays below this
constexpr size_t kStaticSmem = 1024;

// staged (resident) matrix needs 16-bit indices and room beside the vectors
// and the kernel's static shared memory
bool resident(const igaos_pdhg_unrolled_layout* L, size_t vec, int optin) {
    return L->max_m <= 65536 && L->max_n <= 65536 &&
           vec + mat_res(L) + kStaticSmem <= (size_t)optin;
}

template <typename T>
int run_steps(const igaos_pdhg_unrolled_layout* L, const void* ax, double omega, void* tau,
              void* sigma, cudaStream_t st) {
    UArgs<T> a = base_args<T>(L);
    a.ax = static_cast<const T*>(ax);
    a.tau_o = static_cast<T*>(tau);
    a.sigma_o = static_cast<T*>(sigma);
    a.omega = (T)omega;
    const size_t sm = (size_t)(2 * L->max_n + L->max_m) * sizeof(double);
    cudaError_t e = set_smem(k_unroll_steps<T>, sm);
    if (e == cudaSuccess) {
        k_unroll_steps<T><<<L->count, kThreads, sm, st>>>(a);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? igx_set_error(IGAOS_PDHG_OK, "") : fail_cuda(e);
}

template <typename T>
int run_forward(const igaos_pdhg_unrolled_layout* L, const void* c, const void* cl,
                const void* cu, const void* rmin, const void* rmax, const void* ax,
                const void* tau, const void* sigma, void* x, void* y, void* obj, void* ckpt,
                cudaStream_t st, int optin) {
    UArgs<T> a = base_args<T>(L);
    a.c = static_cast<const T*>(c);
    a.cl = static_cast<const T*>(cl);
    a.cu = static_cast<const T*>(cu);
    a.rmin = static_cast<const T*>(rmin);
    a.rmax = static_cast<const T*>(rmax);
    a.ax = static_cast<const T*>(ax);
    a.tau = static_cast<const T*>(tau);
    a.sigma = static_cast<const T*>(sigma);
    a.x = static_cast<T*>(x);
    a.y = static_cast<T*>(y);
    a.obj = static_cast<T*>(obj);
    a.ckpt = static_cast<T*>(ckpt);
    const size_t vec = vec_fwd(L);
    cudaError_t e;
    if (resident(L, vec, optin)) {
        const size_t sm = vec + mat_res(L);
        e = set_smem(k_unroll_fwd<T, true>, sm);
        if (e == cudaSuccess) k_unroll_fwd<T, true><<<L->count, kLT, sm, st>>>(a);
    } else {
        e = set_smem(k_unroll_fwd<T, false>, vec);
        if (e == cudaSuccess) k_unroll_fwd<T, false><<<L->count, kLT, vec, st>>>(a);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? igx_set_error(IGAOS_PDHG_OK, "") : fail_cuda(e);
}

template <typename T>
int run_backward(const igaos_pdhg_unrolled_layout* L, const void* c, const void* cl,
                 const void* cu, const void* rmin, const void* rmax, const void* ax,
                 const void* tau, const void* sigma, const void* ckpt, const void* x,
                 const void* gx, const void* gy, const void* gobj, void* gc, void* gcl,
                 void* gcu, void* grmin, void* grmax, void* gax, void* work, cudaStream_t st,
                 int optin) {
    UArgs<T> a = base_args<T>(L);
    a.c = static_cast<const T*>(c);
    a.cl = static_cast<const T*>(cl);
    a.cu = static_cast<const T*>(cu);
    a.rmin = static_cast<const T*>(rmin);
    a.rmax = static_cast<const T*>(rmax);
    a.ax = static_cast<const T*>(ax);
    a.tau = static_cast<const T*>(tau);
    a.sigma = static_cast<const T*>(sigma);
    a.ckpt = const_cast<T*>(static_cast<const T*>(ckpt));
    a.xK = static_cast<const T*>(x);
    a.gx = static_cast<const T*>(gx);
    a.gy = static_cast<const T*>(gy);
    a.gobj = static_cast<const T*>(gobj);
    a.gc = static_cast<T*>(gc);
    a.gcl = static_cast<T*>(gcl);
    a.gcu = static_cast<T*>(gcu);
    a.grmin = static_cast<T*>(grmin);
    a.grmax = static_cast<T*>(grmax);
    a.gax = static_cast<T*>(gax);
    const long long per = (long long)L->checkpoint * (L->total_n + L->total_m);
    const long long vb = (per * (long long)sizeof(T) + 255) / 256 * 256;
    a.seg = static_cast<T*>(work);
    a.segf = static_cast<unsigned char*>(work) + vb;
    const size_t vec = vec_bwd(L);
    const size_t grad = (size_t)L->max_nnz * sizeof(T);
    cudaError_t e;
    if (resident(L, vec + grad, optin)) {
        const size_t sm = vec + grad + mat_res(L);
        e = set_smem(k_unroll_bwd<T, true>, sm);
        if (e == cudaSuccess) k_unroll_bwd<T, true><<<L->count, kLT, sm, st>>>(a);
    } else {
        e = set_smem(k_unroll_bwd<T, false>, vec);
        if (e == cudaSuccess) k_unroll_bwd<T, false><<<L->count, kLT, vec, st>>>(a);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? igx_set_error(IGAOS_PDHG_OK, "") : fail_cuda(e);
}

// common checks of the three entry points; fills the opt-in shared memory
int prepare(const igaos_pdhg_unrolled_layout* L, int* optin) {
    int rc = check_layout(L);
    if (rc != IGAOS_PDHG_OK) return rc;
    if ((rc = smem_optin(optin)) != IGAOS_PDHG_OK) return rc;
    const size_t need = std::max(vec_bwd(L), (size_t)(2 * L->max_n + L->max_m) * sizeof(double));
    if (need + kStaticSmem > (size_t)*optin) return too_large(need, *optin);
    return IGAOS_PDHG_OK;
}

}  // namespace
}  // namespace igx

extern "C" int64_t igaos_pdhg_unrolled_checkpoint_elems(const igaos_pdhg_unrolled_layout* L) {
    if (igx::check_layout(L) != IGAOS_PDHG_OK) return -1;
    const int64_t nck = (L->iterations + L->checkpoint - 1) / L->checkpoint;
    return nck * (L->total_n + L->total_m);
}

extern "C" int64_t igaos_pdhg_unrolled_workspace_bytes(const igaos_pdhg_unrolled_layout* L) {
    if (igx::check_layout(L) != IGAOS_PDHG_OK) return -1;
    const int64_t per = (int64_t)L->checkpoint * (L->total_n + L->total_m);
    // values, then one clamp-outcome byte per value after a 256-byte boundary
    const int64_t vb = ((per * (int64_t)igx::elem_size(L)) + 255) / 256 * 256;
    return vb + per;
}

extern "C" int igaos_pdhg_unrolled_steps(const igaos_pdhg_unrolled_layout* L, const void* ax,
                                         double omega, void* tau, void* sigma, void* stream) {
    using namespace igx;
    int optin = 0;
    int rc = prepare(L, &optin);
    if (rc != IGAOS_PDHG_OK) return rc;
    if (!ax || !tau || !sigma) return igx_set_error(IGAOS_PDHG_ERR_INVALID, "NULL device pointer");
    if (!(omega > 0.0) || !std::isfinite(omega))
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "omega must be positive and finite");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return L->precision == IGAOS_PDHG_FP64 ? run_steps<double>(L, ax, omega, tau, sigma, st)
                                           : run_steps<float>(L, ax, omega, tau, sigma, st);
}

extern "C" int igaos_pdhg_unrolled_forward(const igaos_pdhg_unrolled_layout* L, const void* c,
                                           const void* cl, const void* cu, const void* rmin,
                                           const void* rmax, const void* ax, const void* tau,
                                           const void* sigma, void* x, void* y, void* obj,
                                           void* ckpt, void* stream) {
    using namespace igx;
    int optin = 0;
    int rc = prepare(L, &optin);
    if (rc != IGAOS_PDHG_OK) return rc;
    if (!c || !cl || !cu || !rmin || !rmax || !ax || !tau || !sigma || !x || !y || !obj || !ckpt)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "NULL device pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return L->precision == IGAOS_PDHG_FP64
               ? run_forward<double>(L, c, cl, cu, rmin, rmax, ax, tau, sigma, x, y, obj, ckpt,
                                     st, optin)
               : run_forward<float>(L, c, cl, cu, rmin, rmax, ax, tau, sigma, x, y, obj, ckpt,
                                    st, optin);
}

extern "C" int igaos_pdhg_unrolled_backward(const igaos_pdhg_unrolled_layout* L, const void* c,
                                            const void* cl, const void* cu, const void* rmin,
                                            const void* rmax, const void* ax, const void* tau,
                                            const void* sigma, const void* ckpt, const void* x,
                                            const void* gx, const void* gy, const void* gobj,
                                            void* gc, void* gcl, void* gcu, void* grmin,
                                            void* grmax, void* gax, void* work, void* stream) {
    using namespace igx;
    int optin = 0;
    int rc = prepare(L, &optin);
    if (rc != IGAOS_PDHG_OK) return rc;
    if (!c || !cl || !cu || !rmin || !rmax || !ax || !tau || !sigma || !ckpt || !x || !gc ||
        !gcl || !gcu || !grmin || !grmax || !gax || !work)
        return igx_set_error(IGAOS_PDHG_ERR_INVALID, "NULL device pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return L->precision == IGAOS_PDHG_FP64
               ? run_backward<double>(L, c, cl, cu, rmin, rmax, ax, tau, sigma, ckpt, x, gx, gy,
                                      gobj, gc, gcl, gcu, grmin, grmax, gax, work, st, optin)
               : run_backward<float>(L, c, cl, cu, rmin, rmax, ax, tau, sigma, ckpt, x, gx, gy,
                                     gobj, gc, gcl, gcu, grmin, grmax, gax, work, st, optin);
}
