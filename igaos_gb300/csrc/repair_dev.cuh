// Kernels of the matrix-free dual repair (device path of dual_repair for LPs
// whose dense m x m normal matrix does not fit: m > kRepairMaxRows).
//
// The reference repair (src/pdhg/pdhg.cu:288-448) alternates, from two
// anchors and for up to 300 rounds, three projections of the dual y:
//   1. onto { y : d_J = 0 } for the columns J strictly inside their bounds,
//      by a dense Cholesky solve of (A_J A_J^T + ridge) dy = -A_J d_J;
//   2. onto each column's sign half-space (d_j >= 0 for a column with only a
//      lower bound, <= 0 with only an upper bound, = 0 when free), one
//      column after the other (Hildreth);
//   3. onto the row cone (y_i >= 0 / <= 0 / = 0 on one-sided / free rows),
// and keeps the dual with the best finite gap. On the device the same three
// sets are projected on matrix-free:
//   1. the regularised least-squares step by CGLS on the Ruiz-scaled matrix
//      (two products per CG step, scalars kept on the device), moving only
//      the duals that are off the row cone's boundary;
//   2. all violated half-spaces at once, each row averaging the steps of the
//      violated columns it meets (component-averaged projections);
//   3. the row cone, fused into step 2.
// Signs, zero patterns and the inner set are invariant under the diagonal
// scaling (d~_j = dc_j d_j, y~_i = dr_i y_i), so the scaled iteration targets
// the same certificate; the gap is evaluated in original units by the KKT
// kernels.
#pragma once

#include "device.cuh"

namespace igx {

// Column setup: sign class (0 >= 0, 1 <= 0, 2 = 0, 3 any) from the original
// bounds, inner flag from the original x (band col_tol (1 + |bound|), as
// the reference), squared scaled column norm.
__global__ void k_rep_cols(int n, const int* __restrict__ cp, const double* __restrict__ acx,
                           const double* __restrict__ xs, const double* __restrict__ dc,
                           const double* __restrict__ cl, const double* __restrict__ cu,
                           double col_tol, signed char* __restrict__ sgn,
                           unsigned char* __restrict__ inj, double* __restrict__ nrm2) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double s2 = 0.0;
        for (int p = cp[j]; p < cp[j + 1]; ++p) s2 = fma(acx[p], acx[p], s2);
        nrm2[j] = s2;
        const double lo = cl[j], hi = cu[j];
        const bool up_inf = !isfinite(hi), lo_inf = !isfinite(lo);
        sgn[j] = (up_inf && lo_inf) ? 2 : up_inf ? 0 : lo_inf ? 1 : 3;
        const double x = xs[j] * dc[j];
        const double blo = col_tol * (1.0 + (isfinite(lo) ? fabs(lo) : 0.0));
        const double bhi = col_tol * (1.0 + (isfinite(hi) ? fabs(hi) : 0.0));
        inj[j] = (x - lo > blo && hi - x > bhi) ? 1 : 0;
    }
}

// Deterministic two-stage sums over n entries of (v * w) and of a 0/1 mask
// (w == nullptr: v alone; mask == nullptr: every entry): out[0] = sum
// mask*v*w, out[1] = sum mask.
struct RepSum {
    const double* v;
    const double* w;
    const unsigned char* mask;
    int n;
    double* part;
    double* out;
    unsigned int* ticket;
};
__global__ void k_rep_sum(RepSum a) {
    __shared__ double red[kWarps * 4];
    double s[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        if (a.mask && !a.mask[i]) continue;
        s[0] = fma(a.v[i], a.w ? a.w[i] : 1.0, s[0]);
        s[1] += 1.0;
    }
    block_sum<2>(s, red);
    if (threadIdx.x == 0) {
        a.part[2 * blockIdx.x] = s[0];
        a.part[2 * blockIdx.x + 1] = s[1];
    }
    if (!last_cta(a.ticket)) return;
    double t[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) {
        t[0] += a.part[2 * i];
        t[1] += a.part[2 * i + 1];
    }
    block_sum<2>(t, red);
    if (threadIdx.x == 0) {
        a.out[0] = t[0];
        a.out[1] = t[1];
    }
}

// Row cone of the dual from the original row bounds.
__device__ __forceinline__ double rep_cone(double y, double lo, double hi) {
    const bool fl = isfinite(lo), fh = isfinite(hi);
    if (fl && fh) return y;
    if (fh) return y < 0.0 ? 0.0 : y;   // <= row: y >= 0
    if (fl) return y > 0.0 ? 0.0 : y;   // >= row: y <= 0
    return 0.0;                         // free row
}

// y = cone(src) (src == nullptr: 0)
__global__ void k_rep_start(int m, const double* __restrict__ src, const double* __restrict__ rmin,
                            const double* __restrict__ rmax, double* __restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        y[i] = rep_cone(src ? src[i] : 0.0, rmin[i], rmax[i]);
}

// CGLS scalars, device side: s[0] gamma, s[3] alpha, s[4] beta, s[5]
// gamma0, s[6] ridge, s[8] active; sums land in s[9] ||q||^2, s[11] ||p||^2,
// s[13] gamma' (each sum also writes the slot after it).
__global__ void k_rep_cg_init(double* s) { s[5] = s[0]; }
__global__ void k_rep_cg_alpha(double* s, double rtol2) {
    const double delta = s[9] + s[6] * s[11];
    const bool active = s[0] > rtol2 * s[5] && delta > 0.0 && isfinite(delta);
    s[8] = active ? 1.0 : 0.0;
    s[3] = active ? s[0] / delta : 0.0;
}
__global__ void k_rep_cg_beta(double* s) {
    const bool active = s[8] != 0.0 && s[0] > 0.0;
    s[4] = active ? s[13] / s[0] : 0.0;
    if (active) s[0] = s[13];
}

// r_j = -(c~_j + (A~^T y)_j) on J, 0 elsewhere (aty holds A~^T y)
__global__ void k_rep_rinit(int n, const double* __restrict__ sc, const double* __restrict__ aty,
                            const unsigned char* __restrict__ inj, double* __restrict__ r) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        r[j] = inj[j] ? -(sc[j] + aty[j]) : 0.0;
}

// q restricted to J (in place)
__global__ void k_rep_mask(int n, const unsigned char* __restrict__ inj, double* __restrict__ q) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        if (!inj[j]) q[j] = 0.0;
}

// z += alpha p (m);  r -= alpha q (n)
__global__ void k_rep_zr(int m, int n, const double* __restrict__ s, const double* __restrict__ p,
                         double* __restrict__ z, const double* __restrict__ q,
                         double* __restrict__ r) {
    const double al = s[3];
    if (al == 0.0) return;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) z[i] = fma(al, p[i], z[i]);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) r[j] = fma(-al, q[j], r[j]);
}

// Rows the least-squares step may move: two-sided rows and one-sided rows
// whose dual is off the cone's boundary (0); free rows (cone {0}) never.
// Holding the rows at the boundary keeps the affine step from pushing duals
// out of the cone only for the clamp to push them back.
__global__ void k_rep_rowmask(int m, const double* __restrict__ y, const double* __restrict__ rmin,
                              const double* __restrict__ rmax, unsigned char* __restrict__ rm) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const bool fl = isfinite(rmin[i]), fh = isfinite(rmax[i]);
        rm[i] = (fl && fh) || ((fl || fh) && y[i] != 0.0) ? 1 : 0;
    }
}

// t = P (A~_J r) - ridge z, P the row mask (t holds A~ r on entry)
__global__ void k_rep_grad(int m, const double* __restrict__ s, const double* __restrict__ z,
                           const unsigned char* __restrict__ rm, double* __restrict__ t) {
    const double ridge = s[6];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        t[i] = rm[i] ? fma(-ridge, z[i], t[i]) : 0.0;
}

// p = t + beta p (first = 1: p = t)
__global__ void k_rep_dir(int m, const double* __restrict__ s, const double* __restrict__ t,
                          double* __restrict__ p, int first) {
    if (!first && s[8] == 0.0) return;
    const double be = first ? 0.0 : s[4];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        p[i] = first ? t[i] : fma(be, p[i], t[i]);
}

// y += z
__global__ void k_rep_addz(int m, const double* __restrict__ z, double* __restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        y[i] += z[i];
}

// Violated sign half-spaces: step_j = -d_j / ||a~_j||^2 where column j's
// reduced cost d_j = c~_j + (A~^T y)_j breaks its sign class, else 0.
__global__ void k_rep_sign(int n, const double* __restrict__ sc, const double* __restrict__ aty,
                           const signed char* __restrict__ sgn, const double* __restrict__ nrm2,
                           double* __restrict__ step) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const double d = sc[j] + aty[j];
        const int sg = sgn[j];
        double v = 0.0;
        if (sg == 0 && d < 0.0) v = -d;
        else if (sg == 1 && d > 0.0) v = -d;
        else if (sg == 2 && d != 0.0) v = -d;
        step[j] = (v != 0.0 && nrm2[j] > 0.0) ? v / nrm2[j] : 0.0;
    }
}

// Row update: y_i += (sum_j a~_ij step_j) / #(violated columns meeting row
// i), then the row cone. One thread per row of the CSR of A~.
__global__ void k_rep_rows(int m, const int* __restrict__ ap, const int* __restrict__ ai,
                           const double* __restrict__ ax, const double* __restrict__ step,
                           const double* __restrict__ rmin, const double* __restrict__ rmax,
                           double* __restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        double acc = 0.0;
        int cnt = 0;
        for (int p = ap[i]; p < ap[i + 1]; ++p) {
            const double st = step[ai[p]];
            if (st != 0.0 && ax[p] != 0.0) {
                acc = fma(ax[p], st, acc);
                ++cnt;
            }
        }
        const double yi = cnt > 0 ? y[i] + acc / (double)cnt : y[i];
        y[i] = rep_cone(yi, rmin[i], rmax[i]);
    }
}

}  // namespace igx
