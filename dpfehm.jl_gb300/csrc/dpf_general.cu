// dpf_general.cu -- CSR (general topology) groundwater solver for sm_103a.
//
// The same algorithms as the structured path (flux-form operator with identity
// Dirichlet rows, aggregation multigrid with Chebyshev smoothing and a dense
// coarsest inverse, FP64 CG or double-float CG with an FP32 V-cycle, rrule adjoint,
// backward-Euler transient with its adjoint) on an arbitrary face list:
//   A h = b, A = groundwater_h, b = -groundwater_residuals(0)   (src/groundwater.jl:75-83)
// Kernels are grid-stride loops over cells, couplings or faces; every reduction is
// deterministic (fixed partial slots, finalised by the last block).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "dpf_direct.h"
#include "dpf_general.h"
#include "dpf_struct_kernels.cuh"

namespace dpf {

#define GSTRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// ------------------------------------------------------------ operator
template <typename T>
struct GOp {
    const int *rp, *ci;
    const T *v, *leak, *idg;
    int n;                         // rows (= columns)
};

// flux form y_i = leak_i x_i + sum_e c_e (x_i - x_j); also returns the diagonal
template <typename T, typename XAt>
__device__ __forceinline__ T g_apply(int i, const GOp<T> &A, T xi, XAt xat, T &diag) {
    T lk = A.leak[i];
    T a = lk * xi, d = lk;
    for (int e = A.rp[i]; e < A.rp[i + 1]; e++) {
        const int j = A.ci[e];
        if (!DPF_INSIDE(CK_CSR_COL, j, 0, A.n)) continue;
        T w = A.v[e];
        a += w * (xi - xat(j));
        d += w;
    }
    diag = d;
    return a;
}

__device__ __forceinline__ int other_end(const int *fa, const int *fb, int f, int i) {
    return fa[f] == i ? fb[f] : fa[f];
}

__device__ __forceinline__ double g_face_k(const double *Ks, const double *kc, int kind, const int *fa, const int *fb,
                                           int f) {
    return Ks ? Ks[f] : face_mean_k(kc[fa[f]], kc[fb[f]], kind);
}

// ------------------------------------------------------------ set-up kernels
__global__ void kg_cell_k(int n, const double *__restrict__ logK, int kind, double *__restrict__ kc) {
    GSTRIDE(i, n) {
        double v = logK[i];
        kc[i] = exp(kind == DPF_MEAN_GEOMETRIC ? 0.5 * v : v);
    }
}

__global__ void kg_faces(int F, const int *__restrict__ fa, const int *__restrict__ fb, const double *__restrict__ kc,
                         int kind, double *__restrict__ Ks) {
    GSTRIDE(f, F) Ks[f] = face_mean_k(kc[fa[f]], kc[fb[f]], kind);
}

// dlogK_i = sum over the faces of i of dK_f/dlogK_i dKs_f
__global__ void kg_vjp(int n, const int *__restrict__ irp, const int *__restrict__ ifc, const int *__restrict__ fa,
                       const int *__restrict__ fb, const double *__restrict__ kc, int kind,
                       const double *__restrict__ dKs, double *__restrict__ g) {
    GSTRIDE(i, n) {
        double ki = kc[i], acc = 0.0;
        for (int k = irp[i]; k < irp[i + 1]; k++) {
            int f = ifc[k];
            double K = face_mean_k(ki, kc[other_end(fa, fb, f, i)], kind);
            acc += face_mean_dlogk(K, ki, kind) * dKs[f];
        }
        g[i] = acc;
    }
}

// leak, right-hand side and initial guess of every cell (src/groundwater.jl:4-20)
__global__ void kg_assemble(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                            const int *__restrict__ fa, const int *__restrict__ fb, const double *__restrict__ faol,
                            const double *__restrict__ Ks, const double *__restrict__ kc, int kind,
                            const uint8_t *__restrict__ dir, const double *__restrict__ dh,
                            const double *__restrict__ Qs, const double *__restrict__ shift, double *__restrict__ leak,
                            double *__restrict__ b, double *__restrict__ x, int init_x) {
    GSTRIDE(i, n) {
        const bool fi = !dir[i];
        double lk = 0.0, rhs = fi ? Qs[i] : dh[i];
        if (fi) {
            for (int k = irp[i]; k < irp[i + 1]; k++) {
                int f = ifc[k];
                int j = other_end(fa, fb, f, i);
                if (!dir[j]) continue;
                double c = g_face_k(Ks, kc, kind, fa, fb, f) * faol[f];
                lk += c;
                rhs += c * dh[j];
            }
            if (shift) lk += shift[i];
        } else {
            lk = 1.0;
        }
        leak[i] = lk;
        b[i] = rhs;
        if (init_x) x[i] = fi ? 0.0 : dh[i];
        else if (!fi) x[i] = dh[i];
    }
}

__global__ void kg_entry_vals(int nnz, const int *__restrict__ e_face, const int *__restrict__ fa,
                              const int *__restrict__ fb, const double *__restrict__ faol,
                              const double *__restrict__ Ks, const double *__restrict__ kc, int kind,
                              double *__restrict__ v) {
    GSTRIDE(e, nnz) {
        int f = e_face[e];
        v[e] = g_face_k(Ks, kc, kind, fa, fb, f) * faol[f];
    }
}

// coarse coupling = sum of the fine couplings between its two aggregates
__global__ void kg_coarse_vals(int nnz_c, const int *__restrict__ crp, const int *__restrict__ cci,
                               const double *__restrict__ vf, double *__restrict__ vc) {
    GSTRIDE(e, nnz_c) {
        double s = 0.0;
        for (int k = crp[e]; k < crp[e + 1]; k++) s += vf[cci[k]];
        vc[e] = s;
    }
}

// coarse leak = sum of the members' leaks (members are free cells)
__global__ void kg_coarse_leak(int nc, const int *__restrict__ mrp, const int *__restrict__ mci,
                               const double *__restrict__ leak_f, double *__restrict__ leak_c, uint8_t *dir_c) {
    GSTRIDE(I, nc) {
        double s = 0.0;
        for (int k = mrp[I]; k < mrp[I + 1]; k++) s += leak_f[mci[k]];
        leak_c[I] = s;
        dir_c[I] = 0;
    }
}

__global__ void kg_invdiag(int n, const int *__restrict__ rp, const double *__restrict__ v,
                           const double *__restrict__ leak, double *__restrict__ idg64, float *__restrict__ idg32) {
    GSTRIDE(i, n) {
        double d = leak[i];
        for (int e = rp[i]; e < rp[i + 1]; e++) d += v[e];
        double g = 1.0 / d;
        if (idg64) idg64[i] = g;
        if (idg32) idg32[i] = (float)g;
    }
}

__global__ void kg_to_float(int n, const double *__restrict__ a, float *__restrict__ b) {
    GSTRIDE(i, n) b[i] = (float)a[i];
}

__global__ void kg_to_df(int n, const double *__restrict__ a, float2 *__restrict__ b) {
    GSTRIDE(i, n) b[i] = df_from_double(a[i]);
}

// dense inverse of the coarsest operator (n <= 64), Gauss-Jordan in shared memory
__global__ void kg_dense_inverse(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                 const double *__restrict__ v, const double *__restrict__ leak, double *Inv,
                                 int *status) {
    __shared__ double A[kMaxCoarse][kMaxCoarse + 1];
    __shared__ double col[kMaxCoarse];
    __shared__ int bad;
    for (int k = threadIdx.x; k < kMaxCoarse * kMaxCoarse; k += blockDim.x) A[k / kMaxCoarse][k % kMaxCoarse] = 0.0;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double d = leak[i];
        for (int e = rp[i]; e < rp[i + 1]; e++) {
            d += v[e];
            A[i][ci[e]] -= v[e];
        }
        A[i][i] += d;
    }
    __syncthreads();
    for (int k = 0; k < n; k++) {
        double piv = A[k][k];
        if (!(piv > 0.0)) { if (threadIdx.x == 0) bad = 1; piv = 1.0; }
        double ip = 1.0 / piv;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) col[i] = A[i][k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) A[k][j] = (j == k ? 1.0 : A[k][j]) * ip;
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            int i = t / n, j = t % n;
            if (i == k) continue;
            A[i][j] = (j == k ? 0.0 : A[i][j]) - col[i] * A[k][j];
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < kMaxCoarse * kMaxCoarse; k += blockDim.x) {
        int i = k / kMaxCoarse, j = k % kMaxCoarse;
        Inv[k] = (i < n && j < n) ? A[i][j] : 0.0;
    }
    if (threadIdx.x == 0 && bad) atomicExch(status, 1);
}

// ------------------------------------------------------------ V-cycle kernels
template <typename T>
__device__ __forceinline__ T g_dinv(const GOp<T> &A, int i, T v, T dg) {
    if constexpr (sizeof(T) == 8) return v * A.idg[i];
    else return __fdividef(v, dg);
}

__device__ __forceinline__ bool g_active(const CgState *st) { return st == nullptr || st[0].active; }

template <typename T>
__global__ void kg_cheb_first2(int n, const CgState *st, GOp<T> A, const T *__restrict__ b, T *__restrict__ xout,
                               T *__restrict__ d, T invtheta, T c1, T c2) {
    if (!g_active(st)) return;
    GSTRIDE(i, n) {
        const T bi = b[i], gi = A.idg[i];
        const T x1 = invtheta * bi * gi;
        T dg;
        T Ax = g_apply<T>(i, A, x1, [&](int j) { return invtheta * b[j] * A.idg[j]; }, dg);
        const T dn = c1 * x1 + c2 * (bi - Ax) * gi;
        d[i] = dn;
        xout[i] = x1 + dn;
    }
}

template <typename T>
__global__ void kg_cheb_first(int n, const CgState *st, GOp<T> A, const T *__restrict__ b, T *__restrict__ x,
                              T *__restrict__ d, T invtheta) {
    if (!g_active(st)) return;
    GSTRIDE(i, n) {
        T v = invtheta * b[i] * A.idg[i];
        x[i] = v;
        d[i] = v;
    }
}

template <typename T, bool FUSE_RZ, bool FIRST>
__global__ void kg_cheb_step(int n, CgState *st, GOp<T> A, const T *__restrict__ b, const T *__restrict__ xin,
                             T *__restrict__ xout, T *__restrict__ d, T c1, T c2, ReduceScratch rs) {
    if (!g_active(st)) return;
    Acc<T> part;
    GSTRIDE(i, n) {
        T xi = xin[i], dg;
        T Ax = g_apply<T>(i, A, xi, [&](int j) { return xin[j]; }, dg);
        T bi = b[i];
        T r = g_dinv(A, i, bi - Ax, dg);
        T dn = FIRST ? c2 * r : c1 * d[i] + c2 * r;
        T xo = xi + dn;
        d[i] = dn;
        xout[i] = xo;
        if (FUSE_RZ) part = part + Acc<T>::prod(bi, xo);
    }
    if (FUSE_RZ) {
        double2 tot;
        if (reduce_last<T>(part, Acc<T>(), rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
            CgState &s = st[0];
            s.rz_old = s.rz;
            s.rz = tot.x;
            s.beta = (s.iters == 0 || s.rz_old == 0.0) ? 0.0 : s.rz / s.rz_old;
        }
    }
}

// Restriction b_c = sum over the aggregate's members of (b - A x), in two passes: the residual of
// every fine cell (a thread per cell, so the work is spread evenly however uneven the aggregates
// are), then per coarse cell the sum over its members in member order. A thread per coarse cell
// applying every member's row in turn was up to 5x slower on coarse levels of fracture networks,
// whose large or uneven aggregates left most threads waiting on a few.
template <typename T>
__global__ void kg_resid(int n, const CgState *st, GOp<T> A, const T *__restrict__ b, const T *__restrict__ x,
                         T *__restrict__ r) {
    if (!g_active(st)) return;
    GSTRIDE(i, n) {
        T dg;
        r[i] = b[i] - g_apply<T>(i, A, x[i], [&](int j) { return x[j]; }, dg);
    }
}
template <typename T>
__global__ void kg_restrict_sum(int nc, const CgState *st, const int *__restrict__ mrp, const int *__restrict__ mci,
                                const T *__restrict__ r, T *__restrict__ bc) {
    if (!g_active(st)) return;
    GSTRIDE(I, nc) {
        T acc = 0;
        for (int k = mrp[I]; k < mrp[I + 1]; k++) acc += r[mci[k]];
        bc[I] = acc;
    }
}

template <typename T>
__global__ void kg_prolong_add(int n, const CgState *st, const int *__restrict__ agg, const uint8_t *__restrict__ dir,
                               T *__restrict__ x, const T *__restrict__ e, T scale) {
    if (!g_active(st)) return;
    GSTRIDE(i, n) {
        int a = agg[i];
        if (a >= 0 && !dir[i]) x[i] += scale * e[a];
    }
}

template <typename T, bool FUSE_RZ>
__global__ void kg_coarse_solve(int n, CgState *st, const double *__restrict__ Inv, const T *__restrict__ b,
                                T *__restrict__ x) {
    if (!g_active(st)) return;
    __shared__ double bs[kMaxCoarse];
    __shared__ double red[kMaxCoarse / 32];
    const int i = threadIdx.x;
    if (i < n) bs[i] = (double)b[i];
    __syncthreads();
    double xi = 0.0;
    if (i < n)
        for (int j = 0; j < n; j++) xi += Inv[j * kMaxCoarse + i] * bs[j];
    T xo = (T)xi;
    if (i < n) x[i] = xo;
    if (FUSE_RZ) {
        double v = i < n ? bs[i] * (double)xo : 0.0;
        v = warp_sum(v);
        if ((i & 31) == 0) red[i >> 5] = v;
        __syncthreads();
        if (i == 0) {
            double rz = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) rz += red[w];
            CgState &s = st[0];
            s.rz_old = s.rz;
            s.rz = rz;
            s.beta = (s.iters == 0 || s.rz_old == 0.0) ? 0.0 : s.rz / s.rz_old;
        }
    }
}

// ------------------------------------------------------------ CG kernels (FP64)
// |b| over the free rows only (identity rows hold their Dirichlet values exactly; the
// reference measures reltol against the free cells' right-hand side)
__global__ void kg_cg_start(int n, CgState *st, int *active_count, ReduceScratch rs, GOp<double> A,
                            const uint8_t *__restrict__ dir, const double *__restrict__ b,
                            const double *__restrict__ x, double *__restrict__ r, double tol2) {
    Acc<double> rr, bb;
    GSTRIDE(i, n) {
        double dg;
        double ri = b[i] - g_apply<double>(i, A, x[i], [&](int j) { return x[j]; }, dg);
        r[i] = ri;
        rr.v += ri * ri;
        if (!dir[i]) bb.v += b[i] * b[i];
    }
    double2 tot;
    if (reduce_last<double, 2>(rr, bb, rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
        CgState &s = st[0];
        s.rr = tot.x;
        s.bb = tot.y;
        s.tol2 = tol2;
        s.iters = 0;
        s.total_iters = 0;
        s.rz = s.rz_old = s.beta = 0.0;
        s.status = DPF_OK;
        bool act = s.bb > 0.0 && s.rr > tol2 * s.bb;
        if (!isfinite(s.rr)) { s.status = DPF_NAN; act = false; }
        s.active = act ? 1 : 0;
        if (act) atomicAdd(active_count, 1);
    }
}

__global__ void kg_spmv_pq(int n, CgState *st, int *active_count, ReduceScratch rs, GOp<double> A,
                           const double *__restrict__ pv, double *__restrict__ q) {
    if (!st[0].active) return;
    Acc<double> part;
    GSTRIDE(i, n) {
        double dg;
        double a = g_apply<double>(i, A, pv[i], [&](int j) { return pv[j]; }, dg);
        q[i] = a;
        part.v += pv[i] * a;
    }
    double2 tot;
    if (reduce_last<double>(part, Acc<double>(), rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
        CgState &s = st[0];
        s.pq = tot.x;
        if (!isfinite(s.pq)) { s.alpha = 0.0; s.status = DPF_NAN; deactivate(s, active_count); }
        else if (!(s.pq > 0.0)) { s.alpha = 0.0; deactivate(s, active_count); }
        else s.alpha = s.rz / s.pq;
    }
}

__global__ void kg_update_xr(int n, CgState *st, int *active_count, ReduceScratch rs, double *__restrict__ x,
                             double *__restrict__ r, const double *__restrict__ pv, const double *__restrict__ q,
                             int maxiter) {
    if (!st[0].active) return;
    const double a = st[0].alpha;
    Acc<double> part;
    GSTRIDE(i, n) {
        x[i] += a * pv[i];
        double ri = r[i] - a * q[i];
        r[i] = ri;
        part.v += ri * ri;
    }
    double2 tot;
    if (reduce_last<double>(part, Acc<double>(), rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
        CgState &s = st[0];
        s.rr = tot.x;
        s.iters++;
        s.total_iters++;
        if (!isfinite(s.rr)) { s.status = DPF_NAN; deactivate(s, active_count); }
        else if (s.rr <= s.tol2 * s.bb) deactivate(s, active_count);
        else if (s.iters >= maxiter) { s.status = DPF_NOT_CONVERGED; deactivate(s, active_count); }
    }
}

__global__ void kg_update_p(int n, const CgState *st, const double *__restrict__ z, double *__restrict__ pv) {
    if (!st[0].active) return;
    const double beta = st[0].beta;
    GSTRIDE(i, n) pv[i] = beta == 0.0 ? z[i] : z[i] + beta * pv[i];
}

// ------------------------------------------------------------ mixed precision (double-float CG)
__global__ void kg_df_spmv_pq(int n, CgState *st, int *active_count, ReduceScratch rs, const int *__restrict__ rp,
                              const int *__restrict__ ci, const float2 *__restrict__ v,
                              const float2 *__restrict__ leak, const float2 *__restrict__ pv, float2 *__restrict__ q) {
    if (!st[0].active) return;
    Acc<float> part;
    GSTRIDE(i, n) {
        const float2 pi = pv[i];
        float2 a = df_mul(leak[i], pi);
        for (int e = rp[i]; e < rp[i + 1]; e++) {
            if (!DPF_INSIDE(CK_CSR_COL, ci[e], 0, n)) continue;
            a = df_add(a, df_mul(v[e], df_sub(pi, pv[ci[e]])));
        }
        q[i] = a;
        part = part + Acc<float>::prod(pi.x, a.x);
    }
    double2 tot;
    if (reduce_last<float>(part, Acc<float>(), rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
        CgState &s = st[0];
        s.pq = tot.x;
        if (!isfinite(s.pq)) { s.alpha = 0.0; s.status = DPF_NAN; deactivate(s, active_count); }
        else if (!(s.pq > 0.0)) { s.alpha = 0.0; deactivate(s, active_count); }
        else s.alpha = s.rz / s.pq;
    }
}

// x64 += (alpha scale) p in FP64 (the solution keeps all 53 bits); r -= alpha q (double-float)
__global__ void kg_df_update_xr(int n, CgState *st, int *active_count, ReduceScratch rs, double *__restrict__ x64,
                                float2 *__restrict__ r, float *__restrict__ r32, const float2 *__restrict__ pv,
                                const float2 *__restrict__ q, int maxiter) {
    if (!st[0].active) return;
    const float2 a = df_from_double(st[0].alpha);
    const double as = st[0].alpha * st[0].scale;
    Acc<float> part;
    GSTRIDE(i, n) {
        const float2 pi = pv[i];
        x64[i] = fma(as, (double)pi.x + (double)pi.y, x64[i]);
        const float2 ri = df_sub(r[i], df_mul(a, q[i]));
        r[i] = ri;
        r32[i] = ri.x;
        part = part + Acc<float>::prod(ri.x, ri.x);
    }
    double2 tot;
    if (reduce_last<float>(part, Acc<float>(), rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
        CgState &s = st[0];
        s.rr = tot.x;
        s.iters++;
        s.total_iters++;
        if (!isfinite(s.rr)) { s.status = DPF_NAN; deactivate(s, active_count); }
        else if (s.rr * s.scale * s.scale <= s.tol2 * s.obb || s.rr <= kRoundDrop2) deactivate(s, active_count);
        else if (s.total_iters >= maxiter) { s.status = DPF_NOT_CONVERGED; deactivate(s, active_count); }
    }
}

__global__ void kg_df_update_p(int n, const CgState *st, const float *__restrict__ z, float2 *__restrict__ pv) {
    if (!st[0].active) return;
    const double beta = st[0].beta;
    const float2 bd = df_from_double(beta);
    GSTRIDE(i, n) {
        const float2 zi = make_float2(z[i], 0.0f);
        pv[i] = beta == 0.0 ? zi : df_add(zi, df_mul(bd, pv[i]));
    }
}

// true FP64 residual; decides whether a (further) double-float round is needed
template <bool FIRST>
__global__ void kg_df_residual(int n, CgState *st, int *active_count, ReduceScratch rs, GOp<double> A,
                               const uint8_t *__restrict__ dir, const double *__restrict__ b,
                               const double *__restrict__ x, double *__restrict__ r, double tol2, int maxiter,
                               int max_rounds) {
    if (!FIRST && !st[0].ru_flag) return;
    Acc<double> rr, bb;  // FIRST: |r|^2, |b|^2; otherwise |r|^2 and the FP64 rounding floor
    GSTRIDE(i, n) {
        double dg;
        const double xi = x[i];
        double ri = b[i] - g_apply<double>(i, A, xi, [&](int j) { return x[j]; }, dg);
        r[i] = ri;
        rr.v += ri * ri;
        if (dir[i]) {
            // identity row: in neither |b| nor the rounding floor
        } else if (FIRST) {
            bb.v += b[i] * b[i];
        } else {
            // the rounding bound of the double-float recurrence (u = 2^-48), as on the structured path
            const double f = 0x1p-48 * fma(2.0 * dg, fabs(xi), fabs(b[i]));
            bb.v += f * f;
        }
    }
    double2 tot;
    if (reduce_last<double, 2>(rr, bb, rs, make_int2(0, gridDim.x), 0, tot) && threadIdx.x == 0) {
        CgState &s = st[0];
        s.orr = tot.x;
        bool go;
        if (FIRST) {
            s.floor2 = 0.0;
            s.obb = tot.y;
            s.tol2 = tol2;
            s.status = DPF_OK;
            s.total_iters = 0;
            s.outer = 0;
            go = s.obb > 0.0 && s.orr > tol2 * s.obb;
            if (!isfinite(s.orr)) { s.status = DPF_NAN; go = false; }
        } else {
            s.outer++;
            s.floor2 = tot.y;
            // at the FP64 rounding floor of b - A x: accept (no further accuracy exists)
            const bool at_floor = s.orr <= s.floor2 || s.orr > 0.25 * s.orr_prev;
            go = true;
            if (!isfinite(s.orr)) { s.status = DPF_NAN; go = false; }
            else if (s.orr <= tol2 * s.obb || at_floor) go = false;
            else if (s.total_iters >= maxiter || s.outer >= max_rounds) { s.status = DPF_NOT_CONVERGED; go = false; }
        }
        s.orr_prev = s.orr;
        s.ru_flag = go ? 1 : 0;
        s.active = go ? 1 : 0;
        s.iters = 0;
        s.rz = s.rz_old = s.beta = 0.0;
        if (go) {
            s.scale = sqrt(s.orr);
            atomicAdd(active_count, 1);
        }
    }
}

__global__ void kg_df_begin(int n, const CgState *st, const double *__restrict__ r64, float2 *__restrict__ r,
                            float *__restrict__ r32) {
    if (!st[0].ru_flag) return;
    const double inv = 1.0 / st[0].scale;
    GSTRIDE(i, n) {
        const float2 v = df_from_double(r64[i] * inv);
        r[i] = v;
        r32[i] = v.x;
    }
}

// ------------------------------------------------------------ misc and gradients
__global__ void kg_state_init(CgState *st) {
    CgState s;
    memset(&s, 0, sizeof(s));
    s.cont = 1.0;
    st[0] = s;
}

__global__ void kg_apply(int n, GOp<double> A, const double *__restrict__ x, double *__restrict__ y) {
    GSTRIDE(i, n) {
        double dg;
        y[i] = g_apply<double>(i, A, x[i], [&](int j) { return x[j]; }, dg);
    }
}

__global__ void kg_adjoint_rhs(int n, const uint8_t *__restrict__ dir, const double *__restrict__ delta,
                               double *__restrict__ rhs, double *__restrict__ x) {
    GSTRIDE(i, n) {
        rhs[i] = dir[i] ? 0.0 : delta[i];
        x[i] = 0.0;
    }
}

__global__ void kg_grad_faces(int F, const int *__restrict__ fa, const int *__restrict__ fb,
                              const double *__restrict__ faol, const double *__restrict__ h,
                              const double *__restrict__ lam, double *__restrict__ dKs, int accumulate) {
    GSTRIDE(f, F) {
        int a = fa[f], b = fb[f];
        double g = -faol[f] * (h[a] - h[b]) * (lam[a] - lam[b]);
        if (accumulate) dKs[f] += g;
        else dKs[f] = g;
    }
}

__global__ void kg_grad_logk(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                             const int *__restrict__ fa, const int *__restrict__ fb, const double *__restrict__ faol,
                             const double *__restrict__ kc, int kind, const double *__restrict__ h,
                             const double *__restrict__ lam, double *__restrict__ g) {
    GSTRIDE(i, n) {
        double ki = kc[i], hi = h[i], li = lam[i], acc = 0.0;
        for (int k = irp[i]; k < irp[i + 1]; k++) {
            int f = ifc[k];
            int j = other_end(fa, fb, f, i);
            double dK = -faol[f] * (hi - h[j]) * (li - lam[j]);
            double K = face_mean_k(ki, kc[j], kind);
            acc += face_mean_dlogk(K, ki, kind) * dK;
        }
        g[i] = acc;
    }
}

// ddirichleths_k = delta_k + sum over faces to free cells of K aol lambda_j; dQs = lambda (free cells)
__global__ void kg_grad_dh_q(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                             const int *__restrict__ fa, const int *__restrict__ fb, const double *__restrict__ faol,
                             const double *__restrict__ Ks, const double *__restrict__ kc, int kind,
                             const uint8_t *__restrict__ dir, const double *__restrict__ delta,
                             const double *__restrict__ lam, double *ddh, double *dQs, int accumulate) {
    GSTRIDE(i, n) {
        const bool isd = dir[i];
        if (dQs) {
            double v = isd ? 0.0 : lam[i];
            if (accumulate) dQs[i] += v;
            else dQs[i] = v;
        }
        if (!ddh) continue;
        double acc = 0.0;
        if (isd) {
            if (delta) acc = delta[i];
            for (int k = irp[i]; k < irp[i + 1]; k++) {
                int f = ifc[k];
                int j = other_end(fa, fb, f, i);
                if (dir[j]) continue;
                acc += g_face_k(Ks, kc, kind, fa, fb, f) * faol[f] * lam[j];
            }
        }
        if (accumulate) ddh[i] += acc;
        else ddh[i] = acc;
    }
}

__global__ void kg_shift(int n, const double *__restrict__ Ss, const double *__restrict__ vol, double inv_dt,
                         double *__restrict__ shift) {
    GSTRIDE(i, n) shift[i] = Ss[i] * vol[i] * inv_dt;
}

__global__ void kg_axpy_rhs(int n, const uint8_t *__restrict__ dir, const double *__restrict__ b0,
                            const double *__restrict__ shift, const double *__restrict__ hprev,
                            double *__restrict__ b) {
    GSTRIDE(i, n) b[i] = dir[i] ? b0[i] : b0[i] + shift[i] * hprev[i];
}

__global__ void kg_trans_adj_rhs(int n, const uint8_t *__restrict__ dir, const double *__restrict__ shift,
                                 const double *__restrict__ mu, const double *__restrict__ gT,
                                 double *__restrict__ rhs) {
    GSTRIDE(i, n) {
        double v = shift[i] * mu[i];
        if (gT) v += gT[i];
        rhs[i] = dir[i] ? 0.0 : v;
    }
}

__global__ void kg_obs_add(int nobs, const long long *__restrict__ obs, const double *__restrict__ w,
                           const uint8_t *__restrict__ dir, const double *__restrict__ h, double *__restrict__ rhs,
                           int skip_dir) {
    GSTRIDE(k, nobs) {
        long long i = obs[k];
        if (skip_dir && dir[i]) continue;
        atomicAdd(&rhs[i], 2.0 * (w ? w[k] : 1.0) * h[i]);
    }
}

__global__ void kg_dh0(int n, const uint8_t *__restrict__ dir, const double *__restrict__ shift,
                       const double *__restrict__ mu, double *__restrict__ out) {
    GSTRIDE(i, n) out[i] = dir[i] ? 0.0 : shift[i] * mu[i];
}

// ================================================================ host side
static void gck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e), e);
    }
}
#define GCK(x) gck((x), #x)
#define GLAUNCH() \
    do {          \
        launches++; \
        gck(cudaGetLastError(), "kernel launch"); \
    } while (0)

// Brackets one kernel launch with a pair of CUDA events on the solver's stream while profiling is
// on (per-kernel device time for dpf_profile_report; launches are counted by GLAUNCH).
struct GTimer {
    GeneralSolver *S;
    int slot = -1;
    GTimer(GeneralSolver *s, const char *name, long long cells) : S(s) {
        if (!S->prof_on || S->prof_recs.size() >= (1u << 20)) return;
        const int e = (int)(2 * S->prof_recs.size());
        while ((int)S->ev_pool.size() < e + 2) {
            cudaEvent_t ev;
            if (cudaEventCreate(&ev) != cudaSuccess) { cudaGetLastError(); return; }
            S->ev_pool.push_back(ev);
        }
        S->prof_recs.push_back(ProfRec{name, e, cells});
        cudaEventRecord(S->ev_pool[e], S->stream);
        slot = e;
    }
    ~GTimer() {
        if (slot >= 0) cudaEventRecord(S->ev_pool[slot + 1], S->stream);
    }
};

void GeneralSolver::profile(bool on) {
    cudaStreamSynchronize(stream);
    prof_recs.clear();
    prof_on = on;
}

int GeneralSolver::profile_report(int cap, const char **names, long long *counts, double *ms, long long *cells) {
    GCK(cudaStreamSynchronize(stream));
    std::vector<const char *> nm;
    std::vector<long long> cnt, cl;
    std::vector<double> tot;
    for (auto &r : prof_recs) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ev_pool[r.ev], ev_pool[r.ev + 1]) != cudaSuccess) { cudaGetLastError(); continue; }
        size_t k = 0;
        while (k < nm.size() && std::strcmp(nm[k], r.name) != 0) k++;
        if (k == nm.size()) { nm.push_back(r.name); cnt.push_back(0); tot.push_back(0.0); cl.push_back(0); }
        cnt[k]++;
        tot[k] += t;
        cl[k] += r.cells;
    }
    for (size_t k = 0; k < nm.size() && (int)k < cap; k++) {
        if (names) names[k] = nm[k];
        if (counts) counts[k] = cnt[k];
        if (ms) ms[k] = tot[k];
        if (cells) cells[k] = cl[k];
    }
    return (int)nm.size();
}

template <typename T>
T *GeneralSolver::dev(size_t n) {
    void *p = nullptr;
    if (dev_malloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        throw OomError("cudaMalloc of " + std::to_string(n * sizeof(T)) + " bytes failed");
    }
    owned.push_back(p);
    return (T *)p;
}

void GeneralSolver::drop(void *p) {
    if (!p) return;
    auto it = std::find(owned.begin(), owned.end(), p);
    if (it != owned.end()) {
        dev_free(p);
        owned.erase(it);
    }
}

void GeneralSolver::to_dev(void *dst, const void *src, size_t bytes) {
    if (bytes) GCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
}
void GeneralSolver::from_dev(void *dst, const void *src, size_t bytes) {
    if (bytes) GCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream));
}

static bool g_is_device(const void *p);

// Observation indices (host or device array) read to the host and range-checked against N.
// A device array is read with one copy on the solver's stream, so it is ordered after the work
// the caller issued there.
std::vector<long long> GeneralSolver::read_indices(const int64_t *idx, long long n) {
    std::vector<long long> out(n);
    if (n <= 0) return out;
    static_assert(sizeof(long long) == sizeof(int64_t), "index width");
    if (g_is_device(idx)) {
        GCK(cudaMemcpyAsync(out.data(), idx, n * sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
        GCK(cudaStreamSynchronize(stream));
    } else {
        std::memcpy(out.data(), idx, n * sizeof(int64_t));
    }
    for (long long v : out)
        if (v < 0 || v >= N) throw BadInput("observation index out of range");
    return out;
}

static bool g_is_device(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

const double *GeneralSolver::stage(const double *src, size_t n, double *dst) {
    if (!src) return nullptr;
    GCK(cudaMemcpyAsync(dst, src, n * sizeof(double),
                        g_is_device(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
    return dst;
}

static void copy_out(double *dst, const double *src, size_t n, cudaStream_t s) {
    if (!dst) return;
    gck(cudaMemcpyAsync(dst, src, n * sizeof(double), g_is_device(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                        s),
        "copy out");
}

GeneralSolver::GeneralSolver(long long N_, long long F_, const int64_t *a, const int64_t *b, const double *aol,
                             const double *volumes, long long nd, const int64_t *dn, const dpf_options &o,
                             cudaStream_t s)
    : opt(o), stream(s) {
    N = N_;
    F = F_;
    if (N >= (1LL << 31) || F >= (1LL << 31)) throw BadInput("general topologies are limited to 2^31 cells and faces");
    if (opt.max_coarse < 1 || opt.max_coarse > kMaxCoarse) opt.max_coarse = kMaxCoarse;
    // defaults of the general path: graph aggregates are larger and less regular than
    // 2x2x2 cubes, and a stronger smoother with a larger over-correction pays (on a 1M-cell
    // 7-point graph with a sigma = 2 field: 32 CG iterations instead of 74 with 2 / 2.0)
    if (opt.cheb_degree == 0) opt.cheb_degree = 3;
    if (!(opt.coarse_scale > 0)) opt.coarse_scale = 3.5;
    if (opt.cheb_degree < 1) opt.cheb_degree = 1;
    if (opt.cheb_degree > 8) opt.cheb_degree = 8;
    mixed = opt.precision == DPF_PREC_MIXED;
    int dev_id = 0, sms = 152;
    GCK(cudaGetDevice(&dev_id));
    GCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
    long long target = (long long)sms * std::max(1, opt.blocks_per_sm);
    nblocks = (int)std::max(1LL, std::min((N + kBlock - 1) / kBlock, target));
    setup_topology(a, b, aol, volumes, nd, dn);
    build_hierarchy();
    // vectors
    h = dev<double>(N); b64 = dev<double>(N); r64 = dev<double>(N); lam = dev<double>(N);
    delta = dev<double>(N); arhs = dev<double>(N); in_Ks = dev<double>(F); in_kc = dev<double>(N);
    aux_kc = dev<double>(N); in_dh = dev<double>(N); in_Q = dev<double>(N); tmpN = dev<double>(N);
    tmpF = dev<double>(F);
    if (!mixed) {
        for (int k = 0; k < 4; k++) cgv[k] = dev<double>(N);
    } else {
        for (int k = 0; k < 2; k++) cgv[k] = dev<float>(N);
        for (int k = 1; k < 4; k++) dfv[k] = dev<float2>(N);  // r, p, q (double-float)
        vdf = dev<float2>(lv[0].nnz);
        leakdf = dev<float2>(N);
    }
    d_state = dev<CgState>(1);
    d_count = dev<int>(4);
    d_status = dev<int>(1);
    rs.partials = dev<double2>(nblocks);
    rs.tickets = dev<unsigned>(1);
    rs.capacity = nblocks;
    GCK(cudaMemsetAsync(rs.tickets, 0, sizeof(unsigned), stream));
    dense_inv = dev<double>(kMaxCoarse * kMaxCoarse);
    h_count = (int *)pinned.alloc(4 * sizeof(int));
    h_state = (CgState *)pinned.alloc(sizeof(CgState));
    if (!h_count || !h_state) throw OomError("pinned host allocation failed");
    // Chebyshev coefficients over [2 cheb_lo, 2] (Gershgorin bound 2 for these M-matrices)
    double lmax = 2.0, lmin = 2.0 * opt.cheb_lo;
    double theta = 0.5 * (lmax + lmin), delt = 0.5 * (lmax - lmin);
    double sigma = theta / delt, rho = 1.0 / sigma;
    inv_theta = 1.0 / theta;
    auto coeffs = [&](int deg, std::vector<double> &c1, std::vector<double> &c2) {
        double rh = 1.0 / sigma;
        c1.assign(deg, 0.0);
        c2.assign(deg, 0.0);
        for (int k = 1; k < deg; k++) {
            double rn = 1.0 / (2.0 * sigma - rh);
            c1[k] = rn * rh;
            c2[k] = 2.0 * rn / delt;
            rh = rn;
        }
    };
    (void)rho;
    coeffs(opt.cheb_degree, cheb_c1, cheb_c2);
    coeffs(8, cheb8_c1, cheb8_c2);
    GCK(cudaStreamSynchronize(stream));
}

GeneralSolver::~GeneralSolver() {
    cudaStreamSynchronize(stream);  // then `owned` and `pinned` free the buffers
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
}

// Host-side topology: the Dirichlet mask, the cell -> face incidence, the CSR of the
// free-free couplings (one entry per face and direction, duplicated faces kept) and
// the entry -> face map.
void GeneralSolver::setup_topology(const int64_t *a, const int64_t *b, const double *aol, const double *volumes,
                                   long long nd, const int64_t *dn) {
    const int n = (int)N, nf = (int)F;
    h_dir.assign(n, 0);
    nfree = N;
    for (long long k = 0; k < nd; k++) {
        if (!h_dir[dn[k]]) nfree--;
        h_dir[dn[k]] = 1;
    }
    std::vector<int> ha(nf), hb(nf);
    for (int f = 0; f < nf; f++) { ha[f] = (int)a[f]; hb[f] = (int)b[f]; }
    // incidence
    std::vector<int> irp_h(n + 1, 0);
    for (int f = 0; f < nf; f++) { irp_h[ha[f] + 1]++; irp_h[hb[f] + 1]++; }
    for (int i = 0; i < n; i++) irp_h[i + 1] += irp_h[i];
    std::vector<int> ifc_h(irp_h[n]), pos(irp_h.begin(), irp_h.end() - 1);
    for (int f = 0; f < nf; f++) { ifc_h[pos[ha[f]]++] = f; ifc_h[pos[hb[f]]++] = f; }
    // couplings between free cells
    std::vector<int> rp_h(n + 1, 0);
    for (int f = 0; f < nf; f++)
        if (!h_dir[ha[f]] && !h_dir[hb[f]]) { rp_h[ha[f] + 1]++; rp_h[hb[f] + 1]++; }
    for (int i = 0; i < n; i++) rp_h[i + 1] += rp_h[i];
    const int nnz = rp_h[n];
    std::vector<int> ci_h(nnz), ef_h(nnz);
    std::copy(rp_h.begin(), rp_h.end() - 1, pos.begin());
    for (int f = 0; f < nf; f++)
        if (!h_dir[ha[f]] && !h_dir[hb[f]]) {
            int p1 = pos[ha[f]]++, p2 = pos[hb[f]]++;
            ci_h[p1] = hb[f]; ef_h[p1] = f;
            ci_h[p2] = ha[f]; ef_h[p2] = f;
        }
    fa = dev<int>(nf); fb = dev<int>(nf); faol = dev<double>(nf);
    irp = dev<int>(n + 1); ifc = dev<int>(irp_h[n]);
    e_face = dev<int>(nnz);
    vol = dev<double>(n);
    to_dev(fa, ha.data(), nf * sizeof(int));
    to_dev(fb, hb.data(), nf * sizeof(int));
    to_dev(faol, aol, nf * sizeof(double));
    to_dev(irp, irp_h.data(), (n + 1) * sizeof(int));
    to_dev(ifc, ifc_h.data(), irp_h[n] * sizeof(int));
    to_dev(e_face, ef_h.data(), nnz * sizeof(int));
    std::vector<double> vv(n, 1.0);
    if (volumes) std::copy(volumes, volumes + n, vv.begin());
    to_dev(vol, vv.data(), n * sizeof(double));
    GLevel L0;
    L0.n = n;
    L0.nnz = nnz;
    L0.rp = dev<int>(n + 1);
    L0.ci = dev<int>(nnz);
    to_dev(L0.rp, rp_h.data(), (n + 1) * sizeof(int));
    to_dev(L0.ci, ci_h.data(), nnz * sizeof(int));
    std::vector<uint8_t> d8(h_dir.begin(), h_dir.end());
    L0.dir = dev<uint8_t>(n);
    to_dev(L0.dir, d8.data(), n);
    lv.push_back(L0);
    // keep the host CSR for the hierarchy
    hrp_ = std::move(rp_h);
    hci_ = std::move(ci_h);
    GCK(cudaStreamSynchronize(stream));
}

// Greedy aggregation of a level's free cells (topology only):
//  1. a cell whose neighbours are all unaggregated forms an aggregate with them;
//  2. a leftover cell joins the aggregate of an already aggregated neighbour;
//  3. what remains becomes a singleton aggregate.
// Identity rows (Dirichlet) are left out (aggregate -1).
static int aggregate(int n, const std::vector<int> &rp, const std::vector<int> &ci, const std::vector<int> &dir,
                     std::vector<int> &agg) {
    agg.assign(n, -1);
    int na = 0;
    for (int i = 0; i < n; i++) {
        if (dir[i] || agg[i] >= 0) continue;
        bool ok = true;
        for (int e = rp[i]; e < rp[i + 1] && ok; e++) ok = agg[ci[e]] < 0;
        if (!ok) continue;
        agg[i] = na;
        for (int e = rp[i]; e < rp[i + 1]; e++) agg[ci[e]] = na;
        na++;
    }
    std::vector<int> snap(agg);
    for (int i = 0; i < n; i++) {
        if (dir[i] || agg[i] >= 0) continue;
        for (int e = rp[i]; e < rp[i + 1]; e++)
            if (snap[ci[e]] >= 0) { agg[i] = snap[ci[e]]; break; }
    }
    for (int i = 0; i < n; i++)
        if (!dir[i] && agg[i] < 0) agg[i] = na++;
    return na;
}

void GeneralSolver::build_hierarchy() {
    NvtxRange range("build hierarchy (CSR)");
    std::vector<int> rp = hrp_, ci = hci_, dir = h_dir;
    int n = (int)N;
    while (n > opt.max_coarse) {
        std::vector<int> agg;
        int nc = aggregate(n, rp, ci, dir, agg);
        if (nc == 0 || nc > (int)(0.9 * n)) break;  // no useful coarsening (e.g. disconnected cells)
        // members of each aggregate
        std::vector<int> mrp(nc + 1, 0);
        for (int i = 0; i < n; i++) if (agg[i] >= 0) mrp[agg[i] + 1]++;
        for (int I = 0; I < nc; I++) mrp[I + 1] += mrp[I];
        std::vector<int> mci(mrp[nc]), pos(mrp.begin(), mrp.end() - 1);
        for (int i = 0; i < n; i++) if (agg[i] >= 0) mci[pos[agg[i]]++] = i;
        // coarse couplings: each fine coupling between different aggregates, merged per pair. The
        // fine entries are bucketed by coarse row with a counting sort into one flat array of
        // (coarse column, fine entry) keys, and each row's short run is sorted by key, so the
        // setup is linear in the couplings up to the sort of a row's few entries.
        std::vector<long long> rstart(nc + 1, 0);
        for (int i = 0; i < n; i++) {
            const int I = agg[i];
            if (I < 0) continue;
            for (int e = rp[i]; e < rp[i + 1]; e++) {
                const int J = agg[ci[e]];
                if (J >= 0 && J != I) rstart[I + 1]++;
            }
        }
        for (int I = 0; I < nc; I++) rstart[I + 1] += rstart[I];
        std::vector<unsigned long long> keys(rstart[nc]);
        {
            std::vector<long long> fill(rstart.begin(), rstart.end() - 1);
            for (int i = 0; i < n; i++) {
                const int I = agg[i];
                if (I < 0) continue;
                for (int e = rp[i]; e < rp[i + 1]; e++) {
                    const int J = agg[ci[e]];
                    if (J >= 0 && J != I) keys[fill[I]++] = ((unsigned long long)(unsigned)J << 32) | (unsigned)e;
                }
            }
        }
        std::vector<int> crp_c(nc + 1, 0), cci_c;     // coarse CSR
        std::vector<int> mrp_e, mci_e;                // coarse entry -> fine entries
        cci_c.reserve(keys.size());
        mci_e.reserve(keys.size());
        mrp_e.reserve(keys.size() + 1);
        mrp_e.push_back(0);
        for (int I = 0; I < nc; I++) {
            std::sort(keys.begin() + rstart[I], keys.begin() + rstart[I + 1]);
            for (long long k = rstart[I]; k < rstart[I + 1];) {
                const unsigned J = (unsigned)(keys[k] >> 32);
                long long k2 = k;
                while (k2 < rstart[I + 1] && (unsigned)(keys[k2] >> 32) == J) {
                    mci_e.push_back((int)(keys[k2] & 0xffffffffu));
                    k2++;
                }
                cci_c.push_back((int)J);
                mrp_e.push_back((int)mci_e.size());
                k = k2;
            }
            crp_c[I + 1] = (int)cci_c.size();
        }
        GLevel &F = lv.back();
        F.agg = dev<int>(n);
        F.mrp = dev<int>(nc + 1);
        F.mci = dev<int>(mci.size());
        F.crp = dev<int>(mrp_e.size());
        F.cci = dev<int>(mci_e.size());
        to_dev(F.agg, agg.data(), n * sizeof(int));
        to_dev(F.mrp, mrp.data(), (nc + 1) * sizeof(int));
        to_dev(F.mci, mci.data(), mci.size() * sizeof(int));
        to_dev(F.crp, mrp_e.data(), mrp_e.size() * sizeof(int));
        to_dev(F.cci, mci_e.data(), mci_e.size() * sizeof(int));
        GLevel C;
        C.n = nc;
        C.nnz = (int)cci_c.size();
        C.rp = dev<int>(nc + 1);
        C.ci = dev<int>(C.nnz);
        C.dir = dev<uint8_t>(nc);
        to_dev(C.rp, crp_c.data(), (nc + 1) * sizeof(int));
        to_dev(C.ci, cci_c.data(), C.nnz * sizeof(int));
        lv.push_back(C);
        rp.swap(crp_c);
        ci.swap(cci_c);
        dir.assign(nc, 0);
        n = nc;
        GCK(cudaStreamSynchronize(stream));
    }
    lv.back().dense = lv.back().n <= kMaxCoarse;
    const size_t vs = mixed ? sizeof(float) : sizeof(double);
    for (auto &L : lv) {
        L.v64 = dev<double>(L.nnz);
        L.leak64 = dev<double>(L.n);
        if (mixed) {
            L.v32 = dev<float>(L.nnz);
            L.leak32 = dev<float>(L.n);
            L.idg32 = dev<float>(L.n);
        } else {
            L.idg64 = dev<double>(L.n);
        }
        for (int k = 0; k < 4; k++) L.work[k] = dev<char>(L.n * vs);
    }
}

int GeneralSolver::read_active() {
    GCK(cudaMemcpyAsync(h_count, d_count, sizeof(int), cudaMemcpyDeviceToHost, stream));
    GCK(cudaStreamSynchronize(stream));
    return h_count[0];
}

bool GeneralSolver::check_due(int it) const {
    const int check = std::max(1, opt.check_every);
    if (it % check != 0) return false;
    return it >= loop_hint - 2 || it % 8 == 0;
}

static unsigned gblocks(long long n, int cap) { return (unsigned)std::max(1LL, std::min((n + kBlock - 1) / kBlock, (long long)cap)); }

void GeneralSolver::assemble(const double *Ks, const double *kc, int kind, const double *shift_, bool init_x) {
    GLevel &L0 = lv[0];
    direct_stale = true;  // a direct factor of the previous operator is out of date
    const int n = (int)N;
    kg_assemble<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, irp, ifc, fa, fb, faol, Ks, kc, kind, L0.dir, in_dh, in_Q,
                                                           shift_, L0.leak64, b64, h, init_x ? 1 : 0);
    GLAUNCH();
    kg_entry_vals<<<gblocks(L0.nnz, nblocks), kBlock, 0, stream>>>(L0.nnz, e_face, fa, fb, faol, Ks, kc, kind, L0.v64);
    GLAUNCH();
    for (size_t l = 0; l + 1 < lv.size(); l++) {
        GLevel &Fl = lv[l], &C = lv[l + 1];
        kg_coarse_vals<<<gblocks(C.nnz, nblocks), kBlock, 0, stream>>>(C.nnz, Fl.crp, Fl.cci, Fl.v64, C.v64);
        GLAUNCH();
        kg_coarse_leak<<<gblocks(C.n, nblocks), kBlock, 0, stream>>>(C.n, Fl.mrp, Fl.mci, Fl.leak64, C.leak64, C.dir);
        GLAUNCH();
    }
    for (auto &L : lv) {
        kg_invdiag<<<gblocks(L.n, nblocks), kBlock, 0, stream>>>(L.n, L.rp, L.v64, L.leak64, L.idg64, L.idg32);
        GLAUNCH();
        if (mixed) {
            kg_to_float<<<gblocks(L.nnz, nblocks), kBlock, 0, stream>>>(L.nnz, L.v64, L.v32);
            GLAUNCH();
            kg_to_float<<<gblocks(L.n, nblocks), kBlock, 0, stream>>>(L.n, L.leak64, L.leak32);
            GLAUNCH();
        }
    }
    if (mixed) {
        kg_to_df<<<gblocks(L0.nnz, nblocks), kBlock, 0, stream>>>(L0.nnz, L0.v64, vdf);
        GLAUNCH();
        kg_to_df<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, L0.leak64, leakdf);
        GLAUNCH();
    }
    GCK(cudaMemsetAsync(d_status, 0, sizeof(int), stream));
    GLevel &Lc = lv.back();
    if (Lc.dense) {
        kg_dense_inverse<<<1, kBlock, 0, stream>>>(Lc.n, Lc.rp, Lc.ci, Lc.v64, Lc.leak64, dense_inv, d_status);
        GLAUNCH();
    }
}

template <typename T>
static GOp<T> gop(GLevel &L);
template <>
GOp<double> gop<double>(GLevel &L) { return GOp<double>{L.rp, L.ci, L.v64, L.leak64, L.idg64, (int)L.n}; }
template <>
GOp<float> gop<float>(GLevel &L) { return GOp<float>{L.rp, L.ci, L.v32, L.leak32, L.idg32, (int)L.n}; }

// V-cycle: z = M r on the finest level
template <typename T>
void GeneralSolver::vcycle(const T *r, T *z) {
    const int deg = opt.cheb_degree;
    const T invth = (T)inv_theta, sc = (T)opt.coarse_scale;
    const int nl = (int)lv.size();
    std::vector<T *> pre(nl, nullptr);
    for (int l = 0; l < nl; l++) {
        GLevel &L = lv[l];
        GOp<T> A = gop<T>(L);
        const T *b = l == 0 ? r : (const T *)L.work[2];
        T *xa = (T *)L.work[0], *xb = (T *)L.work[1], *d = (T *)L.work[3];
        const unsigned g = gblocks(L.n, nblocks);
        if (l == nl - 1) {
            T *out = l == 0 ? z : xb;
            if (L.dense) {
                if (l == 0) { GTimer _gt(this, kname("kg_coarse_solve", l, sizeof(T) == 4), L.n); kg_coarse_solve<T, true><<<1, kMaxCoarse, 0, stream>>>(L.n, d_state, dense_inv, b, out); }
                else { GTimer _gt(this, kname("kg_coarse_solve", l, sizeof(T) == 4), L.n); kg_coarse_solve<T, false><<<1, kMaxCoarse, 0, stream>>>(L.n, d_state, dense_inv, b, out); }
                GLAUNCH();
            } else {
                // no useful coarsening left: a long Chebyshev sweep stands in for the solve
                { GTimer _gt(this, kname("kg_cheb_first", l, sizeof(T) == 4), L.n); kg_cheb_first<T><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, xa, d, invth); }
                GLAUNCH();
                T *cur = xa;
                for (int k = 1; k < 8; k++) {
                    T *o = (k == 7) ? out : (cur == xa ? xb : xa);
                    if (o == cur) o = cur == xa ? xb : xa;
                    { GTimer _gt(this, kname("kg_cheb_step", l, sizeof(T) == 4), L.n); kg_cheb_step<T, false, false><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, o, d,
                                                                           (T)cheb8_c1[k], (T)cheb8_c2[k], rs); }
                    GLAUNCH();
                    cur = o;
                }
                if (cur != out) GCK(cudaMemcpyAsync(out, cur, L.n * sizeof(T), cudaMemcpyDeviceToDevice, stream));
            }
            break;
        }
        T *cur = xa;
        if (deg >= 2) {
            { GTimer _gt(this, kname("kg_cheb_first2", l, sizeof(T) == 4), L.n); kg_cheb_first2<T><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, xb, d, invth, (T)cheb_c1[1], (T)cheb_c2[1]); }
            GLAUNCH();
            cur = xb;
            for (int k = 2; k < deg; k++) {
                T *o = cur == xa ? xb : xa;
                { GTimer _gt(this, kname("kg_cheb_step", l, sizeof(T) == 4), L.n); kg_cheb_step<T, false, false><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, o, d, (T)cheb_c1[k],
                                                                       (T)cheb_c2[k], rs); }
                GLAUNCH();
                cur = o;
            }
        } else {
            { GTimer _gt(this, kname("kg_cheb_first", l, sizeof(T) == 4), L.n); kg_cheb_first<T><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, xa, d, invth); }
            GLAUNCH();
        }
        pre[l] = cur;
        GLevel &C = lv[l + 1];
        // the fine residual in the level's Chebyshev direction buffer (d is written afresh by the
        // first post-smoothing step), then the sums over the aggregates
        { GTimer _gt(this, kname("kg_restrict_resid", l, sizeof(T) == 4), L.n); kg_resid<T><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, d); }
        GLAUNCH();
        { GTimer _gt(this, kname("kg_restrict", l, sizeof(T) == 4), C.n); kg_restrict_sum<T><<<gblocks(C.n, nblocks), kBlock, 0, stream>>>(C.n, d_state, L.mrp, L.mci, d,
                                                                    (T *)C.work[2]); }
        GLAUNCH();
    }
    for (int l = nl - 2; l >= 0; l--) {
        GLevel &L = lv[l], &C = lv[l + 1];
        GOp<T> A = gop<T>(L);
        const T *b = l == 0 ? r : (const T *)L.work[2];
        T *xa = (T *)L.work[0], *xb = (T *)L.work[1], *d = (T *)L.work[3];
        const unsigned g = gblocks(L.n, nblocks);
        T *cur = pre[l];
        { GTimer _gt(this, kname("kg_prolong_add", l, sizeof(T) == 4), L.n); kg_prolong_add<T><<<g, kBlock, 0, stream>>>(L.n, d_state, L.agg, L.dir, cur, (const T *)C.work[1], sc); }
        GLAUNCH();
        for (int k = 0; k < deg; k++) {
            const bool last = k == deg - 1;
            T *o = (l == 0 && last) ? z : (cur == xa ? xb : xa);
            const T c1 = (T)cheb_c1[k], c2 = k == 0 ? invth : (T)cheb_c2[k];
            if (l == 0 && last) {
                // the fused reduction needs the level-0 grid used by every other reduction
                if (k == 0)
                    { GTimer _gt(this, kname("kg_cheb_step0", l, sizeof(T) == 4), L.n); kg_cheb_step<T, true, true><<<nblocks, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, o, d, c1, c2, rs); }
                else
                    { GTimer _gt(this, kname("kg_cheb_step", l, sizeof(T) == 4), L.n); kg_cheb_step<T, true, false><<<nblocks, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, o, d, c1, c2,
                                                                                rs); }
            } else {
                if (k == 0)
                    { GTimer _gt(this, kname("kg_cheb_step0", l, sizeof(T) == 4), L.n); kg_cheb_step<T, false, true><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, o, d, c1, c2, rs); }
                else
                    { GTimer _gt(this, kname("kg_cheb_step", l, sizeof(T) == 4), L.n); kg_cheb_step<T, false, false><<<g, kBlock, 0, stream>>>(L.n, d_state, A, b, cur, o, d, c1, c2, rs); }
            }
            GLAUNCH();
            cur = o;
        }
    }
}

template <typename T>
void GeneralSolver::pcg(const T *b, T *x, double tol2) {
    GLevel &L0 = lv[0];
    const int n = (int)N;
    T *r = (T *)cgv[0], *z = (T *)cgv[1], *pv = (T *)cgv[2], *q = (T *)cgv[3];
    GOp<double> A = gop<double>(L0);
    GCK(cudaMemsetAsync(d_count, 0, sizeof(int), stream));
    { GTimer _gt(this, kname("kg_cg_start", 0, sizeof(T) == 4), n); kg_cg_start<<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, A, L0.dir, b, x, r, tol2); }
    GLAUNCH();
    vcycle<T>(r, z);
    { GTimer _gt(this, kname("kg_update_p", 0, sizeof(T) == 4), n); kg_update_p<<<nblocks, kBlock, 0, stream>>>(n, d_state, z, pv); }
    GLAUNCH();
    for (int it = 1; it <= opt.maxiter + 1; it++) {
        { GTimer _gt(this, kname("kg_spmv_pq", 0, sizeof(T) == 4), n); kg_spmv_pq<<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, A, pv, q); }
        GLAUNCH();
        { GTimer _gt(this, kname("kg_update_xr", 0, sizeof(T) == 4), n); kg_update_xr<<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, x, r, pv, q, opt.maxiter); }
        GLAUNCH();
        if (check_due(it) && read_active() <= 0) {
            loop_hint = it;
            return;
        }
        vcycle<T>(r, z);
        { GTimer _gt(this, kname("kg_update_p", 0, sizeof(T) == 4), n); kg_update_p<<<nblocks, kBlock, 0, stream>>>(n, d_state, z, pv); }
        GLAUNCH();
    }
}

void GeneralSolver::df_pcg(const double *b, double *x, double tol2) {
    GLevel &L0 = lv[0];
    const int n = (int)N;
    float *r32 = (float *)cgv[0], *z32 = (float *)cgv[1];
    GOp<double> A = gop<double>(L0);
    GCK(cudaMemsetAsync(d_count, 0, sizeof(int), stream));
    { GTimer _gt(this, kname("kg_df_residual", 0, false), n); kg_df_residual<true><<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, A, L0.dir, b, x, r64, tol2,
                                                         opt.maxiter, opt.max_outer); }
    GLAUNCH();
    const int check = std::max(1, opt.check_every);
    for (int round = 0; round < opt.max_outer && read_active() > 0; round++) {
        { GTimer _gt(this, kname("kg_df_begin", 0, false), n); kg_df_begin<<<nblocks, kBlock, 0, stream>>>(n, d_state, r64, dfv[1], r32); }
        GLAUNCH();
        vcycle<float>(r32, z32);
        { GTimer _gt(this, kname("kg_df_update_p", 0, true), n); kg_df_update_p<<<nblocks, kBlock, 0, stream>>>(n, d_state, z32, dfv[2]); }
        GLAUNCH();
        for (int it = 1; it <= opt.maxiter + 1; it++) {
            { GTimer _gt(this, kname("kg_df_spmv_pq", 0, true), n); kg_df_spmv_pq<<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, L0.rp, L0.ci, vdf, leakdf, dfv[2],
                                                          dfv[3]); }
            GLAUNCH();
            { GTimer _gt(this, kname("kg_df_update_xr", 0, true), n); kg_df_update_xr<<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, x, dfv[1], r32, dfv[2],
                                                            dfv[3], opt.maxiter); }
            GLAUNCH();
            if ((round == 0 ? check_due(it) : it % check == 0) && read_active() <= 0) {
                if (round == 0) loop_hint = it;
                break;
            }
            vcycle<float>(r32, z32);
            { GTimer _gt(this, kname("kg_df_update_p", 0, true), n); kg_df_update_p<<<nblocks, kBlock, 0, stream>>>(n, d_state, z32, dfv[2]); }
            GLAUNCH();
        }
        GCK(cudaMemsetAsync(d_count, 0, sizeof(int), stream));
        { GTimer _gt(this, kname("kg_df_residual", 0, false), n); kg_df_residual<false><<<nblocks, kBlock, 0, stream>>>(n, d_state, d_count, rs, A, L0.dir, b, x, r64, tol2,
                                                              opt.maxiter, opt.max_outer); }
        GLAUNCH();
    }
}

// The FP64 operator in the banded Cholesky's storage: per row its diagonal leak + the sum of
// its couplings, and from the row with the smaller index of each coupling -c at (max, min) of the
// two band rows (added: a pair of cells joined by several faces has several couplings).
__global__ void kg_band_fill(int n, GOp<double> A, const long long *__restrict__ iperm, long long w,
                             double *__restrict__ band) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long k = iperm[i];
        double d = A.leak[i];
        for (int e = A.rp[i]; e < A.rp[i + 1]; e++) {
            const int j = A.ci[e];
            d += A.v[e];
            if (j > i) {
                const long long kj = iperm[j];
                const long long r = max(k, kj), q = min(k, kj);
                if (r - q <= w) atomicAdd(&band[q * (w + 1) + (r - q)], -A.v[e]);
            }
        }
        band[k * (w + 1)] = d;
    }
}

bool GeneralSolver::direct_solve(const double *b, double *x) {
    GLevel &L0 = lv[0];
    if (!direct_tried) {
        direct_tried = true;
        const BandOrder ord = band_order_rcm(N, hrp_, hci_);
        size_t free_b = 0, total_b = 0;
        GCK(cudaMemGetInfo(&free_b, &total_b));
        if (BandCholesky::fits(N, ord.w, free_b / 2)) direct.reset(new BandCholesky(ord, stream));
    }
    if (!direct) return false;
    NvtxRange range("direct solve (banded Cholesky, CSR)");
    BandCholesky &D = *direct;
    D.set_stream(stream);
    const long long l0 = D.launches;
    if (direct_stale) {
        D.clear();
        kg_band_fill<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, gop<double>(L0), D.iperm(), D.w, D.band());
        GLAUNCH();
        direct_ok = D.factor();
        direct_stale = false;
    }
    stats_iters = 0;
    stats_outer = 0;
    stats_relres = 0.0;
    h_state->total_iters = 0;
    h_state->outer = 0;
    if (!direct_ok) {
        h_state->status = DPF_BAD_INPUT;
        last_message = "the operator is not positive definite (is there a Dirichlet cell?)";
        launches += D.launches - l0;
        return true;
    }
    D.solve(b, x);
    kg_apply<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, gop<double>(L0), x, r64);
    GLAUNCH();
    if (!d_direct_acc) d_direct_acc = dev<double>(2);
    stats_relres = BandCholesky::relres(stream, N, L0.dir, b, r64, d_direct_acc);
    h_state->status = std::isfinite(stats_relres) ? DPF_OK : DPF_NAN;
    launches += D.launches - l0 + 2;
    return true;
}

void GeneralSolver::solve(const double *b, double *x) {
    if (opt.solver == DPF_SOLVER_CHOLESKY && direct_solve(b, x)) return;
    NvtxRange range("CG + AMG solve (CSR)");
    kg_state_init<<<1, 1, 0, stream>>>(d_state);
    GLAUNCH();
    const double tol2 = opt.reltol * opt.reltol;
    if (!mixed) pcg<double>(b, x, tol2);
    else df_pcg(b, x, tol2);
    from_dev(h_state, d_state, sizeof(CgState));
    GCK(cudaStreamSynchronize(stream));
    stats_iters = h_state->total_iters;
    stats_outer = mixed ? h_state->outer : 0;
    stats_relres = mixed ? (h_state->obb > 0 ? std::sqrt(h_state->orr / h_state->obb) : 0.0)
                         : (h_state->bb > 0 ? std::sqrt(h_state->rr / h_state->bb) : 0.0);
}

int GeneralSolver::finish_status() {
    int fst = 0;
    GCK(cudaMemcpyAsync(h_count + 1, d_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    GCK(cudaStreamSynchronize(stream));
    fst = h_count[1];
    if (fst) {
        last_message = "coarsest operator is not positive definite (is there a Dirichlet cell?)";
        return DPF_BAD_INPUT;
    }
    if (h_state->status != DPF_OK)
        last_message = h_state->status == DPF_NOT_CONVERGED ? "CG did not converge within maxiter" : "non-finite residual";
    return h_state->status;
}

int GeneralSolver::forward(const double *Ks, const double *logK, int kind, const double *dh, const double *Qs,
                           double *h_out) {
    if (nfree == N) throw BadInput("the problem has no Dirichlet cell: the steady-state operator is singular");
    stage(dh, N, in_dh);
    stage(Qs, N, in_Q);
    if (logK) {
        stage(logK, N, tmpN);
        kg_cell_k<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, tmpN, kind, in_kc);
        GLAUNCH();
        assemble(nullptr, in_kc, kind, nullptr, true);
    } else {
        stage(Ks, F, in_Ks);
        assemble(in_Ks, nullptr, kind, nullptr, true);
    }
    solve(b64, h);
    fwd_kind = logK ? 1 : 0;
    mean_kind = kind;
    have_forward = true;
    copy_out(h_out, h, N, stream);
    GCK(cudaStreamSynchronize(stream));
    return finish_status();
}

void GeneralSolver::adjoint_solve(const double *delta_dev) {
    kg_adjoint_rhs<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, lv[0].dir, delta_dev, arhs, lam);
    GLAUNCH();
    solve(arhs, lam);
}

int GeneralSolver::adjoint(const double *delta_in, double *dKs, double *dlogK, double *ddh, double *dQs) {
    if (!have_forward) {
        last_message = "adjoint called before a forward solve";
        return DPF_STATE;
    }
    if (dlogK && fwd_kind != 1) {
        last_message = "the adjoint to logK needs a preceding forward from logK";
        return DPF_STATE;
    }
    stage(delta_in, N, delta);
    adjoint_solve(delta);
    int rc = finish_status();
    const int n = (int)N;
    if (dKs) {
        kg_grad_faces<<<gblocks(F, nblocks), kBlock, 0, stream>>>((int)F, fa, fb, faol, h, lam, tmpF, 0);
        GLAUNCH();
        copy_out(dKs, tmpF, F, stream);
    }
    if (dlogK) {
        kg_grad_logk<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, irp, ifc, fa, fb, faol, in_kc, mean_kind, h, lam,
                                                                tmpN);
        GLAUNCH();
        copy_out(dlogK, tmpN, N, stream);
        GCK(cudaStreamSynchronize(stream));
    }
    if (ddh || dQs) {
        const double *Kp = fwd_kind ? nullptr : in_Ks, *kcp = fwd_kind ? in_kc : nullptr;
        kg_grad_dh_q<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, irp, ifc, fa, fb, faol, Kp, kcp, mean_kind,
                                                                lv[0].dir, delta, lam, ddh ? r64 : nullptr,
                                                                dQs ? arhs : nullptr, 0);
        GLAUNCH();
        copy_out(ddh, r64, N, stream);
        copy_out(dQs, arhs, N, stream);
    }
    GCK(cudaStreamSynchronize(stream));
    return rc;
}

int GeneralSolver::logk_to_faces(const double *logK, int kind, double *Ks) {
    stage(logK, N, tmpN);
    kg_cell_k<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, tmpN, kind, aux_kc);
    GLAUNCH();
    kg_faces<<<gblocks(F, nblocks), kBlock, 0, stream>>>((int)F, fa, fb, aux_kc, kind, tmpF);
    GLAUNCH();
    copy_out(Ks, tmpF, F, stream);
    GCK(cudaStreamSynchronize(stream));
    return DPF_OK;
}

int GeneralSolver::logk_vjp(const double *logK, int kind, const double *dKs, double *dlogK) {
    stage(logK, N, tmpN);
    kg_cell_k<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, tmpN, kind, aux_kc);
    GLAUNCH();
    stage(dKs, F, tmpF);
    kg_vjp<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, aux_kc, kind, tmpF, tmpN);
    GLAUNCH();
    copy_out(dlogK, tmpN, N, stream);
    GCK(cudaStreamSynchronize(stream));
    return DPF_OK;
}

int GeneralSolver::solve_grad_logk(const double *logK, int kind, const double *dh, const double *Qs, long long nobs,
                                   const int64_t *obs, double *h_out, double *dlogK) {
    int rc = forward(nullptr, logK, kind, dh, Qs, h_out);
    if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) return rc;
    const std::vector<long long> ho = read_indices(obs, nobs);
    long long *d_obs = dev<long long>(nobs);
    to_dev(d_obs, ho.data(), nobs * sizeof(long long));
    GCK(cudaMemsetAsync(delta, 0, N * sizeof(double), stream));
    if (nobs) {
        kg_obs_add<<<gblocks(nobs, nblocks), kBlock, 0, stream>>>((int)nobs, d_obs, nullptr, lv[0].dir, h, delta, 0);
        GLAUNCH();
    }
    int rc2 = adjoint(delta, nullptr, dlogK, nullptr, nullptr);
    GCK(cudaStreamSynchronize(stream));
    drop(d_obs);
    return rc != DPF_OK ? rc : rc2;
}

int GeneralSolver::apply(const double *x, double *y) {
    if (!have_forward && !tr_nsteps) {
        last_message = "no operator assembled yet";
        return DPF_STATE;
    }
    stage(x, N, tmpN);
    kg_apply<<<gblocks(N, nblocks), kBlock, 0, stream>>>((int)N, gop<double>(lv[0]), tmpN, r64);
    GLAUNCH();
    copy_out(y, r64, N, stream);
    GCK(cudaStreamSynchronize(stream));
    return DPF_OK;
}

int GeneralSolver::transient_forward(const double *Ks, const double *dh, const double *Qs, const double *Ss,
                                     double dt, int nsteps, const double *h0, double *states, double *hT) {
    const int n = (int)N;
    if (!shift) shift = dev<double>(N);
    if (!tr_b0) tr_b0 = dev<double>(N);
    if (tr_states && tr_nsteps != nsteps) tr_states = nullptr;  // reallocated below (old buffer stays owned)
    if (!tr_states) tr_states = dev<double>((size_t)nsteps * N);
    tr_nsteps = nsteps;
    stage(Ks, F, in_Ks);
    stage(dh, N, in_dh);
    stage(Qs, N, in_Q);
    stage(Ss, N, tmpN);
    stage(h0, N, h);
    kg_shift<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, tmpN, vol, 1.0 / dt, shift);
    GLAUNCH();
    assemble(in_Ks, nullptr, 0, shift, false);
    fwd_kind = 0;
    mean_kind = 0;
    GCK(cudaMemcpyAsync(tr_b0, b64, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    int worst = DPF_OK;
    long long tot = 0;
    for (int s = 0; s < nsteps; s++) {
        kg_axpy_rhs<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, lv[0].dir, tr_b0, shift, h, b64);
        GLAUNCH();
        solve(b64, h);
        tot += stats_iters;
        int rc = finish_status();
        if (rc != DPF_OK && worst == DPF_OK) worst = rc;
        GCK(cudaMemcpyAsync(tr_states + (size_t)s * N, h, N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        if (states) copy_out(states + (size_t)s * N, h, N, stream);
    }
    stats_iters = (int)std::min<long long>(tot, 1 << 30);
    copy_out(hT, h, N, stream);
    GCK(cudaStreamSynchronize(stream));
    have_forward = false;
    return worst;
}

int GeneralSolver::transient_adjoint(long long nobs, const int64_t *obs, const double *w, const double *gT,
                                     double *dKs, double *ddh, double *dQs, double *dh0) {
    if (tr_nsteps <= 0) {
        last_message = "transient adjoint needs a preceding transient forward";
        return DPF_STATE;
    }
    const int n = (int)N;
    const std::vector<long long> ho = read_indices(obs, nobs);
    long long *d_obs = dev<long long>(std::max(nobs, 1LL));
    to_dev(d_obs, ho.data(), nobs * sizeof(long long));
    double *d_w = nullptr, *d_gT = nullptr;
    if (w) { d_w = dev<double>(nobs); stage(w, nobs, d_w); }
    if (gT) { d_gT = dev<double>(N); stage(gT, N, d_gT); }
    double *aK = dev<double>(F), *adh = dev<double>(N), *aQ = dev<double>(N);
    GCK(cudaMemsetAsync(aK, 0, F * sizeof(double), stream));
    GCK(cudaMemsetAsync(adh, 0, N * sizeof(double), stream));
    GCK(cudaMemsetAsync(aQ, 0, N * sizeof(double), stream));
    GCK(cudaMemsetAsync(lam, 0, N * sizeof(double), stream));
    int worst = DPF_OK;
    for (int s = tr_nsteps - 1; s >= 0; s--) {
        const double *hn = tr_states + (size_t)s * N;
        kg_trans_adj_rhs<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, lv[0].dir, shift, lam,
                                                                    s == tr_nsteps - 1 ? d_gT : nullptr, arhs);
        GLAUNCH();
        if (nobs) {
            kg_obs_add<<<gblocks(nobs, nblocks), kBlock, 0, stream>>>((int)nobs, d_obs, d_w, lv[0].dir, hn, arhs, 1);
            GLAUNCH();
        }
        solve(arhs, lam);
        int rc = finish_status();
        if (rc != DPF_OK && worst == DPF_OK) worst = rc;
        kg_grad_faces<<<gblocks(F, nblocks), kBlock, 0, stream>>>((int)F, fa, fb, faol, hn, lam, aK, 1);
        GLAUNCH();
        kg_grad_dh_q<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, irp, ifc, fa, fb, faol, in_Ks, nullptr, 0,
                                                                lv[0].dir, nullptr, lam, adh, aQ, 1);
        GLAUNCH();
    }
    if (dh0) {
        kg_dh0<<<gblocks(n, nblocks), kBlock, 0, stream>>>(n, lv[0].dir, shift, lam, tmpN);
        GLAUNCH();
        copy_out(dh0, tmpN, N, stream);
    }
    copy_out(dKs, aK, F, stream);
    copy_out(ddh, adh, N, stream);
    copy_out(dQs, aQ, N, stream);
    GCK(cudaStreamSynchronize(stream));
    for (void *p : {(void *)d_obs, (void *)d_w, (void *)d_gT, (void *)aK, (void *)adh, (void *)aQ}) drop(p);
    return worst;
}

template void GeneralSolver::vcycle<double>(const double *, double *);
template void GeneralSolver::vcycle<float>(const float *, float *);

}  // namespace dpf
