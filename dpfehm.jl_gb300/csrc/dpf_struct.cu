// dpf_struct.cu -- structured-grid groundwater solver for sm_103a.
//
// A StructBatch holds nprob regular grids (a single problem is a batch of one):
// the multigrid hierarchy (2x2x2 aggregation, Galerkin 7-point coarse operators,
// dense inverse of the coarsest level), the CG / iterative-refinement state, and the
// kernels that solve and differentiate
//   A h = b,   A = groundwater_h, b = -groundwater_residuals(0)   (src/groundwater.jl:75-83)
//   A lambda = delta[free]                                        (src/groundwater.jl:93-107)
// for every problem at once. Converged problems drop out of the launches (their
// blocks exit at entry), so uneven batches cost what their unconverged members cost.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <stdexcept>

#include <cooperative_groups.h>

#include "dpf_direct.h"
#include "dpf_struct.h"
#include "dpf_struct_kernels.cuh"
#include "dpf_plane.cuh"
#include "dpf_plane2.cuh"

namespace dpf {
namespace cg = cooperative_groups;

// ================================================================ kernels
// Conductance of the face between cell c and its neighbour j in direction d (0..2)
// and side s (+1: neighbour at +, -1: neighbour at -).
struct FaceK {
    const double *Ks;       // face list (reference order), or null
    const double *kc;       // per-cell values of k_cell_k, or null
    int kind;
    __device__ __forceinline__ double operator()(const LevelDesc &L, const ProbParam &P, const Cell &c, int d, int s,
                                                long long j) const {
        if (Ks) {
            int ax = c.ix, ay = c.iy, az = c.iz;  // face is owned by the lower cell
            if (s < 0) { if (d == 0) ax--; else if (d == 1) ay--; else az--; }
            return Ks[P.face_off + regular_face_index(L.nx, L.ny, L.nz, ax, ay, az, d)];
        }
        return face_mean_k(kc[c.i], kc[j], kind);
    }
};

// Fine-level operator, right-hand side and initial guess (src/groundwater.jl:4-20 with
// S = V = 1; storage shift for transient). Writes FP64 coefficients and, when fx != null,
// the bf16 copies of the FP32 V-cycle.
__global__ void k_assemble(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                           const ProbParam *__restrict__ prm, FaceK fk, const double *__restrict__ dh,
                           const double *__restrict__ Qs, const double *__restrict__ shift,
                           const uint8_t *__restrict__ dir, double *cx, double *cy, double *cz, double *leak,
                           __nv_bfloat16 *fx, __nv_bfloat16 *fy, __nv_bfloat16 *fz, __nv_bfloat16 *fleak,
                           float2 *dfx, float2 *dfy, float2 *dfz,
                           float2 *dfleak, double *b, double *x, int init_x) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const ProbParam P = prm[bm.x];
        const long long i = c.i;
        const long long st[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
        const int co[3] = {c.ix, c.iy, c.iz};
        const int nn[3] = {L.nx, L.ny, L.nz};
        bool fi = !dir[i];
        double lk = 0.0, rhs = fi ? Qs[i] : dh[i];
        double cp[3] = {0.0, 0.0, 0.0};
        if (fi) {
    #pragma unroll
            for (int d = 0; d < 3; d++) {
                if (co[d] + 1 < nn[d]) {
                    long long j = i + st[d];
                    double cf = fk(L, P, c, d, +1, j) * P.aol[d];
                    if (!dir[j]) cp[d] = cf;
                    else { lk += cf; rhs += cf * dh[j]; }
                }
                if (co[d] > 0) {
                    long long j = i - st[d];
                    if (dir[j]) {
                        double cf = fk(L, P, c, d, -1, j) * P.aol[d];
                        lk += cf;
                        rhs += cf * dh[j];
                    }
                }
            }
            if (shift) lk += shift[i];
        } else {
            lk = 1.0;
        }
        double *cv[4] = {&cp[0], &cp[1], &cp[2], &lk};
        if (dfx) {
            // mixed precision: the FP64 operator is the exact value of its double-float copy
            // (each coefficient rounded to 48 of its 53 bits: a relative change of at most 2^-48),
            // so the double-float CG and the FP64 residual check see the same operator; the bf16
            // copies of the FP32 V-cycle are rounded from the leading floats
            float2 *dv[4] = {dfx, dfy, dfz, dfleak};
            __nv_bfloat16 *bv[4] = {fx, fy, fz, fleak};
    #pragma unroll
            for (int k = 0; k < 4; k++) {
                float2 q;
                double v48;
                if (!split48(*cv[k], q.x, q.y, v48)) {
                    q = df_from_double(*cv[k]);
                    v48 = df_to_double(q);
                }
                dv[k][i] = q;
                *cv[k] = v48;
                if (fx) bv[k][i] = __float2bfloat16(q.x);
            }
        } else if (fx) {
            fx[i] = __double2bfloat16(cp[0]); fy[i] = __double2bfloat16(cp[1]);
            fz[i] = __double2bfloat16(cp[2]); fleak[i] = __double2bfloat16(lk);
        }
        cx[i] = cp[0]; cy[i] = cp[1]; cz[i] = cp[2]; leak[i] = lk;
        b[i] = rhs;
        if (init_x) x[i] = fi ? 0.0 : dh[i];
        else if (!fi) x[i] = dh[i];
    }
}

// ----------------------------------------------------------- coarsening
// Galerkin coarse operator of piecewise-constant 2x2x2 aggregation that leaves out
// Dirichlet (identity) cells: a coarse face carries the sum of the fine faces that
// cross it, a coarse leak is the sum of the free children's leaks. An aggregate
// with no free child becomes an identity row.
__global__ void k_coarsen(const LevelDesc *__restrict__ fdesc, const LevelDesc *__restrict__ cdesc,
                          const int4 *__restrict__ bmap, const double *__restrict__ fcx,
                          const double *__restrict__ fcy, const double *__restrict__ fcz,
                          const double *__restrict__ fleak, const uint8_t *__restrict__ fdir, double *ccx,
                          double *ccy, double *ccz, double *cleak, uint8_t *cdir, __nv_bfloat16 *gx,
                          __nv_bfloat16 *gy, __nv_bfloat16 *gz, __nv_bfloat16 *gleak) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    LevelDesc Lc = cdesc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)Lc.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(Lc, li_, c);
        LevelDesc Lf = fdesc[bm.x];
        const long long fsy = Lf.nz, fsx = (long long)Lf.ny * Lf.nz;
        int x0 = 2 * c.ix, y0 = 2 * c.iy, z0 = 2 * c.iz;
        int x1 = min(x0 + 1, Lf.nx - 1), y1 = min(y0 + 1, Lf.ny - 1), z1 = min(z0 + 1, Lf.nz - 1);
        double lk = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
        bool anyfree = false;
        for (int fx = x0; fx <= x1; fx++)
            for (int fy = y0; fy <= y1; fy++)
                for (int fz = z0; fz <= z1; fz++) {
                    long long j = Lf.off + fx * fsx + fy * fsy + fz;
                    if (!fdir[j]) { anyfree = true; lk += fleak[j]; }
                    if (fx == x0 + 1 && c.ix + 1 < Lc.nx) sx += fcx[j];
                    if (fy == y0 + 1 && c.iy + 1 < Lc.ny) sy += fcy[j];
                    if (fz == z0 + 1 && c.iz + 1 < Lc.nz) sz += fcz[j];
                }
        if (!anyfree) { lk = 1.0; sx = sy = sz = 0.0; }
        const long long i = c.i;
        ccx[i] = sx; ccy[i] = sy; ccz[i] = sz; cleak[i] = lk; cdir[i] = anyfree ? 0 : 1;
        if (gx) {
            gx[i] = __double2bfloat16(sx); gy[i] = __double2bfloat16(sy);
            gz[i] = __double2bfloat16(sz); gleak[i] = __double2bfloat16(lk);
        }
    }
}

// ------------------------------------------------------ coarsest level
// Dense inverse of each listed problem's coarsest operator (n <= 64), one block
// per problem, by in-place Gauss-Jordan elimination in shared memory (no pivoting:
// the operator is symmetric positive definite, so every pivot is a positive Schur
// complement). The coarsest solve is then one small matrix-vector product.
// The inverse is stored row-major with stride kMaxCoarse.
__global__ void k_coarse_factor(const LevelDesc *__restrict__ desc, const int *__restrict__ plist,
                                const double *__restrict__ cx, const double *__restrict__ cy,
                                const double *__restrict__ cz, const double *__restrict__ leak, double *Inv,
                                int *status) {
    pdl_enter();
    __shared__ double A[kMaxCoarse][kMaxCoarse + 1];
    __shared__ double col[kMaxCoarse];
    __shared__ int bad;
    int p = plist[blockIdx.x];
    LevelDesc L = desc[p];
    int n = (int)L.n;
    const int sy = L.nz, sx = L.ny * L.nz;
    for (int k = threadIdx.x; k < kMaxCoarse * kMaxCoarse; k += blockDim.x) A[k / kMaxCoarse][k % kMaxCoarse] = 0.0;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int li = threadIdx.x; li < n; li += blockDim.x) {
        int q = li / L.nz, iz = li - q * L.nz, iy = q % L.ny, ix = q / L.ny;
        long long i = L.off + li;
        double d = leak[i];
        if (iz + 1 < L.nz) { double w = cz[i];      d += w; A[li][li + 1] = -w; }
        if (iz > 0)        { double w = cz[i - 1];  d += w; A[li][li - 1] = -w; }
        if (iy + 1 < L.ny) { double w = cy[i];      d += w; A[li][li + sy] = -w; }
        if (iy > 0)        { double w = cy[i - sy]; d += w; A[li][li - sy] = -w; }
        if (ix + 1 < L.nx) { double w = cx[i];      d += w; A[li][li + sx] = -w; }
        if (ix > 0)        { double w = cx[i - sx]; d += w; A[li][li - sx] = -w; }
        A[li][li] = d;
    }
    __syncthreads();
    for (int k = 0; k < n; k++) {
        // pivot row k scaled by 1/A[k][k] (with the identity column folded in); save column k
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
            double rk = A[k][j];
            A[i][j] = (j == k ? 0.0 : A[i][j]) - col[i] * rk;
        }
        __syncthreads();
    }
    double *Ip = Inv + (long long)p * kMaxCoarse * kMaxCoarse;
    for (int k = threadIdx.x; k < kMaxCoarse * kMaxCoarse; k += blockDim.x) {
        int i = k / kMaxCoarse, j = k % kMaxCoarse;
        Ip[k] = (i < n && j < n) ? A[i][j] : 0.0;
    }
    if (threadIdx.x == 0 && bad) atomicExch(status, 1);
}

// ---- per-cell bodies of the V-cycle steps, shared by the per-level kernels (one launch
// per level, all problems) and the fused tail kernel (all small levels of one problem).
// CG: vectors written earlier in the same kernel by other blocks of a cluster are read
// through L2 (ld.global.cg), so no block sees a stale L1 line.
template <bool CG, typename T>
__device__ __forceinline__ T ldv(const T *p, long long i) {
    if constexpr (CG) return __ldcg(p + i);
    else return p[i];
}

// first Chebyshev step from a zero guess: x = d = invtheta D^-1 b
template <typename T, bool CG = false>
__device__ __forceinline__ void cell_cheb_first(const LevelDesc &L, const Cell &c, const Coeffs<T> &C,
                                                const T *__restrict__ b, T *__restrict__ x, T *__restrict__ d,
                                                T invtheta) {
    T v;
    if constexpr (sizeof(T) == 8) v = invtheta * ldv<CG>(b, c.i) * C.idg[c.i];
    else v = invtheta * __fdividef(ldv<CG>(b, c.i), diag7(L, c, C));
    x[c.i] = v;
    d[c.i] = v;
}

// the first two Chebyshev steps from a zero guess (see k_cheb_first2)
template <typename T, bool CG = false>
__device__ __forceinline__ void cell_cheb_first2(const LevelDesc &L, const Cell &c, const Coeffs<T> &C,
                                                 const T *__restrict__ b, T *__restrict__ xout, T *__restrict__ d,
                                                 T invtheta, T c1, T c2) {
    const T *__restrict__ g = C.idg;
    const T bi = ldv<CG>(b, c.i), gi = g[c.i];
    const T x1 = invtheta * bi * gi;
    T Ax, dg;
    apply7(L, c, C, x1, [&](long long j, int, int, int) { return invtheta * ldv<CG>(b, j) * g[j]; }, Ax, dg);
    const T dn = c1 * x1 + c2 * (bi - Ax) * gi;
    d[c.i] = dn;
    xout[c.i] = x1 + dn;
}

// one Chebyshev step (see k_cheb_step); returns the new iterate
template <typename T, bool FIRST, bool CG = false>
__device__ __forceinline__ T cell_cheb_step(const LevelDesc &L, const Cell &c, const Coeffs<T> &C,
                                            const T *__restrict__ b, const T *__restrict__ xin,
                                            T *__restrict__ xout, T *__restrict__ d, T c1, T c2, T &bi) {
    T xi = ldv<CG>(xin, c.i), Ax, dg;
    apply7(L, c, C, xi, [&](long long j, int, int, int) { return ldv<CG>(xin, j); }, Ax, dg);
    bi = ldv<CG>(b, c.i);
    T r = dinv_times(C, c.i, bi - Ax, dg);
    T dn = FIRST ? c2 * r : c1 * ldv<CG>((const T *)d, c.i) + c2 * r;
    T xo = xi + dn;
    d[c.i] = dn;
    xout[c.i] = xo;
    return xo;
}

// restricted residual of coarse cell cc: sum over its children i of b_i - (A x)_i
template <typename T, bool CG = false>
__device__ __forceinline__ T cell_restrict(const LevelDesc &L, const Cell &cc, const Coeffs<T> &C,
                                           const T *__restrict__ b, const T *__restrict__ x) {
    const long long fsy = L.nz, fsx = (long long)L.ny * L.nz;
    int x0 = 2 * cc.ix, y0 = 2 * cc.iy, z0 = 2 * cc.iz;
    int x1 = min(x0 + 1, L.nx - 1), y1 = min(y0 + 1, L.ny - 1), z1 = min(z0 + 1, L.nz - 1);
    T acc = 0;
    for (int fx = x0; fx <= x1; fx++)
        for (int fy = y0; fy <= y1; fy++)
            for (int fz = z0; fz <= z1; fz++) {
                Cell c;
                c.ix = fx; c.iy = fy; c.iz = fz;
                c.i = L.off + fx * fsx + fy * fsy + fz;
                T xi = ldv<CG>(x, c.i), Ax, dg;
                apply7(L, c, C, xi, [&](long long j, int, int, int) { return ldv<CG>(x, j); }, Ax, dg);
                acc += ldv<CG>(b, c.i) - Ax;
            }
    return acc;
}

#define DPF_BLOCK_PROLOGUE(DESC, BMAP, ST)                 \
    int4 bm = (BMAP)[blockIdx.x];                          \
    const int p = bm.x;                                    \
    if ((ST) && !(ST)[p].active) return;                   \
    const LevelDesc L = (DESC)[p];


template <typename T>
__global__ void k_cheb_first(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                             Coeffs<T> C, const T *__restrict__ b, T *__restrict__ x, T *__restrict__ d,
                             T invtheta) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        cell_cheb_first(L, c, C, b, x, d, invtheta);
    }
}

// The first two Chebyshev steps from a zero initial guess in one pass: the first
// iterate is x1 = d0 = invtheta D^-1 b pointwise, so its value at a neighbour is formed
// on the fly from b and the stored inverse diagonal; then
// r1 = D^-1 (b - A x1), d1 = c1 d0 + c2 r1, xout = x1 + d1.
template <typename T>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 8 : 5) k_cheb_first2(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                              Coeffs<T> C, const T *__restrict__ b, T *__restrict__ xout, T *__restrict__ d,
                              T invtheta, T c1, T c2) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        cell_cheb_first2(L, c, C, b, xout, d, invtheta, c1, c2);
    }
}

// One Chebyshev step on D^-1 A: r = D^-1 (b - A xin); d = c1 d + c2 r; xout = xin + d.
// FIRST: the first step from a nonzero iterate, d = c2 r (d is not read).
// With FUSE_RZ the kernel is the last of the level-0 V-cycle: it also reduces b . xout
// (b is the CG residual, xout the preconditioned residual) and finalises beta.
template <typename T, bool FUSE_RZ, bool FIRST = false>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 8 : 6)
k_cheb_step(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st, Coeffs<T> C,
            const T *__restrict__ b, const T *__restrict__ xin, T *__restrict__ xout, T *__restrict__ d, T c1, T c2,
            ReduceScratch rs, const int2 *__restrict__ pinfo) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    Acc<T> part;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        T bi;
        const T xo = cell_cheb_step<T, FIRST>(L, c, C, b, xin, xout, d, c1, c2, bi);
        if (FUSE_RZ) part = part + Acc<T>::prod(bi, xo);
    }
    if (FUSE_RZ) {
        double2 tot;
        if (reduce_last<T>(part, Acc<T>(), rs, pinfo[p], p, tot) && threadIdx.x == 0) {
            CgState &s = st[p];
            s.rz_old = s.rz;
            s.rz = tot.x;
            s.beta = (s.iters == 0 || s.rz_old == 0.0) ? 0.0 : s.rz / s.rz_old * s.cont;
            s.cont = 1.0;
        }
    }
}

// Restriction of the residual: bc[I] = sum over the children i of I of (b_i - (A x)_i).
template <typename T>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 8 : 5) k_restrict(const LevelDesc *__restrict__ fdesc, const LevelDesc *__restrict__ cdesc,
                           const int4 *__restrict__ bmap, CgState *st, Coeffs<T> C, const T *__restrict__ b,
                           const T *__restrict__ x, T *__restrict__ bc) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const int p = bm.x;
    if (st && !st[p].active) return;
    const LevelDesc Lc = cdesc[p];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)Lc.n; li_ += bm.z * kBlock) {
        Cell cc;
        cell_at(Lc, li_, cc);
        const LevelDesc L = fdesc[p];
        bc[cc.i] = cell_restrict(L, cc, C, b, x);
    }
}

// Prolongation of the coarse correction, in place: x += s * e[aggregate] (not at
// identity rows). Pointwise, so it streams at bandwidth; the first post-smoothing step
// then runs as a plain Chebyshev step on the corrected iterate.
template <typename T>
__global__ void k_prolong_add(const LevelDesc *__restrict__ desc, const LevelDesc *__restrict__ cdesc,
              const int4 *__restrict__ bmap, CgState *st, const uint8_t *__restrict__ dir, T *__restrict__ x,
              const T *__restrict__ e, T scale) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    const LevelDesc Lc = cdesc[p];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        if (dir[c.i]) continue;
        x[c.i] += scale * e[agg_index(Lc, c)];
    }
}

// Coarsest level: x = A^-1 b with the stored dense inverse (symmetric), one block of
// kMaxCoarse threads per problem. With FUSE_RZ (a problem whose finest level is its
// coarsest) it also sets rz and beta.
template <typename T, bool FUSE_RZ>
__global__ void k_coarse_solve(const LevelDesc *__restrict__ desc, const int *__restrict__ plist, CgState *st,
                               const double *__restrict__ Inv, const T *__restrict__ b, T *__restrict__ x) {
    pdl_enter();
    const int p = plist[blockIdx.x];
    if (st && !st[p].active) return;
    const LevelDesc L = desc[p];
    const int n = (int)L.n;
    const double *Ip = Inv + (long long)p * kMaxCoarse * kMaxCoarse;
    __shared__ double bs[kMaxCoarse];
    __shared__ double red[kMaxCoarse / 32];
    const int i = threadIdx.x;
    if (i < n) bs[i] = (double)b[L.off + i];
    __syncthreads();
    double xi = 0.0;
    if (i < n)
        for (int j = 0; j < n; j++) xi += Ip[j * kMaxCoarse + i] * bs[j];
    T xo = (T)xi;
    if (i < n) x[L.off + i] = xo;
    if (FUSE_RZ) {
        double v = i < n ? bs[i] * (double)xo : 0.0;
        v = warp_sum(v);
        if ((i & 31) == 0) red[i >> 5] = v;
        __syncthreads();
        if (i == 0) {
            double rz = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) rz += red[w];
            CgState &s = st[p];
            s.rz_old = s.rz;
            s.rz = rz;
            s.beta = (s.iters == 0 || s.rz_old == 0.0) ? 0.0 : s.rz / s.rz_old * s.cont;
            s.cont = 1.0;
        }
    }
}

// ---------------------------------------------------------------- fused tail
// The small levels of one problem (from level `lt`, where the problem first has at most
// tail_cells cells, down to its coarsest) run as one block: pre-smoothing, restriction,
// the dense coarsest solve, prolongation and post-smoothing, with block barriers between
// steps instead of kernel boundaries (on a 1M-cell grid this replaces about a dozen
// launches of a few thousand cells each per V-cycle). Same arithmetic, same buffers
// and the same result as the per-level kernels: the corrected iterate of level lt
// lands in its xb buffer.

template <typename T, bool CLUSTER>
__global__ void __launch_bounds__(kTailThreads) k_tail_cycle(const TailLevel<T> *__restrict__ tl,
                                                             const int4 *__restrict__ tails, const CgState *st,
                                                             const double *__restrict__ Inv, TailParams<T> tp) {
    pdl_enter();
    // one problem per block, or (CLUSTER) per thread-block cluster: its blocks share every
    // step's cells and meet at hardware cluster barriers
    unsigned rank = 0, nranks = 1;
    if constexpr (CLUSTER) {
        rank = cg::this_cluster().block_rank();
        nranks = cg::this_cluster().num_blocks();
    }
    const int4 t = tails[blockIdx.x / nranks];  // problem, first tail level, coarsest level
    const int p = t.x, lt = t.y, lc = t.z;
    if (st && !st[p].active) return;  // uniform over the problem's blocks
    auto sync = [&]() {
        if constexpr (CLUSTER) cg::this_cluster().sync();
        else __syncthreads();
    };
    const int first = (int)(rank * blockDim.x + threadIdx.x);
    const int stride = (int)(nranks * blockDim.x);
    const int deg = tp.deg;
    // descend
    for (int l = lt; l < lc; l++) {
        const TailLevel<T> V = tl[l];
        const LevelDesc L = V.desc[p];
        T *cur = V.xa, *oth = V.xb;
        int k0 = 1;
        if (deg >= 2) {
            for (int li = first; li < (int)L.n; li += stride) {
                Cell c;
                cell_at(L, li, c);
                cell_cheb_first2<T, CLUSTER>(L, c, V.C, V.b, V.xb, V.d, tp.invtheta, tp.c1[1], tp.c2[1]);
            }
            cur = V.xb;
            oth = V.xa;
            k0 = 2;
        } else {
            for (int li = first; li < (int)L.n; li += stride) {
                Cell c;
                cell_at(L, li, c);
                cell_cheb_first<T, CLUSTER>(L, c, V.C, V.b, V.xa, V.d, tp.invtheta);
            }
        }
        sync();
        for (int k = k0; k < deg; k++) {
            for (int li = first; li < (int)L.n; li += stride) {
                Cell c;
                cell_at(L, li, c);
                T bi;
                cell_cheb_step<T, false, CLUSTER>(L, c, V.C, V.b, cur, oth, V.d, tp.c1[k], tp.c2[k], bi);
            }
            sync();
            T *tmp = cur; cur = oth; oth = tmp;
        }
        const TailLevel<T> W = tl[l + 1];
        const LevelDesc Lc = W.desc[p];
        for (int li = first; li < (int)Lc.n; li += stride) {
            Cell cc;
            cell_at(Lc, li, cc);
            W.b[cc.i] = cell_restrict<T, CLUSTER>(L, cc, V.C, V.b, cur);
        }
        sync();
    }
    // coarsest: x = A^-1 b with the stored dense inverse (first block of the problem)
    {
        const TailLevel<T> V = tl[lc];
        const LevelDesc L = V.desc[p];
        const double *Ip = Inv + (long long)p * kMaxCoarse * kMaxCoarse;
        const int i = threadIdx.x;
        if (rank == 0 && i < (int)L.n) {
            double xi = 0.0;
            for (int j = 0; j < (int)L.n; j++) xi += Ip[j * kMaxCoarse + i] * (double)ldv<CLUSTER>(V.b, L.off + j);
            V.xb[L.off + i] = (T)xi;
        }
        sync();
    }
    // ascend: prolongation in place into the pre-smoothed iterate, then deg steps
    for (int l = lc - 1; l >= lt; l--) {
        const TailLevel<T> V = tl[l];
        const LevelDesc L = V.desc[p];
        const TailLevel<T> W = tl[l + 1];
        const LevelDesc Lc = W.desc[p];
        T *cur = (deg % 2 == 0) ? V.xb : V.xa;  // where pre-smoothing left its iterate
        for (int li = first; li < (int)L.n; li += stride) {
            Cell c;
            cell_at(L, li, c);
            if (V.dir[c.i]) continue;
            cur[c.i] += tp.coarse_scale *
                        ldv<CLUSTER>(W.xb, agg_index(Lc, c));
        }
        sync();
        for (int k = 0; k < deg; k++) {
            T *o = cur == V.xa ? V.xb : V.xa;
            for (int li = first; li < (int)L.n; li += stride) {
                Cell c;
                cell_at(L, li, c);
                T bi;
                if (k == 0) cell_cheb_step<T, true, CLUSTER>(L, c, V.C, V.b, cur, o, V.d, tp.c1[0], tp.invtheta, bi);
                else cell_cheb_step<T, false, CLUSTER>(L, c, V.C, V.b, cur, o, V.d, tp.c1[k], tp.c2[k], bi);
            }
            sync();
            cur = o;
        }
    }
}

// ---------------------------------------------------------------- CG kernels
// r = b - A x; reduce (r.r, b.b); activate the problem unless already converged. b.b runs over
// the free rows only: an identity row holds its Dirichlet value exactly, and the reference's
// solve (src/groundwater.jl:45-49, 78) measures reltol against the right-hand side of the free
// cells, so large Dirichlet heads must not loosen the test.
template <typename T>
__global__ void k_cg_start(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                           int *active_count, ReduceScratch rs, const int2 *__restrict__ pinfo, Coeffs<T> C,
                           const uint8_t *__restrict__ dir, const T *__restrict__ b, const T *__restrict__ x,
                           T *__restrict__ r, double tol2) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const int p = bm.x;
    const LevelDesc L = desc[p];
    Acc<T> rr, bb;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        T xi = x[c.i], Ax, dg;
        apply7(L, c, C, xi, [&](long long j, int, int, int) { return x[j]; }, Ax, dg);
        T bi = b[c.i];
        T ri = bi - Ax;
        r[c.i] = ri;
        rr = rr + Acc<T>::prod(ri, ri);
        if (!dir[c.i]) bb = bb + Acc<T>::prod(bi, bi);
    }
    double2 tot;
    if (reduce_last<T, 2>(rr, bb, rs, pinfo[p], p, tot) && threadIdx.x == 0) {
        CgState &s = st[p];
        s.rr = tot.x;
        s.bb = tot.y;
        s.tol2 = tol2;
        s.iters = 0;
        s.rz = 0.0;
        s.rz_old = 0.0;
        s.beta = 0.0;
        s.status = DPF_OK;
        bool act = s.bb > 0.0 && s.rr > tol2 * s.bb;
        if (!isfinite(s.rr)) { s.status = DPF_NAN; act = false; }
        s.active = act ? 1 : 0;
        if (act) atomicAdd(active_count, 1);
    }
}

// q = A p; alpha = rz / (p . q)
template <typename T>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_spmv_pq(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                          int *active_count, ReduceScratch rs, const int2 *__restrict__ pinfo, Coeffs<T> C,
                          const T *__restrict__ pv, T *__restrict__ q) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    Acc<T> part;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        T pi = pv[c.i], Ax, dg;
        apply7(L, c, C, pi, [&](long long j, int, int, int) { return pv[j]; }, Ax, dg);
        q[c.i] = Ax;
        part = part + Acc<T>::prod(pi, Ax);
    }
    double2 tot;
    if (reduce_last<T>(part, Acc<T>(), rs, pinfo[p], p, tot) && threadIdx.x == 0) {
        CgState &s = st[p];
        s.pq = tot.x;
        if (!isfinite(s.pq)) { s.alpha = 0.0; s.status = DPF_NAN; deactivate(s, active_count); }
        else if (!(s.pq > 0.0)) { s.alpha = 0.0; deactivate(s, active_count); }   // p = 0: exact solution
        else s.alpha = s.rz / s.pq;
    }
}

// x += alpha p; r -= alpha q; convergence test on r . r.
template <typename T>
__global__ void k_update_xr(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                            int *active_count, ReduceScratch rs, const int2 *__restrict__ pinfo, T *__restrict__ x,
                            T *__restrict__ r, const T *__restrict__ pv, const T *__restrict__ q, int maxiter) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    const double alpha = st[p].alpha;
    Acc<T> part;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        T a = (T)alpha;
        x[c.i] += a * pv[c.i];
        T ri = r[c.i] - a * q[c.i];
        r[c.i] = ri;
        part = part + Acc<T>::prod(ri, ri);
    }
    double2 tot;
    if (reduce_last<T>(part, Acc<T>(), rs, pinfo[p], p, tot) && threadIdx.x == 0) {
        CgState &s = st[p];
        s.rr = tot.x;
        s.iters++;
        s.total_iters++;
        if (!isfinite(s.rr)) { s.status = DPF_NAN; deactivate(s, active_count); }
        else if (s.rr <= s.tol2 * s.bb) deactivate(s, active_count);
        else if (s.iters >= maxiter) { s.status = DPF_NOT_CONVERGED; deactivate(s, active_count); }
    }
}

// p = z + beta p
template <typename T>
__global__ void k_update_p(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                           const T *__restrict__ z, T *__restrict__ pv) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    const T beta = (T)st[p].beta;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        pv[c.i] = beta == (T)0 ? z[c.i] : z[c.i] + beta * pv[c.i];
    }
}

// ----------------------------------- mixed precision: double-float CG recurrence
// The CG recurrence (iterate, residual, search direction, SpMV with the finest-level
// operator) runs on double-float numbers: an unevaluated sum hi + lo of two floats
// (about 48 significant bits) handled with FP32 arithmetic only (GB300's FP32 rate is
// many times its FP64 rate). The V-cycle preconditioner runs in plain FP32 on the
// rounded residual. FP32 storage alone is not enough here: with few Dirichlet cells
// the operator is nearly singular and the search directions are dominated by a
// smooth near-null mode whose small variations FP32 cannot resolve, so an FP32
// recurrence stagnates; 48 bits resolve them like FP64 does.
// Each solve round starts from the true FP64 residual (normalised by its norm) and
// ends by adding the correction to the FP64 solution; convergence is then confirmed
// on the true FP64 residual, and another round runs if it is not met.


// q = A p in double-float (flux form); alpha = rz / (p . q) (hi parts: q is accurate, so
// its leading float is too)
#ifndef DPF_DF_SPMV_MINB
#define DPF_DF_SPMV_MINB 8
#endif
__global__ void __launch_bounds__(kBlock, DPF_DF_SPMV_MINB) k_df_spmv_pq(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                             int *active_count, ReduceScratch rs, const int2 *__restrict__ pinfo, CoeffsDF C,
                             const float2 *__restrict__ pv, float2 *__restrict__ q) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    Acc<float> part;
    const long long sy = L.nz, sx = (long long)L.ny * L.nz;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const long long i = c.i;
        const float2 pi = pv[i];
        float2 a = df_mul(C.leak[i], pi);
        if (c.iz + 1 < L.nz) a = df_add(a, df_mul(C.cz[i], df_sub(pi, pv[i + 1])));
        if (c.iz > 0) a = df_add(a, df_mul(C.cz[i - 1], df_sub(pi, pv[i - 1])));
        if (c.iy + 1 < L.ny) a = df_add(a, df_mul(C.cy[i], df_sub(pi, pv[i + sy])));
        if (c.iy > 0) a = df_add(a, df_mul(C.cy[i - sy], df_sub(pi, pv[i - sy])));
        if (c.ix + 1 < L.nx) a = df_add(a, df_mul(C.cx[i], df_sub(pi, pv[i + sx])));
        if (c.ix > 0) a = df_add(a, df_mul(C.cx[i - sx], df_sub(pi, pv[i - sx])));
        q[i] = a;
        part = part + Acc<float>::prod(pi.x, a.x);
    }
    double2 tot;
    if (reduce_last<float>(part, Acc<float>(), rs, pinfo[p], p, tot) && threadIdx.x == 0)
        finish_pq(st[p], tot.x, active_count);
}

// x64 += (alpha scale) p in FP64 (the solution keeps all 53 bits: a 48-bit double-float
// solution would put the FP64 check's floor 32x higher and cost extra rounds);
// r -= alpha q (double-float); r32 = leading float of r for the V-cycle; convergence test
// on the recursive residual (r is normalised by `scale`)
__global__ void k_df_update_xr(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                               int *active_count, ReduceScratch rs, const int2 *__restrict__ pinfo,
                               double *__restrict__ x64, float2 *__restrict__ r, float *__restrict__ r32,
                               const float2 *__restrict__ pv, const float2 *__restrict__ q, int maxiter) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    const float2 a = df_from_double(st[p].alpha);
    const double as = st[p].alpha * st[p].scale;
    Acc<float> part;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        const long long i = L.off + li_;  // pointwise: no cell decode
        const float2 pi = pv[i];
        x64[i] = fma(as, (double)pi.x + (double)pi.y, x64[i]);
        const float2 ri = df_sub(r[i], df_mul(a, q[i]));
        r[i] = ri;
        r32[i] = ri.x;
        part = part + Acc<float>::prod(ri.x, ri.x);
    }
    double2 tot;
    if (reduce_last<float>(part, Acc<float>(), rs, pinfo[p], p, tot) && threadIdx.x == 0) {
        CgState &s = st[p];
        s.rr = tot.x;
        s.iters++;
        s.total_iters++;
        if (!isfinite(s.rr)) { s.status = DPF_NAN; deactivate(s, active_count); }
        else if (s.rr * s.scale * s.scale <= s.tol2 * s.obb || s.rr <= kRoundDrop2) deactivate(s, active_count);
        else if (s.total_iters >= maxiter) { s.status = DPF_NOT_CONVERGED; deactivate(s, active_count); }
    }
}

// p = z + beta p (double-float; z is the FP32 preconditioned residual)
__global__ void k_df_update_p(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                              const float *__restrict__ z, float2 *__restrict__ pv) {
    pdl_enter();
    DPF_BLOCK_PROLOGUE(desc, bmap, st)
    const double beta = st[p].beta;
    const float2 b = df_from_double(beta);
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        const long long i = L.off + li_;  // pointwise: no cell decode
        const float2 zi = make_float2(z[i], 0.0f);
        pv[i] = beta == 0.0 ? zi : df_add(zi, df_mul(b, pv[i]));
    }
}

// True residual r64 = b - A x64 in FP64 flux form; decides whether a (further) round is
// needed. FIRST: the start of a solve. ZERO (with FIRST): the initial guess is zero on
// free cells and the Dirichlet value on identity rows, so r = b on free rows and 0 on
// identity rows (free rows have no coupling to identity rows) and no product is formed.
template <bool FIRST, bool ZERO = false>
__global__ void k_df_residual(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, CgState *st,
                              int *active_count, ReduceScratch rs, const int2 *__restrict__ pinfo,
                              Coeffs<double> C, Coeffs<float> C16, const uint8_t *__restrict__ dir,
                              const double *__restrict__ b, const double *__restrict__ x, double *__restrict__ r,
                              double tol2, int maxiter, int max_rounds) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const int p = bm.x;
    if (!FIRST && st[p].ru_flag == 0) return;  // finished in an earlier round
    const LevelDesc L = desc[p];
    Acc<double> rr, bb;  // FIRST: |r|^2, |b|^2; otherwise |r|^2 and the rounding floor / 2^-96
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        double ri, bi, xi = 0.0;
        float dg = 0.0f;
        if (ZERO) {
            c.i = L.off + li_;
            bi = b[c.i];
            ri = dir[c.i] ? 0.0 : bi;
        } else {
            cell_at(L, li_, c);
            xi = x[c.i];
            double Ax;
            apply7_f32diag(L, c, C, C16, xi, x, Ax, dg);
            bi = b[c.i];
            ri = bi - Ax;
        }
        r[c.i] = ri;
        rr.v += ri * ri;
        if (dir[c.i]) {
            // identity row: holds its Dirichlet value exactly; in neither |b| nor the floor
        } else if (FIRST) {
            bb.v += bi * bi;
        } else {
            // rounding bound of b_i - (A x)_i and of x itself, u (|b_i| + 2 diag_i |x_i|) (neighbours
            // of x_i taken as |x_i|), with the unit roundoff of the double-float recurrence that
            // produced x, u = 2^-48: its search directions and residuals carry about 48 bits, so the
            // true residual of a converged round settles near this bound, about 32 times the FP64
            // one; a round that reaches it is accepted without a further round that cannot improve it.
            // An estimate: formed in FP32 (u applied to the sum), squared and summed in FP64.
            const double f = (double)fmaf(2.0f * dg, abs_float_trunc(xi), abs_float_trunc(bi));
            bb.v = fma(f, f, bb.v);
        }
    }
    if (!FIRST) bb.v *= 0x1p-96;
    double2 tot;
    if (reduce_last<double, 2>(rr, bb, rs, pinfo[p], p, tot) && threadIdx.x == 0) {
        CgState &s = st[p];
        s.orr = tot.x;
        bool go;
        if (FIRST) {
            s.floor2 = 0.0;
            s.obb = tot.y;
            s.tol2 = tol2;
            s.status = DPF_OK;
            s.total_iters = 0;
            s.outer = 0;
            s.stall = 0;
            go = s.obb > 0.0 && s.orr > tol2 * s.obb;
            if (!isfinite(s.orr)) { s.status = DPF_NAN; go = false; }
        } else {
            s.outer++;
            s.floor2 = tot.y;
            // the true residual is at the FP64 rounding floor of b - A x when it is within the
            // floor's bound, or when a whole round did not even halve it: no further accuracy
            // exists in FP64, so the solve is accepted there
            const bool at_floor = s.orr <= s.floor2 || s.orr > 0.25 * s.orr_prev;
            go = true;
            if (!isfinite(s.orr)) { s.status = DPF_NAN; go = false; }
            else if (s.orr <= tol2 * s.obb || at_floor) go = false;
            else if (s.total_iters >= maxiter || s.outer >= max_rounds) { s.status = DPF_NOT_CONVERGED; go = false; }
        }
        s.orr_prev = s.orr;
        s.ru_flag = go ? 1 : 0;  // problem takes part in the next round
        s.active = go ? 1 : 0;
        if (FIRST) {
            s.iters = 0;
            s.rz = 0.0;
            s.rz_old = 0.0;
            s.beta = 0.0;
            s.cont = 1.0;
        }
        if (go) {
            // a further round continues the Krylov process on the true residual (residual
            // replacement): the direction is kept, and the next beta is rescaled by the change
            // of normalisation new/old so that p = z + beta p holds in the new units
            const double sc = sqrt(s.orr);
            if (!FIRST) s.cont = sc / s.scale;
            s.scale = sc;
            atomicAdd(active_count, 1);
        }
    }
}

// start of a round: r = r64 / scale (double-float and its leading float)
__global__ void k_df_begin(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, const CgState *st,
                           const double *__restrict__ r64, float2 *__restrict__ r, float *__restrict__ r32) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const int p = bm.x;
    if (!st[p].ru_flag) return;
    const LevelDesc L = desc[p];
    const double inv = 1.0 / st[p].scale;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        const long long i = L.off + li_;
        const double w = r64[i] * inv;
        float2 v;
        double w48;
        if (!split48(w, v.x, v.y, w48)) v = df_from_double(w);  // 48 bits either way
        r[i] = v;
        r32[i] = v.x;
    }
}

// ------------------------------------------------------------ misc vector kernels
__global__ void k_state_init(CgState *st, int nprob) {
    pdl_enter();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    CgState s;
    memset(&s, 0, sizeof(s));
    s.cont = 1.0;
    st[p] = s;
}

// adjoint right-hand side: rhs = delta at free cells, 0 at Dirichlet cells; x = 0
__global__ void k_adjoint_rhs(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                              const uint8_t *__restrict__ dir, const double *__restrict__ delta,
                              double *__restrict__ rhs, double *__restrict__ x) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        rhs[c.i] = dir[c.i] ? 0.0 : delta[c.i];
        x[c.i] = 0.0;
    }
}

// delta = 2 h at observation cells (J = sum h[obs]^2), 0 elsewhere (delta zeroed before)
__global__ void k_obs_delta(const long long *__restrict__ obs_global, long long nobs, const double *__restrict__ h,
                            double *__restrict__ delta) {
    pdl_enter();
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nobs) return;
    long long i = obs_global[k];
    atomicAdd(&delta[i], 2.0 * h[i]);
}

// storage shift S_i V_i / dt (transient)
__global__ void k_shift(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                        const ProbParam *__restrict__ prm, const double *__restrict__ Ss, double inv_dt,
                        double *__restrict__ shift) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        shift[c.i] = Ss[c.i] * prm[bm.x].vol * inv_dt;
    }
}

// b_n = b0 + shift * h_prev (transient right-hand side); Dirichlet rows keep b0 = dirichleths
__global__ void k_axpy_rhs(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                           const uint8_t *__restrict__ dir, const double *__restrict__ b0,
                           const double *__restrict__ shift, const double *__restrict__ hprev,
                           double *__restrict__ b) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        b[c.i] = dir[c.i] ? b0[c.i] : b0[c.i] + shift[c.i] * hprev[c.i];
    }
}

// ------------------------------------------------------------- gradients
// dKs_f = -aol_f (h_a - h_b)(lambda_a - lambda_b), in the reference face order; with
// accumulate != 0 it adds to dKs (transient adjoint sums over steps).
__global__ void k_grad_faces(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                             const ProbParam *__restrict__ prm, const double *__restrict__ h,
                             const double *__restrict__ lam, double *__restrict__ dKs, int accumulate) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const ProbParam P = prm[bm.x];
        const long long st3[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
        const int co[3] = {c.ix, c.iy, c.iz};
        const int nn[3] = {L.nx, L.ny, L.nz};
        const double hi = h[c.i], li = lam[c.i];
    #pragma unroll
        for (int d = 0; d < 3; d++) {
            if (co[d] + 1 < nn[d]) {
                long long j = c.i + st3[d];
                double g = -P.aol[d] * (hi - h[j]) * (li - lam[j]);
                long long f = P.face_off + regular_face_index(L.nx, L.ny, L.nz, c.ix, c.iy, c.iz, d);
                if (accumulate) dKs[f] += g; else dKs[f] = g;
            }
        }
    }
}

// dlogK_i = sum over the faces of i of dK_f/dlogK_i * dKs_f, with dKs_f formed on the fly
// from h and lambda; K_f and its derivative come from the per-cell values kc.
__global__ void k_grad_logk(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                            const ProbParam *__restrict__ prm, const double *__restrict__ kc, int kind,
                            const double *__restrict__ h, const double *__restrict__ lam, double *__restrict__ g) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const ProbParam P = prm[bm.x];
        const long long st3[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
        const int co[3] = {c.ix, c.iy, c.iz};
        const int nn[3] = {L.nx, L.ny, L.nz};
        const double hi = h[c.i], li = lam[c.i], ki = kc[c.i];
        double acc = 0.0;
        if (kind == DPF_MEAN_GEOMETRIC) {
            // dK_f/dlogK_i = K_f / 2 = kc_i kc_j / 2: per direction sum kc_j (h_i-h_j)(l_i-l_j),
            // then scale by -aol kc_i / 2 (4 FP64 operations per face)
    #pragma unroll
            for (int d = 0; d < 3; d++) {
                double sd = 0.0;
                if (co[d] + 1 < nn[d]) {
                    const long long j = c.i + st3[d];
                    sd = fma(kc[j], (hi - h[j]) * (li - lam[j]), sd);
                }
                if (co[d] > 0) {
                    const long long j = c.i - st3[d];
                    sd = fma(kc[j], (hi - h[j]) * (li - lam[j]), sd);
                }
                acc = fma(-0.5 * P.aol[d] * ki, sd, acc);
            }
            g[c.i] = acc;
            continue;
        }
    #pragma unroll
        for (int d = 0; d < 3; d++) {
    #pragma unroll
            for (int s = -1; s <= 1; s += 2) {
                bool ok = s > 0 ? co[d] + 1 < nn[d] : co[d] > 0;
                if (!ok) continue;
                long long j = c.i + s * st3[d];
                double dK = -P.aol[d] * (hi - h[j]) * (li - lam[j]);
                double K = face_mean_k(ki, kc[j], kind);
                acc += face_mean_dlogk(K, ki, kind) * dK;
            }
        }
        g[c.i] = acc;
    }
}

// Mixed handles, geometric means: d/dlogK of k_grad_logk in double-float arithmetic on the FP32
// pipe (the FP64 form is bound by GB300's FP64 rate). A pre-pass splits h, lambda and the cell
// factors kc into double-floats (integer operations, 48 bits); the differences h_i - h_j and
// lambda_i - lambda_j are then formed from those, which keeps about 48 bits of each difference
// relative to |h| (a relative error of 2^-48 |h| / |h_i - h_j|, far inside the gradient's 1e-6).
__global__ void k_grad_split(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                             const double *__restrict__ h, const double *__restrict__ lam,
                             const double *__restrict__ kc, float2 *__restrict__ hd, float2 *__restrict__ ld,
                             float2 *__restrict__ kd) {
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    auto split = [](double v) {
        float2 q;
        double v48;
        if (!split48(v, q.x, q.y, v48)) q = df_from_double(v);
        return q;
    };
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        const long long i = L.off + li_;
        hd[i] = split(h[i]);
        ld[i] = split(lam[i]);
        kd[i] = split(kc[i]);
    }
}

__global__ void k_grad_logk_df(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                               const ProbParam *__restrict__ prm, const float2 *__restrict__ kd,
                               const float2 *__restrict__ hd, const float2 *__restrict__ ld, double *__restrict__ g) {
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    const ProbParam P = prm[bm.x];
    const float2 w3[3] = {df_from_double(-0.5 * P.aol[0]), df_from_double(-0.5 * P.aol[1]),
                          df_from_double(-0.5 * P.aol[2])};
    const long long st3[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const int co[3] = {c.ix, c.iy, c.iz};
        const int nn[3] = {L.nx, L.ny, L.nz};
        const float2 hi = hd[c.i], li = ld[c.i], ki = kd[c.i];
        float2 acc = make_float2(0.f, 0.f);
    #pragma unroll
        for (int d = 0; d < 3; d++) {
            float2 sd = make_float2(0.f, 0.f);
            if (co[d] + 1 < nn[d]) {
                const long long j = c.i + st3[d];
                sd = df_add(sd, df_mul(kd[j], df_mul(df_sub(hi, hd[j]), df_sub(li, ld[j]))));
            }
            if (co[d] > 0) {
                const long long j = c.i - st3[d];
                sd = df_add(sd, df_mul(kd[j], df_mul(df_sub(hi, hd[j]), df_sub(li, ld[j]))));
            }
            acc = df_add(acc, df_mul(df_mul(w3[d], ki), sd));
        }
        g[c.i] = df_to_double(acc);
    }
}

// per-cell values for the face means: exp(logK / 2) (geometric) or exp(logK) (harmonic)
__global__ void k_cell_k(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                         const double *__restrict__ logK, int kind, double *__restrict__ kc) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        double v = logK[c.i];
        kc[c.i] = exp(kind == DPF_MEAN_GEOMETRIC ? 0.5 * v : v);
    }
}

// inverse diagonal of a level from its FP64 coefficients (the smoothers multiply
// instead of dividing); written in FP64 and/or FP32
__global__ void k_invdiag(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, Coeffs<double> C,
                          Coeffs<float> C16, double *__restrict__ idg, float *__restrict__ idg32) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        if (idg) {
            const double v = 1.0 / diag7(L, c, C);
            idg[c.i] = v;
            if (idg32) idg32[c.i] = (float)v;
        } else {
            // the FP32 V-cycle: the diagonal its kernels form from the bf16 coefficients
            idg32[c.i] = 1.0f / diag7(L, c, C16);
        }
    }
}

// ddirichleths_k = delta_k + sum over free neighbours j of K_f aol_f lambda_j (Dirichlet k);
// 0 at free cells. dQs = lambda (0 at Dirichlet cells). Either output may be null.
__global__ void k_grad_dh_q(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                            const ProbParam *__restrict__ prm, FaceK fk, const uint8_t *__restrict__ dir,
                            const double *__restrict__ delta, const double *__restrict__ lam, double *ddh,
                            double *dQs, int accumulate) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const ProbParam P = prm[bm.x];
        const bool isd = dir[c.i];
        if (dQs) {
            double v = isd ? 0.0 : lam[c.i];
            if (accumulate) dQs[c.i] += v; else dQs[c.i] = v;
        }
        if (!ddh) continue;
        double acc = 0.0;
        if (isd) {
            if (delta) acc = delta[c.i];
            const long long st3[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
            const int co[3] = {c.ix, c.iy, c.iz};
            const int nn[3] = {L.nx, L.ny, L.nz};
            for (int d = 0; d < 3; d++)
                for (int s = -1; s <= 1; s += 2) {
                    bool ok = s > 0 ? co[d] + 1 < nn[d] : co[d] > 0;
                    if (!ok) continue;
                    long long j = c.i + s * st3[d];
                    if (dir[j]) continue;
                    acc += fk(L, P, c, d, s, j) * P.aol[d] * lam[j];
                }
        }
        if (accumulate) ddh[c.i] += acc; else ddh[c.i] = acc;
    }
}

// Ks in the reference face order from the per-cell values kc
__global__ void k_logk_to_faces(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                                const ProbParam *__restrict__ prm, const double *__restrict__ kc, int kind,
                                double *__restrict__ Ks) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const ProbParam P = prm[bm.x];
        const long long st3[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
        const int co[3] = {c.ix, c.iy, c.iz};
        const int nn[3] = {L.nx, L.ny, L.nz};
        for (int d = 0; d < 3; d++)
            if (co[d] + 1 < nn[d])
                Ks[P.face_off + regular_face_index(L.nx, L.ny, L.nz, c.ix, c.iy, c.iz, d)] =
                    face_mean_k(kc[c.i], kc[c.i + st3[d]], kind);
    }
}

// dlogK from dKs (gather over the six faces of each cell)
__global__ void k_logk_vjp(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                           const ProbParam *__restrict__ prm, const double *__restrict__ kc, int kind,
                           const double *__restrict__ dKs, double *__restrict__ g) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const ProbParam P = prm[bm.x];
        const long long st3[3] = {(long long)L.ny * L.nz, (long long)L.nz, 1};
        const int co[3] = {c.ix, c.iy, c.iz};
        const int nn[3] = {L.nx, L.ny, L.nz};
        const double ki = kc[c.i];
        double acc = 0.0;
        for (int d = 0; d < 3; d++)
            for (int s = -1; s <= 1; s += 2) {
                bool ok = s > 0 ? co[d] + 1 < nn[d] : co[d] > 0;
                if (!ok) continue;
                long long j = c.i + s * st3[d];
                int ax = c.ix, ay = c.iy, az = c.iz;
                if (s < 0) { if (d == 0) ax--; else if (d == 1) ay--; else az--; }
                long long f = P.face_off + regular_face_index(L.nx, L.ny, L.nz, ax, ay, az, d);
                double K = face_mean_k(ki, kc[j], kind);
                acc += face_mean_dlogk(K, ki, kind) * dKs[f];
            }
        g[c.i] = acc;
    }
}

// y = A x (FP64 fine operator; Dirichlet rows identity)
__global__ void k_apply(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, Coeffs<double> C,
                        const double *__restrict__ x, double *__restrict__ y) {
    pdl_enter();
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        double Ax, dg;
        apply7(L, c, C, x[c.i], [&](long long j, int, int, int) { return x[j]; }, Ax, dg);
        y[c.i] = Ax;
    }
}

// The FP64 operator in the banded Cholesky's storage (dpf_direct.h): per cell its diagonal
// leak + the sum of its face coefficients, and, from the cell on the lower side of each face,
// the coupling -c at (max, min) of the two cells' band rows. Dirichlet rows are identity rows.
__global__ void k_band_fill(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap, Coeffs<double> C,
                            const long long *__restrict__ iperm, long long w, double *__restrict__ band) {
    int4 bm = bmap[blockIdx.x];
    const LevelDesc L = desc[bm.x];
    const long long sy = L.nz, sx = (long long)L.ny * L.nz;
    for (int li_ = bm.y * kBlock + (int)threadIdx.x; li_ < (int)L.n; li_ += bm.z * kBlock) {
        Cell c;
        cell_at(L, li_, c);
        const long long i = c.i, k = iperm[i];
        double d = C.leak[i];
        const bool up[3] = {c.iz + 1 < L.nz, c.iy + 1 < L.ny, c.ix + 1 < L.nx};
        const long long st[3] = {1, sy, sx};
        const double *cf[3] = {C.cz, C.cy, C.cx};
        if (c.iz > 0) d += C.cz[i - 1];
        if (c.iy > 0) d += C.cy[i - sy];
        if (c.ix > 0) d += C.cx[i - sx];
    #pragma unroll
        for (int a = 0; a < 3; a++) {
            if (!up[a]) continue;
            const double v = cf[a][i];
            d += v;
            if (v != 0.0) {
                const long long kj = iperm[i + st[a]];
                const long long r = max(k, kj), q = min(k, kj);
                if (r - q <= w) band[q * (w + 1) + (r - q)] = -v;
            }
        }
        band[k * (w + 1)] = d;
    }
}

// ================================================================ host side
static void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e), e);
}
#define CK(x) ck((x), #x)
#define LAUNCH_CHECK() ck(cudaGetLastError(), "kernel launch")

static void configure_kernels();

// Launch with programmatic stream serialization: the launch is prepared while the previous
// kernel on the stream runs and its blocks start as that kernel's blocks exit; each solver
// kernel's pdl_enter() waits for the previous kernel's completion and memory before it
// touches memory, so the order is that of plain launches (also inside captured graphs).
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args &&...args) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = at;
#ifndef DPF_PDL
#define DPF_PDL 1
#endif
    cfg.numAttrs = DPF_PDL;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
    if (e != cudaSuccess) {
        cudaGetLastError();
        const char *name = nullptr;
        if (cudaFuncGetName(&name, (const void *)kernel) != cudaSuccess) {
            cudaGetLastError();
            name = "?";
        }
        throw CudaError(std::string("kernel launch (") + name + ", grid " + std::to_string(grid.x) + ", block " +
                            std::to_string(block.x) + ", dynamic shared " + std::to_string(smem) +
                            " B): " + cudaGetErrorString(e),
                        e);
    }
}

template <typename T>
static T *dalloc(size_t n, DevList &owned) {
    void *p = nullptr;
    if (n == 0) n = 1;
    // 64 bytes of padding: bulk copies widen their ranges to 16-byte boundaries
    cudaError_t e = dev_malloc(&p, n * sizeof(T) + 64);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw OomError(std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) + " bytes failed");
    }
    owned.push_back(p);
    return (T *)p;
}

// host check of the invariant-integer division on the numerators a level can produce
static void check_fast_div(unsigned d, unsigned m, int l, unsigned nmax) {
    auto q = [&](unsigned n) { return (unsigned)(((unsigned long long)n * m >> 32) + n) >> l; };
    unsigned probes[] = {0u, 1u, d - 1, d, d + 1, 2 * d - 1, nmax > 0 ? nmax - 1 : 0, nmax, nmax / 2, nmax / 3};
    for (unsigned n : probes)
        if (q(n) != n / d) throw DpfError("invariant-integer division self-check failed", DPF_CUDA);
    for (unsigned n = 0; n < nmax && n < 4096; n++)
        if (q(n) != n / d) throw DpfError("invariant-integer division self-check failed", DPF_CUDA);
}

// Launch map over the problems marked in `take`. Kernels loop over their cells with a
// stride of (blocks of the problem) x kBlock, so a problem's block count is chosen to
// fill the GPU once: about `target` blocks in total (SMs x resident blocks per SM),
// split in proportion to the problems' cells, never more than one cell per thread.
static BlockMap build_map(const std::vector<LevelDesc> &desc, const std::vector<int> &take, DevList &own,
                         int nprob, long long target) {
    BlockMap m;
    long long total = 0;
    for (int p = 0; p < nprob; p++)
        if (take[p]) total += desc[p].n;
    std::vector<int4> map;
    std::vector<int2> pinfo(nprob, make_int2(0, 0));
    for (int p = 0; p < nprob; p++) {
        if (!take[p]) continue;
        long long full = (desc[p].n + kBlock - 1) / kBlock;
        long long share = total > 0 ? (long long)((double)target * (double)desc[p].n / (double)total + 0.5) : 1;
        int nb = (int)std::max(1LL, std::min(full, share));
        pinfo[p] = make_int2((int)map.size(), nb);
        for (int b = 0; b < nb; b++) map.push_back(make_int4(p, b, nb, 0));
    }
    m.nblocks = (int)map.size();
    m.d_map = dalloc<int4>(map.size(), own);
    m.d_pinfo = dalloc<int2>(nprob, own);
    if (!map.empty()) CK(cudaMemcpy(m.d_map, map.data(), map.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m.d_pinfo, pinfo.data(), nprob * sizeof(int2), cudaMemcpyHostToDevice));
    return m;
}

// Plane-marching work of a level. Per smoothed problem the grid is cut into slabs of whole
// rows (plane_rows: up to `cells` cells, so a slab is contiguous in every array), and the
// planes of all slabs of all problems form one sequence of plane pairs (the restriction sums
// pairs of planes) weighted by their cells. The sequence is cut into contiguous runs of about
// equal weight, one per block (SMs x blocks_per_sm blocks, fewer on small levels), so
// every block of a launch gets the same work whatever the batch's sizes; a run that crosses a
// slab boundary becomes several items, which the block marches through one after another.
// Items start on even planes and end on one, or on the grid's last plane.
void StructBatch::build_plane_items(PlaneItems &P, const Level &L, const std::vector<int> &take, int sms,
                                    int cells, int blocks_per_sm,
                                    const std::vector<std::vector<std::array<int, 3>>> *shapes, int l) {
    P.ok = false;
    P.cells = cells;
    // FP32 V-cycles only: with 8-byte values the stages of a 768-cell slab allow one block
    // per SM, and the FP64 smoothers are faster as grid-stride kernels
    if (cells <= 0 || !mixed) return;
    long long total = 0;
    for (int p = 0; p < nprob; p++) {
        if (!take[p]) continue;
        const LevelDesc &D = L.h_desc[p];
        if (D.nz > cells) return;  // a row must fit a slab
        total += D.n;
    }
    if (total == 0) return;
    // the units: plane pairs of every slab, in problem, slab, plane order
    struct Unit {
        int p, y0, x0, x1;
        long long w;
    };
    std::vector<Unit> units;
    for (int p = 0; p < nprob; p++) {
        if (!take[p]) continue;
        const LevelDesc &D = L.h_desc[p];
        const int Ty = plane_rows(D.ny, D.nz, cells);
        for (int y0 = 0; y0 < D.ny; y0 += Ty) {
            const long long rc = (long long)std::min(Ty, D.ny - y0) * D.nz;
            for (int x0 = 0; x0 < D.nx; x0 += 2) {
                const int x1 = std::min(x0 + 2, D.nx);
                units.push_back(Unit{p, y0, x0, x1, rc * (x1 - x0)});
            }
        }
        P.halo = std::max(P.halo, (Ty + 2) * D.nz);
        P.cy = std::max(P.cy, (Ty + 1) * D.nz);
        P.slab = std::max(P.slab, Ty * D.nz);
        P.halo2 = std::max(P.halo2, (Ty + 4) * D.nz);
        P.cy2 = std::max(P.cy2, (Ty + 3) * D.nz);
        if (shapes && l + 1 < (int)(*shapes)[p].size()) {
            const int cnz = (*shapes)[p][l + 1][2];
            P.coarse = std::max(P.coarse, ((Ty + 2) / 2 + 2) * cnz);
            P.coarse2 = std::max(P.coarse2, ((Ty + 4) / 2 + 2) * cnz);
        }
    }
    // on the finest level at least 4 plane pairs per block where the level allows: every run also
    // stages the plane on each side of it, which for shorter runs costs more bandwidth than the
    // parallelism gains; the coarser levels are latency-bound and take as many blocks as they can
    const long long target = (long long)sms * std::max(1, blocks_per_sm);
    const long long min_pairs = l == 0 ? 4 : 1;
    const int nb = (int)std::max(1LL, std::min<long long>(target, ((long long)units.size() + min_pairs - 1) / min_pairs));
    std::vector<int4> items;
    std::vector<int> first(nb + 1, 0);
    std::vector<int2> pinfo(nprob, make_int2(0, 0));
    long long acc = 0;
    size_t u = 0;
    for (int blk = 0; blk < nb; blk++) {
        first[blk] = (int)items.size();
        // units up to the block's share of the cumulative weight (at least one; the last block
        // takes what is left)
        const long long end = blk + 1 == nb ? -1 : (long long)((double)total * (blk + 1) / nb + 0.5);
        bool took = false;
        while (u < units.size() && (!took || end < 0 || acc + units[u].w / 2 <= end) &&
               (units.size() - u) > (size_t)(nb - 1 - blk)) {
            const Unit &U = units[u];
            if (!items.empty() && (int)items.size() > first[blk] && items.back().x == U.p && items.back().y == U.y0 &&
                items.back().w == U.x0)
                items.back().w = U.x1;  // extend the block's current item
            else
                items.push_back(make_int4(U.p, U.y0, U.x0, U.x1));
            acc += U.w;
            took = true;
            u++;
        }
    }
    first[nb] = (int)items.size();
    if (u != units.size()) throw std::logic_error("plane work partition left units unassigned");
    for (int w = 0; w < (int)items.size(); w++) {
        const int p = items[w].x;
        if (pinfo[p].y == 0) pinfo[p].x = w;
        pinfo[p].y++;
    }
    P.n = (int)items.size();
    P.nb = nb;
    P.items = dalloc<int4>(items.size(), owned);
    P.first = dalloc<int>(first.size(), owned);
    P.pinfo = dalloc<int2>(nprob, owned);
    CK(cudaMemcpy(P.items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.first, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.pinfo, pinfo.data(), nprob * sizeof(int2), cudaMemcpyHostToDevice));
    P.ok = true;
}

StructBatch::StructBatch(const std::vector<GridSpec> &grids, const std::vector<std::vector<int64_t>> &dnodes,
                         const dpf_options &o, cudaStream_t s)
    : opt(o), stream(s) {
    nprob = (int)grids.size();
    if (nprob <= 0) throw BadInput("empty batch");
    if (opt.max_coarse < 1 || opt.max_coarse > kMaxCoarse) opt.max_coarse = kMaxCoarse;
    if (opt.cheb_degree == 0) opt.cheb_degree = 2;  // regular grids' defaults (2x2x2 aggregates)
    if (!(opt.coarse_scale > 0)) opt.coarse_scale = 2.0;
    if (opt.cheb_degree < 1) opt.cheb_degree = 1;
    if (opt.cheb_degree > 8) opt.cheb_degree = 8;
    mixed = opt.precision == DPF_PREC_MIXED;
    // per-problem hierarchy shapes
    nlev.resize(nprob);
    std::vector<std::vector<std::array<int, 3>>> shapes(nprob);
    nlev_max = 0;
    for (int p = 0; p < nprob; p++) {
        auto g = grids[p];
        if (g.n[0] < 1 || g.n[1] < 1 || g.n[2] < 1) throw BadInput("grid dimensions must be >= 1");
        long long n = (long long)g.n[0] * g.n[1] * g.n[2];
        if (n >= (1LL << 31)) throw BadInput("a single grid must have fewer than 2^31 cells");
        std::array<int, 3> d = {g.n[0], g.n[1], g.n[2]};
        shapes[p].push_back(d);
        while ((long long)d[0] * d[1] * d[2] > opt.max_coarse) {
            d = {(d[0] + 1) / 2, (d[1] + 1) / 2, (d[2] + 1) / 2};
            shapes[p].push_back(d);
        }
        nlev[p] = (int)shapes[p].size();
        nlev_max = std::max(nlev_max, nlev[p]);
    }
    // function attributes of this device's kernels, set once before any launch
    configure_kernels();
    // launch shape: grids sized to the resident capacity of the device
    int dev = 0, sms = 152;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long target_blocks = (long long)sms * std::max(1, opt.blocks_per_sm);
    // fused tail: from the first level (>= 1) at which a problem has at most tail_cells cells
    std::vector<int> tail_at(nprob);
    for (int p = 0; p < nprob; p++) {
        tail_at[p] = nlev[p];  // none
        if (opt.tail_cells <= 0 || nlev[p] < 2) continue;
        for (int l = 1; l < nlev[p]; l++) {
            auto d = shapes[p][l];
            if ((long long)d[0] * d[1] * d[2] <= opt.tail_cells) { tail_at[p] = l; break; }
        }
        if (tail_at[p] < nlev[p]) tails.push_back(make_int4(p, tail_at[p], nlev[p] - 1, 0));
    }
    // level descriptors
    lv.resize(nlev_max);
    int maxblocks = 0;
    for (int l = 0; l < nlev_max; l++) {
        Level &L = lv[l];
        LevelDesc unit{1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
        fast_div_magic(1u, unit.mag_nz, unit.sh_nz);
        fast_div_magic(1u, unit.mag_ny, unit.sh_ny);
        L.h_desc.assign(nprob, unit);
        long long off = 0;
        std::vector<int> has(nprob, 0), smooth(nprob, 0), restr(nprob, 0);
        for (int p = 0; p < nprob; p++) {
            if (l >= nlev[p]) continue;
            auto d = shapes[p][l];
            LevelDesc &D = L.h_desc[p];
            D.nx = d[0]; D.ny = d[1]; D.nz = d[2];
            D.n = (long long)d[0] * d[1] * d[2];
            D.off = off;
            fast_div_magic((unsigned)d[2], D.mag_nz, D.sh_nz);
            fast_div_magic((unsigned)d[1], D.mag_ny, D.sh_ny);
            check_fast_div((unsigned)d[2], D.mag_nz, D.sh_nz, (unsigned)D.n);
            check_fast_div((unsigned)d[1], D.mag_ny, D.sh_ny, (unsigned)(D.n / d[2]));
            off += D.n;
            has[p] = 1;
            smooth[p] = l < nlev[p] - 1 && l < tail_at[p];
            restr[p] = l >= 1 && l <= tail_at[p];
            if (l == nlev[p] - 1) {
                L.coarse_list.push_back(p);
                if (tail_at[p] == nlev[p]) {
                    L.csolve_list.push_back(p);
                    L.csolve_cells += D.n;
                }
            }
            if (l == tail_at[p]) tail_cells_total += D.n;
        }
        L.ntot = off;
        L.d_desc = dalloc<LevelDesc>(nprob, owned);
        CK(cudaMemcpy(L.d_desc, L.h_desc.data(), nprob * sizeof(LevelDesc), cudaMemcpyHostToDevice));
        L.all = build_map(L.h_desc, has, owned, nprob, target_blocks);
        L.smooth = build_map(L.h_desc, smooth, owned, nprob, target_blocks);
        L.restr = build_map(L.h_desc, restr, owned, nprob, target_blocks);
        // plane-marching smoothers where the batch is large enough to fill the GPU with their
        // work runs: a finest level of 2^21 cells or more (an 800k-cell single problem ran 8 %
        // faster on the grid-stride kernels), or at any size with plane >= 2
        const long long fine_cells = l == 0 ? off : lv[0].ntot;
        const bool plane_on = opt.plane >= 2 || (opt.plane > 0 && fine_cells >= (1LL << 21));
        const bool plane_here = plane_on && (opt.plane_levels <= 0 || l < opt.plane_levels);
        build_plane_items(L.pm, L, smooth, sms, plane_here ? opt.plane_cells : 0, opt.plane_blocks_per_sm, &shapes,
                          l);
        if (l == 0)
            build_plane_items(L.pa, L, has, sms, opt.df_plane_cells > 0 ? kPlaneThreads : 0, opt.df_plane_blocks_per_sm,
                              nullptr, l);
        for (int p = 0; p < nprob; p++) {
            if (has[p]) L.all_cells += L.h_desc[p].n;
            if (smooth[p]) L.smooth_cells += L.h_desc[p].n;
            if (restr[p]) L.restr_cells += L.h_desc[p].n;
            if (has[p] && l == nlev[p] - 1) L.coarse_cells += L.h_desc[p].n;
        }
        maxblocks = std::max(maxblocks, std::max(L.all.nblocks, std::max(L.pm.n, L.pa.n)));
        L.d_coarse = dalloc<int>(L.coarse_list.size(), owned);
        if (!L.coarse_list.empty())
            CK(cudaMemcpy(L.d_coarse, L.coarse_list.data(), L.coarse_list.size() * sizeof(int),
                          cudaMemcpyHostToDevice));
        L.d_csolve = dalloc<int>(L.csolve_list.size(), owned);
        if (!L.csolve_list.empty())
            CK(cudaMemcpy(L.d_csolve, L.csolve_list.data(), L.csolve_list.size() * sizeof(int),
                          cudaMemcpyHostToDevice));
        size_t n = (size_t)L.ntot;
        L.dir = dalloc<uint8_t>(n, owned);
        L.c64[0] = dalloc<double>(n, owned); L.c64[1] = dalloc<double>(n, owned);
        L.c64[2] = dalloc<double>(n, owned); L.c64[3] = dalloc<double>(n, owned);
        if (mixed) {
            for (int k = 0; k < 4; k++) L.c16[k] = dalloc<__nv_bfloat16>(n, owned);
            L.idg32 = dalloc<float>(n, owned);
        } else {
            L.idg64 = dalloc<double>(n, owned);
        }
        size_t vs = mixed ? sizeof(float) : sizeof(double);
        for (int k = 0; k < 4; k++) L.work[k] = dalloc<char>(n * vs, owned);
    }
    N = lv[0].ntot;
    // faces and parameters
    prm.resize(nprob);
    long long foff = 0;
    cell_off.resize(nprob + 1);
    face_off.resize(nprob + 1);
    for (int p = 0; p < nprob; p++) {
        auto g = grids[p];
        int nx = g.n[0], ny = g.n[1], nz = g.n[2];
        double dxyz[3];
        for (int k = 0; k < 3; k++) dxyz[k] = g.n[k] > 1 ? (g.maxs[k] - g.mins[k]) / (g.n[k] - 1) : 1.0;
        ProbParam &P = prm[p];
        P.aol[0] = dxyz[1] * dxyz[2] / dxyz[0];
        P.aol[1] = dxyz[0] * dxyz[2] / dxyz[1];
        P.aol[2] = dxyz[0] * dxyz[1] / dxyz[2];
        if (g.aol_override) for (int k = 0; k < 3; k++) P.aol[k] = g.aol[k];
        P.vol = g.vol_override ? g.vol : dxyz[0] * dxyz[1] * dxyz[2];
        for (int k = 0; k < 3; k++) {
            P.x0[k] = g.mins[k];
            P.dx[k] = dxyz[k];
        }
        long long Fp = 3LL * nx * ny * nz - (long long)nx * ny - (long long)nx * nz - (long long)ny * nz;
        P.face_off = foff;
        P.F = Fp;
        cell_off[p] = lv[0].h_desc[p].off;
        face_off[p] = foff;
        foff += Fp;
    }
    cell_off[nprob] = N;
    face_off[nprob] = foff;
    F = foff;
    d_prm = dalloc<ProbParam>(nprob, owned);
    CK(cudaMemcpy(d_prm, prm.data(), nprob * sizeof(ProbParam), cudaMemcpyHostToDevice));
    // Dirichlet mask of the finest level
    std::vector<uint8_t> dir(N, 0);
    nfree_total = N;
    ndir.assign(nprob, 0);
    for (int p = 0; p < nprob; p++) {
        for (int64_t k : dnodes[p]) {
            if (k < 0 || k >= lv[0].h_desc[p].n) throw BadInput("Dirichlet node index out of range");
            if (!dir[cell_off[p] + k]) { nfree_total--; ndir[p]++; }
            dir[cell_off[p] + k] = 1;
        }
    }
    CK(cudaMemcpy(lv[0].dir, dir.data(), N, cudaMemcpyHostToDevice));
    // fine-level vectors
    h = dalloc<double>(N, owned);
    b64 = dalloc<double>(N, owned);
    r64 = dalloc<double>(N, owned);
    lam = dalloc<double>(N, owned);
    delta = dalloc<double>(N, owned);
    arhs = dalloc<double>(N, owned);
    in_dh = dalloc<double>(N, owned);
    in_Q = dalloc<double>(N, owned);
    in_logK = dalloc<double>(N, owned);
    in_kc = dalloc<double>(N, owned);
    aux_kc = dalloc<double>(N, owned);
    in_Ks = dalloc<double>(F, owned);
    if (!mixed) {
        for (int k = 0; k < 4; k++) cgv[k] = dalloc<double>(N, owned);  // r, z, p, q
    } else {
        for (int k = 0; k < 2; k++) cgv[k] = dalloc<float>(N, owned);   // r32, z32
        for (int k = 1; k < 4; k++) dfv[k] = dalloc<float2>(N, owned);  // r, p, q (double-float)
        for (int k = 0; k < 4; k++) cdf[k] = dalloc<float2>(N, owned);  // finest operator (double-float)
    }
    // state, reductions, coarse factors
    d_state = dalloc<CgState>(nprob, owned);
    d_count = dalloc<int>(4, owned);
    d_factor_status = dalloc<int>(2, owned);
    CK(cudaMemset(d_factor_status, 0, 2 * sizeof(int)));
    rs.partials = dalloc<double2>(std::max(maxblocks, 1), owned);
    rs.tickets = dalloc<unsigned>(nprob, owned);
    rs.capacity = maxblocks;
    CK(cudaMemset(rs.tickets, 0, nprob * sizeof(unsigned)));
    d_coarseL = dalloc<double>((size_t)nprob * kMaxCoarse * kMaxCoarse, owned);
    if (!tails.empty()) {
        d_tails = dalloc<int4>(tails.size(), owned);
        CK(cudaMemcpy(d_tails, tails.data(), tails.size() * sizeof(int4), cudaMemcpyHostToDevice));
        tail_first_level = nlev_max;
        for (auto &t : tails) tail_first_level = std::min(tail_first_level, t.y);
    }
    h_count = (int *)pinned.alloc(4 * sizeof(int));
    h_misc = (int *)pinned.alloc(4 * sizeof(int));
    h_state_buf = pinned.alloc(nprob * sizeof(CgState));
    if (!h_count || !h_misc || !h_state_buf) throw OomError("pinned host allocation failed");
    // Chebyshev coefficients on D^-1 A over [lo*2, 2] (Gershgorin: the spectrum of
    // D^-1 A of a weakly diagonally dominant symmetric M-matrix lies in [0, 2]).
    double lmax = 2.0, lmin = 2.0 * opt.cheb_lo;
    double theta = 0.5 * (lmax + lmin), delt = 0.5 * (lmax - lmin);
    double sigma = theta / delt, rho = 1.0 / sigma;
    inv_theta = 1.0 / theta;
    cheb_c1.assign(opt.cheb_degree, 0.0);
    cheb_c2.assign(opt.cheb_degree, 0.0);
    for (int k = 1; k < opt.cheb_degree; k++) {
        double rn = 1.0 / (2.0 * sigma - rho);
        cheb_c1[k] = rn * rho;
        cheb_c2[k] = 2.0 * rn / delt;
        rho = rn;
    }
    if (!tails.empty()) write_tail_table();
    // the uploads above are synchronous copies on the legacy stream, some from pageable memory
    // (which may return before the DMA lands): the device is drained before the handle is used
    // from any stream
    CK(cudaDeviceSynchronize());
}

// Stable names "kernel<f64|f32>/L<level>" for the per-kernel timing report. Every launch asks
// for its name, from the host threads of all the handles (and of a batch's concurrent parts)
// at once, so the shared set is guarded.
const char *kname(const char *base, int level, bool fp32) {
    static std::mutex mu;
    static std::set<std::string> names;
    std::string n = std::string(base) + (fp32 ? "<f32>" : "<f64>") + "/L" + std::to_string(level);
    std::lock_guard<std::mutex> lk(mu);
    return names.insert(n).first->c_str();
}

KTimer::KTimer(StructBatch *s, const char *name, long long cells) : S(s) {
    S->launches++;
    if (!S->prof_on || S->prof_recs.size() >= (1u << 20)) return;
    int e = (int)(2 * S->prof_recs.size());
    while ((int)S->ev_pool.size() < e + 2) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) { cudaGetLastError(); return; }
        S->ev_pool.push_back(ev);
    }
    S->prof_recs.push_back(ProfRec{name, e, cells});
    cudaEventRecord(S->ev_pool[e], S->stream);
    slot = e;
}

KTimer::~KTimer() {
    if (slot >= 0) cudaEventRecord(S->ev_pool[slot + 1], S->stream);
}

void StructBatch::profile(bool on) {
    cudaStreamSynchronize(stream);
    prof_recs.clear();
    prof_on = on;
}

int StructBatch::profile_report(int cap, const char **names, long long *counts, double *ms, long long *cells) {
    CK(cudaStreamSynchronize(stream));
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

StructBatch::~StructBatch() {
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    for (auto &kv : graphs) {
        cudaGraphExecDestroy(kv.second.exec);
        cudaGraphDestroy(kv.second.graph);
    }
    if (cap_stream) cudaStreamDestroy(cap_stream);
    cudaStreamSynchronize(stream);  // then `owned` and `pinned` free the buffers
}

static inline unsigned nb_of(const BlockMap &m) { return (unsigned)m.nblocks; }

// ---- assembly and hierarchy
template <typename T>
static Coeffs<T> coeffs_of(StructBatch::Level &L, bool mixed);
template <>
Coeffs<double> coeffs_of<double>(StructBatch::Level &L, bool) {
    return Coeffs<double>{L.c64[0], L.c64[1], L.c64[2], L.c64[3], L.idg64};
}
template <>
Coeffs<float> coeffs_of<float>(StructBatch::Level &L, bool) {
    return Coeffs<float>{L.c16[0], L.c16[1], L.c16[2], L.c16[3], L.idg32};
}

// The fused tail's per-level pointer table, written once at construction: staged in pinned
// memory, copied on the handle's stream and waited for, so no kernel on any stream can read
// the table before its copy has landed. (A pageable cudaMemcpy may return before its DMA
// completes, and the legacy stream it runs on is not ordered with non-blocking streams.)
template <typename T>
static void fill_tail_table(StructBatch &S, void *host) {
    TailLevel<T> *tab = (TailLevel<T> *)host;
    for (int l = 0; l < S.nlev_max; l++) {
        StructBatch::Level &L = S.lv[l];
        tab[l] = TailLevel<T>{L.d_desc, coeffs_of<T>(L, S.mixed), (T *)L.work[0], (T *)L.work[1],
                              (T *)L.work[2], (T *)L.work[3], L.dir};
    }
}

void StructBatch::write_tail_table() {
    const size_t bytes = (size_t)nlev_max * (mixed ? sizeof(TailLevel<float>) : sizeof(TailLevel<double>));
    void *host = pinned.alloc(bytes);
    if (!host) throw OomError("pinned host allocation failed");
    if (mixed) fill_tail_table<float>(*this, host);
    else fill_tail_table<double>(*this, host);
    d_tail_lv = dalloc<char>(bytes, owned);
    CK(cudaMemcpyAsync(d_tail_lv, host, bytes, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
}

void StructBatch::assemble(const double *Ks, const double *kc, int kind, const double *shift, bool init_x) {
    NvtxRange range("assemble operator and hierarchy");
    direct_stale = true;  // a direct factor of the previous operator is out of date
    Level &L0 = lv[0];
    FaceK fk{Ks, kc, kind};
    if (nb_of(L0.all))
        {
            KTimer _kt(this, kname("k_assemble", 0, false), L0.all_cells);
            k_assemble<<<nb_of(L0.all), kBlock, 0, stream>>>(
                L0.d_desc, L0.all.d_map, d_prm, fk, in_dh, in_Q, shift, L0.dir, L0.c64[0], L0.c64[1], L0.c64[2],
                L0.c64[3], mixed ? L0.c16[0] : nullptr, mixed ? L0.c16[1] : nullptr, mixed ? L0.c16[2] : nullptr,
                mixed ? L0.c16[3] : nullptr, mixed ? cdf[0] : nullptr, mixed ? cdf[1] : nullptr,
                mixed ? cdf[2] : nullptr, mixed ? cdf[3] : nullptr, b64, h, init_x ? 1 : 0);
        }
    LAUNCH_CHECK();
    for (int l = 0; l + 1 < nlev_max; l++) {
        Level &F = lv[l], &C = lv[l + 1];
        if (!nb_of(C.all)) continue;
        {
            KTimer _kt(this, kname("k_coarsen", l + 1, false), C.all_cells);
            k_coarsen<<<nb_of(C.all), kBlock, 0, stream>>>(
                F.d_desc, C.d_desc, C.all.d_map, F.c64[0], F.c64[1], F.c64[2], F.c64[3], F.dir, C.c64[0], C.c64[1],
                C.c64[2], C.c64[3], C.dir, mixed ? C.c16[0] : nullptr, mixed ? C.c16[1] : nullptr,
                mixed ? C.c16[2] : nullptr, mixed ? C.c16[3] : nullptr);
        }
        LAUNCH_CHECK();
    }
    CK(cudaMemsetAsync(d_factor_status, 0, sizeof(int), stream));
    for (int l = 0; l < nlev_max; l++) {
        Level &L = lv[l];
        if (L.coarse_list.empty()) continue;
        {
            KTimer _kt(this, kname("k_coarse_factor", l, false), L.coarse_cells);
            k_coarse_factor<<<(unsigned)L.coarse_list.size(), kBlock, 0, stream>>>(
                L.d_desc, L.d_coarse, L.c64[0], L.c64[1], L.c64[2], L.c64[3], d_coarseL, d_factor_status);
        }
        LAUNCH_CHECK();
    }
    for (int l = 0; l < nlev_max; l++) {
        Level &L = lv[l];
        if (!nb_of(L.all)) continue;
        {
            KTimer _kt(this, kname("k_invdiag", l, false), L.all_cells);
            k_invdiag<<<nb_of(L.all), kBlock, 0, stream>>>(L.d_desc, L.all.d_map, coeffs_of<double>(L, false),
                                                           mixed ? coeffs_of<float>(L, true) : Coeffs<float>{},
                                                           mixed ? nullptr : L.idg64, mixed ? L.idg32 : nullptr);
        }
        LAUNCH_CHECK();
    }
    have_operator = true;
}

// ---- V-cycle: z = M r on the fine level (vector precision T)
// ---- plane-marching launches
static int pm_region(int count, int es) { return ((count * es + 32) + 15) & ~15; }

// Function attributes are set once per device, at the first handle's construction and before
// any launch: the plane kernels' dynamic shared memory limit (all that a block may hold beside
// its static shared memory) and the fused tail's permission for non-portable cluster sizes (up
// to 16 blocks). An attribute is then never changed while kernels of another handle, or of
// another part of a split batch on another host thread, run or are being captured into a graph.
template <int MODE>
static void raise_pm_cheb(const std::function<void(const void *)> &raise) {
    raise((const void *)k_pm_cheb<float, MODE, 1>);
    raise((const void *)k_pm_cheb<float, MODE, 2>);
    raise((const void *)k_pm_cheb<float, MODE, 3>);
    raise((const void *)k_pm_cheb<float, MODE, 4>);
}

static void configure_kernels() {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return;
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const std::function<void(const void *)> raise = [&](const void *f) {
        cudaFuncAttributes a;
        CK(cudaFuncGetAttributes(&a, f));
        CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes));
    };
    raise_pm_cheb<PM_FIRST2>(raise);
    raise_pm_cheb<PM_FIRST2 | PM_NOD>(raise);
    raise_pm_cheb<0>(raise);
    raise_pm_cheb<PM_NOD>(raise);
    raise_pm_cheb<PM_PROLONG | PM_FIRST>(raise);
    raise_pm_cheb<PM_PROLONG | PM_FIRST | PM_NOD>(raise);
    raise_pm_cheb<PM_PROLONG | PM_FIRST | PM_NOD | PM_RZ>(raise);
    raise_pm_cheb<PM_NOD | PM_RZ>(raise);
    raise((const void *)k_pm_restrict<float, 1>);
    raise((const void *)k_pm_restrict<float, 2>);
    raise((const void *)k_pm_restrict<float, 3>);
    raise((const void *)k_pm_restrict<float, 4>);
    raise((const void *)k_pm_post2<float, false>);
    raise((const void *)k_pm_post2<float, true>);
    raise((const void *)k_pm_pre2r<float>);
    CK(cudaFuncSetAttribute(k_tail_cycle<float, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    CK(cudaFuncSetAttribute(k_tail_cycle<double, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    done.insert(dev);
}

template <typename T, int MODE, int CPT>
static void pm_kernel(unsigned nblocks, size_t smem, cudaStream_t stream, const LevelDesc *desc,
                      const LevelDesc *cdesc, PlaneWork items, CgState *st, Coeffs<T> C, const T *b,
                      const T *xin, T *xout, T *d, const uint8_t *dir, const T *e, T c1, T c2, T invth, T sc,
                      PlaneLayout lay, ReduceScratch rs, const int2 *pinfo, int *err) {
    launch_pdl(k_pm_cheb<T, MODE, CPT>, nblocks, kPlaneThreads + 32, smem, stream, desc, cdesc, items, st, C, b, xin, xout, d,
                                                                       dir, e, c1, c2, invth, sc, lay, rs, pinfo, err);
}

template <typename T, int MODE>
static void pm_kernel_cpt(int cpt, unsigned nblocks, size_t smem, cudaStream_t stream, const LevelDesc *desc,
                          const LevelDesc *cdesc, PlaneWork items, CgState *st, Coeffs<T> C, const T *b,
                          const T *xin, T *xout, T *d, const uint8_t *dir, const T *e, T c1, T c2, T invth, T sc,
                          PlaneLayout lay, ReduceScratch rs, const int2 *pinfo, int *err) {
#define DPF_PM_CPT(N)                                                                                              \
    case N:                                                                                                        \
        pm_kernel<T, MODE, N>(nblocks, smem, stream, desc, cdesc, items, st, C, b, xin, xout, d, dir, e, c1, c2, invth, \
                              sc, lay, rs, pinfo, err);                                                            \
        break;
    switch (cpt) {
        DPF_PM_CPT(1)
        DPF_PM_CPT(2)
        DPF_PM_CPT(3)
        DPF_PM_CPT(4)
        default:
            throw std::logic_error("plane slab must hold 1..4 cells per thread");
    }
#undef DPF_PM_CPT
}

// One plane-marching Chebyshev launch over the smoothed problems of level l (mode: PM_* bits).
template <typename T>
void StructBatch::pm_launch(int mode, int l, const T *b, const T *xin, T *xout, T *d, const T *e, T c1, T c2,
                            T invth, T sc) {
    if constexpr (sizeof(T) != 4) {
        throw std::logic_error("plane-marching kernels run FP32 V-cycles only");
    } else {
    Level &L = lv[l];
    const int cpt = L.pm.cells / kPlaneThreads;
    const int es = (int)sizeof(T);
    PlaneLayout lay{};
    int off = 0;
    auto take = [&](int bytes) { int o = off; off += bytes; return o; };
    const bool f2 = mode & PM_FIRST2, first = mode & PM_FIRST, prol = mode & PM_PROLONG;
    lay.oX = f2 ? -1 : take(pm_region(L.pm.halo, es));
    lay.oB = take(pm_region(f2 ? L.pm.halo : L.pm.slab, es));
    lay.oD = (f2 || first) ? -1 : take(pm_region(L.pm.slab, es));
    lay.oG = f2 ? take(pm_region(L.pm.halo, es)) : -1;
    const int ec = (int)sizeof(coef_t<T>);
    lay.oCX = take(pm_region(L.pm.slab, ec));
    lay.oCY = take(pm_region(L.pm.cy, ec));
    lay.oCZ = take(pm_region(L.pm.slab, ec));
    lay.oLK = take(pm_region(L.pm.slab, ec));
    lay.oDIR = prol ? take(pm_region(L.pm.halo, 1)) : -1;
    lay.oE = prol ? take(pm_region(L.pm.coarse, es)) : -1;
    lay.slot_bytes = (off + 127) & ~127;
    const size_t smem = (size_t)kPlaneStages * lay.slot_bytes;
    Coeffs<T> C = coeffs_of<T>(L, mixed);
    const LevelDesc *cd = l + 1 < nlev_max ? lv[l + 1].d_desc : nullptr;
    const unsigned nb = (unsigned)L.pm.nb;
    const PlaneWork wk{L.pm.items, L.pm.first};
    int *err = d_factor_status + 1;
#define DPF_PM_CASE(M)                                                                                           \
    case M:                                                                                                      \
        pm_kernel_cpt<T, M>(cpt, nb, smem, stream, L.d_desc, cd, wk, d_state, C, b, xin, xout, d, L.dir, e, \
                            c1, c2, invth, sc, lay, rs, L.pm.pinfo, err);                                         \
        break;
    switch (mode) {
        DPF_PM_CASE(PM_FIRST2)
        DPF_PM_CASE(PM_FIRST2 | PM_NOD)
        DPF_PM_CASE(0)
        DPF_PM_CASE(PM_NOD)
        DPF_PM_CASE(PM_PROLONG | PM_FIRST)
        DPF_PM_CASE(PM_PROLONG | PM_FIRST | PM_NOD)
        DPF_PM_CASE(PM_PROLONG | PM_FIRST | PM_NOD | PM_RZ)
        DPF_PM_CASE(PM_NOD | PM_RZ)
        default:
            throw std::logic_error("unsupported plane kernel mode");
    }
#undef DPF_PM_CASE
    }
}

// Plane-marching restriction of level l's residual into level l+1 (the smoothed problems).
template <typename T, int CPT>
static void pm_restrict_kernel(unsigned nblocks, size_t smem, cudaStream_t stream, const LevelDesc *desc,
                               const LevelDesc *cdesc, PlaneWork items, const CgState *st, Coeffs<T> C, const T *b,
                               const T *x, T *bc, PlaneLayout lay, int *err) {
    launch_pdl(k_pm_restrict<T, CPT>, nblocks, kPlaneThreads + 32, smem, stream, desc, cdesc, items, st, C, b, x, bc, lay, err);
}

template <typename T>
void StructBatch::pm_restrict(int l, const T *b, const T *x, T *bc) {
    if constexpr (sizeof(T) != 4) {
        throw std::logic_error("plane-marching kernels run FP32 V-cycles only");
    } else {
    Level &L = lv[l];
    const int es = (int)sizeof(T);
    PlaneLayout lay{};
    int off = 0;
    auto take = [&](int bytes) { int o = off; off += bytes; return o; };
    lay.oX = take(pm_region(L.pm.halo, es));
    lay.oB = take(pm_region(L.pm.slab, es));
    const int ec = (int)sizeof(coef_t<T>);
    lay.oCX = take(pm_region(L.pm.slab, ec));
    lay.oCY = take(pm_region(L.pm.cy, ec));
    lay.oCZ = take(pm_region(L.pm.slab, ec));
    lay.oLK = take(pm_region(L.pm.slab, ec));
    lay.oD = lay.oG = lay.oDIR = lay.oE = -1;
    lay.slot_bytes = (off + 127) & ~127;
    const size_t smem = (size_t)kPlaneStages * lay.slot_bytes;
    const unsigned nb = (unsigned)L.pm.nb;
    const PlaneWork wk{L.pm.items, L.pm.first};
    const Coeffs<T> C = coeffs_of<T>(L, mixed);
    switch (L.pm.cells / kPlaneThreads) {
        case 1: pm_restrict_kernel<T, 1>(nb, smem, stream, L.d_desc, lv[l + 1].d_desc, wk, d_state, C, b, x, bc, lay, d_factor_status + 1); break;
        case 2: pm_restrict_kernel<T, 2>(nb, smem, stream, L.d_desc, lv[l + 1].d_desc, wk, d_state, C, b, x, bc, lay, d_factor_status + 1); break;
        case 3: pm_restrict_kernel<T, 3>(nb, smem, stream, L.d_desc, lv[l + 1].d_desc, wk, d_state, C, b, x, bc, lay, d_factor_status + 1); break;
        case 4: pm_restrict_kernel<T, 4>(nb, smem, stream, L.d_desc, lv[l + 1].d_desc, wk, d_state, C, b, x, bc, lay, d_factor_status + 1); break;
        default: throw std::logic_error("plane slab must hold 1..4 cells per thread");
    }
    }
}

// Layout of the fused kernels' shared memory for level l: the staged regions of one plane (kFusedStages
// of them), then the rings of first-step results, directions and residual pairs.
static FusedLayout fused_layout(const StructBatch::PlaneItems &P, bool post, int es, int ec) {
    FusedLayout lay{};
    int off = 0;
    auto take = [&](int bytes) { int o = off; off += bytes; return o; };
    lay.oX = lay.oDIR = lay.oE = lay.oB = lay.oG = lay.oCX = lay.oCY = lay.oCZ = lay.oLK = -1;
    if (post) {
        lay.oX = take(pm_region(P.halo2, es));
        lay.oDIR = take(pm_region(P.halo2, 1));
        lay.oE = take(pm_region(P.coarse2, es));
        lay.oB = take(pm_region(P.halo, es));
    } else {
        lay.oB = take(pm_region(P.halo2, es));
        lay.oG = take(pm_region(P.halo2, es));
    }
    lay.oCX = take(pm_region(P.halo, ec));
    lay.oCY = take(pm_region(P.cy2, ec));
    lay.oCZ = take(pm_region(P.halo, ec));
    lay.oLK = take(pm_region(P.halo, ec));
    lay.slot_bytes = (off + 127) & ~127;
    int ring = kFusedStages * lay.slot_bytes;
    lay.v_stride = (P.halo * es + 127) & ~127;
    lay.oV = ring;
    ring += 4 * lay.v_stride;
    lay.d_stride = lay.r_stride = (P.slab * es + 127) & ~127;
    lay.oD = lay.oR = ring;  // the post-smoothing's directions or the pre-smoothing's residual pairs
    ring += 2 * lay.d_stride;
    lay.slot_bytes = lay.slot_bytes;
    return lay;
}
static size_t fused_smem(const FusedLayout &lay) { return (size_t)lay.oD + 2 * (size_t)lay.d_stride; }

// Fused pre-smoothing (two Chebyshev steps from zero) and restriction of level l into level l+1.
template <typename T>
void StructBatch::pm_pre2r(int l, const T *b, T *xout, T *bc, T c1, T c2, T invth) {
    if constexpr (sizeof(T) != 4) {
        throw std::logic_error("plane-marching kernels run FP32 V-cycles only");
    } else {
        Level &L = lv[l];
        const FusedLayout lay = fused_layout(L.pm, false, (int)sizeof(T), (int)sizeof(coef_t<T>));
        launch_pdl(k_pm_pre2r<T>, (unsigned)L.pm.nb, kFusedThreads + 32, fused_smem(lay), stream, L.d_desc,
                   lv[l + 1].d_desc, PlaneWork{L.pm.items, L.pm.first}, L.pm.cells, (const CgState *)d_state,
                   coeffs_of<T>(L, mixed), b, xout, bc, c1, c2, invth, lay, d_factor_status + 1);
    }
}

// Fused prolongation and post-smoothing (two Chebyshev steps) of level l; on the finest level it
// also forms r . z and beta.
template <typename T>
void StructBatch::pm_post2(int l, const T *b, const T *xin, T *xout, const T *e, T c2a, T c1b, T c2b, T sc) {
    if constexpr (sizeof(T) != 4) {
        throw std::logic_error("plane-marching kernels run FP32 V-cycles only");
    } else {
        Level &L = lv[l];
        const FusedLayout lay = fused_layout(L.pm, true, (int)sizeof(T), (int)sizeof(coef_t<T>));
        const PlaneWork wk{L.pm.items, L.pm.first};
        if (l == 0)
            launch_pdl(k_pm_post2<T, true>, (unsigned)L.pm.nb, kFusedThreads + 32, fused_smem(lay), stream, L.d_desc,
                       lv[l + 1].d_desc, wk, L.pm.cells, d_state, coeffs_of<T>(L, mixed), b, xin, xout,
                       (const uint8_t *)L.dir, e, c2a, c1b, c2b, sc, lay, rs, (const int2 *)L.pm.pinfo,
                       d_factor_status + 1);
        else
            launch_pdl(k_pm_post2<T, false>, (unsigned)L.pm.nb, kFusedThreads + 32, fused_smem(lay), stream, L.d_desc,
                       lv[l + 1].d_desc, wk, L.pm.cells, d_state, coeffs_of<T>(L, mixed), b, xin, xout,
                       (const uint8_t *)L.dir, e, c2a, c1b, c2b, sc, lay, rs, (const int2 *)L.pm.pinfo,
                       d_factor_status + 1);
    }
}

// The fused tail: one block per problem, or a cluster of tail_cs blocks per problem when
// the device can co-schedule that many 1024-thread blocks (halved until it can).
template <typename T>
void StructBatch::launch_tail(const TailParams<T> &tp) {
    const unsigned nt = (unsigned)tails.size();
    if (tail_cs == 0) {
        int cs = std::max(1, std::min(16, opt.tail_cluster));
        while (cs > 1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(nt * cs);
            cfg.blockDim = dim3(kTailThreads);
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, k_tail_cycle<T, true>, &cfg) == cudaSuccess && nclusters > 0)
                break;
            cudaGetLastError();
            cs /= 2;
        }
        tail_cs = cs;
    }
    if (tail_cs <= 1) {
        launch_pdl(k_tail_cycle<T, false>, nt, kTailThreads, 0, stream, (const TailLevel<T> *)d_tail_lv, d_tails, d_state,
                                                               d_coarseL, tp);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nt * tail_cs);
    cfg.blockDim = dim3(kTailThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = tail_cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelEx(&cfg, k_tail_cycle<T, true>, (const TailLevel<T> *)d_tail_lv, (const int4 *)d_tails,
                          (const CgState *)d_state, (const double *)d_coarseL, tp));
}

template <typename T>
void StructBatch::vcycle(const T *r, T *z) {
    const int deg = opt.cheb_degree;
    const T invth = (T)inv_theta, sc = (T)opt.coarse_scale;
    std::vector<T *> pre(nlev_max, nullptr);
    // Every level leaves its final iterate (the coarse correction of the next finer level) in
    // work[1] (xb), whichever kernels ran it for a problem: per-level passes, the fused tail or the
    // coarsest solve. Problems of an uneven batch reach the tail at different levels, so this must
    // hold for every problem. The fused passes keep it: the pre-smoothed iterate goes to work[0]
    // and the post-smoothing (which cannot run in place) reads it there and writes work[1].
    const bool fused = opt.fuse > 0 && deg == 2;
    // descend
    for (int l = 0; l < nlev_max; l++) {
        Level &L = lv[l];
        Coeffs<T> C = coeffs_of<T>(L, mixed);
        const T *b = l == 0 ? r : (const T *)L.work[2];
        T *xa = (T *)L.work[0], *xb = (T *)L.work[1], *d = (T *)L.work[3];
        if (nb_of(L.smooth) && L.pm.ok && fused) {
            // one pass: two pre-smoothing steps from zero and the restriction of their residual
            Level &Cn = lv[l + 1];
            {
                KTimer _kt(this, kname("k_pm_pre2r", l, sizeof(T) == 4), L.smooth_cells);
                pm_pre2r<T>(l, b, xa, (T *)Cn.work[2], (T)cheb_c1[1], (T)cheb_c2[1], invth);
            }
            LAUNCH_CHECK();
            pre[l] = xa;
        } else if (nb_of(L.smooth) && L.pm.ok && deg >= 2) {
            // plane-marching pre-smoothing: two fused first steps, then the rest
            {
                KTimer _kt(this, kname("k_pm_first2", l, sizeof(T) == 4), L.smooth_cells);
                pm_launch<T>(deg == 2 ? (PM_FIRST2 | PM_NOD) : PM_FIRST2, l, b, nullptr, xb, d, nullptr,
                             (T)cheb_c1[1], (T)cheb_c2[1], invth, sc);
            }
            LAUNCH_CHECK();
            T *cur = xb, *oth = xa;
            for (int k = 2; k < deg; k++) {
                {
                    KTimer _kt(this, kname("k_pm_step", l, sizeof(T) == 4), L.smooth_cells);
                    pm_launch<T>(k == deg - 1 ? PM_NOD : 0, l, b, cur, oth, d, nullptr, (T)cheb_c1[k],
                                 (T)cheb_c2[k], invth, sc);
                }
                LAUNCH_CHECK();
                std::swap(cur, oth);
            }
            pre[l] = cur;
            Level &Cn = lv[l + 1];
            {
                KTimer _kt(this, kname("k_pm_restrict", l + 1, sizeof(T) == 4), Cn.restr_cells);
                pm_restrict<T>(l, b, cur, (T *)Cn.work[2]);
            }
            LAUNCH_CHECK();
        } else if (nb_of(L.smooth)) {
            T *cur = xa, *oth = xb;
            int k0 = 1;
            if (deg >= 2) {
                // steps 0 and 1 fused; the iterate lands where step 1 would leave it (xb)
                {
                    KTimer _kt(this, kname("k_cheb_first2", l, sizeof(T) == 4), L.smooth_cells);
                    launch_pdl(k_cheb_first2<T>, nb_of(L.smooth), kBlock, 0, stream, L.d_desc, L.smooth.d_map, d_state, C, b,
                                                                             xb, d, invth, (T)cheb_c1[1],
                                                                             (T)cheb_c2[1]);
                }
                LAUNCH_CHECK();
                cur = xb;
                oth = xa;
                k0 = 2;
            } else {
                {
                    KTimer _kt(this, kname("k_cheb_first", l, sizeof(T) == 4), L.smooth_cells);
                    launch_pdl(k_cheb_first<T>, nb_of(L.smooth), kBlock, 0, stream, L.d_desc, L.smooth.d_map, d_state, C, b,
                                                                            xa, d, invth);
                }
                LAUNCH_CHECK();
            }
            for (int k = k0; k < deg; k++) {
                {
                    KTimer _kt(this, kname("k_cheb_step", l, sizeof(T) == 4), L.smooth_cells);
                    launch_pdl(k_cheb_step<T, false>, nb_of(L.smooth), kBlock, 0, stream, 
                        L.d_desc, L.smooth.d_map, d_state, C, b, cur, oth, d, (T)cheb_c1[k], (T)cheb_c2[k], rs,
                        L.smooth.d_pinfo);
                }
                LAUNCH_CHECK();
                std::swap(cur, oth);
            }
            pre[l] = cur;
            Level &Cn = lv[l + 1];
            {
                KTimer _kt(this, kname("k_restrict", l + 1, sizeof(T) == 4), Cn.restr_cells);
                launch_pdl(k_restrict<T>, nb_of(Cn.restr), kBlock, 0, stream, L.d_desc, Cn.d_desc, Cn.restr.d_map, d_state, C, b,
                                                                   cur, (T *)Cn.work[2]);
            }
            LAUNCH_CHECK();
        }
        if (!L.csolve_list.empty()) {
            // the coarse solution goes where the post-smoother of this level would
            // leave its result: work[1] (always, see below), or z on the finest level
            T *out = l == 0 ? z : xb;
            if (l == 0)
                {
                    KTimer _kt(this, kname("k_coarse_solve", l, sizeof(T) == 4), L.csolve_cells);
                    launch_pdl(k_coarse_solve<T, true>, (unsigned)L.csolve_list.size(), kMaxCoarse, 0, stream, 
                        L.d_desc, L.d_csolve, d_state, d_coarseL, b, out);
                }
            else
                {
                    KTimer _kt(this, kname("k_coarse_solve", l, sizeof(T) == 4), L.csolve_cells);
                    launch_pdl(k_coarse_solve<T, false>, (unsigned)L.csolve_list.size(), kMaxCoarse, 0, stream, 
                        L.d_desc, L.d_csolve, d_state, d_coarseL, b, out);
                }
            LAUNCH_CHECK();
        }
    }
    // the small levels: one fused block per problem
    if (!tails.empty()) {
        // the level table is written once, at construction, for the V-cycle precision in use
        if (!d_tail_lv || (sizeof(T) == 4) != mixed) throw std::logic_error("fused-tail level table missing");
        TailParams<T> tp{};
        for (int k = 0; k < deg && k < 8; k++) {
            tp.c1[k] = (T)cheb_c1[k];
            tp.c2[k] = (T)cheb_c2[k];
        }
        tp.invtheta = invth;
        tp.coarse_scale = sc;
        tp.deg = deg;
        {
            KTimer _kt(this, kname("k_tail_cycle", tail_first_level, sizeof(T) == 4), tail_cells_total);
            launch_tail<T>(tp);
        }
        LAUNCH_CHECK();
    }
    // ascend: the coarse correction is added in place to the pre-smoothed iterate, then
    // deg Chebyshev steps alternate buffers. Pre-smoothing wrote deg iterates starting in
    // work[0] and post-smoothing writes deg more, so the final iterate always lands in
    // work[1] (or z on the finest level).
    for (int l = nlev_max - 2; l >= 0; l--) {
        Level &L = lv[l];
        if (!nb_of(L.smooth)) continue;
        Level &Cn = lv[l + 1];
        Coeffs<T> C = coeffs_of<T>(L, mixed);
        const T *b = l == 0 ? r : (const T *)L.work[2];
        T *xa = (T *)L.work[0], *xb = (T *)L.work[1], *d = (T *)L.work[3];
        T *cur = pre[l];
        const T *e = (const T *)Cn.work[1];
        if (L.pm.ok && fused) {
            // one pass: prolongation and both post-smoothing steps (the finest level also forms r . z)
            {
                KTimer _kt(this, kname("k_pm_post2", l, sizeof(T) == 4), L.smooth_cells);
                pm_post2<T>(l, b, cur, l == 0 ? z : xb, e, invth, (T)cheb_c1[1], (T)cheb_c2[1], sc);
            }
            LAUNCH_CHECK();
            continue;
        }
        if (L.pm.ok && deg >= 2) {
            // plane-marching post-smoothing: prolongation fused into the first step; the
            // last step writes no direction (and on the finest level also forms r . z)
            for (int k = 0; k < deg; k++) {
                const bool last = k == deg - 1;
                T *o = (l == 0 && last) ? z : (cur == xa ? xb : xa);
                int mode = k == 0 ? (PM_PROLONG | PM_FIRST) : 0;
                if (last) mode |= PM_NOD;
                if (last && l == 0) mode |= PM_RZ;
                {
                    KTimer _kt(this, kname(k == 0 ? "k_pm_prolong_step" : "k_pm_step", l, sizeof(T) == 4),
                               L.smooth_cells);
                    pm_launch<T>(mode, l, b, cur, o, d, e, (T)cheb_c1[k], k == 0 ? invth : (T)cheb_c2[k], invth, sc);
                }
                LAUNCH_CHECK();
                cur = o;
            }
            continue;
        }
        {
            KTimer _kt(this, kname("k_prolong_add", l, sizeof(T) == 4), L.smooth_cells);
            launch_pdl(k_prolong_add<T>, nb_of(L.smooth), kBlock, 0, stream, L.d_desc, Cn.d_desc, L.smooth.d_map, d_state,
                                                                     L.dir, cur, e, sc);
        }
        LAUNCH_CHECK();
        for (int k = 0; k < deg; k++) {
            const bool last = k == deg - 1;
            T *o = (l == 0 && last) ? z : (cur == xa ? xb : xa);
            const T c1 = (T)cheb_c1[k], c2 = k == 0 ? invth : (T)cheb_c2[k];
            {
                KTimer _kt(this, kname(k == 0 ? "k_cheb_step0" : "k_cheb_step", l, sizeof(T) == 4), L.smooth_cells);
                if (l == 0 && last) {
                    if (k == 0)
                        launch_pdl(k_cheb_step<T, true, true>, nb_of(L.smooth), kBlock, 0, stream, 
                            L.d_desc, L.smooth.d_map, d_state, C, b, cur, o, d, c1, c2, rs, L.smooth.d_pinfo);
                    else
                        launch_pdl(k_cheb_step<T, true, false>, nb_of(L.smooth), kBlock, 0, stream, 
                            L.d_desc, L.smooth.d_map, d_state, C, b, cur, o, d, c1, c2, rs, L.smooth.d_pinfo);
                } else {
                    if (k == 0)
                        launch_pdl(k_cheb_step<T, false, true>, nb_of(L.smooth), kBlock, 0, stream, 
                            L.d_desc, L.smooth.d_map, d_state, C, b, cur, o, d, c1, c2, rs, L.smooth.d_pinfo);
                    else
                        launch_pdl(k_cheb_step<T, false, false>, nb_of(L.smooth), kBlock, 0, stream, 
                            L.d_desc, L.smooth.d_map, d_state, C, b, cur, o, d, c1, c2, rs, L.smooth.d_pinfo);
                }
            }
            LAUNCH_CHECK();
            cur = o;
        }
    }
}

int StructBatch::read_count(int which) {
    CK(cudaMemcpyAsync(h_count, d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return h_count[which];
}

int StructBatch::read_stats() {
    CK(cudaMemcpyAsync(h_state_buf, d_state, nprob * sizeof(CgState), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h_misc, d_factor_status, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h_misc + 2, d_count + 2, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h_count, d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return h_count[0];
}

// One PCG iteration (FP64 mode): q = A p, alpha; x, r update and convergence test;
// z = M r, beta; p update.
template <typename T>
void StructBatch::pcg_iteration(T *x) {
    Level &L0 = lv[0];
    Coeffs<T> C = coeffs_of<T>(L0, mixed);
    T *r = (T *)cgv[0], *z = (T *)cgv[1], *pv = (T *)cgv[2], *q = (T *)cgv[3];
    const unsigned nb = nb_of(L0.all);
    {
        KTimer _kt(this, kname("k_spmv_pq", 0, sizeof(T) == 4), L0.all_cells);
        launch_pdl(k_spmv_pq<T>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs, L0.all.d_pinfo, C,
                                                pv, q);
    }
    LAUNCH_CHECK();
    {
        KTimer _kt(this, kname("k_update_xr", 0, sizeof(T) == 4), L0.all_cells);
        launch_pdl(k_update_xr<T>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs, L0.all.d_pinfo, x, r,
                                                  pv, q, opt.maxiter);
    }
    LAUNCH_CHECK();
    vcycle<T>(r, z);
    {
        KTimer _kt(this, kname("k_update_p", 0, sizeof(T) == 4), L0.all_cells);
        launch_pdl(k_update_p<T>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, z, pv);
    }
    LAUNCH_CHECK();
}

// Plane-marching double-float CG product over all problems of the finest level (each face flux
// computed once; slabs of at most 256 cells, one per thread).
void StructBatch::pm_df_spmv(const CoeffsDF &C) {
    Level &L0 = lv[0];
    const unsigned nb = (unsigned)L0.pa.nb;
    const PlaneWork wk{L0.pa.items, L0.pa.first};
    if (L0.pa.cells != kPlaneThreads) throw std::logic_error("the marching product holds one cell per thread");
    launch_pdl(k_pm_df_flux<1>, nb, kPlaneThreads, 0, stream, L0.d_desc, wk, d_state, d_count, rs, L0.pa.pinfo, C, dfv[2],
               dfv[3]);
}

// One iteration of the mixed-precision CG: double-float q = A p, alpha, x/r update,
// FP32 V-cycle on the rounded residual, double-float p update.
void StructBatch::df_iteration(double *x64) {
    Level &L0 = lv[0];
    const unsigned nb = nb_of(L0.all);
    float *r32 = (float *)cgv[0], *z32 = (float *)cgv[1];
    CoeffsDF C{cdf[0], cdf[1], cdf[2], cdf[3]};
    if (L0.pa.ok) {
        KTimer _kt(this, kname("k_pm_df_flux", 0, true), L0.all_cells);
        pm_df_spmv(C);
    } else {
        KTimer _kt(this, kname("k_df_spmv_pq", 0, true), L0.all_cells);
        launch_pdl(k_df_spmv_pq, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs, L0.all.d_pinfo, C,
                                                dfv[2], dfv[3]);
    }
    LAUNCH_CHECK();
    {
        KTimer _kt(this, kname("k_df_update_xr", 0, true), L0.all_cells);
        launch_pdl(k_df_update_xr, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs, L0.all.d_pinfo,
                                                  x64, dfv[1], r32, dfv[2], dfv[3], opt.maxiter);
    }
    LAUNCH_CHECK();
    vcycle<float>(r32, z32);
    {
        KTimer _kt(this, kname("k_df_update_p", 0, true), L0.all_cells);
        launch_pdl(k_df_update_p, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, z32, dfv[2]);
    }
    LAUNCH_CHECK();
}

// Keeps iterating while any problem is active (bounded by maxiter + 2 passes).
__global__ void k_loop_cond(cudaGraphConditionalHandle h, const int *count, int *iters, int maxiter) {
    pdl_enter();
    int it = ++(*iters);
    cudaGraphSetConditional(h, (*count > 0 && it < maxiter + 2) ? 1u : 0u);
}

// The CG loop as one graph: a conditional WHILE node whose body is one iteration followed
// by k_loop_cond. Built once per (kind, iterate buffer); kind 0: FP64 CG, 1: mixed.
cudaGraphExec_t StructBatch::loop_graph(int kind, void *x) {
    GraphKey key{kind, x};
    auto it = graphs.find(key);
    if (it != graphs.end()) return it->second.exec;
    if (!cap_stream) CK(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle cond;
    CK(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t saved = stream;
    long long l0 = launches;
    stream = cap_stream;
    cudaError_t ce = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) {
        stream = saved;
        cudaGraphDestroy(g);
        ck(ce, "cudaStreamBeginCaptureToGraph");
    }
    try {
        if (kind == 0) pcg_iteration<double>((double *)x);
        else df_iteration((double *)x);
        launch_pdl(k_loop_cond, 1, 1, 0, stream, cond, d_count, d_count + 2, opt.maxiter);
        launches++;
        LAUNCH_CHECK();
    } catch (...) {
        cudaGraph_t junk;
        cudaStreamEndCapture(cap_stream, &junk);
        stream = saved;
        cudaGraphDestroy(g);
        throw;
    }
    CK(cudaStreamEndCapture(stream, &body));
    stream = saved;
    GraphRec rec;
    rec.graph = g;
    rec.body_kernels = launches - l0;
    launches = l0;
    CK(cudaGraphInstantiate(&rec.exec, g, 0));
    graphs[key] = rec;
    return rec.exec;
}

void StructBatch::run_loop(int kind, void *x) {
    if (opt.use_graphs && !prof_on) {
        cudaGraphExec_t ex = loop_graph(kind, x);
        CK(cudaGraphLaunch(ex, stream));
        // the graph's kernel launches (body kernels times passes) are counted when the solve
        // reads its statistics, with no synchronisation here
        graph_body_kernels = graphs[GraphKey{kind, x}].body_kernels;
        return;
    }
    const int check = std::max(1, opt.check_every);
    for (int it = 1; it <= opt.maxiter + 1; it++) {
        if (kind == 0) pcg_iteration<double>((double *)x);
        else df_iteration((double *)x);
        if (it % check == 0 && read_count(0) <= 0) return;
    }
    read_count(0);
}

// ---- FP64 preconditioned CG on all problems: A x = b
template <typename T>
void StructBatch::pcg(const T *b, T *x, double tol2) {
    Level &L0 = lv[0];
    Coeffs<T> C = coeffs_of<T>(L0, mixed);
    T *r = (T *)cgv[0], *z = (T *)cgv[1], *pv = (T *)cgv[2];
    const unsigned nb = nb_of(L0.all);
    CK(cudaMemsetAsync(d_count, 0, 4 * sizeof(int), stream));  // active problems, -, loop passes, -
    {
        KTimer _kt(this, kname("k_cg_start", 0, sizeof(T) == 4), L0.all_cells);
        launch_pdl(k_cg_start<T>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs, L0.all.d_pinfo, C,
                   (const uint8_t *)L0.dir, b, x, r, tol2);
    }
    LAUNCH_CHECK();
    vcycle<T>(r, z);
    {
        KTimer _kt(this, kname("k_update_p", 0, sizeof(T) == 4), L0.all_cells);
        launch_pdl(k_update_p<T>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, z, pv);
    }
    LAUNCH_CHECK();
    run_loop(0, (void *)x);
}

// ---- mixed precision: rounds of double-float CG with the FP32 V-cycle, each started
// from and checked against the true FP64 residual b64 - A x64
void StructBatch::df_pcg(const double *b64, double *x64, double tol2) {
    Level &L0 = lv[0];
    const unsigned nb = nb_of(L0.all);
    float *r32 = (float *)cgv[0], *z32 = (float *)cgv[1];
    CK(cudaMemsetAsync(d_count, 0, 4 * sizeof(int), stream));
    {
        KTimer _kt(this, kname(zero_guess ? "k_df_residual0" : "k_df_residual", 0, false), L0.all_cells);
        if (zero_guess)
            launch_pdl(k_df_residual<true, true>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs,
                                                                 L0.all.d_pinfo, coeffs_of<double>(L0, true),
                                                                 coeffs_of<float>(L0, true), L0.dir, b64, x64, r64, tol2,
                                                                 opt.maxiter, opt.max_outer);
        else
            launch_pdl(k_df_residual<true>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs,
                                                           L0.all.d_pinfo, coeffs_of<double>(L0, true),
                                                           coeffs_of<float>(L0, true), L0.dir, b64, x64, r64, tol2,
                                                           opt.maxiter, opt.max_outer);
    }
    LAUNCH_CHECK();
    for (int round = 0; round < opt.max_outer; round++) {
        // the last check's outcome, read together with the statistics: when no round follows
        // (warm-started transient steps often pass the first check), that is the solve's final
        // synchronisation. Running round 0 without reading the first check was slower: when no
        // problem needs it, its launches (all skipping) cost more than the synchronisation.
        if (read_stats() <= 0) {
            stats_fresh = true;
            break;
        }
        {
            KTimer _kt(this, kname("k_df_begin", 0, false), L0.all_cells);
            launch_pdl(k_df_begin, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, r64, dfv[1], r32);
        }
        LAUNCH_CHECK();
        vcycle<float>(r32, z32);
        {
            KTimer _kt(this, kname("k_df_update_p", 0, true), L0.all_cells);
            launch_pdl(k_df_update_p, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, z32, dfv[2]);
        }
        LAUNCH_CHECK();
        run_loop(1, x64);
        CK(cudaMemsetAsync(d_count, 0, sizeof(int), stream));
        {
            KTimer _kt(this, kname("k_df_residual", 0, false), L0.all_cells);
            launch_pdl(k_df_residual<false>, nb, kBlock, 0, stream, L0.d_desc, L0.all.d_map, d_state, d_count, rs,
                                                            L0.all.d_pinfo, coeffs_of<double>(L0, true),
                                                            coeffs_of<float>(L0, true), L0.dir, b64, x64, r64, tol2,
                                                            opt.maxiter, opt.max_outer);
        }
        LAUNCH_CHECK();
    }
}

// ---- full solve of A x = b for every problem (x holds the initial guess)
void StructBatch::solve(const double *b, double *x, double reltol) {
    if (opt.solver == DPF_SOLVER_CHOLESKY && direct_solve(b, x)) return;
    NvtxRange range("CG + AMG solve");
    const double tol2 = reltol * reltol;
    struct ZeroGuessReset {
        bool &f;
        ~ZeroGuessReset() { f = false; }
    } zg{zero_guess};
    {
        KTimer _kt(this, kname("k_state_init", 0, false), 0);
        launch_pdl(k_state_init, (nprob + 127) / 128, 128, 0, stream, d_state, nprob);
    }
    LAUNCH_CHECK();
    CK(cudaMemsetAsync(d_factor_status + 1, 0, sizeof(int), stream));  // expired-wait word of this solve
    graph_body_kernels = 0;
    stats_fresh = false;
    if (!mixed) {
        pcg<double>(b, x, tol2);
        stats_outer = 0;
    } else {
        df_pcg(b, x, tol2);
    }
    // statistics, the error words and the graph passes in one synchronisation (already read when
    // the rounds ended on reading them)
    if (!stats_fresh) read_stats();
    stats_fresh = false;
    if (graph_body_kernels) launches += graph_body_kernels * (long long)h_misc[2];
    CgState *hs = (CgState *)h_state_buf;
    last_status = DPF_OK;
    stats_iters = 0;
    stats_relres = 0.0;
    if (mixed) stats_outer = 0;
    for (int p = 0; p < nprob; p++) {
        if (mixed) stats_outer = std::max(stats_outer, hs[p].outer);
        stats_iters = std::max(stats_iters, mixed ? hs[p].total_iters : hs[p].iters);
        double rel = mixed ? (hs[p].obb > 0 ? std::sqrt(hs[p].orr / hs[p].obb) : 0.0)
                           : (hs[p].bb > 0 ? std::sqrt(hs[p].rr / hs[p].bb) : 0.0);
        stats_relres = std::max(stats_relres, rel);
        if (hs[p].status != DPF_OK && last_status == DPF_OK) last_status = hs[p].status;
    }
    if (h_misc[0]) {
        last_status = DPF_BAD_INPUT;
        last_message = "coarsest operator is not positive definite (does every problem have a Dirichlet cell?)";
    }
    if (h_misc[1]) {
        last_status = DPF_TIMEOUT;
        last_message = "a shared-memory staging wait of a smoother kernel expired";
    }
}


// ---- public operations
void StructBatch::forward(const double *Ks, const double *logK, int kind) {
    for (int p = 0; p < nprob; p++)
        if (ndir[p] == 0)
            throw BadInput("problem " + std::to_string(p) +
                           " has no Dirichlet cell: the steady-state operator is singular");
    if (logK) cell_k(logK, kind, in_kc);
    assemble(Ks, logK ? in_kc : nullptr, kind, nullptr, true);
    zero_guess = true;
    solve(b64, h, opt.reltol);
    fwd_kind = logK ? 1 : 0;
    mean_kind = kind;
    have_forward = true;
}

void StructBatch::adjoint_solve() {
    NvtxRange range("adjoint solve");
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_adjoint_rhs", 0, false), L0.all_cells);
        k_adjoint_rhs<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, L0.dir, delta, arhs, lam);
    }
    LAUNCH_CHECK();
    zero_guess = true;
    solve(arhs, lam, opt.reltol);
}

void *StructBatch::dalloc_bytes(size_t bytes) { return (void *)dalloc<char>(bytes, owned); }

long long *StructBatch::obs_buffer(size_t n) {
    if (n > obs_cap || !d_obs_buf) {
        const size_t cap = std::max<size_t>(n, 1024);
        d_obs_buf = dalloc<long long>(cap, owned);  // the previous buffer stays owned until destruction
        obs_cap = cap;
    }
    return d_obs_buf;
}

void StructBatch::obs_delta(const long long *d_obs, long long nobs) {
    CK(cudaMemsetAsync(delta, 0, N * sizeof(double), stream));
    if (nobs > 0) {
        {
            KTimer _kt(this, kname("k_obs_delta", 0, false), nobs);
            k_obs_delta<<<(unsigned)((nobs + 255) / 256), 256, 0, stream>>>(d_obs, nobs, h, delta);
        }
        LAUNCH_CHECK();
    }
}

void StructBatch::grad_faces(const double *hv, const double *lv_, double *dKs, bool accumulate) {
    NvtxRange range("face gradient");
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_grad_faces", 0, false), L0.all_cells);
        k_grad_faces<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, hv, lv_, dKs,
                                                           accumulate ? 1 : 0);
    }
    LAUNCH_CHECK();
}

void StructBatch::grad_logk(double *g) {
    Level &L0 = lv[0];
    if (mixed && mean_kind == DPF_MEAN_GEOMETRIC) {
        // the CG's double-float vectors are free once the solves are done
        {
            KTimer _kt(this, kname("k_grad_split", 0, false), L0.all_cells);
            k_grad_split<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, h, lam, in_kc, dfv[2],
                                                               dfv[3], dfv[1]);
        }
        LAUNCH_CHECK();
        {
            KTimer _kt(this, kname("k_grad_logk", 0, true), L0.all_cells);
            k_grad_logk_df<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, dfv[1], dfv[2],
                                                                 dfv[3], g);
        }
        LAUNCH_CHECK();
        return;
    }
    {
        KTimer _kt(this, kname("k_grad_logk", 0, false), L0.all_cells);
        k_grad_logk<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, in_kc, mean_kind, h, lam,
                                                          g);
    }
    LAUNCH_CHECK();
}

void StructBatch::grad_dh_q(const double *lv_, double *ddh, double *dQs, bool with_delta, bool accumulate) {
    Level &L0 = lv[0];
    FaceK fk{fwd_kind ? nullptr : in_Ks, fwd_kind ? in_kc : nullptr, mean_kind};
    {
        KTimer _kt(this, kname("k_grad_dh_q", 0, false), L0.all_cells);
        k_grad_dh_q<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, fk, L0.dir,
                                                          with_delta ? delta : nullptr, lv_, ddh, dQs,
                                                          accumulate ? 1 : 0);
    }
    LAUNCH_CHECK();
}

void StructBatch::cell_k(const double *logK, int kind, double *kc) {
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_cell_k", 0, false), L0.all_cells);
        k_cell_k<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, logK, kind, kc);
    }
    LAUNCH_CHECK();
}

void StructBatch::logk_to_faces(const double *logK, int kind, double *Ks) {
    Level &L0 = lv[0];
    cell_k(logK, kind, aux_kc);
    {
        KTimer _kt(this, kname("k_logk_to_faces", 0, false), L0.all_cells);
        k_logk_to_faces<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, aux_kc, kind, Ks);
    }
    LAUNCH_CHECK();
}

void StructBatch::logk_vjp(const double *logK, int kind, const double *dKs, double *g) {
    Level &L0 = lv[0];
    cell_k(logK, kind, aux_kc);
    {
        KTimer _kt(this, kname("k_logk_vjp", 0, false), L0.all_cells);
        k_logk_vjp<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, aux_kc, kind, dKs, g);
    }
    LAUNCH_CHECK();
}

void StructBatch::apply(const double *x, double *y) {
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_apply", 0, false), L0.all_cells);
        k_apply<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, coeffs_of<double>(L0, true), x, y);
    }
    LAUNCH_CHECK();
}

bool StructBatch::direct_solve(const double *b, double *x) {
    Level &L0 = lv[0];
    if (!direct_tried) {
        direct_tried = true;
        std::vector<std::array<int, 3>> dims;
        std::vector<long long> off;
        for (int p = 0; p < nprob; p++) {
            const LevelDesc &D = L0.h_desc[p];
            dims.push_back({D.nx, D.ny, D.nz});
            off.push_back(D.off);
        }
        const BandOrder ord = band_order_regular(dims, off);
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b));
        if (BandCholesky::fits(N, ord.w, free_b / 2)) direct.reset(new BandCholesky(ord, stream));
    }
    if (!direct) return false;
    NvtxRange range("direct solve (banded Cholesky)");
    BandCholesky &D = *direct;
    D.set_stream(stream);
    const long long l0 = D.launches;
    if (direct_stale) {
        D.clear();
        k_band_fill<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, coeffs_of<double>(L0, true),
                                                         D.iperm(), D.w, D.band());
        LAUNCH_CHECK();
        direct_ok = D.factor();
        direct_stale = false;
    }
    stats_iters = 0;
    stats_outer = 0;
    stats_relres = 0.0;
    if (!direct_ok) {
        last_status = DPF_BAD_INPUT;
        last_message = "the operator is not positive definite (does every problem have a Dirichlet cell?)";
        launches += D.launches - l0;
        return true;
    }
    D.solve(b, x);
    // the relative residual over the free cells, for the statistics
    apply(x, r64);
    if (!d_direct_acc) d_direct_acc = (double *)dalloc_bytes(2 * sizeof(double));
    stats_relres = BandCholesky::relres(stream, N, L0.dir, b, r64, d_direct_acc);
    last_status = std::isfinite(stats_relres) ? DPF_OK : DPF_NAN;
    if (last_status != DPF_OK) last_message = "non-finite residual after the direct solve";
    launches += D.launches - l0 + 2;
    return true;
}

// ---- transient backward Euler with checkpointed adjoint
void StructBatch::set_shift(const double *Ss, double dt) {
    if (!shift) shift = dalloc<double>(N, owned);
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_shift", 0, false), L0.all_cells);
        k_shift<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, d_prm, Ss, 1.0 / dt, shift);
    }
    LAUNCH_CHECK();
}

void StructBatch::transient_step(const double *b0, const double *hprev) {
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_axpy_rhs", 0, false), L0.all_cells);
        k_axpy_rhs<<<nb_of(L0.all), kBlock, 0, stream>>>(L0.d_desc, L0.all.d_map, L0.dir, b0, shift, hprev, b64);
    }
    LAUNCH_CHECK();
    solve(b64, h, opt.reltol);
}

template void StructBatch::vcycle<double>(const double *, double *);
template void StructBatch::vcycle<float>(const float *, float *);
template void StructBatch::pcg<double>(const double *, double *, double);

}  // namespace dpf
