// dpf_struct_kernels.cuh -- sm_103a kernels of the structured (regular-grid) path.
//
// All kernels are memory-bound sparse/vector work (about 0.1-0.3 flop/byte), so
// they are written for HBM/L2 streaming: one cell per thread, structure-of-arrays
// coefficients, neighbour values re-read through L1/L2, block reductions with
// warp shuffles, and a deterministic "last block finalises" reduction that puts
// CG scalars on the device (no host round trip per reduction).
#pragma once
#include "dpf_internal.h"

namespace dpf {

// ------------------------------------------------------------------ helpers
struct Cell {
    long long i;   // global index in the level arrays
    int ix, iy, iz;
};

__device__ __forceinline__ unsigned fast_div(unsigned n, unsigned m, int l) { return (__umulhi(n, m) + n) >> l; }

// Coordinates of the li-th cell of a grid (li < n), without integer division.
__device__ __forceinline__ void cell_at(const LevelDesc &L, int li, Cell &c) {
    unsigned u = (unsigned)li;
    unsigned q = fast_div(u, L.mag_nz, L.sh_nz);
    c.iz = (int)(u - q * (unsigned)L.nz);
    unsigned x = fast_div(q, L.mag_ny, L.sh_ny);
    c.iy = (int)(q - x * (unsigned)L.ny);
    c.ix = (int)x;
    c.i = L.off + li;
}

// Face index of the reference face list (regulargrid3d, src/grid.jl:163-185) of the
// face leaving cell (ix,iy,iz) in direction d (0:+x, 1:+y, 2:+z). Faces are emitted
// per cell in the order +x, +y, +z when the neighbour exists.
__host__ __device__ __forceinline__ long long regular_face_index(int nx, int ny, int nz, int ix, int iy, int iz,
                                                                 int d) {
    long long ex = ix < nx - 1, ey = iy < ny - 1;
    long long base = (long long)ix * (3LL * ny * nz - nz - ny) + (long long)iy * (ex * nz + nz + nz - 1) +
                     (long long)iz * (ex + ey + 1);
    if (d == 0) return base;
    if (d == 1) return base + ex;
    return base + ex + ey;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Reduction accumulators. FP64 kernels sum in double. FP32 kernels avoid FP64
// arithmetic per cell (GB300's FP64 rate is a small fraction of its FP32 rate):
// each product is formed exactly as an unevaluated float pair (fmaf error term)
// and pairs are added with Knuth's two-sum, giving about 48 significant bits;
// only the per-block result is converted to double.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    float h = s + e;
    return DF{h, e - (h - s)};
}
__device__ __forceinline__ DF df_shfl(DF a, int o) {
    return DF{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}

template <typename T>
struct Acc;
template <>
struct Acc<double> {
    double v = 0.0;
    __device__ __forceinline__ static Acc prod(double a, double b) { Acc r; r.v = a * b; return r; }
    __device__ __forceinline__ Acc operator+(Acc o) const { Acc r; r.v = v + o.v; return r; }
    __device__ __forceinline__ Acc shfl(int o) const { Acc r; r.v = __shfl_xor_sync(0xffffffffu, v, o); return r; }
    __device__ __forceinline__ double to_double() const { return v; }
};
template <>
struct Acc<float> {
    DF v = DF{0.f, 0.f};
    __device__ __forceinline__ static Acc prod(float a, float b) {
        Acc r;
        float p = a * b;
        r.v = DF{p, fmaf(a, b, -p)};
        return r;
    }
    __device__ __forceinline__ Acc operator+(Acc o) const { Acc r; r.v = df_add(v, o.v); return r; }
    __device__ __forceinline__ Acc shfl(int o) const { Acc r; r.v = df_shfl(v, o); return r; }
    __device__ __forceinline__ double to_double() const { return (double)v.hi + (double)v.lo; }
};

// Block-wide sum of NV (1 or 2) accumulators, converted to double; valid in thread 0.
// Every thread of the block must call it.
template <typename T, int NV>
__device__ __forceinline__ double2 block_sum(Acc<T> a, Acc<T> b) {
    __shared__ Acc<T> sh[NV][kBlock / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = a + a.shfl(o);
        if (NV == 2) b = b + b.shfl(o);
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sh[0][w] = a;
        if (NV == 2) sh[NV - 1][w] = b;
    }
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (w == 0) {
        Acc<T> x, y;
        if (l < (int)(blockDim.x >> 5)) {
            x = sh[0][l];
            if (NV == 2) y = sh[NV - 1][l];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x = x + x.shfl(o);
            if (NV == 2) y = y + y.shfl(o);
        }
        r = make_double2(x.to_double(), NV == 2 ? y.to_double() : 0.0);
    }
    return r;
}

// Write this block's partial; return true (in every thread) in the last block of
// problem p to arrive, with the problem total in `tot`. Deterministic: the total is
// always summed over the partial slots in the same order. Each block reduces once
// per launch (kernels loop over their cells), so this runs about once per resident
// block rather than once per 256 cells.
template <typename T, int NV = 1>
__device__ __forceinline__ bool reduce_last(Acc<T> a, Acc<T> b, ReduceScratch rs, int2 pinfo, int p, double2 &tot) {
    __shared__ int amlast;
    __shared__ double2 total;
    double2 s = block_sum<T, NV>(a, b);
    if (threadIdx.x == 0) {
        rs.partials[blockIdx.x] = s;
        __threadfence();
        unsigned t = atomicAdd(&rs.tickets[p], 1u);
        amlast = (t == (unsigned)(pinfo.y - 1));
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
    Acc<double> ax, ay;
    for (int k = threadIdx.x; k < pinfo.y; k += blockDim.x) {
        double2 q = __ldcg(&rs.partials[pinfo.x + k]);
        ax.v += q.x;
        if (NV == 2) ay.v += q.y;
    }
    double2 r = block_sum<double, 2>(ax, ay);
    if (threadIdx.x == 0) {
        total = r;
        rs.tickets[p] = 0u;
    }
    __syncthreads();
    tot = total;
    return true;
}

// Flux-form 7-point operator at one cell: Ax = leak x_i + sum_f c_f (x_i - x_j) and
// the diagonal. XAt(j, jx, jy, jz) returns x at neighbour j.
template <typename T, typename XAt>
__device__ __forceinline__ void apply7(const LevelDesc &L, const Cell &c, const Coeffs<T> &C, T xi, XAt xat, T &Ax,
                                       T &diag) {
    const long long i = c.i;
    const long long sy = L.nz, sx = (long long)L.ny * L.nz;
    T lk = C.leak[i];
    T a = lk * xi, d = lk;
    if (c.iz + 1 < L.nz) { T w = C.cz[i];      a += w * (xi - xat(i + 1, c.ix, c.iy, c.iz + 1));   d += w; }
    if (c.iz > 0)        { T w = C.cz[i - 1];  a += w * (xi - xat(i - 1, c.ix, c.iy, c.iz - 1));   d += w; }
    if (c.iy + 1 < L.ny) { T w = C.cy[i];      a += w * (xi - xat(i + sy, c.ix, c.iy + 1, c.iz));  d += w; }
    if (c.iy > 0)        { T w = C.cy[i - sy]; a += w * (xi - xat(i - sy, c.ix, c.iy - 1, c.iz));  d += w; }
    if (c.ix + 1 < L.nx) { T w = C.cx[i];      a += w * (xi - xat(i + sx, c.ix + 1, c.iy, c.iz));  d += w; }
    if (c.ix > 0)        { T w = C.cx[i - sx]; a += w * (xi - xat(i - sx, c.ix - 1, c.iy, c.iz));  d += w; }
    Ax = a;
    diag = d;
}

// v / diag for the smoothers: FP64 levels multiply by the stored inverse diagonal
// (a DP division per cell per sweep is expensive on GB300), FP32 levels use the fast
// approximate division (about 2 ulp, ample for a smoother).
template <typename T>
__device__ __forceinline__ T dinv_times(const Coeffs<T> &C, long long i, T v, T dg) {
    if constexpr (sizeof(T) == 8) {
        return v * C.idg[i];
    } else {
        return __fdividef(v, dg);
    }
}

template <typename T>
__device__ __forceinline__ T diag7(const LevelDesc &L, const Cell &c, const Coeffs<T> &C) {
    const long long i = c.i;
    const long long sy = L.nz, sx = (long long)L.ny * L.nz;
    T d = C.leak[i];
    if (c.iz + 1 < L.nz) d += C.cz[i];
    if (c.iz > 0) d += C.cz[i - 1];
    if (c.iy + 1 < L.ny) d += C.cy[i];
    if (c.iy > 0) d += C.cy[i - sy];
    if (c.ix + 1 < L.nx) d += C.cx[i];
    if (c.ix > 0) d += C.cx[i - sx];
    return d;
}

// -------------------------------------------------------------- assembly
// Face conductances from cell values kc, computed once per cell by k_cell_k
// (GB300 has little FP64 throughput, so exp runs once per cell, not once per face):
//   geometric  kc = exp(logK / 2):  K_f = exp((logK_a + logK_b)/2) = kc_a kc_b
//   harmonic   kc = exp(logK):      K_f = 2 / (1/K_a + 1/K_b) = 2 kc_a kc_b / (kc_a + kc_b)
__device__ __forceinline__ double face_mean_k(double ka, double kb, int kind) {
    if (kind == DPF_MEAN_GEOMETRIC) return ka * kb;
    return 2.0 * ka * kb / (ka + kb);
}
// dK_f / dlogK_a:  geometric K_f / 2;  harmonic K_f^2 / (2 K_a)
__device__ __forceinline__ double face_mean_dlogk(double Kf, double ka, int kind) {
    if (kind == DPF_MEAN_GEOMETRIC) return 0.5 * Kf;
    return 0.5 * Kf * Kf / ka;
}

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
// FP32 copies.
__global__ void k_assemble(const LevelDesc *__restrict__ desc, const int4 *__restrict__ bmap,
                           const ProbParam *__restrict__ prm, FaceK fk, const double *__restrict__ dh,
                           const double *__restrict__ Qs, const double *__restrict__ shift,
                           const uint8_t *__restrict__ dir, double *cx, double *cy, double *cz, double *leak,
                           float *fx, float *fy, float *fz, float *fleak, double *b, double *x, int init_x) {
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
        cx[i] = cp[0]; cy[i] = cp[1]; cz[i] = cp[2]; leak[i] = lk;
        if (fx) { fx[i] = (float)cp[0]; fy[i] = (float)cp[1]; fz[i] = (float)cp[2]; fleak[i] = (float)lk; }
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
                          double *ccy, double *ccz, double *cleak, uint8_t *cdir, float *gx, float *gy, float *gz,
                          float *gleak) {
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
        if (gx) { gx[i] = (float)sx; gy[i] = (float)sy; gz[i] = (float)sz; gleak[i] = (float)lk; }
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

}  // namespace dpf
