// dpf_struct_kernels.cuh -- sm_103a kernels of the structured (regular-grid) path.
//
// All kernels are memory-bound sparse/vector work (about 0.1-0.3 flop/byte), so
// they are written for HBM/L2 streaming: one cell per thread, structure-of-arrays
// coefficients, neighbour values re-read through L1/L2, block reductions with
// warp shuffles, and a deterministic "last block finalises" reduction that puts
// CG scalars on the device (no host round trip per reduction).
#pragma once
#include "dpf_check.cuh"
#include "dpf_internal.h"

namespace dpf {

// ------------------------------------------------------------------ helpers
struct Cell {
    long long i;   // global index in the level arrays
    int ix, iy, iz;
};

__device__ __forceinline__ unsigned fast_div(unsigned n, unsigned m, int l) { return (__umulhi(n, m) + n) >> l; }

// Programmatic dependent launch. Every solver kernel begins by waiting for the kernels it
// follows on its stream (griddepcontrol.wait returns once they have completed and their
// writes are visible, at once when the launch carried no such dependency), so launches with
// the programmatic serialization attribute run in stream order while the next launch is
// prepared during the previous kernel. Kernels do not signal their dependents early
// (griddepcontrol.launch_dependents at block start): on the benchmark solve that made the
// graphs 10 % slower, as waiting blocks of the next kernel took SM slots.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Coordinates of the li-th cell of a grid (li < n), without integer division.
__device__ __forceinline__ void cell_at(const LevelDesc &L, int li, Cell &c) {
    unsigned u = (unsigned)li;
    unsigned q = fast_div(u, L.mag_nz, L.sh_nz);
    c.iz = (int)(u - q * (unsigned)L.nz);
    unsigned x = fast_div(q, L.mag_ny, L.sh_ny);
    c.iy = (int)(q - x * (unsigned)L.ny);
    c.ix = (int)x;
    c.i = L.off + li;
#if DPF_CHECKED
    if (!DPF_INSIDE(CK_CELL, li, 0, L.n) || !DPF_INSIDE(CK_CELL, c.ix, 0, L.nx) || !DPF_INSIDE(CK_CELL, c.iy, 0, L.ny) ||
        !DPF_INSIDE(CK_CELL, ((long long)c.ix * L.ny + c.iy) * L.nz + c.iz, li, (long long)li + 1)) {
        c.ix = c.iy = c.iz = 0;  // the problem's first cell: no access outside it
        c.i = L.off;
    }
#endif
}

// A stored coefficient as the arithmetic type of its level.
__device__ __forceinline__ float cf(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float cf(float v) { return v; }
__device__ __forceinline__ double cf(double v) { return v; }

// Index in the coarse level arrays of the 2x2x2 aggregate that holds fine cell c.
__device__ __forceinline__ long long agg_index(const LevelDesc &Lc, const Cell &c) {
    const int ax = c.ix >> 1, ay = c.iy >> 1, az = c.iz >> 1;
#if DPF_CHECKED
    if (!DPF_INSIDE(CK_AGGREGATE, ax, 0, Lc.nx) || !DPF_INSIDE(CK_AGGREGATE, ay, 0, Lc.ny) ||
        !DPF_INSIDE(CK_AGGREGATE, az, 0, Lc.nz))
        return Lc.off;
#endif
    return Lc.off + ((long long)ax * Lc.ny + ay) * Lc.nz + az;
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
// Double-float (hi + lo) arithmetic. Additions and products inside an error-free
// transformation use the _rn intrinsics, which the compiler never contracts into a fused
// multiply-add (a contraction would make the captured rounding errors inexact).
#ifndef DPF_DF_STRICT_ACC
#define DPF_DF_STRICT_ACC 1
#endif
#ifndef DPF_DF_STRICT_VEC
#define DPF_DF_STRICT_VEC 1
#endif
#if DPF_DF_STRICT_ACC
#define DPF_ACC_ADD(a, b) __fadd_rn(a, b)
#define DPF_ACC_SUB(a, b) __fsub_rn(a, b)
#define DPF_ACC_MUL(a, b) __fmul_rn(a, b)
#else
#define DPF_ACC_ADD(a, b) ((a) + (b))
#define DPF_ACC_SUB(a, b) ((a) - (b))
#define DPF_ACC_MUL(a, b) ((a) * (b))
#endif
#if DPF_DF_STRICT_VEC
#define DPF_VEC_ADD(a, b) __fadd_rn(a, b)
#define DPF_VEC_SUB(a, b) __fsub_rn(a, b)
#define DPF_VEC_MUL(a, b) __fmul_rn(a, b)
#else
#define DPF_VEC_ADD(a, b) ((a) + (b))
#define DPF_VEC_SUB(a, b) ((a) - (b))
#define DPF_VEC_MUL(a, b) ((a) * (b))
#endif
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = DPF_ACC_ADD(a.hi, b.hi);
    const float bb = DPF_ACC_SUB(s, a.hi);
    float e = DPF_ACC_ADD(DPF_ACC_SUB(a.hi, DPF_ACC_SUB(s, bb)), DPF_ACC_SUB(b.hi, bb));
    e = DPF_ACC_ADD(e, DPF_ACC_ADD(a.lo, b.lo));
    const float h = DPF_ACC_ADD(s, e);
    return DF{h, DPF_ACC_SUB(e, DPF_ACC_SUB(h, s))};
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
        const float p = DPF_ACC_MUL(a, b);
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
    __shared__ Acc<T> sh[NV][32];  // one slot per warp of any block size
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
__device__ __forceinline__ bool reduce_last(Acc<T> a, Acc<T> b, ReduceScratch rs, int2 pinfo, int p, double2 &tot,
                                            int slot = -1) {
    __shared__ int amlast;
    __shared__ double2 total;
    double2 s = block_sum<T, NV>(a, b);
    if (threadIdx.x == 0) {
        rs.partials[slot >= 0 ? slot : (int)blockIdx.x] = s;
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

// reduce_last for launches whose blocks each contribute one partial per work item (the
// plane-marching kernels): the partial goes to the item's slot, and pinfo = {first slot, slots}
// of problem p.
template <typename T>
__device__ __forceinline__ bool reduce_last_slot(Acc<T> a, ReduceScratch rs, int2 pinfo, int p, int slot,
                                                 double2 &tot) {
    return reduce_last<T, 1>(a, Acc<T>(), rs, pinfo, p, tot, slot);
}

// Flux-form 7-point operator at one cell: Ax = leak x_i + sum_f c_f (x_i - x_j) and
// the diagonal. XAt(j, jx, jy, jz) returns x at neighbour j.
template <typename T, typename XAt>
__device__ __forceinline__ void apply7(const LevelDesc &L, const Cell &c, const Coeffs<T> &C, T xi, XAt xat, T &Ax,
                                       T &diag) {
    const long long i = c.i;
    const long long sy = L.nz, sx = (long long)L.ny * L.nz;
    T lk = cf(C.leak[i]);
    T a = lk * xi, d = lk;
#if DPF_CHECKED
    // every neighbour the flags below admit lies inside the problem's cells
    if (!(DPF_INSIDE(CK_NEIGHBOUR, c.iz + 1 < L.nz ? i + 1 : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.iz > 0 ? i - 1 : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.iy + 1 < L.ny ? i + sy : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.iy > 0 ? i - sy : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.ix + 1 < L.nx ? i + sx : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.ix > 0 ? i - sx : i, L.off, L.off + L.n))) {
        Ax = a;
        diag = d;
        return;
    }
#endif
    if (c.iz + 1 < L.nz) { T w = cf(C.cz[i]);      a += w * (xi - xat(i + 1, c.ix, c.iy, c.iz + 1));   d += w; }
    if (c.iz > 0)        { T w = cf(C.cz[i - 1]);  a += w * (xi - xat(i - 1, c.ix, c.iy, c.iz - 1));   d += w; }
    if (c.iy + 1 < L.ny) { T w = cf(C.cy[i]);      a += w * (xi - xat(i + sy, c.ix, c.iy + 1, c.iz));  d += w; }
    if (c.iy > 0)        { T w = cf(C.cy[i - sy]); a += w * (xi - xat(i - sy, c.ix, c.iy - 1, c.iz));  d += w; }
    if (c.ix + 1 < L.nx) { T w = cf(C.cx[i]);      a += w * (xi - xat(i + sx, c.ix + 1, c.iy, c.iz));  d += w; }
    if (c.ix > 0)        { T w = cf(C.cx[i - sx]); a += w * (xi - xat(i - sx, c.ix - 1, c.iy, c.iz));  d += w; }
    Ax = a;
    diag = d;
}

// |v| as a float, truncated, from v's bits (integer operations only): 0 below 2^-126, 3e38 at or
// above 2^128 (Inf and NaN included). For rounding-floor estimates, where a relative error of
// 2^-23 is immaterial and an FP64-to-FP32 conversion would occupy GB300's FP64 pipe.
__device__ __forceinline__ float abs_float_trunc(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
    const int e = (int)(u >> 52);
    if (e >= 1023 + 128) return 3.0e38f;
    if (e <= 1023 - 127) return 0.0f;
    return __uint_as_float(((unsigned)(e - 1023 + 127) << 23) | ((unsigned)(u >> 29) & 0x7FFFFFu));
}

// apply7 in FP64 (the same arithmetic in the same order: A x is bitwise apply7's) with the
// diagonal summed in FP32 from the level's bf16 coefficients: the diagonal only scales a
// rounding-floor estimate, where bf16 precision is ample, and FP64 additions cost as much as
// the flux terms on GB300's FP64 pipe.
__device__ __forceinline__ void apply7_f32diag(const LevelDesc &L, const Cell &c, const Coeffs<double> &C,
                                               const Coeffs<float> &C16, double xi, const double *__restrict__ x,
                                               double &Ax, float &diag) {
    const long long i = c.i;
    const long long sy = L.nz, sx = (long long)L.ny * L.nz;
    double a = C.leak[i] * xi;
    float d = cf(C16.leak[i]);
#if DPF_CHECKED
    if (!(DPF_INSIDE(CK_NEIGHBOUR, c.iz + 1 < L.nz ? i + 1 : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.iz > 0 ? i - 1 : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.iy + 1 < L.ny ? i + sy : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.iy > 0 ? i - sy : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.ix + 1 < L.nx ? i + sx : i, L.off, L.off + L.n) &&
          DPF_INSIDE(CK_NEIGHBOUR, c.ix > 0 ? i - sx : i, L.off, L.off + L.n))) {
        Ax = a;
        diag = d;
        return;
    }
#endif
    if (c.iz + 1 < L.nz) { a += C.cz[i] * (xi - x[i + 1]);       d += cf(C16.cz[i]); }
    if (c.iz > 0)        { a += C.cz[i - 1] * (xi - x[i - 1]);   d += cf(C16.cz[i - 1]); }
    if (c.iy + 1 < L.ny) { a += C.cy[i] * (xi - x[i + sy]);      d += cf(C16.cy[i]); }
    if (c.iy > 0)        { a += C.cy[i - sy] * (xi - x[i - sy]); d += cf(C16.cy[i - sy]); }
    if (c.ix + 1 < L.nx) { a += C.cx[i] * (xi - x[i + sx]);      d += cf(C16.cx[i]); }
    if (c.ix > 0)        { a += C.cx[i - sx] * (xi - x[i - sx]); d += cf(C16.cx[i - sx]); }
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
    T d = cf(C.leak[i]);
    if (c.iz + 1 < L.nz) d += cf(C.cz[i]);
    if (c.iz > 0) d += cf(C.cz[i - 1]);
    if (c.iy + 1 < L.ny) d += cf(C.cy[i]);
    if (c.iy > 0) d += cf(C.cy[i - sy]);
    if (c.ix + 1 < L.nx) d += cf(C.cx[i]);
    if (c.ix > 0) d += cf(C.cx[i - sx]);
    return d;
}

// -------------------------------------------------------------- assembly
// ---------------------------------------------------------- shared helpers
__device__ __forceinline__ void deactivate(CgState &s, int *count) {
    if (s.active) {
        s.active = 0;
        atomicSub(count, 1);
    }
}

// double-float arithmetic: unevaluated sums hi + lo of two floats (about 48 bits)
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = DPF_VEC_ADD(a, b);
    const float bb = DPF_VEC_SUB(s, a);
    return make_float2(s, DPF_VEC_ADD(DPF_VEC_SUB(a, DPF_VEC_SUB(s, bb)), DPF_VEC_SUB(b, bb)));
}
__device__ __forceinline__ float2 df_quick(float a, float b) {
    const float s = DPF_VEC_ADD(a, b);
    return make_float2(s, DPF_VEC_SUB(b, DPF_VEC_SUB(s, a)));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float2 s = df_two_sum(a.x, b.x);
    s.y = DPF_VEC_ADD(s.y, DPF_VEC_ADD(a.y, b.y));
    return df_quick(s.x, s.y);
}
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = DPF_VEC_MUL(a.x, b.x);
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_quick(p, e);
}
__device__ __forceinline__ float2 df_from_double(double v) {
    float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }
// v rounded to 48 significant bits (to nearest, ties away from zero), v48, and its exact split
// v48 = hi + lo into two floats, formed from v's bits with integer operations only: conversions
// between FP64 and FP32 run on GB300's FP64 pipe, a small fraction of its FP32 rate, and the
// split is needed per cell. hi is v48 with its low 29 fraction bits cleared (exactly a float), lo
// the next 24 bits (a 24-bit integer times a power of two: exact). Handles zero and
// 2^-79 <= |v48| < 2^128; returns false for anything else (subnormals, tiny or huge values, Inf,
// NaN), where the caller takes the FP64 route.
__device__ __forceinline__ bool split48(double v, float &hi, float &lo, double &v48) {
    const unsigned long long u0 = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(u0 >> 32) & 0x80000000u;
    if ((u0 << 1) == 0ull) {  // +0 or -0
        hi = lo = __uint_as_float(sign);
        v48 = v;
        return true;
    }
    if (((u0 >> 52) & 0x7FFull) == 0x7FFull) return false;  // Inf, NaN
    // add half of the 5 dropped bits, then drop them (a carry runs into the exponent correctly)
    const unsigned long long u = (u0 + 0x10ull) & ~0x1Full;
    const int e = (int)((u >> 52) & 0x7FFull);
    const int E = e - 1023;
    if (e == 0 || E < -79 || E > 127) return false;
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    hi = __uint_as_float(sign | ((unsigned)(E + 127) << 23) | (unsigned)(m >> 29));
    const unsigned r24 = (unsigned)(m >> 5) & 0xFFFFFFu;
    const float lo_mag = __uint2float_rn(r24) * __uint_as_float((unsigned)(E - 47 + 127) << 23);
    lo = __uint_as_float(__float_as_uint(lo_mag) | sign);
    v48 = __longlong_as_double((long long)u);
    return true;
}

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

}  // namespace dpf
