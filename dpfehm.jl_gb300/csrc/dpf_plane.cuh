// dpf_plane.cuh -- plane-marching Chebyshev kernels for the structured multigrid levels.
//
// A block owns a slab of `rows` consecutive y-rows of a problem's grid (all nz cells of
// each row, so the slab is one contiguous range of each array per x-plane) and marches
// along x over a chunk of planes. Every array the step reads is streamed plane by plane
// into a ring of shared-memory stages with 1-D bulk asynchronous copies
// (cp.async.bulk, completion on an mbarrier); the x-plane of the iterate is staged with one
// halo row on each side, so all six neighbours of a cell come from shared memory and each
// value is read from HBM once. A producer warp issues the copies, so the copies in flight
// do not occupy registers and the ring keeps planes ahead in flight per block.
//
// The arithmetic is that of the per-cell bodies in dpf_struct.cu in the same order
// (apply7: z+, z-, y+, y-, x+, x-), so results are bitwise identical to the grid-stride
// kernels, except in the two fused pre-smoothing steps from zero (PM_FIRST2), which stage the
// first step's iterate in place of b and recover the cell's own b from it (a few ulps of FP32).
// Every mbarrier wait is bounded (one second); on expiry the kernel records an error in
// *err, and the producer drains its copies (bounded, an expiry recorded too) before the block returns.
#pragma once
#include <cstdint>

#include "dpf_check.cuh"
#include "dpf_struct_kernels.cuh"

namespace dpf {

#ifndef DPF_PLANE_THREADS
#define DPF_PLANE_THREADS 256
#endif
constexpr int kPlaneThreads = DPF_PLANE_THREADS;  // consumer threads per block (plus one producer warp)
#ifndef DPF_PLANE_STAGES
#define DPF_PLANE_STAGES 4
#endif
constexpr int kPlaneStages = DPF_PLANE_STAGES;  // planes x-1, x, x+1 resident, the rest in flight
constexpr int kMaxCellsPerThread = 4;  // slab capacity CPT x kPlaneThreads cells, CPT = 1..4 (a template parameter)
// Rows per slab: the fewest slabs of at most `cells` cells of whole rows, with the rows
// spread evenly over them, and an even count (so that slabs align with the 2x2x2
// aggregates of the next level) unless one slab holds the whole plane. Host and device
// both use it, so the work items and the kernels agree.
__host__ __device__ __forceinline__ int plane_rows(int ny, int nz, int cells) {
    int t = cells / nz;
    if (t >= 2) t &= ~1;
    if (t < 1) t = 1;
    if (t >= ny) return ny;
    const int tiles = (ny + t - 1) / t;
    int u = (ny + tiles - 1) / tiles;  // <= t
    if (t >= 2) u += u & 1;            // still <= t: t is even
    return u;
}

// per-cell flags: inside the slab, and which of the z+/z-/y+/y- neighbours exist
constexpr unsigned CF_VALID = 1u, CF_ZP = 2u, CF_ZM = 4u, CF_YP = 8u, CF_YM = 16u;
constexpr uint64_t kWaitNs = 1000000000ull;       // a bounded mbarrier wait ends after one second ...
constexpr uint32_t kWaitTries = 1u << 28;         // ... or, should the global timer stall, 2^28 polls

enum : int { PM_FIRST2 = 1, PM_FIRST = 2, PM_PROLONG = 4, PM_NOD = 8, PM_RZ = 16 };

// byte offsets of the per-stream regions in one stage, and the stage size (host computed)
struct PlaneLayout {
    int slot_bytes;
    int oX, oB, oD, oCX, oCY, oCZ, oLK, oG, oDIR, oE;
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred P;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, P;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// bounded wait for the phase with the given parity: one second by the global timer (a poll
// count far above what a second of polling takes is only a backstop); false and *err set on
// expiry. The bound is by time so that a block descheduled or slowed by other work on the GPU
// does not see a wait expire that would have completed.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t k = 0; k < kWaitTries; k++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((k & 63) == 63 && global_ns() - t0 > kWaitNs) break;
    }
    atomicExch(err, 1);
    return false;
}
// barrier 1 over the `count` consumer threads only (the producer warp does not take part),
// returning the OR of `pred` over them: a shared error flag makes every consumer leave
// together, so no consumer is left waiting at the barrier
__device__ __forceinline__ bool consumer_sync_or(bool pred, int count) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(count)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// order this thread's generic-proxy shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbarrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// One staged range: global elements [a0, a1) of `base` land in the stage region at
// element position delta + (a0 - l0), where l0 is the logical start of the region and
// delta = (l0 * es mod 16) / es puts source and destination on the same 16-byte phase.
// Both ends are widened to 16-byte boundaries (allocations carry 64 bytes of padding).
struct BulkRange {
    const char *src;
    char *dst;
    uint32_t bytes;
};

__device__ __forceinline__ int stage_delta(long long l0, int es) { return (int)(((l0 * es) & 15) / es); }

__device__ __forceinline__ BulkRange make_range(const void *base, int es, long long l0, long long a0, long long a1,
                                                char *region) {
    BulkRange r;
    const uintptr_t s0 = (uintptr_t)base + (uintptr_t)(a0 * es);
    const uintptr_t res = s0 & 15u;
    const uintptr_t s1 = (uintptr_t)base + (uintptr_t)(a1 * es);
    r.src = (const char *)(s0 - res);
    r.dst = region + (stage_delta(l0, es) + (a0 - l0)) * es - res;
    r.bytes = (uint32_t)(((s1 - (s0 - res)) + 15u) & ~(uintptr_t)15u);
    return r;
}

// Announces (expect_tx) and issues the bulk copy of elements [a0, a1) of `base` into the
// stage region `region` (see make_range). In a checked build the range must lie in the array
// section [lo, hi), the copy inside its slot [slot, slot + slot_bytes) and on 16-byte
// boundaries; a violation is recorded and the copy is not issued (the phase then completes
// without it).
__device__ __forceinline__ void stage_range(uint64_t *bar, const void *base, int es, long long l0, long long a0,
                                            long long a1, char *region, long long lo, long long hi, const char *slot,
                                            int slot_bytes) {
    const BulkRange r = make_range(base, es, l0, a0, a1, region);
#if DPF_CHECKED
    if (a1 > a0 && !(DPF_INSIDE(CK_STAGE_SRC, a0, lo, hi) && DPF_INSIDE(CK_STAGE_SRC, a1 - 1, lo, hi))) return;
    if (!DPF_INSIDE(CK_STAGE_DST, r.dst - slot, 0, slot_bytes) ||
        !DPF_INSIDE(CK_STAGE_DST, r.dst + r.bytes - slot, 0, slot_bytes + 1))
        return;
    if (!DPF_INSIDE(CK_STAGE_ALIGN, (long long)(((uintptr_t)r.src | smem_addr(r.dst) | r.bytes) & 15u), 0, 1)) return;
#else
    (void)lo;
    (void)hi;
    (void)slot;
    (void)slot_bytes;
#endif
    mbar_expect_tx(bar, r.bytes);
    bulk_copy_g2s(r.dst, r.src, r.bytes, bar);
}

// Fast division of k (< 2^31) by nz with the level's invariant-integer constants.
__device__ __forceinline__ int div_nz(const LevelDesc &L, int k) { return (int)fast_div((unsigned)k, L.mag_nz, L.sh_nz); }

// Work of a plane-marching launch: items {p, y0, x0, x1} (a slab of rows y0.. of problem p,
// planes x0..x1-1; x0 even, x1 even or the grid's last plane), and per block the contiguous
// range of items it marches through, first[b] .. first[b+1]-1. The host cuts the items so that
// every block gets about the same number of cells. A block's planes are numbered across its
// items (g = 0, 1, ...): ring slot g % R, phase (g / R) & 1, so the ring runs on from one item to
// the next.
struct PlaneWork {
    const int4 *items;
    const int *first;
};

// Producer of one item, run by lane 0 of the producer warp: stages planes pl_lo..pl_hi (block
// plane numbers g0, g0 + 1, ...) into the ring as the consumer warps release slots.
// stage_plane(q, slot, bar) announces (mbarrier expect_tx) and issues the copies of plane q;
// the one pending arrival made here afterwards keeps the phase open until every copy has been
// announced. Returns the planes issued (fewer than the item's when a bounded wait expired).
template <int R, typename F>
__device__ __forceinline__ int pm_produce(int pl_lo, int pl_hi, int g0, uint64_t *full, uint64_t *empty,
                                          unsigned char *sm, int slot_bytes, int *err, F stage_plane) {
    for (int q = pl_lo; q <= pl_hi; q++) {
        const int g = g0 + (q - pl_lo), s = g % R;
        if (g >= R && !mbar_wait(&empty[s], (uint32_t)((g / R - 1) & 1), err)) return q - pl_lo;
        fence_proxy_async_smem();
        stage_plane(q, (char *)sm + s * slot_bytes, &full[s]);
        mbar_arrive(&full[s]);
    }
    return pl_hi - pl_lo + 1;
}

// Before the block may end, the last phase of every filled slot (the last min(R, issued) planes)
// is waited for (bounded), so no copy is still in flight into the block's shared memory. Should
// one of those waits expire, copies may still land after the block ends: the error word is set,
// the solve reports DPF_TIMEOUT and the host treats the device's results as suspect.
template <int R>
__device__ __forceinline__ void pm_drain(int issued, uint64_t *full, int *err) {
    for (int g = max(0, issued - R); g < issued; g++) mbar_wait(&full[g % R], (uint32_t)((g / R) & 1), err);
}

// x / y for the plane smoothers: FP32 takes the fast approximate division (about 2 ulp, ample in
// a smoother), FP64 the exact one
__device__ __forceinline__ float pm_div(float x, float y) { return __fdividef(x, y); }
__device__ __forceinline__ double pm_div(double x, double y) { return x / y; }

// Chebyshev step family on the plane ring. MODE bits:
//   PM_FIRST2  the first two steps from a zero guess (reads b and the inverse diagonal
//              with halos instead of an iterate; the first step's iterate invtheta b g is
//              formed once per staged plane, in place of b, before the plane is used)
//   PM_FIRST   d = c2 r (d not read)
//   PM_PROLONG the iterate is corrected on arrival: x += scale * e[aggregate] (not at
//              identity rows), i.e. the prolongation fused into the first post-step
//   PM_NOD     d not written (last step of a sweep)
//   PM_RZ      reduce b . xout per problem and finalise beta (last step of the cycle)
//
// Warp-specialised pipeline: warp kPlaneThreads/32 is the producer (its lane 0 stages
// plane after plane as ring slots free up), warps 0..7 consume. Per slot three mbarriers:
// full (copies landed), empty (all consumer warps are done with the plane), ready (with
// PM_PROLONG or PM_FIRST2: every consumer thread has applied its share of the correction or of
// the first step). A block marches
// through its items one after another; at the end of each item every thread meets (a block
// barrier that also carries the error flag, and with PM_RZ the item's partial of b . xout in its
// own reduction slot, so the sum per problem is formed in a fixed order).
template <typename T, int MODE, int CPT>
__global__ void __launch_bounds__(kPlaneThreads + 32) k_pm_cheb(
    const LevelDesc *__restrict__ desc, const LevelDesc *__restrict__ cdesc, PlaneWork work,
    CgState *st, Coeffs<T> C, const T *__restrict__ b, const T *__restrict__ xin, T *__restrict__ xout,
    T *__restrict__ d, const uint8_t *__restrict__ dir, const T *__restrict__ e, T c1, T c2, T invtheta, T scale,
    PlaneLayout lay, ReduceScratch rs, const int2 *__restrict__ pinfo, int *err) {
    pdl_enter();
    constexpr bool F2 = (MODE & PM_FIRST2) != 0, FIRST = (MODE & PM_FIRST) != 0,
                   PROL = (MODE & PM_PROLONG) != 0, NOD = (MODE & PM_NOD) != 0, RZ = (MODE & PM_RZ) != 0;
    constexpr int R = kPlaneStages;
    constexpr int es = (int)sizeof(T);
    using CT = coef_t<T>;
    constexpr int ec = (int)sizeof(CT);  // coefficient streams
    constexpr int kConsumerWarps = kPlaneThreads / 32;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[R], empty[R], ready[R];

    const int t = threadIdx.x;
    const int warp = t >> 5, lane = t & 31;
    auto slot_of = [&](int g) { return (char *)sm + ((unsigned)g % (unsigned)R) * lay.slot_bytes; };
    if (t == 0) {
        for (int s = 0; s < R; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
            mbar_init(&ready[s], kPlaneThreads);
        }
        fence_mbarrier_init();
    }
    __syncthreads();
    int g0 = 0;      // block plane number of the current item's first plane
    int issued = 0;  // planes the producer has staged (producer lane 0)
    for (int w = work.first[blockIdx.x]; w < work.first[blockIdx.x + 1]; w++) {
        const int4 it = work.items[w];
        const int p = it.x, y0 = it.y, xa = it.z, xe = it.w;
        if (st && !st[p].active) continue;  // uniform over the block
        const LevelDesc L = desc[p];
        const int nz = L.nz, ny = L.ny, nx = L.nx;
        const long long sx = (long long)ny * nz;
        const int Ty = plane_rows(ny, nz, CPT * kPlaneThreads);
        const int rows = min(Ty, ny - y0);
        const int ncell = rows * nz;
        const int pl_lo = max(xa - 1, 0), pl_hi = min(xe, nx - 1);
        const int h0 = max(y0 - 1, 0), h1 = min(y0 + rows + 1, ny);
        LevelDesc Lc{};
        if (PROL) Lc = cdesc[p];
        const long long csx = PROL ? (long long)Lc.ny * Lc.nz : 0;
        const int cr_lo = (y0 - 1) >> 1;  // logical first coarse row of the halo (may be -1)
        auto gof = [&](int q) { return g0 + (q - pl_lo); };
        Acc<T> part;
        bool bad = false;

        if (warp == kConsumerWarps) {
            // ---------------- producer
            if (lane == 0) {
                const int n = pm_produce<R>(pl_lo, pl_hi, g0, full, empty, sm, lay.slot_bytes, err,
                                            [&](int q, char *slot, uint64_t *bar) {
                    const long long pb = L.off + (long long)q * sx;
                    const long long lh = pb + (long long)(y0 - 1) * nz, lp = pb + (long long)y0 * nz;
                    const long long hA = pb + (long long)h0 * nz, hB = pb + (long long)h1 * nz, pE = lp + ncell;
                    auto stage = [&](const void *base, int esz, long long l0, long long a0, long long a1, int off) {
                        stage_range(bar, base, esz, l0, a0, a1, slot + off, L.off, L.off + L.n, slot, lay.slot_bytes);
                    };
                    if (F2) {
                        stage(b, es, lh, hA, hB, lay.oB);
                        stage(C.idg, es, lh, hA, hB, lay.oG);
                    } else {
                        stage(xin, es, lh, hA, hB, lay.oX);
                        stage(b, es, lp, lp, pE, lay.oB);
                        if (!FIRST) stage(d, es, lp, lp, pE, lay.oD);
                    }
                    stage(C.cx, ec, lp, lp, pE, lay.oCX);
                    stage(C.cy, ec, lh, hA, pE, lay.oCY);
                    stage(C.cz, ec, lp, lp, pE, lay.oCZ);
                    stage(C.leak, ec, lp, lp, pE, lay.oLK);
                    if (PROL) {
                        stage(dir, 1, lh, hA, hB, lay.oDIR);
                        const long long cb = Lc.off + (long long)(q >> 1) * csx;
                        const int c0 = max(cr_lo, 0), c1r = min((y0 + rows) >> 1, Lc.ny - 1) + 1;
                        stage_range(bar, e, es, cb + (long long)cr_lo * Lc.nz, cb + (long long)c0 * Lc.nz,
                                    cb + (long long)c1r * Lc.nz, slot + lay.oE, Lc.off, Lc.off + Lc.n, slot,
                                    lay.slot_bytes);
                    }
                });
                issued += n;
                bad = n != pl_hi - pl_lo + 1;
            }
            __syncwarp();
        } else {
            // ---------------- consumers
            // this thread's cells of the slab (the same in every plane) and their y/z neighbours
            unsigned cfl[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                const int tc = t + k * kPlaneThreads;
                unsigned f = 0;
                if (tc < ncell) {
                    const int ty = div_nz(L, tc), z = tc - ty * nz, y = y0 + ty;
                    f = CF_VALID | (z + 1 < nz ? CF_ZP : 0u) | (z > 0 ? CF_ZM : 0u) | (y + 1 < ny ? CF_YP : 0u) |
                        (y > 0 ? CF_YM : 0u);
                }
                cfl[k] = f;
            }
            // PM_PROLONG: this thread's first kHaloSlots elements k = t + m kPlaneThreads of a staged
            // plane and its halo rows, and the offset of each one's aggregate in the staged coarse
            // plane (-1: past the halo, or a row outside the grid); the same in every plane
            constexpr int kHaloSlots = PROL ? CPT + 2 : 1;
            int eoff[kHaloSlots];
#pragma unroll
            for (int m = 0; m < kHaloSlots; m++) {
                const int k = t + m * kPlaneThreads;
                eoff[m] = -1;
                if (PROL && k < (rows + 2) * nz) {
                    const int rr = div_nz(L, k);
                    const int row = y0 - 1 + rr;
                    if (row >= 0 && row < ny) eoff[m] = ((row >> 1) - cr_lo) * Lc.nz + ((k - rr * nz) >> 1);
                }
            }
            int waited = pl_lo - 1, released = pl_lo;
            for (int x = xa; x < xe && !bad; x++) {
                const int need = min(x + 1, pl_hi);
                const int first_new = waited + 1;
                while (waited < need) {
                    const int q = waited + 1, g = gof(q);
                    if (!mbar_wait(&full[g % R], (uint32_t)((g / R) & 1), err)) {
                        bad = true;
                        break;
                    }
                    waited = q;
                    if (F2) {
                        // the first step's iterate x1 = invtheta b g of every staged cell, once per
                        // plane, in place of b (the cell's own b is recovered as x1 / (invtheta g))
                        char *sl = slot_of(g);
                        const long long lh = L.off + (long long)q * sx + (long long)(y0 - 1) * nz;
                        T *Bq_ = (T *)(sl + lay.oB) + stage_delta(lh, es);
                        const T *Gq_ = (const T *)(sl + lay.oG) + stage_delta(lh, es);
                        const int nh = (rows + 2) * nz;
                        for (int k = t; k < nh; k += kPlaneThreads) Bq_[k] = invtheta * Bq_[k] * Gq_[k];
                        mbar_arrive(&ready[g % R]);
                    }
                    if (PROL) {
                        // prolongation on arrival: this thread's share of the slab and its halo rows
                        char *sl = slot_of(g);
                        const long long pb = L.off + (long long)q * sx;
                        const long long lh = pb + (long long)(y0 - 1) * nz;
                        T *X = (T *)(sl + lay.oX) + stage_delta(lh, es);
                        const uint8_t *DR = (const uint8_t *)(sl + lay.oDIR) + stage_delta(lh, 1);
                        const long long cb = Lc.off + (long long)(q >> 1) * csx;
                        const T *E = (const T *)(sl + lay.oE) + stage_delta(cb + (long long)cr_lo * Lc.nz, es);
                        const int nh = (rows + 2) * nz;
#pragma unroll
                        for (int m = 0; m < kHaloSlots; m++)  // offsets worked out once per item
                            if (eoff[m] >= 0 && !DR[t + m * kPlaneThreads]) X[t + m * kPlaneThreads] += scale * E[eoff[m]];
                        for (int k = t + kHaloSlots * kPlaneThreads; k < nh; k += kPlaneThreads) {
                            const int rr = div_nz(L, k);
                            const int row = y0 - 1 + rr;
                            if (row < 0 || row >= ny || DR[k]) continue;
                            const int zz = k - rr * nz;
                            X[k] += scale * E[((row >> 1) - cr_lo) * Lc.nz + (zz >> 1)];
                        }
                        mbar_arrive(&ready[g % R]);
                    }
                }
                if (bad) break;
                if (PROL || F2) {
                    for (int q = first_new; q <= waited; q++) {
                        const int g = gof(q);
                        if (!mbar_wait(&ready[g % R], (uint32_t)((g / R) & 1), err)) {
                            bad = true;
                            break;
                        }
                    }
                    if (bad) break;
                }
                {
                    // per-plane addresses, shared by this thread's cells
                    const long long pb = L.off + (long long)x * sx;
                    const long long lh = pb + (long long)(y0 - 1) * nz, lp = pb + (long long)y0 * nz;
                    const int dh = stage_delta(lh, es), dp = stage_delta(lp, es);
                    char *sc = slot_of(gof(x));
                    const bool xp = x + 1 < nx, xm = x > 0;
                    char *sn = xp ? slot_of(gof(x + 1)) : sc;
                    char *sq = xm ? slot_of(gof(x - 1)) : sc;
                    const int dn_ = xp ? stage_delta(lh + sx, es) : dh;
                    const int dq = xm ? stage_delta(lh - sx, es) : dh;
                    const int ch = stage_delta(lh, ec), cp = stage_delta(lp, ec);
                    const int cqp = xm ? stage_delta(lp - sx, ec) : cp;
                    const CT *CX = (const CT *)(sc + lay.oCX) + cp;
                    const CT *CXq = (const CT *)(sq + lay.oCX) + cqp;
                    const CT *CY = (const CT *)(sc + lay.oCY) + ch;  // logical row 0 = y0 - 1
                    const CT *CZ = (const CT *)(sc + lay.oCZ) + cp;
                    const CT *LK = (const CT *)(sc + lay.oLK) + cp;
#pragma unroll
                    for (int k = 0; k < CPT; k++) {
                        const unsigned f = cfl[k];
                        if (!(f & CF_VALID)) continue;
                        const int tc = t + k * kPlaneThreads;
                        const long long i = lp + tc;
                        const int c = nz + tc;  // own cell in halo coordinates
                        if (F2) {
                            // x1 = invtheta b g, staged in place of b for every cell of the plane
                            // and its halo; the cell's own b is x1 / (invtheta g) (g > 0)
                            const T *X1 = (const T *)(sc + lay.oB) + dh;
                            const T *G = (const T *)(sc + lay.oG) + dh;
                            const T gi = G[c];
                            const T x1 = X1[c];
                            const T bi = pm_div(x1, invtheta * gi);
                            T a = cf(LK[tc]) * x1;
                            if (f & CF_ZP) a += cf(CZ[tc]) * (x1 - X1[c + 1]);
                            if (f & CF_ZM) a += cf(CZ[tc - 1]) * (x1 - X1[c - 1]);
                            if (f & CF_YP) a += cf(CY[c]) * (x1 - X1[c + nz]);
                            if (f & CF_YM) a += cf(CY[tc]) * (x1 - X1[c - nz]);
                            if (xp) a += cf(CX[tc]) * (x1 - ((const T *)(sn + lay.oB) + dn_)[c]);
                            if (xm) a += cf(CXq[tc]) * (x1 - ((const T *)(sq + lay.oB) + dq)[c]);
                            const T dn = c1 * x1 + c2 * (bi - a) * gi;
                            if (!NOD) d[i] = dn;
                            xout[i] = x1 + dn;
                        } else {
                            const T *X = (const T *)(sc + lay.oX) + dh;
                            const T xi = X[c];
                            const T lk = cf(LK[tc]);
                            T a = lk * xi, dg = lk;
                            if (f & CF_ZP) { T w_ = cf(CZ[tc]);     a += w_ * (xi - X[c + 1]);  dg += w_; }
                            if (f & CF_ZM) { T w_ = cf(CZ[tc - 1]); a += w_ * (xi - X[c - 1]);  dg += w_; }
                            if (f & CF_YP) { T w_ = cf(CY[c]);      a += w_ * (xi - X[c + nz]); dg += w_; }
                            if (f & CF_YM) { T w_ = cf(CY[tc]);     a += w_ * (xi - X[c - nz]); dg += w_; }
                            if (xp) {
                                const T *Xn = (const T *)(sn + lay.oX) + dn_;
                                T w_ = cf(CX[tc]);
                                a += w_ * (xi - Xn[c]);
                                dg += w_;
                            }
                            if (xm) {
                                const T *Xq = (const T *)(sq + lay.oX) + dq;
                                T w_ = cf(CXq[tc]);
                                a += w_ * (xi - Xq[c]);
                                dg += w_;
                            }
                            const T bi = ((const T *)(sc + lay.oB) + dp)[tc];
                            T r;
                            if constexpr (sizeof(T) == 8) r = (bi - a) * C.idg[i];
                            else r = __fdividef(bi - a, dg);
                            T dn;
                            if (FIRST) dn = c2 * r;
                            else dn = c1 * ((const T *)(sc + lay.oD) + dp)[tc] + c2 * r;
                            const T xo = xi + dn;
                            if (!NOD) d[i] = dn;
                            xout[i] = xo;
                            if (RZ) part = part + Acc<T>::prod(bi, xo);
                        }
                    }
                }
                // this warp is done with plane x-1
                __syncwarp();
                if (lane == 0 && x - 1 >= released) mbar_arrive(&empty[gof(x - 1) % R]);
                released = max(released, x);
            }
            // the item's remaining planes go back to the producer
            if (!bad) {
                __syncwarp();
                for (int q = released; q <= waited; q++)
                    if (lane == 0) mbar_arrive(&empty[gof(q) % R]);
            }
        }
        g0 += pl_hi - pl_lo + 1;
        if (RZ) {
            double2 tot;
            if (reduce_last_slot<T>(part, rs, pinfo[p], p, w, tot) && threadIdx.x == 0) {
                CgState &s = st[p];
                s.rz_old = s.rz;
                s.rz = tot.x;
                s.beta = (s.iters == 0 || s.rz_old == 0.0) ? 0.0 : s.rz / s.rz_old * s.cont;
                s.cont = 1.0;
            }
        }
        if (__syncthreads_or(bad)) break;  // every thread leaves together after an expired wait
    }
    if (warp == kConsumerWarps && lane == 0) pm_drain<R>(issued, full, err);
}

__device__ __forceinline__ void finish_pq(CgState &s, double pq, int *active_count) {
    s.pq = pq;
    if (!isfinite(s.pq)) { s.alpha = 0.0; s.status = DPF_NAN; deactivate(s, active_count); }
    else if (!(s.pq > 0.0)) { s.alpha = 0.0; deactivate(s, active_count); }
    else s.alpha = s.rz / s.pq;
}

// Restriction on the plane ring: residuals b - A x of each fine plane of the slab go to a
// shared buffer (two planes), and after every odd plane (or the grid's last) the coarse
// cells of the slab sum their children in the order of cell_restrict (x, then y, then z),
// so the coarse right-hand side is bitwise that of k_restrict. Slabs start on even rows and
// items on even planes (and end on one, or on the grid's last plane). Streams per plane: x with
// halo rows, b, cx, cy (+ row below), cz, leak. A block marches through its items like k_pm_cheb.
template <typename T, int CPT>
__global__ void __launch_bounds__(kPlaneThreads + 32) k_pm_restrict(
    const LevelDesc *__restrict__ desc, const LevelDesc *__restrict__ cdesc, PlaneWork work,
    const CgState *st, Coeffs<T> C, const T *__restrict__ b, const T *__restrict__ xin, T *__restrict__ bc,
    PlaneLayout lay, int *err) {
    pdl_enter();
    constexpr int R = kPlaneStages;
    constexpr int es = (int)sizeof(T);
    using CT = coef_t<T>;
    constexpr int ec = (int)sizeof(CT);  // coefficient streams
    constexpr int kConsumerWarps = kPlaneThreads / 32;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[R], empty[R];
    __shared__ T res[2][CPT * kPlaneThreads];

    const int t = threadIdx.x;
    const int warp = t >> 5, lane = t & 31;
    auto slot_of = [&](int g) { return (char *)sm + ((unsigned)g % (unsigned)R) * lay.slot_bytes; };
    if (t == 0) {
        for (int s = 0; s < R; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
        fence_mbarrier_init();
    }
    __syncthreads();
    int g0 = 0, issued = 0;
    for (int w = work.first[blockIdx.x]; w < work.first[blockIdx.x + 1]; w++) {
        const int4 it = work.items[w];
        const int p = it.x, y0 = it.y, xa = it.z, xe = it.w;
        if (st && !st[p].active) continue;  // uniform over the block
        const LevelDesc L = desc[p];
        const LevelDesc Lc = cdesc[p];
        const int nz = L.nz, ny = L.ny, nx = L.nx;
        const long long sx = (long long)ny * nz;
        const int Ty = plane_rows(ny, nz, CPT * kPlaneThreads);
        const int rows = min(Ty, ny - y0);
        const int ncell = rows * nz;
        const int pl_lo = max(xa - 1, 0), pl_hi = min(xe, nx - 1);
        const int h0 = max(y0 - 1, 0), h1 = min(y0 + rows + 1, ny);
        auto gof = [&](int q) { return g0 + (q - pl_lo); };
        // coarse cells of the slab: rows y0/2 .. (y0+rows-1)/2, all coarse z
        const int cy0 = y0 >> 1, crows = ((y0 + rows - 1) >> 1) - cy0 + 1;
        const int ncc = crows * Lc.nz;
        bool bad = false;

        if (warp == kConsumerWarps) {
            if (lane == 0) {
                const int n = pm_produce<R>(pl_lo, pl_hi, g0, full, empty, sm, lay.slot_bytes, err,
                                            [&](int q, char *slot, uint64_t *bar) {
                    const long long pb = L.off + (long long)q * sx;
                    const long long lh = pb + (long long)(y0 - 1) * nz, lp = pb + (long long)y0 * nz;
                    const long long hA = pb + (long long)h0 * nz, hB = pb + (long long)h1 * nz, pE = lp + ncell;
                    auto stage = [&](const void *base, int esz, long long l0, long long a0, long long a1, int off) {
                        stage_range(bar, base, esz, l0, a0, a1, slot + off, L.off, L.off + L.n, slot, lay.slot_bytes);
                    };
                    stage(xin, es, lh, hA, hB, lay.oX);
                    stage(b, es, lp, lp, pE, lay.oB);
                    stage(C.cx, ec, lp, lp, pE, lay.oCX);
                    stage(C.cy, ec, lh, hA, pE, lay.oCY);
                    stage(C.cz, ec, lp, lp, pE, lay.oCZ);
                    stage(C.leak, ec, lp, lp, pE, lay.oLK);
                });
                issued += n;
                bad = n != pl_hi - pl_lo + 1;
            }
            __syncwarp();
        } else {
            // ---------------- consumers
            unsigned cfl[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                const int tc = t + k * kPlaneThreads;
                unsigned f = 0;
                if (tc < ncell) {
                    const int ty = div_nz(L, tc), z = tc - ty * nz, y = y0 + ty;
                    f = CF_VALID | (z + 1 < nz ? CF_ZP : 0u) | (z > 0 ? CF_ZM : 0u) | (y + 1 < ny ? CF_YP : 0u) |
                        (y > 0 ? CF_YM : 0u);
                }
                cfl[k] = f;
            }
            int waited = pl_lo - 1, released = pl_lo;
            for (int x = xa; x < xe; x++) {
                const int need = min(x + 1, pl_hi);
                while (!bad && waited < need) {
                    const int g = gof(waited + 1);
                    if (!mbar_wait(&full[g % R], (uint32_t)((g / R) & 1), err)) bad = true;
                    else waited++;
                }
                if (!bad) {
                    const long long pb = L.off + (long long)x * sx;
                    const long long lh = pb + (long long)(y0 - 1) * nz, lp = pb + (long long)y0 * nz;
                    const int dh = stage_delta(lh, es), dp = stage_delta(lp, es);
                    char *sc = slot_of(gof(x));
                    const bool xp = x + 1 < nx, xm = x > 0;
                    char *sn = xp ? slot_of(gof(x + 1)) : sc;
                    char *sq = xm ? slot_of(gof(x - 1)) : sc;
                    const int dn_ = xp ? stage_delta(lh + sx, es) : dh;
                    const int dq = xm ? stage_delta(lh - sx, es) : dh;
                    const T *X = (const T *)(sc + lay.oX) + dh;
                    const T *B = (const T *)(sc + lay.oB) + dp;
                    const int ch = stage_delta(lh, ec), cp = stage_delta(lp, ec);
                    const int cqp = xm ? stage_delta(lp - sx, ec) : cp;
                    const CT *CX = (const CT *)(sc + lay.oCX) + cp;
                    const CT *CXq = (const CT *)(sq + lay.oCX) + cqp;
                    const CT *CY = (const CT *)(sc + lay.oCY) + ch;
                    const CT *CZ = (const CT *)(sc + lay.oCZ) + cp;
                    const CT *LK = (const CT *)(sc + lay.oLK) + cp;
                    const T *Xn = (const T *)(sn + lay.oX) + dn_;
                    const T *Xq = (const T *)(sq + lay.oX) + dq;
                    T *rsd = res[x & 1];
#pragma unroll
                    for (int k = 0; k < CPT; k++) {
                        const unsigned f = cfl[k];
                        if (!(f & CF_VALID)) continue;
                        const int tc = t + k * kPlaneThreads;
                        const int c = nz + tc;
                        const T xi = X[c];
                        T a = cf(LK[tc]) * xi;
                        if (f & CF_ZP) a += cf(CZ[tc]) * (xi - X[c + 1]);
                        if (f & CF_ZM) a += cf(CZ[tc - 1]) * (xi - X[c - 1]);
                        if (f & CF_YP) a += cf(CY[c]) * (xi - X[c + nz]);
                        if (f & CF_YM) a += cf(CY[tc]) * (xi - X[c - nz]);
                        if (xp) a += cf(CX[tc]) * (xi - Xn[c]);
                        if (xm) a += cf(CXq[tc]) * (xi - Xq[c]);
                        rsd[tc] = B[tc] - a;
                    }
                }
                // plane x-1 is no longer needed by this warp
                __syncwarp();
                if (!bad && lane == 0 && x - 1 >= released) mbar_arrive(&empty[gof(x - 1) % R]);
                released = max(released, x);
                const bool pair_done = (x & 1) || x + 1 == nx;
                if (!pair_done) continue;
                if (consumer_sync_or(bad, kPlaneThreads)) {  // residuals of the pair are in res[]
                    bad = true;
                    break;
                }
                const int X0 = x & ~1;
                const int cx = X0 >> 1;
                const bool two = X0 + 1 < nx;
                const long long cb = Lc.off + (long long)cx * Lc.ny * Lc.nz + (long long)cy0 * Lc.nz;
                for (int tcc = t; tcc < ncc; tcc += kPlaneThreads) {
                    const int cr = div_nz(Lc, tcc), czz = tcc - cr * Lc.nz;
                    const int fy0 = 2 * (cy0 + cr) - y0, fz0 = 2 * czz;
                    const bool y2 = 2 * (cy0 + cr) + 1 < ny, z2 = fz0 + 1 < nz;
                    T acc = 0;
                    for (int ix = 0; ix < (two ? 2 : 1); ix++) {
                        const T *r = res[(X0 + ix) & 1];
                        acc += r[fy0 * nz + fz0];
                        if (z2) acc += r[fy0 * nz + fz0 + 1];
                        if (y2) {
                            acc += r[(fy0 + 1) * nz + fz0];
                            if (z2) acc += r[(fy0 + 1) * nz + fz0 + 1];
                        }
                    }
                    bc[cb + tcc] = acc;
                }
                if (consumer_sync_or(bad, kPlaneThreads)) {  // res[] may be overwritten
                    bad = true;
                    break;
                }
            }
            // the item's remaining planes go back to the producer
            if (!bad) {
                __syncwarp();
                for (int q = released; q <= waited; q++)
                    if (lane == 0) mbar_arrive(&empty[gof(q) % R]);
            }
        }
        g0 += pl_hi - pl_lo + 1;
        if (__syncthreads_or(bad)) break;  // every thread leaves together after an expired wait
    }
    if (warp == kConsumerWarps && lane == 0) pm_drain<R>(issued, full, err);
}

// Double-float CG product q = A p (flux form, double-float coefficients) and the problem's p . q
// (leading floats), marching along x through the plane work items with every face flux computed
// once. A cell computes the fluxes c_f (p_i - p_j) through its z+, y+ and x+ faces; the cell
// above takes the z+ and y+ fluxes of the cell below it from shared memory (two buffers by plane
// parity, so one block barrier per plane), and the x+ flux is carried in a register to the next
// plane, where it is that cell's x- flux. A slab's first row computes its y- flux itself (the cell
// below is in the slab underneath), and so does an item's first plane its x- flux.
// The double-float difference and product are odd functions of their arguments (round to nearest
// is symmetric and the two-sum error is exact), so the negated flux of a neighbour equals the
// term the cell would compute itself, up to the sign of a zero: q is the six-face product of
// k_df_spmv_pq term for term, with the terms summed in its order (z+, z-, y+, y-, x+, x-). The
// leading-float p . q is summed per thread along x, so its rounding differs from k_df_spmv_pq's.
// Global reads per cell: p of the next plane (once from HBM) and of the z+ and y+ neighbours
// (loaded by those cells' threads a plane earlier, mostly cache hits), and the four coefficients.
// Every value a plane needs is loaded into registers one plane ahead, so the loads of plane x + 1
// are in flight while plane x is computed.
#ifndef DPF_DF_FLUX_MINB
#define DPF_DF_FLUX_MINB 4
#endif
struct FluxPlane {  // one cell's operands of one plane
    float2 pz, py, pym, pn;  // p at z+1, y+1, y-1 (slab's first row only), x+1
    float2 cz, cy, cym, cx, lk;
};
template <int CPT>
__global__ void __launch_bounds__(kPlaneThreads, (DPF_DF_FLUX_MINB / CPT > 0 ? DPF_DF_FLUX_MINB / CPT : 1))
    k_pm_df_flux(const LevelDesc *__restrict__ desc, PlaneWork work, CgState *st, int *active_count,
                 ReduceScratch rs, const int2 *__restrict__ pinfo, CoeffsDF C, const float2 *__restrict__ pv,
                 float2 *__restrict__ qv) {
    pdl_enter();
    constexpr unsigned CF_YIN = 32u;  // the y- neighbour is inside the slab
    // z fluxes with one leading zero entry (the z- flux of the slab's first cell, z = 0), y fluxes
    __shared__ float2 fz_s[2][CPT * kPlaneThreads + 1], fy_s[2][CPT * kPlaneThreads];
    const int t = threadIdx.x;
    const float2 zero = make_float2(0.f, 0.f);
    if (t < 2) fz_s[t][0] = zero;  // written before the first block barrier of the first item
    for (int w = work.first[blockIdx.x]; w < work.first[blockIdx.x + 1]; w++) {
        const int4 it = work.items[w];
        const int p = it.x, y0 = it.y, xa = it.z, xe = it.w;
        if (!st[p].active) continue;  // uniform over the block
        const LevelDesc L = desc[p];
        const int nz = L.nz, ny = L.ny, nx = L.nx;
        const long long sx = (long long)ny * nz;
        const int Ty = plane_rows(ny, nz, CPT * kPlaneThreads);
        const int ncell = min(Ty, ny - y0) * nz;
        unsigned cfl[CPT];
        long long ic[CPT];
        float2 pi[CPT], fxm[CPT];
        FluxPlane cur[CPT];
        // the operands of the plane at ic (x < nx, so the x+1 load is guarded by x + 1 < nx). The
        // z+ and y+ operands are read unconditionally: the assembly stores a zero coefficient for
        // a face that does not exist (the grid's last z or y) or that leads to a Dirichlet cell, so
        // such a flux is exactly zero and adding it leaves the (normalised) double-float sum as it
        // is; the neighbour index is clamped to the problem's last cell, so the p read there is a
        // finite value of the same array.
        const long long ilast = L.off + L.n - 1;
        auto fetch = [&](FluxPlane &o, unsigned f, long long i, int x) {
            o.pz = pv[min(i + 1, ilast)];
            o.py = pv[min(i + nz, ilast)];
            const bool ylo = (f & CF_YM) && !(f & CF_YIN);
            o.pym = ylo ? pv[i - nz] : zero;
            o.pn = x + 1 < nx ? pv[i + sx] : zero;
            o.cz = C.cz[i];
            o.cy = C.cy[i];
            o.cym = ylo ? C.cy[i - nz] : zero;
            o.cx = x + 1 < nx ? C.cx[i] : zero;
            o.lk = C.leak[i];
        };
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            const int tc = t + k * kPlaneThreads;
            unsigned f = 0;
            ic[k] = L.off + (long long)xa * sx + (long long)y0 * nz + tc;
            pi[k] = fxm[k] = zero;
            if (tc < ncell) {
                const int ty = div_nz(L, tc), z = tc - ty * nz, y = y0 + ty;
                f = CF_VALID | (z + 1 < nz ? CF_ZP : 0u) | (z > 0 ? CF_ZM : 0u) | (y + 1 < ny ? CF_YP : 0u) |
                    (y > 0 ? CF_YM : 0u) | (ty > 0 ? CF_YIN : 0u);
#if DPF_CHECKED
                // every neighbour the flags admit, on the item's first and last planes
                for (int e = 0; e < 2 && f; e++) {
                    const long long i = ic[k] + (e ? (long long)(xe - 1 - xa) * sx : 0);
                    const int x = e ? xe - 1 : xa;
                    if (!(DPF_INSIDE(CK_NEIGHBOUR, i, L.off, L.off + L.n) &&
                          DPF_INSIDE(CK_NEIGHBOUR, (f & CF_ZP) ? i + 1 : i, L.off, L.off + L.n) &&
                          DPF_INSIDE(CK_NEIGHBOUR, (f & CF_YP) ? i + nz : i, L.off, L.off + L.n) &&
                          DPF_INSIDE(CK_NEIGHBOUR, (f & CF_YM) ? i - nz : i, L.off, L.off + L.n) &&
                          DPF_INSIDE(CK_NEIGHBOUR, x + 1 < nx ? i + sx : i, L.off, L.off + L.n) &&
                          DPF_INSIDE(CK_NEIGHBOUR, x > 0 ? i - sx : i, L.off, L.off + L.n)))
                        f = 0;
                }
#endif
            }
            cfl[k] = f;
            if (f) {
                pi[k] = pv[ic[k]];
                fetch(cur[k], f, ic[k], xa);
                if (xa > 0) fxm[k] = df_mul(C.cx[ic[k] - sx], df_sub(pv[ic[k] - sx], pi[k]));
            }
        }
        Acc<float> part;
        for (int x = xa; x < xe; x++) {
            const bool xp = x + 1 < nx, xm = x > 0;
            float2 *fzb = fz_s[x & 1] + 1, *fyb = fy_s[x & 1];
            float2 fz[CPT], fy[CPT], fx[CPT];
            FluxPlane nxt[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                const unsigned f = cfl[k];
                const int tc = t + k * kPlaneThreads;
                fz[k] = fy[k] = fx[k] = zero;
                if (!f) continue;
                if (x + 1 < xe) fetch(nxt[k], f, ic[k] + sx, x + 1);
                const FluxPlane &o = cur[k];
                fz[k] = df_mul(o.cz, df_sub(pi[k], o.pz));  // zero where no z+ face
                fy[k] = df_mul(o.cy, df_sub(pi[k], o.py));  // zero where no y+ face
                if (xp) fx[k] = df_mul(o.cx, df_sub(pi[k], o.pn));
                fzb[tc] = fz[k];
                fyb[tc] = fy[k];
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                const unsigned f = cfl[k];
                const int tc = t + k * kPlaneThreads;
                if (!f) continue;
                const FluxPlane &o = cur[k];
                float2 a = df_mul(o.lk, pi[k]);
                a = df_add(a, fz[k]);
                a = df_sub(a, fzb[tc - 1]);  // zero at z = 0: the row below ends with a zero z+ flux
                a = df_add(a, fy[k]);
                if (f & CF_YM) a = (f & CF_YIN) ? df_sub(a, fyb[tc - nz]) : df_add(a, df_mul(o.cym, df_sub(pi[k], o.pym)));
                if (xp) a = df_add(a, fx[k]);
                if (xm) a = df_sub(a, fxm[k]);
                qv[ic[k]] = a;
                part = part + Acc<float>::prod(pi[k].x, a.x);
                fxm[k] = fx[k];
                pi[k] = o.pn;
                ic[k] += sx;
                cur[k] = nxt[k];
            }
        }
        // reduce_last_slot's block barriers also keep the next item's first flux writes
        // behind this item's last reads
        double2 tot;
        if (reduce_last_slot<float>(part, rs, pinfo[p], p, w, tot) && t == 0) finish_pq(st[p], tot.x, active_count);
    }
}

}  // namespace dpf
