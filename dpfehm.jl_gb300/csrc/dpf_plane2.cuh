// dpf_plane2.cuh -- plane-marching kernels that fuse two V-cycle passes of a level into one
// (temporal blocking): the post-smoothing (prolongation and two Chebyshev steps) and the
// pre-smoothing from a zero guess together with the restriction of its residual.
//
// Both march along x over the work runs of dpf_plane.cuh (same items, same slabs of whole rows)
// and stream their inputs through a ring of shared-memory stages with bulk asynchronous copies
// issued by a producer warp. The first of the two steps runs one plane ahead of the second and
// also on the slab's two halo rows, so the second step finds the first step's result at all six
// neighbours of a cell in shared memory (a ring of four planes): the intermediate iterate never
// goes through HBM. To feed the first step on the halo rows, the iterate (or b and the inverse
// diagonal) is staged with two halo rows on each side and the coefficients with one.
//
// Per cell the arithmetic is that of the separate passes (cell_cheb_first2, cell_cheb_step,
// cell_restrict in dpf_struct.cu; apply7's face order z+, z-, y+, y-, x+, x-), in the same order.
// Every wait is bounded (one second); an expired wait sets *err, and every consumer leaves at the
// next consumer barrier (which carries the flag); the producer drains its copies before the block
// ends.
#pragma once
#include "dpf_plane.cuh"

namespace dpf {

constexpr int kFusedThreads = 512;  // consumer threads per block (plus one producer warp)
constexpr int kFusedStages = 6;     // staged planes s-2 .. s+1 resident, two more in flight

// Byte offsets inside one staged plane and of the rings after the staged slots (host computed).
// Row origins: y0 - 2 for the regions with two halo rows (iterate, identity flags, b and the
// inverse diagonal of the pre-smoother, cy), y0 - 1 for those with one (b of the post-smoother,
// cx, cz, leak, and the ring of first-step results).
struct FusedLayout {
    int slot_bytes;
    int oX, oDIR, oE, oB, oG, oCX, oCY, oCZ, oLK;  // -1: not staged
    int oV, v_stride;                              // 4 planes of first-step results
    int oD, d_stride;                              // 2 planes of first-step directions (post-smoothing)
    int oR, r_stride;                              // 2 planes of residuals (restriction)
};

// consumer-only barrier 2 (barrier 1 is used by the other plane kernels) with the OR of pred
__device__ __forceinline__ bool fused_sync_or(bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.or.pred q, 2, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(kFusedThreads)
        : "memory");
    return r != 0;
}

// Post-smoothing of a level in one pass (degree 2):
//   x3 = x + s e[aggregate]            at free cells, on arrival of each plane (prolongation)
//   d1 = invtheta D^-1 (b - A x3),  x4 = x3 + d1                (first step, one plane ahead)
//   z  = x4 + c1 d1 + c2 D^-1 (b - A x4)                        (second step) -> xout
// With RZ (the finest level) it also reduces b . z per problem and finalises beta.
template <typename T, bool RZ>
__global__ void __launch_bounds__(kFusedThreads + 32) k_pm_post2(
    const LevelDesc *__restrict__ desc, const LevelDesc *__restrict__ cdesc, PlaneWork work, int cells,
    CgState *st, Coeffs<T> C, const T *__restrict__ b, const T *__restrict__ xin, T *__restrict__ xout,
    const uint8_t *__restrict__ dir, const T *__restrict__ e, T c2a, T c1b, T c2b, T scale, FusedLayout lay,
    ReduceScratch rs, const int2 *__restrict__ pinfo, int *err) {
    pdl_enter();
    constexpr int R = kFusedStages;
    constexpr int es = (int)sizeof(T);
    using CT = coef_t<T>;
    constexpr int ec = (int)sizeof(CT);
    constexpr int kConsumerWarps = kFusedThreads / 32;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[R], empty[R];

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
        const int nz = L.nz, ny = L.ny, nx = L.nx, cnz = Lc.nz;
        const long long sx = (long long)ny * nz, csx = (long long)Lc.ny * cnz;
        const int Ty = plane_rows(ny, nz, cells);
        const int rows = min(Ty, ny - y0);
        const int pl_lo = max(xa - 2, 0), pl_hi = min(xe + 1, nx - 1);  // staged planes
        const int s_lo = max(xa - 1, 0), s_hi = min(xe, nx - 1);        // first-step planes
        const int r2a = max(y0 - 2, 0), r2b = min(y0 + rows + 2, ny);   // rows with two halo rows
        const int r1a = max(y0 - 1, 0), r1b = min(y0 + rows + 1, ny);   // rows with one
        const int cr_lo = (y0 - 2) >> 1;                                // logical first coarse row (>= -1)
        const int c0 = max(cr_lo, 0), c1r = min((y0 + rows + 1) >> 1, Lc.ny - 1) + 1;
        auto gof = [&](int q) { return g0 + (q - pl_lo); };
        Acc<T> part;
        bool bad = false;

        if (warp == kConsumerWarps) {
            // ---------------- producer
            if (lane == 0) {
                const int n = pm_produce<R>(pl_lo, pl_hi, g0, full, empty, sm, lay.slot_bytes, err,
                                            [&](int q, char *slot, uint64_t *bar) {
                    const long long pb = L.off + (long long)q * sx;
                    const long long l2 = pb + (long long)(y0 - 2) * nz, l1 = pb + (long long)(y0 - 1) * nz;
                    auto stage = [&](const void *base, int esz, long long l0, int ra, int rb, int off) {
                        stage_range(bar, base, esz, l0, pb + (long long)ra * nz, pb + (long long)rb * nz, slot + off,
                                    L.off, L.off + L.n, slot, lay.slot_bytes);
                    };
                    stage(xin, es, l2, r2a, r2b, lay.oX);
                    stage(dir, 1, l2, r2a, r2b, lay.oDIR);
                    stage(b, es, l1, r1a, r1b, lay.oB);
                    stage(C.cx, ec, l1, r1a, r1b, lay.oCX);
                    stage(C.cy, ec, l2, r2a, r1b, lay.oCY);
                    stage(C.cz, ec, l1, r1a, r1b, lay.oCZ);
                    stage(C.leak, ec, l1, r1a, r1b, lay.oLK);
                    const long long cb = Lc.off + (long long)(q >> 1) * csx;
                    stage_range(bar, e, es, cb + (long long)cr_lo * cnz, cb + (long long)c0 * cnz,
                                cb + (long long)c1r * cnz, slot + lay.oE, Lc.off, Lc.off + Lc.n, slot,
                                lay.slot_bytes);
                });
                issued += n;
                bad = n != pl_hi - pl_lo + 1;
            }
            __syncwarp();
        } else {
            // ---------------- consumers
            const int n2 = (rows + 4) * nz, n1 = (rows + 2) * nz, ns = rows * nz;
            int waited = pl_lo - 1, released = pl_lo;
            for (int s = s_lo; s <= s_hi + 1 && !bad; s++) {
                // planes up to s + 1 arrive; each thread corrects its share of them (prolongation)
                const int need = min(s + 1, pl_hi);
                while (waited < need) {
                    const int q = waited + 1, g = gof(q);
                    if (!mbar_wait(&full[g % R], (uint32_t)((g / R) & 1), err)) {
                        bad = true;
                        break;
                    }
                    waited = q;
                    char *sl = slot_of(g);
                    const long long pb = L.off + (long long)q * sx;
                    T *X = (T *)(sl + lay.oX) + stage_delta(pb + (long long)(y0 - 2) * nz, es);
                    const uint8_t *DR = (const uint8_t *)(sl + lay.oDIR) + stage_delta(pb + (long long)(y0 - 2) * nz, 1);
                    const long long cb = Lc.off + (long long)(q >> 1) * csx;
                    const T *E = (const T *)(sl + lay.oE) + stage_delta(cb + (long long)cr_lo * cnz, es);
                    for (int k = t; k < n2; k += kFusedThreads) {
                        const int rr = div_nz(L, k);
                        const int row = y0 - 2 + rr;
                        if (row < 0 || row >= ny || DR[k]) continue;
                        const int zz = k - rr * nz;
                        X[k] += scale * E[((row >> 1) - cr_lo) * cnz + (zz >> 1)];
                    }
                }
                if (fused_sync_or(bad)) {  // corrections of the new planes visible
                    bad = true;
                    break;
                }
                if (s <= s_hi) {
                    // first step on plane s, slab rows and one halo row each side -> V ring, D ring
                    const long long pb = L.off + (long long)s * sx;
                    const long long l2 = pb + (long long)(y0 - 2) * nz, l1 = pb + (long long)(y0 - 1) * nz;
                    char *sc = slot_of(gof(s));
                    const bool xp = s + 1 < nx, xm = s > 0;
                    char *sn = xp ? slot_of(gof(s + 1)) : sc;
                    char *sq = xm ? slot_of(gof(s - 1)) : sc;
                    const T *X = (const T *)(sc + lay.oX) + stage_delta(l2, es);
                    const T *Xn = (const T *)(sn + lay.oX) + (xp ? stage_delta(l2 + sx, es) : 0);
                    const T *Xq = (const T *)(sq + lay.oX) + (xm ? stage_delta(l2 - sx, es) : 0);
                    const T *B = (const T *)(sc + lay.oB) + stage_delta(l1, es);
                    const CT *CX = (const CT *)(sc + lay.oCX) + stage_delta(l1, ec);
                    const CT *CXq = (const CT *)(sq + lay.oCX) + (xm ? stage_delta(l1 - sx, ec) : 0);
                    const CT *CY = (const CT *)(sc + lay.oCY) + stage_delta(l2, ec);
                    const CT *CZ = (const CT *)(sc + lay.oCZ) + stage_delta(l1, ec);
                    const CT *LK = (const CT *)(sc + lay.oLK) + stage_delta(l1, ec);
                    T *V = (T *)(sm + lay.oV + ((s - s_lo) & 3) * lay.v_stride);
                    T *D = (T *)(sm + lay.oD + ((s - s_lo) & 1) * lay.d_stride);
                    for (int k = t; k < n1; k += kFusedThreads) {
                        const int rr = div_nz(L, k);
                        const int y = y0 - 1 + rr, z = k - rr * nz;
                        if (y < 0 || y >= ny) continue;
                        const int kx = k + nz;  // the cell in the two-halo-row regions
                        const T xi = X[kx];
                        const T lk = cf(LK[k]);
                        T a = lk * xi, dg = lk;
                        if (z + 1 < nz) { T w_ = cf(CZ[k]);     a += w_ * (xi - X[kx + 1]);  dg += w_; }
                        if (z > 0)      { T w_ = cf(CZ[k - 1]); a += w_ * (xi - X[kx - 1]);  dg += w_; }
                        if (y + 1 < ny) { T w_ = cf(CY[kx]);    a += w_ * (xi - X[kx + nz]); dg += w_; }
                        if (y > 0)      { T w_ = cf(CY[k]);     a += w_ * (xi - X[kx - nz]); dg += w_; }
                        if (xp)         { T w_ = cf(CX[k]);     a += w_ * (xi - Xn[kx]);     dg += w_; }
                        if (xm)         { T w_ = cf(CXq[k]);    a += w_ * (xi - Xq[kx]);     dg += w_; }
                        const T r = __fdividef(B[k] - a, dg);
                        const T d1 = c2a * r;
                        V[k] = xi + d1;
                        if (rr >= 1 && rr <= rows) D[k - nz] = d1;
                    }
                }
                if (fused_sync_or(bad)) {  // first-step results of plane s visible
                    bad = true;
                    break;
                }
                const int tp = s - 1;
                if (tp >= xa && tp <= xe - 1) {
                    // second step on plane tp (slab rows) from the V ring -> xout
                    const long long pb = L.off + (long long)tp * sx;
                    const long long l2 = pb + (long long)(y0 - 2) * nz, l1 = pb + (long long)(y0 - 1) * nz;
                    char *sc = slot_of(gof(tp));
                    const bool xp = tp + 1 < nx, xm = tp > 0;
                    char *sq = xm ? slot_of(gof(tp - 1)) : sc;
                    const T *Vc = (const T *)(sm + lay.oV + ((tp - s_lo) & 3) * lay.v_stride);
                    const T *Vn = xp ? (const T *)(sm + lay.oV + ((tp + 1 - s_lo) & 3) * lay.v_stride) : Vc;
                    const T *Vq = xm ? (const T *)(sm + lay.oV + ((tp - 1 - s_lo) & 3) * lay.v_stride) : Vc;
                    const T *D = (const T *)(sm + lay.oD + ((tp - s_lo) & 1) * lay.d_stride);
                    const T *B = (const T *)(sc + lay.oB) + stage_delta(l1, es);
                    const CT *CX = (const CT *)(sc + lay.oCX) + stage_delta(l1, ec);
                    const CT *CXq = (const CT *)(sq + lay.oCX) + (xm ? stage_delta(l1 - sx, ec) : 0);
                    const CT *CY = (const CT *)(sc + lay.oCY) + stage_delta(l2, ec);
                    const CT *CZ = (const CT *)(sc + lay.oCZ) + stage_delta(l1, ec);
                    const CT *LK = (const CT *)(sc + lay.oLK) + stage_delta(l1, ec);
                    const long long lp = pb + (long long)y0 * nz;
                    for (int kk = t; kk < ns; kk += kFusedThreads) {
                        const int rr = div_nz(L, kk);
                        const int y = y0 + rr, z = kk - rr * nz;
                        const int k = kk + nz;  // halo1 coordinates
                        const T xi = Vc[k];
                        const T lk = cf(LK[k]);
                        T a = lk * xi, dg = lk;
                        if (z + 1 < nz) { T w_ = cf(CZ[k]);      a += w_ * (xi - Vc[k + 1]);  dg += w_; }
                        if (z > 0)      { T w_ = cf(CZ[k - 1]);  a += w_ * (xi - Vc[k - 1]);  dg += w_; }
                        if (y + 1 < ny) { T w_ = cf(CY[k + nz]); a += w_ * (xi - Vc[k + nz]); dg += w_; }
                        if (y > 0)      { T w_ = cf(CY[k]);      a += w_ * (xi - Vc[k - nz]); dg += w_; }
                        if (xp)         { T w_ = cf(CX[k]);      a += w_ * (xi - Vn[k]);      dg += w_; }
                        if (xm)         { T w_ = cf(CXq[k]);     a += w_ * (xi - Vq[k]);      dg += w_; }
                        const T bi = B[k];
                        const T r = __fdividef(bi - a, dg);
                        const T zo = xi + (c1b * D[kk] + c2b * r);
                        xout[lp + kk] = zo;
                        if (RZ) part = part + Acc<T>::prod(bi, zo);
                    }
                }
                // planes below s - 1 are no longer read
                __syncwarp();
                for (int q = released; q <= s - 2 && q <= waited; q++)
                    if (lane == 0) mbar_arrive(&empty[gof(q) % R]);
                released = max(released, min(s - 1, waited + 1));
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

// Pre-smoothing of a level from a zero guess (degree 2) and the restriction of its residual in
// one pass:
//   x1 = invtheta D^-1 b (pointwise, formed at every neighbour from the staged b and inverse
//   diagonal), x2 = x1 + c1 x1 + c2 D^-1 (b - A x1)   (first step, one plane ahead) -> V ring, xout
//   bc[I] = sum over the children i of I of (b - A x2)_i  (second step, the order of cell_restrict)
template <typename T>
__global__ void __launch_bounds__(kFusedThreads + 32) k_pm_pre2r(
    const LevelDesc *__restrict__ desc, const LevelDesc *__restrict__ cdesc, PlaneWork work, int cells,
    const CgState *st, Coeffs<T> C, const T *__restrict__ b, T *__restrict__ xout, T *__restrict__ bc, T c1, T c2,
    T invtheta, FusedLayout lay, int *err) {
    pdl_enter();
    constexpr int R = kFusedStages;
    constexpr int es = (int)sizeof(T);
    using CT = coef_t<T>;
    constexpr int ec = (int)sizeof(CT);
    constexpr int kConsumerWarps = kFusedThreads / 32;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[R], empty[R];

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
        const int Ty = plane_rows(ny, nz, cells);
        const int rows = min(Ty, ny - y0);
        const int pl_lo = max(xa - 2, 0), pl_hi = min(xe + 1, nx - 1);
        const int s_lo = max(xa - 1, 0), s_hi = min(xe, nx - 1);
        const int r2a = max(y0 - 2, 0), r2b = min(y0 + rows + 2, ny);
        const int r1a = max(y0 - 1, 0), r1b = min(y0 + rows + 1, ny);
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
                    const long long l2 = pb + (long long)(y0 - 2) * nz, l1 = pb + (long long)(y0 - 1) * nz;
                    auto stage = [&](const void *base, int esz, long long l0, int ra, int rb, int off) {
                        stage_range(bar, base, esz, l0, pb + (long long)ra * nz, pb + (long long)rb * nz, slot + off,
                                    L.off, L.off + L.n, slot, lay.slot_bytes);
                    };
                    stage(b, es, l2, r2a, r2b, lay.oB);
                    stage(C.idg, es, l2, r2a, r2b, lay.oG);
                    stage(C.cx, ec, l1, r1a, r1b, lay.oCX);
                    stage(C.cy, ec, l2, r2a, r1b, lay.oCY);
                    stage(C.cz, ec, l1, r1a, r1b, lay.oCZ);
                    stage(C.leak, ec, l1, r1a, r1b, lay.oLK);
                });
                issued += n;
                bad = n != pl_hi - pl_lo + 1;
            }
            __syncwarp();
        } else {
            const int n1 = (rows + 2) * nz, ns = rows * nz;
            int waited = pl_lo - 1, released = pl_lo;
            for (int s = s_lo; s <= s_hi + 1 && !bad; s++) {
                const int need = min(s + 1, pl_hi);
                while (waited < need) {
                    const int g = gof(waited + 1);
                    if (!mbar_wait(&full[g % R], (uint32_t)((g / R) & 1), err)) {
                        bad = true;
                        break;
                    }
                    waited++;
                }
                if (!bad && s <= s_hi) {
                    // first step on plane s (slab rows and one halo row each side) -> V ring; the
                    // slab rows also to xout (the pre-smoothed iterate the post-smoothing corrects)
                    const long long pb = L.off + (long long)s * sx;
                    const long long l2 = pb + (long long)(y0 - 2) * nz, l1 = pb + (long long)(y0 - 1) * nz;
                    char *sc = slot_of(gof(s));
                    const bool xp = s + 1 < nx, xm = s > 0;
                    char *sn = xp ? slot_of(gof(s + 1)) : sc;
                    char *sq = xm ? slot_of(gof(s - 1)) : sc;
                    const T *B = (const T *)(sc + lay.oB) + stage_delta(l2, es);
                    const T *G = (const T *)(sc + lay.oG) + stage_delta(l2, es);
                    const T *Bn = (const T *)(sn + lay.oB) + (xp ? stage_delta(l2 + sx, es) : 0);
                    const T *Gn = (const T *)(sn + lay.oG) + (xp ? stage_delta(l2 + sx, es) : 0);
                    const T *Bq = (const T *)(sq + lay.oB) + (xm ? stage_delta(l2 - sx, es) : 0);
                    const T *Gq = (const T *)(sq + lay.oG) + (xm ? stage_delta(l2 - sx, es) : 0);
                    const CT *CX = (const CT *)(sc + lay.oCX) + stage_delta(l1, ec);
                    const CT *CXq = (const CT *)(sq + lay.oCX) + (xm ? stage_delta(l1 - sx, ec) : 0);
                    const CT *CY = (const CT *)(sc + lay.oCY) + stage_delta(l2, ec);
                    const CT *CZ = (const CT *)(sc + lay.oCZ) + stage_delta(l1, ec);
                    const CT *LK = (const CT *)(sc + lay.oLK) + stage_delta(l1, ec);
                    T *V = (T *)(sm + lay.oV + ((s - s_lo) & 3) * lay.v_stride);
                    const long long lp = pb + (long long)y0 * nz;
                    for (int k = t; k < n1; k += kFusedThreads) {
                        const int rr = div_nz(L, k);
                        const int y = y0 - 1 + rr, z = k - rr * nz;
                        if (y < 0 || y >= ny) continue;
                        const int kx = k + nz;
                        const T bi = B[kx], gi = G[kx];
                        const T x1 = invtheta * bi * gi;
                        T a = cf(LK[k]) * x1;
                        if (z + 1 < nz) a += cf(CZ[k]) * (x1 - invtheta * B[kx + 1] * G[kx + 1]);
                        if (z > 0)      a += cf(CZ[k - 1]) * (x1 - invtheta * B[kx - 1] * G[kx - 1]);
                        if (y + 1 < ny) a += cf(CY[kx]) * (x1 - invtheta * B[kx + nz] * G[kx + nz]);
                        if (y > 0)      a += cf(CY[k]) * (x1 - invtheta * B[kx - nz] * G[kx - nz]);
                        if (xp)         a += cf(CX[k]) * (x1 - invtheta * Bn[kx] * Gn[kx]);
                        if (xm)         a += cf(CXq[k]) * (x1 - invtheta * Bq[kx] * Gq[kx]);
                        const T dn = c1 * x1 + c2 * (bi - a) * gi;
                        const T x2 = x1 + dn;
                        V[k] = x2;
                        if (rr >= 1 && rr <= rows) xout[lp + (k - nz)] = x2;
                    }
                }
                if (fused_sync_or(bad)) {  // first-step results of plane s visible
                    bad = true;
                    break;
                }
                const int tp = s - 1;
                if (tp < xa || tp > xe - 1) {
                    __syncwarp();
                    for (int q = released; q <= s - 2 && q <= waited; q++)
                        if (lane == 0) mbar_arrive(&empty[gof(q) % R]);
                    released = max(released, min(s - 1, waited + 1));
                    continue;
                }
                {
                    // residual b - A x2 on plane tp (slab rows) -> the pair buffer
                    const long long pb = L.off + (long long)tp * sx;
                    const long long l2 = pb + (long long)(y0 - 2) * nz, l1 = pb + (long long)(y0 - 1) * nz;
                    char *sc = slot_of(gof(tp));
                    const bool xp = tp + 1 < nx, xm = tp > 0;
                    char *sq = xm ? slot_of(gof(tp - 1)) : sc;
                    const T *Vc = (const T *)(sm + lay.oV + ((tp - s_lo) & 3) * lay.v_stride);
                    const T *Vn = xp ? (const T *)(sm + lay.oV + ((tp + 1 - s_lo) & 3) * lay.v_stride) : Vc;
                    const T *Vq = xm ? (const T *)(sm + lay.oV + ((tp - 1 - s_lo) & 3) * lay.v_stride) : Vc;
                    const T *B = (const T *)(sc + lay.oB) + stage_delta(l2, es);
                    const CT *CX = (const CT *)(sc + lay.oCX) + stage_delta(l1, ec);
                    const CT *CXq = (const CT *)(sq + lay.oCX) + (xm ? stage_delta(l1 - sx, ec) : 0);
                    const CT *CY = (const CT *)(sc + lay.oCY) + stage_delta(l2, ec);
                    const CT *CZ = (const CT *)(sc + lay.oCZ) + stage_delta(l1, ec);
                    const CT *LK = (const CT *)(sc + lay.oLK) + stage_delta(l1, ec);
                    T *res = (T *)(sm + lay.oR + (tp & 1) * lay.r_stride);
                    for (int kk = t; kk < ns; kk += kFusedThreads) {
                        const int rr = div_nz(L, kk);
                        const int y = y0 + rr, z = kk - rr * nz;
                        const int k = kk + nz;
                        const T xi = Vc[k];
                        T a = cf(LK[k]) * xi;
                        if (z + 1 < nz) a += cf(CZ[k]) * (xi - Vc[k + 1]);
                        if (z > 0)      a += cf(CZ[k - 1]) * (xi - Vc[k - 1]);
                        if (y + 1 < ny) a += cf(CY[k + nz]) * (xi - Vc[k + nz]);
                        if (y > 0)      a += cf(CY[k]) * (xi - Vc[k - nz]);
                        if (xp)         a += cf(CX[k]) * (xi - Vn[k]);
                        if (xm)         a += cf(CXq[k]) * (xi - Vq[k]);
                        res[kk] = B[k + nz] - a;
                    }
                }
                __syncwarp();
                for (int q = released; q <= s - 2 && q <= waited; q++)
                    if (lane == 0) mbar_arrive(&empty[gof(q) % R]);
                released = max(released, min(s - 1, waited + 1));
                const bool pair_done = (tp & 1) || tp + 1 == nx;
                if (!pair_done) continue;
                if (fused_sync_or(bad)) {  // residuals of the pair are in the pair buffer
                    bad = true;
                    break;
                }
                const int X0 = tp & ~1;
                const int cx = X0 >> 1;
                const bool two = X0 + 1 < nx;
                const long long cb = Lc.off + (long long)cx * Lc.ny * Lc.nz + (long long)cy0 * Lc.nz;
                for (int tcc = t; tcc < ncc; tcc += kFusedThreads) {
                    const int cr = div_nz(Lc, tcc), czz = tcc - cr * Lc.nz;
                    const int fy0 = 2 * (cy0 + cr) - y0, fz0 = 2 * czz;
                    const bool y2 = 2 * (cy0 + cr) + 1 < ny, z2 = fz0 + 1 < nz;
                    T acc = 0;
                    for (int ix = 0; ix < (two ? 2 : 1); ix++) {
                        const T *r = (const T *)(sm + lay.oR + ((X0 + ix) & 1) * lay.r_stride);
                        acc += r[fy0 * nz + fz0];
                        if (z2) acc += r[fy0 * nz + fz0 + 1];
                        if (y2) {
                            acc += r[(fy0 + 1) * nz + fz0];
                            if (z2) acc += r[(fy0 + 1) * nz + fz0 + 1];
                        }
                    }
                    bc[cb + tcc] = acc;
                }
                if (fused_sync_or(bad)) {  // the pair buffer may be overwritten
                    bad = true;
                    break;
                }
            }
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

}  // namespace dpf
