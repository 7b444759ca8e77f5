// dpf_direct.cu -- banded Cholesky factorisation and solves (see dpf_direct.h).
//
// Factorisation: right-looking, in blocks of kNB = 32 columns. Per block two launches: the
// 32 x 32 diagonal block factored in shared memory by every CTA of the panel solve, which then
// solves the panel below it (up to w rows, a thread per row); and the symmetric update of the
// trailing window, at most (w + 32)^2 / 2 entries inside the band, in 32 x 32 tiles. Triangular solves: one CTA that walks the blocks in order (forward) and in reverse
// (backward); per block one warp solves the 32 x 32 triangle and the CTA applies the block's
// columns to the up to w rows (forward) or columns (backward) that depend on it.
// All arithmetic is FP64.
#include "dpf_direct.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "dpf_struct.h"

namespace dpf {

namespace {

constexpr int kNB = 32;            // block columns
constexpr int kSolveThreads = 1024;

__device__ __forceinline__ long long bidx(long long r, long long c, long long w) { return c * (w + 1) + (r - c); }

// One block step's diagonal factorisation and panel solve, in one launch: every CTA factors the
// 32 x 32 diagonal block [j0, j0 + jb) in shared memory (the same arithmetic in every CTA, so the
// same result; CTA 0 stores it and reports a non-positive pivot), then solves its 256 rows of the
// panel r in [j0 + jb, r_end): L[r, c] = (A[r, c] - sum_{k < c} L[r, k] L[c, k]) / L[c, c];
// columns c < r - w are outside the band and stay zero.
constexpr int kPanelThreads = 256;
__global__ void __launch_bounds__(kPanelThreads) k_band_panel(double *__restrict__ B, long long w, long long j0,
                                                              int jb, long long r_end, int *err) {
    __shared__ double d[kNB][kNB + 1];
    __shared__ double inv[kNB];
    const int t = threadIdx.x;
    for (int e = t; e < kNB * kNB; e += kPanelThreads) {
        const int j = e / kNB, i = e % kNB;  // consecutive threads: consecutive rows of column j
        d[i][j] = (j <= i && i < jb && (long long)(i - j) <= w) ? B[bidx(j0 + i, j0 + j, w)] : 0.0;
    }
    for (int k = 0; k < jb; k++) {
        __syncthreads();
        if (t == 0) {
            double v = d[k][k];
            if (!(v > 0.0)) {  // not positive definite: recorded; a unit pivot keeps the rest finite
                if (blockIdx.x == 0) atomicExch(err, 1);
                v = 1.0;
            }
            d[k][k] = sqrt(v);
            inv[k] = 1.0 / d[k][k];
        }
        __syncthreads();
        if (t > k && t < jb) d[t][k] *= inv[k];
        __syncthreads();
        // trailing entries (i, j), k < j <= i < jb (zero outside the band stays zero: a factor of
        // each product is zero there)
        for (int e = t; e < kNB * kNB; e += kPanelThreads) {
            const int i = e / kNB, j = e % kNB;
            if (j > k && j <= i && i < jb) d[i][j] -= d[i][k] * d[j][k];
        }
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int e = t; e < kNB * kNB; e += kPanelThreads) {
            const int j = e / kNB, i = e % kNB;
            if (j <= i && i < jb && (long long)(i - j) <= w) B[bidx(j0 + i, j0 + j, w)] = d[i][j];
        }
    const long long r = j0 + jb + (long long)blockIdx.x * kPanelThreads + t;
    if (r >= r_end) return;
    const int cmin = (int)max(0LL, r - w - j0);
    double x[kNB];
#pragma unroll
    for (int c = 0; c < kNB; c++) {
        x[c] = 0.0;
        if (c < cmin || c >= jb) continue;
        double v = B[bidx(r, j0 + c, w)];
#pragma unroll
        for (int k = 0; k < c; k++) v -= x[k] * d[c][k];
        x[c] = v * inv[c];
        B[bidx(r, j0 + c, w)] = x[c];
    }
}

// trailing update: A[r, q] -= sum_c L[r, c] L[q, c] over the block's columns, for q <= r,
// r - q <= w, r and q in [m0, m1); tile (blockIdx.y, blockIdx.x) of 32 rows x 32 columns,
// thread (tx, ty) = row r0 + tx, column q0 + ty (consecutive rows are consecutive in the band)
__global__ void __launch_bounds__(kNB * kNB) k_band_syrk(double *__restrict__ B, long long w, long long j0, int jb,
                                                         long long m0, long long m1) {
    const long long r0 = m0 + (long long)blockIdx.y * kNB, q0 = m0 + (long long)blockIdx.x * kNB;
    if (q0 > r0 + kNB - 1 || r0 - (q0 + kNB - 1) > w) return;  // above the diagonal or outside the band
    __shared__ double lr[kNB][kNB + 1], lq[kNB][kNB + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    {
        const int c = ty;  // column of the block, row of the tile tx
        const long long r = r0 + tx, q = q0 + tx, cc = j0 + c;
        lr[tx][c] = (c < jb && r < m1 && r - cc <= w) ? B[bidx(r, cc, w)] : 0.0;
        lq[tx][c] = (c < jb && q < m1 && q - cc <= w) ? B[bidx(q, cc, w)] : 0.0;
    }
    __syncthreads();
    const long long r = r0 + tx, q = q0 + ty;
    if (r >= m1 || q > r || r - q > w) return;
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kNB; c++) s = fma(lr[tx][c], lq[ty][c], s);
    B[bidx(r, q, w)] -= s;
}

// y[k] = b[perm[k]]  /  x[perm[k]] = y[k]
__global__ void k_gather(long long n, const long long *__restrict__ perm, const double *__restrict__ b,
                         double *__restrict__ y) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        y[k] = b[perm[k]];
}
__global__ void k_scatter(long long n, const long long *__restrict__ perm, const double *__restrict__ y,
                          double *__restrict__ x) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        x[perm[k]] = y[k];
}

// the lower triangle of diagonal block [j0, j0 + jb) into d (zeros elsewhere), by all threads
// (consecutive threads read consecutive rows of one column: consecutive in the band), with the
// reciprocals of its diagonal on the diagonal (one FP64 division per entry, in parallel, instead
// of 32 in the sequential solve)
__device__ __forceinline__ void load_diag(const double *__restrict__ B, long long w, long long j0, int jb,
                                          double (*d)[kNB + 1]) {
    for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) {
        const int j = e / kNB, i = e % kNB;
        double v = (j <= i && i < jb && (long long)(i - j) <= w) ? B[bidx(j0 + i, j0 + j, w)] : 0.0;
        if (i == j) v = i < jb ? 1.0 / v : 0.0;
        d[i][j] = v;
    }
}

// L z = y, then L^T x = z, in place in y, by one CTA walking the blocks. Forward, per block: warp
// 0 solves the 32 x 32 triangle (lane i holds row j0 + i) from the block's entries staged in
// shared memory, then every thread applies the block's columns to its rows below (up to w rows,
// consecutive rows consecutive in the band), while the next block's triangle is staged. Backward,
// per block from the last: warp 0 solves the transposed triangle, then the CTA applies the
// block's rows to the columns above it that reach them (each thread one column, its entries in
// the block's rows contiguous in the band).
__global__ void __launch_bounds__(kSolveThreads) k_band_solve(const double *__restrict__ B, long long n, long long w,
                                                               double *__restrict__ y) {
    __shared__ double d[2][kNB][kNB + 1];
    const int t = threadIdx.x, lane = t & 31;
    const long long nblk = (n + kNB - 1) / kNB;
    load_diag(B, w, 0, (int)min((long long)kNB, n), d[0]);
    __syncthreads();
    for (long long b = 0; b < nblk; b++) {
        const long long j0 = b * kNB;
        const int jb = (int)min((long long)kNB, n - j0);
        double(*D)[kNB + 1] = d[b & 1];
        if (t < 32) {
            double v = lane < jb ? y[j0 + lane] : 0.0;
            for (int k = 0; k < jb; k++) {
                double z = v * D[k][k];  // meaningful in lane k (D[k][k] holds 1 / L[k][k])
                z = __shfl_sync(0xffffffffu, z, k);
                if (lane == k) v = z;
                else if (lane > k) v -= D[lane][k] * z;  // zero outside the band and past jb
            }
            if (lane < jb) y[j0 + lane] = v;
        }
        __syncthreads();
        if (b + 1 < nblk) load_diag(B, w, j0 + kNB, (int)min((long long)kNB, n - j0 - kNB), d[(b + 1) & 1]);
        const long long r_end = min(n, j0 + jb + w);
        for (long long r = j0 + jb + t; r < r_end; r += kSolveThreads) {
            double s = 0.0;
            const int cmin = (int)max(0LL, r - w - j0);
            for (int c = cmin; c < jb; c++) s = fma(B[bidx(r, j0 + c, w)], y[j0 + c], s);
            y[r] -= s;
        }
        __syncthreads();
    }
    // backward step s = nblk - 1 - b uses d[s & 1] and stages the next block into d[(s + 1) & 1]
    load_diag(B, w, (nblk - 1) * kNB, (int)(n - (nblk - 1) * kNB), d[0]);
    __syncthreads();
    for (long long b = nblk - 1; b >= 0; b--) {
        const long long j0 = b * kNB;
        const int jb = (int)min((long long)kNB, n - j0);
        double(*D)[kNB + 1] = d[(nblk - 1 - b) & 1];
        if (t < 32) {
            double v = lane < jb ? y[j0 + lane] : 0.0;
            for (int k = jb - 1; k >= 0; k--) {
                double x = v * D[k][k];
                x = __shfl_sync(0xffffffffu, x, k);
                if (lane == k) v = x;
                else if (lane < k) v -= D[k][lane] * x;
            }
            if (lane < jb) y[j0 + lane] = v;
        }
        __syncthreads();
        if (b > 0) load_diag(B, w, j0 - kNB, kNB, d[(nblk - b) & 1]);
        const long long c_lo = max(0LL, j0 - w);
        for (long long c = c_lo + t; c < j0; c += kSolveThreads) {
            double s = 0.0;
            const long long r_hi = min(j0 + jb - 1, c + w);
            for (long long r = j0; r <= r_hi; r++) s = fma(B[bidx(r, c, w)], y[r], s);
            y[c] -= s;
        }
        __syncthreads();
    }
}

__global__ void k_direct_resid(long long n, const uint8_t *__restrict__ dir, const double *__restrict__ b,
                               const double *__restrict__ Ax, double *acc) {
    double rr = 0.0, bb = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (dir[i]) continue;
        const double r = b[i] - Ax[i];
        rr = fma(r, r, rr);
        bb = fma(b[i], b[i], bb);
    }
    for (int o = 16; o > 0; o >>= 1) {
        rr += __shfl_xor_sync(0xffffffffu, rr, o);
        bb += __shfl_xor_sync(0xffffffffu, bb, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], rr);
        atomicAdd(&acc[1], bb);
    }
}

void dck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaError(std::string("direct solve, ") + what + ": " + cudaGetErrorString(e), e);
    }
}

}  // namespace

BandOrder band_order_regular(const std::vector<std::array<int, 3>> &dims, const std::vector<long long> &off) {
    BandOrder o;
    long long n = 0;
    for (size_t p = 0; p < dims.size(); p++) n = std::max(n, off[p] + (long long)dims[p][0] * dims[p][1] * dims[p][2]);
    o.perm.assign(n, 0);
    for (size_t p = 0; p < dims.size(); p++) {
        const int nn[3] = {dims[p][0], dims[p][1], dims[p][2]};
        const long long st[3] = {(long long)nn[1] * nn[2], nn[2], 1};
        int ax[3] = {0, 1, 2};
        std::stable_sort(ax, ax + 3, [&](int a, int b) { return nn[a] > nn[b]; });  // longest slowest
        const long long w = (long long)nn[ax[1]] * nn[ax[2]];
        if (nn[ax[0]] > 1) o.w = std::max(o.w, w);
        else if (nn[ax[1]] > 1) o.w = std::max(o.w, (long long)nn[ax[2]]);
        else if (nn[ax[2]] > 1) o.w = std::max(o.w, 1LL);
        long long k = off[p];
        for (int a = 0; a < nn[ax[0]]; a++)
            for (int b = 0; b < nn[ax[1]]; b++)
                for (int c = 0; c < nn[ax[2]]; c++)
                    o.perm[k++] = off[p] + a * st[ax[0]] + b * st[ax[1]] + c * st[ax[2]];
    }
    return o;
}

BandOrder band_order_rcm(long long n, const std::vector<int> &rp, const std::vector<int> &ci) {
    BandOrder o;
    std::vector<int> deg(n);
    for (long long i = 0; i < n; i++) deg[i] = rp[i + 1] - rp[i];
    std::vector<char> seen(n, 0);
    std::vector<long long> order;
    order.reserve(n);
    std::vector<int> level(n, -1);
    // breadth-first levels from s over the unvisited component; returns the vertex of smallest
    // degree in the deepest level
    auto bfs_far = [&](long long s, std::vector<long long> &comp) {
        comp.clear();
        comp.push_back(s);
        level[s] = 0;
        for (size_t h = 0; h < comp.size(); h++) {
            const long long v = comp[h];
            for (int e = rp[v]; e < rp[v + 1]; e++) {
                const int u = ci[e];
                if (u != v && level[u] < 0 && !seen[u]) {
                    level[u] = level[v] + 1;
                    comp.push_back(u);
                }
            }
        }
        long long best = comp.back();
        for (long long v : comp)
            if (level[v] == level[comp.back()] && deg[v] < deg[best]) best = v;
        for (long long v : comp) level[v] = -1;
        return best;
    };
    std::vector<long long> comp;
    std::vector<int> nb;
    for (long long s0 = 0; s0 < n; s0++) {
        if (seen[s0]) continue;
        // pseudo-peripheral start: twice the farthest lowest-degree vertex
        long long s = bfs_far(s0, comp);
        s = bfs_far(s, comp);
        // Cuthill-McKee from s: neighbours in order of increasing degree
        const size_t first = order.size();
        order.push_back(s);
        seen[s] = 1;
        for (size_t h = first; h < order.size(); h++) {
            const long long v = order[h];
            nb.clear();
            for (int e = rp[v]; e < rp[v + 1]; e++)
                if (!seen[ci[e]] && ci[e] != v) {
                    seen[ci[e]] = 1;
                    nb.push_back(ci[e]);
                }
            std::sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b] || (deg[a] == deg[b] && a < b); });
            for (int u : nb) order.push_back(u);
        }
        std::reverse(order.begin() + first, order.end());
    }
    o.perm = order;
    std::vector<long long> pos(n);
    for (long long k = 0; k < n; k++) pos[order[k]] = k;
    for (long long i = 0; i < n; i++)
        for (int e = rp[i]; e < rp[i + 1]; e++) o.w = std::max(o.w, std::llabs(pos[i] - pos[ci[e]]));
    return o;
}

bool BandCholesky::fits(long long n, long long w, size_t mem_bytes) {
    if (n <= 0) return false;
    const double bytes = 8.0 * (double)n * (double)(w + 1) + 24.0 * (double)n;
    return bytes <= (double)mem_bytes && (double)n * (double)w * (double)w <= 2e13;
}

BandCholesky::BandCholesky(const BandOrder &ord, cudaStream_t s) : n((long long)ord.perm.size()), w(ord.w), stream(s) {
    std::vector<long long> iperm(n);
    for (long long k = 0; k < n; k++) iperm[ord.perm[k]] = k;
    auto alloc = [&](void **p, size_t bytes) {
        if (dev_malloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            throw OomError("direct solve: cudaMalloc of " + std::to_string(bytes) + " bytes failed");
        }
    };
    try {
        alloc((void **)&B, (size_t)n * (size_t)(w + 1) * sizeof(double));
        alloc((void **)&y, (size_t)n * sizeof(double));
        alloc((void **)&d_perm, (size_t)n * sizeof(long long));
        alloc((void **)&d_iperm, (size_t)n * sizeof(long long));
        alloc((void **)&d_err, sizeof(int));
        dck(cudaMemcpyAsync(d_perm, ord.perm.data(), n * sizeof(long long), cudaMemcpyHostToDevice, stream), "perm");
        dck(cudaMemcpyAsync(d_iperm, iperm.data(), n * sizeof(long long), cudaMemcpyHostToDevice, stream), "perm");
        dck(cudaStreamSynchronize(stream), "perm");  // the host vectors go out of scope
    } catch (...) {
        dev_free(B);
        dev_free(y);
        dev_free(d_perm);
        dev_free(d_iperm);
        dev_free(d_err);
        throw;
    }
}

BandCholesky::~BandCholesky() {
    if (stream) cudaStreamSynchronize(stream);
    dev_free(B);
    dev_free(y);
    dev_free(d_perm);
    dev_free(d_iperm);
    dev_free(d_err);
}

void BandCholesky::clear() {
    dck(cudaMemsetAsync(B, 0, (size_t)n * (size_t)(w + 1) * sizeof(double), stream), "clear");
}

bool BandCholesky::factor() {
    NvtxRange range("banded Cholesky factorisation");
    dck(cudaMemsetAsync(d_err, 0, sizeof(int), stream), "factor");
    for (long long j0 = 0; j0 < n; j0 += kNB) {
        const int jb = (int)std::min<long long>(kNB, n - j0);
        const long long r_end = std::min(n, j0 + jb + w);
        const long long m = r_end - (j0 + jb);
        k_band_panel<<<(unsigned)std::max(1LL, (m + kPanelThreads - 1) / kPanelThreads), kPanelThreads, 0, stream>>>(
            B, w, j0, jb, r_end, d_err);
        launches++;
        if (m > 0) {
            const unsigned nt = (unsigned)((m + kNB - 1) / kNB);
            k_band_syrk<<<dim3(nt, nt), dim3(kNB, kNB), 0, stream>>>(B, w, j0, jb, j0 + jb, r_end);
            launches++;
        }
    }
    dck(cudaGetLastError(), "factor launch");
    int h_err = 0;
    dck(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "factor");
    dck(cudaStreamSynchronize(stream), "factor");
    return h_err == 0;
}

void BandCholesky::solve(const double *b, double *x) {
    NvtxRange range("banded Cholesky solves");
    const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 4096);
    k_gather<<<g, 256, 0, stream>>>(n, d_perm, b, y);
    k_band_solve<<<1, kSolveThreads, 0, stream>>>(B, n, w, y);
    k_scatter<<<g, 256, 0, stream>>>(n, d_perm, y, x);
    launches += 3;
    dck(cudaGetLastError(), "solve launch");
}

double BandCholesky::relres(cudaStream_t s, long long n, const uint8_t *dir, const double *b, const double *Ax,
                            double *acc) {
    dck(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s), "residual");
    k_direct_resid<<<(unsigned)std::min<long long>((n + 255) / 256, 1024), 256, 0, s>>>(n, dir, b, Ax, acc);
    dck(cudaGetLastError(), "residual launch");
    double h[2] = {0.0, 0.0};
    dck(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s), "residual");
    dck(cudaStreamSynchronize(s), "residual");
    return h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
}

}  // namespace dpf
