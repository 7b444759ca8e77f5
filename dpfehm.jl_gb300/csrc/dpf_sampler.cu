// dpf_sampler.cu -- seeded Gaussian log-conductivity fields with Matern (nu = 1) covariance, drawn on
// the GPU for every problem of a regular-grid batch, so that an inverse or uncertainty-quantification
// loop (draw fields, solve, differentiate) needs no host or third-party step between its launches.
//
// Method: spectral synthesis (the randomization method). With M modes,
//   f(x) = mean + sigma sqrt(2 / M) sum_k cos(w_k . x + phi_k),
// phi_k uniform on [0, 2 pi) and the frequencies w_k drawn from the normalised spectral density of
// the Matern covariance, S(w) ~ (kappa^2 + |w|^2)^-(nu + 3/2) with kappa^2 = 2 nu / ell^2 (the same
// convention as the package's FFT sampler, fields.matern_field). That density is a Gaussian scale
// mixture: w = sqrt(s) z with z ~ N(0, I_3) and s = kappa^2 / (2 G), G ~ Gamma(nu, 1); for nu = 1,
// G is exponential. The field then has mean `mean`, variance sigma^2 and, in expectation over the
// modes, exactly the Matern correlation (kappa r) K_1(kappa r); by the central limit theorem it is
// close to Gaussian for a few hundred modes. It is periodic-free (no padding) and every cell costs
// M cosines, independent of the grid's extent.
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC 2011), a counter-based generator: the draws of mode k of a problem are a pure
// function of (seed, k), so a field depends only on its seed, grid and M -- not on its position in
// the batch, the launch shape or the device -- and repeated calls give it bit for bit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "dpf_struct.h"
#include "dpf_struct_kernels.cuh"

namespace dpf {

struct SampleParam {
    unsigned long long seed;
    double ell, sigma, mean;
};

constexpr unsigned kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;  // round multipliers
constexpr unsigned kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;  // key increments (Weyl sequence)
constexpr unsigned kModeTag = 0x4d415445u;                            // counter word 2 of the sampler's draws

__host__ __device__ __forceinline__ void philox4x32_10(unsigned c[4], unsigned k0, unsigned k1) {
    for (int r = 0; r < 10; r++) {
        const unsigned long long p0 = (unsigned long long)kPhiloxM0 * c[0];
        const unsigned long long p1 = (unsigned long long)kPhiloxM1 * c[2];
        const unsigned hi0 = (unsigned)(p0 >> 32), lo0 = (unsigned)p0;
        const unsigned hi1 = (unsigned)(p1 >> 32), lo1 = (unsigned)p1;
        const unsigned n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
}

__device__ __forceinline__ double u01(unsigned x) { return ((double)x + 0.5) * 0x1p-32; }  // in (0, 1)

// One thread per (problem, mode): the mode's frequency per grid step along each axis and its phase
// at the grid's centre, reduced to [0, 2 pi), so the field kernel works in a centred frame in FP32.
__global__ void k_matern_modes(int nprob, int M, const SampleParam *__restrict__ sp, const ProbParam *__restrict__ prm,
                               const LevelDesc *__restrict__ desc, float4 *__restrict__ modes) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nprob * M) return;
    const int p = (int)(t / M), k = (int)(t % M);
    const SampleParam q = sp[p];
    const unsigned k0 = (unsigned)q.seed, k1 = (unsigned)(q.seed >> 32);
    unsigned a[4] = {(unsigned)k, 0u, kModeTag, 0u}, b[4] = {(unsigned)k, 1u, kModeTag, 0u};
    philox4x32_10(a, k0, k1);
    philox4x32_10(b, k0, k1);
    const double two_pi = 6.283185307179586476925286766559;
    const double r1 = sqrt(-2.0 * log(u01(a[0]))), r2 = sqrt(-2.0 * log(u01(a[2])));
    const double z1 = r1 * cos(two_pi * u01(a[1])), z2 = r1 * sin(two_pi * u01(a[1]));
    const double z3 = r2 * cos(two_pi * u01(a[3]));
    const double G = -log(u01(b[0]));             // Gamma(1, 1)
    const double s = 1.0 / (q.ell * sqrt(G));    // sqrt(kappa^2 / (2 G)) with kappa^2 = 2 / ell^2
    const LevelDesc L = desc[p];
    const ProbParam P = prm[p];
    const double w[3] = {s * z1, s * z2, s * z3};
    const int n[3] = {L.nx, L.ny, L.nz};
    double ph = two_pi * u01(b[1]);
    for (int d = 0; d < 3; d++) ph += w[d] * (P.x0[d] + 0.5 * (n[d] - 1) * P.dx[d]);
    ph -= two_pi * floor(ph / two_pi);
    modes[t] = make_float4((float)(w[0] * P.dx[0]), (float)(w[1] * P.dx[1]), (float)(w[2] * P.dx[2]), (float)ph);
}

// The field at every cell of every problem (block map over the problems' cells): the problem's M
// modes are staged through shared memory in tiles, each thread sums its cell's cosines in mode
// order (FP32; a fixed order, so the result is reproducible bit for bit).
constexpr int kModeTile = 256;
__global__ void __launch_bounds__(kModeTile) k_matern_field(const LevelDesc *__restrict__ desc,
                                                            const int4 *__restrict__ bmap,
                                                            const SampleParam *__restrict__ sp,
                                                            const float4 *__restrict__ modes, int M,
                                                            double *__restrict__ logK) {
    __shared__ float4 tile[kModeTile];
    const int4 bm = bmap[blockIdx.x];
    const int p = bm.x;
    const LevelDesc L = desc[p];
    const SampleParam q = sp[p];
    const float cx = 0.5f * (float)(L.nx - 1), cy = 0.5f * (float)(L.ny - 1), cz = 0.5f * (float)(L.nz - 1);
    const double amp = q.sigma * sqrt(2.0 / (double)M);
    const float4 *mp = modes + (long long)p * M;
    for (int base = bm.y * kModeTile; base < (int)L.n; base += bm.z * kModeTile) {
        const int li = base + (int)threadIdx.x;
        const bool valid = li < (int)L.n;
        Cell c{};
        if (valid) cell_at(L, li, c);
        const float fx = (float)c.ix - cx, fy = (float)c.iy - cy, fz = (float)c.iz - cz;
        float acc = 0.0f;
        for (int m0 = 0; m0 < M; m0 += kModeTile) {
            __syncthreads();
            if (m0 + (int)threadIdx.x < M) tile[threadIdx.x] = mp[m0 + threadIdx.x];
            __syncthreads();
            const int mm = min(kModeTile, M - m0);
            for (int k = 0; k < mm; k++) {
                const float4 w = tile[k];
                acc += cosf(fmaf(w.z, fz, fmaf(w.y, fy, fmaf(w.x, fx, w.w))));
            }
        }
        if (valid) logK[c.i] = q.mean + amp * (double)acc;
    }
}

static void sck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e), e);
    }
}

void StructBatch::sample_logk(int M, const unsigned long long *seeds, const double *ell, const double *sigma,
                              const double *mean, double *out) {
    NvtxRange range("Matern field sampler");
    if (M < 1 || M > (1 << 16)) throw BadInput("the number of modes must be in 1..65536");
    for (int p = 0; p < nprob; p++)
        if (!(ell[p] > 0.0) || !(sigma[p] >= 0.0) || !std::isfinite(mean[p]))
            throw BadInput("correlation lengths must be positive, sigmas non-negative, means finite");
    if (!d_sample) {
        d_sample = (void *)dalloc_bytes(nprob * sizeof(SampleParam));
        h_sample = pinned.alloc(nprob * sizeof(SampleParam));
        if (!h_sample) throw OomError("pinned host allocation failed");
    }
    if ((long long)M * nprob > modes_cap) {
        d_modes = (void *)dalloc_bytes((size_t)M * nprob * sizeof(float4));  // the old buffer stays owned
        modes_cap = (long long)M * nprob;
    }
    SampleParam *hs = (SampleParam *)h_sample;
    for (int p = 0; p < nprob; p++) hs[p] = SampleParam{seeds[p], ell[p], sigma[p], mean[p]};
    sck(cudaMemcpyAsync(d_sample, h_sample, nprob * sizeof(SampleParam), cudaMemcpyHostToDevice, stream),
        "sampler parameters");
    const long long nm = (long long)M * nprob;
    {
        KTimer _kt(this, kname("k_matern_modes", 0, false), nm);
        k_matern_modes<<<(unsigned)((nm + 255) / 256), 256, 0, stream>>>(nprob, M, (const SampleParam *)d_sample,
                                                                         d_prm, lv[0].d_desc, (float4 *)d_modes);
    }
    sck(cudaGetLastError(), "kernel launch");
    Level &L0 = lv[0];
    {
        KTimer _kt(this, kname("k_matern_field", 0, true), L0.all_cells);
        k_matern_field<<<(unsigned)L0.all.nblocks, kModeTile, 0, stream>>>(L0.d_desc, L0.all.d_map,
                                                                          (const SampleParam *)d_sample,
                                                                          (const float4 *)d_modes, M, out);
    }
    sck(cudaGetLastError(), "kernel launch");
}

}  // namespace dpf
