// dpf_debug.cu -- test hooks: the bounded waits of the staging kernels, the integer-only
// 48-bit split of doubles that the assembly and the round start use, and the band orderings of
// the direct solver (host code, callable without a GPU).
//
// dpf_debug_expired_wait runs one block whose threads wait on a shared-memory mbarrier
// that nothing arrives on, through the same bounded wait (mbar_wait) that every staging
// kernel uses, so that a test sees that wait end by its bound, the error word set and the
// device still usable, without any kernel of a solve being made to fail.
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "dpf_direct.h"
#include "dpf_plane.cuh"

namespace dpf {

void set_global_error(const std::string &msg);

__global__ void k_expired_wait(int *err, unsigned long long *waited_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);  // one arrival completes phase 0; none is made
    __syncthreads();
    const uint64_t t0 = global_ns();
    const bool done = mbar_wait(&bar, 0, err);
    __syncthreads();
    if (threadIdx.x == 0) {
        waited_ns[0] = global_ns() - t0;
        if (done) atomicExch(err, 2);  // the phase cannot complete: a defect of the wait
    }
}

__global__ void k_split48(long long n, const double *v, float *hi, float *lo, double *v48, int *ok) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float h = 0.f, l = 0.f;
    double w = 0.0;
    ok[i] = split48(v[i], h, l, w) ? 1 : 0;
    hi[i] = h;
    lo[i] = l;
    v48[i] = w;
}

}  // namespace dpf

extern "C" int dpf_debug_split48(int64_t n, const double *v, float *hi, float *lo, double *v48, int *ok) {
    if (n < 0 || (n > 0 && (!v || !hi || !lo || !v48 || !ok))) return DPF_BAD_INPUT;
    if (n == 0) return DPF_OK;
    dpf::k_split48<<<(unsigned)((n + 255) / 256), 256>>>((long long)n, v, hi, lo, v48, ok);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaGetLastError();
        dpf::set_global_error(std::string("split probe: ") + cudaGetErrorString(e));
        return DPF_CUDA;
    }
    return DPF_OK;
}

extern "C" int dpf_debug_expired_wait(double *waited_ms) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        dpf::set_global_error("no CUDA device");
        return DPF_NO_DEVICE;
    }
    void *buf = nullptr;
    if (dpf::dev_malloc(&buf, 16) != cudaSuccess) {
        cudaGetLastError();
        dpf::set_global_error("device allocation failed");
        return DPF_OOM;
    }
    int *d_err = (int *)buf;
    unsigned long long *d_ns = (unsigned long long *)((char *)buf + 8);
    int h_err = -1;
    unsigned long long h_ns = 0;
    cudaError_t e = cudaMemset(buf, 0, 16);
    if (e == cudaSuccess) {
        dpf::k_expired_wait<<<1, 32>>>(d_err, d_ns);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&h_ns, d_ns, sizeof(h_ns), cudaMemcpyDeviceToHost);
    dpf::dev_free(buf);
    if (e != cudaSuccess) {
        cudaGetLastError();
        dpf::set_global_error(std::string("expired-wait probe: ") + cudaGetErrorString(e));
        return DPF_CUDA;
    }
    if (waited_ms) *waited_ms = 1e-6 * (double)h_ns;
    if (h_err != 1) {
        dpf::set_global_error("the bounded wait did not report its expiry");
        return DPF_STATE;
    }
    dpf::set_global_error("a bounded staging wait expired after " + std::to_string(1e-6 * (double)h_ns) + " ms");
    return DPF_TIMEOUT;
}

// The direct solver's band orderings, run on the host: perm[k] = the original row of band row k,
// *w = the half-bandwidth the ordering gives.
extern "C" int dpf_debug_band_order_graph(int64_t n, const int32_t *rp, const int32_t *ci, int64_t *perm,
                                          int64_t *w) {
    if (n < 0 || !rp || !perm || !w || n > (int64_t)1 << 30) return DPF_BAD_INPUT;
    if (rp[0] != 0) return DPF_BAD_INPUT;
    for (int64_t i = 0; i < n; i++)
        if (rp[i + 1] < rp[i]) return DPF_BAD_INPUT;
    const int64_t nnz = rp[n];
    if (nnz > 0 && !ci) return DPF_BAD_INPUT;
    for (int64_t e = 0; e < nnz; e++)
        if (ci[e] < 0 || ci[e] >= n) return DPF_BAD_INPUT;
    try {
        std::vector<int> r(rp, rp + n + 1), c(ci, ci + nnz);
        const dpf::BandOrder o = dpf::band_order_rcm((long long)n, r, c);
        for (int64_t k = 0; k < n; k++) perm[k] = o.perm[k];
        *w = o.w;
    } catch (const std::bad_alloc &) {
        return DPF_OOM;
    }
    return DPF_OK;
}

extern "C" int dpf_debug_band_order_grids(int nprob, const int32_t *dims, int64_t *perm, int64_t *w) {
    if (nprob < 0 || (nprob > 0 && !dims) || !perm || !w) return DPF_BAD_INPUT;
    try {
        std::vector<std::array<int, 3>> d(nprob);
        std::vector<long long> off(nprob);
        long long n = 0;
        for (int p = 0; p < nprob; p++) {
            for (int a = 0; a < 3; a++) {
                if (dims[3 * p + a] < 1) return DPF_BAD_INPUT;
                d[p][a] = dims[3 * p + a];
            }
            off[p] = n;
            n += (long long)d[p][0] * d[p][1] * d[p][2];
            if (n > (1LL << 30)) return DPF_BAD_INPUT;
        }
        const dpf::BandOrder o = dpf::band_order_regular(d, off);
        for (long long k = 0; k < n; k++) perm[k] = o.perm[k];
        *w = o.w;
    } catch (const std::bad_alloc &) {
        return DPF_OOM;
    }
    return DPF_OK;
}
