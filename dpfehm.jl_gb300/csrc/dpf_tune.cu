// dpf_tune.cu -- autotuner for the batched steady solve: chooses the Chebyshev degree, the
// plane-marching slab size and blocks per SM, the fused-tail threshold, the grid-stride
// blocks per SM and the form of the double-float CG product for a given batch by timing
// real forward + adjoint solves.
//
// Coordinate descent from the caller's options: each parameter in turn is set to each of
// its candidate values with the others held at the best so far; a candidate is adopted
// when its solve converges and is at least 2 % faster. Every evaluation creates the batch
// through the public API, runs one untimed solve (graph capture, warm caches) and then
// `repeats` timed solves with CUDA events on the library's stream (the legacy default
// stream). Only the public C ABI is used, so what is timed is what a caller runs.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "dpfehm_gpu.h"
#include "dpf_internal.h"

namespace dpf {
void set_global_error(const std::string &msg);
}

namespace {

struct DevCopy {
    const double *ptr = nullptr;
    double *owned = nullptr;
    ~DevCopy() {
        dpf::dev_free(owned);
    }
};

bool on_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int to_device(const double *src, size_t n, DevCopy &out) {
    if (on_device(src)) {
        out.ptr = src;
        return DPF_OK;
    }
    if (dpf::dev_malloc((void **)&out.owned, n * sizeof(double)) != cudaSuccess) return DPF_OOM;
    if (cudaMemcpy(out.owned, src, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return DPF_CUDA;
    out.ptr = out.owned;
    return DPF_OK;
}

}  // namespace

extern "C" int dpf_batch_autotune(int nprob, const int *dims, const double *mins, const double *maxs, const int64_t *nd,
                                  const int64_t *dn, const dpf_options *base, const double *logK, int kind,
                                  const double *dh, const double *Qs, const int64_t *obs_offsets, const int64_t *obs,
                                  int repeats, dpf_options *best, double *best_ms) {
    if (nprob <= 0 || !dims || !mins || !maxs || !nd || !logK || !dh || !Qs || !obs_offsets || !best)
        return DPF_BAD_INPUT;
    if (repeats < 1) repeats = 1;
    size_t N = 0;
    for (int p = 0; p < nprob; p++) N += (size_t)dims[3 * p] * dims[3 * p + 1] * dims[3 * p + 2];
    dpf_options cur;
    dpf_default_options(&cur);
    if (base) cur = *base;
    // batches are regular grids: resolve the "path default" values to the regular-grid ones
    if (cur.cheb_degree == 0) cur.cheb_degree = 2;
    if (!(cur.coarse_scale > 0)) cur.coarse_scale = 2.0;
    DevCopy dlk, ddh, dq;
    int rc;
    if ((rc = to_device(logK, N, dlk)) || (rc = to_device(dh, N, ddh)) || (rc = to_device(Qs, N, dq))) return rc;
    // a copy from pageable memory may return before its DMA lands: complete it before any
    // candidate's stream reads the inputs
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return DPF_CUDA;
    }
    double *hout = nullptr, *gout = nullptr;
    if (dpf::dev_malloc((void **)&hout, N * sizeof(double)) != cudaSuccess ||
        dpf::dev_malloc((void **)&gout, N * sizeof(double)) != cudaSuccess) {
        dpf::dev_free(hout);
        return DPF_OOM;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);

    // one evaluation: create, warm up, time `repeats` solves; DPF_OK and the mean ms per solve
    auto evaluate = [&](const dpf_options &o, double &ms) -> int {
        dpf_problem *h = nullptr;
        int r = dpf_batch_create(nprob, dims, mins, maxs, nd, dn, &o, &h);
        if (r != DPF_OK) return r;
        r = dpf_batch_solve_grad_logk(h, dlk.ptr, kind, ddh.ptr, dq.ptr, obs_offsets, obs, hout, gout);
        if (r == DPF_OK) {
            cudaEventRecord(e0, 0);
            for (int k = 0; k < repeats && r == DPF_OK; k++)
                r = dpf_batch_solve_grad_logk(h, dlk.ptr, kind, ddh.ptr, dq.ptr, obs_offsets, obs, hout, gout);
            cudaEventRecord(e1, 0);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            ms = (double)t / repeats;
        }
        dpf_destroy(h);
        return r;
    };

    double cur_ms = 0.0;
    rc = evaluate(cur, cur_ms);
    if (rc == DPF_CUDA)
        dpf::set_global_error(std::string("autotune: the starting options: ") +
                              cudaGetErrorString(cudaGetLastError()));
    if (rc == DPF_OK) {
        const bool mixed = cur.precision == DPF_PREC_MIXED && cur.plane > 0;
        struct Knob {
            const char *name;
            int *field;
            std::vector<int> values;
            bool active;
        };
        const Knob knobs[] = {
            {"cheb_degree", &cur.cheb_degree, {1, 2, 3}, true},
            {"plane_cells", &cur.plane_cells, {512, 768, 1024}, mixed},
            {"plane_blocks_per_sm", &cur.plane_blocks_per_sm, {1, 2, 3}, mixed},
            {"tail_cells", &cur.tail_cells, {-1, 1024, 4096, 16384}, true},
            {"blocks_per_sm", &cur.blocks_per_sm, {8, 16, 24}, true},
            {"df_plane_cells", &cur.df_plane_cells, {-1, 256}, mixed},
            {"tail_cluster", &cur.tail_cluster, {1, 8}, true},
            {"plane_levels", &cur.plane_levels, {0, 1, 2}, mixed},
            {"streams", &cur.streams, {1, 2, 4}, nprob >= 2},
            {"fuse", &cur.fuse, {-1, 1}, mixed},
        };
        for (const Knob &k : knobs) {
            if (!k.active || rc != DPF_OK) continue;
            const int keep = *k.field;
            int pick = keep;
            for (int v : k.values) {
                if (v == keep) continue;
                *k.field = v;
                double ms = 0.0;
                const int r = evaluate(cur, ms);
                if (r == DPF_CUDA) {
                    // a CUDA error is not a slow candidate: stop and name the candidate
                    dpf::set_global_error(std::string("autotune: candidate ") + k.name + " = " + std::to_string(v) +
                                          ": " + cudaGetErrorString(cudaGetLastError()));
                    rc = DPF_CUDA;
                    break;
                }
                if (r == DPF_OK && ms < 0.98 * cur_ms) {
                    cur_ms = ms;
                    pick = v;
                }
            }
            *k.field = pick;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dpf::dev_free(hout);
    dpf::dev_free(gout);
    *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return rc;
}
