// dpf_api.cu -- the extern "C" boundary of libdpfehm_gpu.so (see include/dpfehm_gpu.h).
//
// Each entry point validates its arguments, moves host arrays to the device when
// needed (device pointers are used in place), runs the solver on the handle's
// stream and maps exceptions to dpf_status codes. There is no CPU code path for
// any computation: without a CUDA device every call returns DPF_NO_DEVICE.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dpf_check.cuh"
#include "dpf_general.h"
#include "dpf_struct.h"

using namespace dpf;

namespace {

// Persistent workers of a batch handle split into concurrent parts: run(f) calls f(i) for
// every part i, f(0) on the calling thread and f(1..n-1) on the workers, and returns when
// all have returned. Each worker has made the handle's device current.
class PartPool {
public:
    PartPool(int n, int device) : n_(n) {
        for (int i = 1; i < n; i++)
            th_.emplace_back([this, i, device]() {
                cudaSetDevice(device);
                unsigned long long seen = 0;
                for (;;) {
                    std::function<void(int)> job;
                    {
                        std::unique_lock<std::mutex> lk(m_);
                        cv_.wait(lk, [&]() { return stop_ || gen_ != seen; });
                        if (stop_) return;
                        seen = gen_;
                        job = job_;
                    }
                    job(i);
                    {
                        std::lock_guard<std::mutex> lk(m_);
                        if (--pending_ == 0) done_.notify_all();
                    }
                }
            });
    }
    ~PartPool() {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    void run(const std::function<void(int)> &f) {
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = f;
            pending_ = n_ - 1;
            gen_++;
        }
        cv_.notify_all();
        f(0);
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [&]() { return pending_ == 0; });
    }

private:
    int n_;
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    std::function<void(int)> job_;
    unsigned long long gen_ = 0;
    int pending_ = 0;
    bool stop_ = false;
};

}  // namespace

struct dpf_problem {
    int device = 0;
    cudaStream_t stream = 0;
    bool own_stream = false;           // a part's stream, created and destroyed with it
    dpf_options opt;
    std::unique_ptr<StructBatch> sb;   // structured path (one problem or a batch)
    std::unique_ptr<GeneralSolver> gs; // CSR path
    std::string err;
    // transient bookkeeping (structured path)
    int tr_nsteps = 0, tr_ck = 0;
    double *tr_b0 = nullptr, *tr_ck_states = nullptr, *tr_seg = nullptr, *tr_Ss = nullptr;
    double tr_dt = 0;
    std::vector<void *> scratch;       // device scratch owned by the handle
    // a batch split into concurrent parts (options.streams): each part is a complete batch
    // handle over consecutive problems, on its own stream, driven by its own host thread;
    // `stream` then only orders the parts' work with the caller's stream
    std::vector<dpf_problem *> parts;
    std::vector<int> part_first;       // first problem of each part, and the problem count last
    std::vector<cudaEvent_t> part_events;
    std::vector<cudaEvent_t> input_events;  // a part's host inputs have landed (split batches)
    std::unique_ptr<PartPool> pool;
    // the copy of the heads to a host buffer runs on its own stream during the adjoint solve
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_events[2] = {nullptr, nullptr};
    ~dpf_problem() {
        // a part's own stream is drained before anything its work may still use is released
        if (own_stream && stream) cudaStreamSynchronize(stream);
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        pool.reset();
        for (dpf_problem *q : parts) delete q;
        for (cudaEvent_t e : part_events) cudaEventDestroy(e);
        for (cudaEvent_t e : input_events) cudaEventDestroy(e);
        for (cudaEvent_t e : copy_events)
            if (e) cudaEventDestroy(e);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        sb.reset();
        gs.reset();
        for (void *p : scratch) dev_free(p);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

static thread_local std::string g_create_error;

namespace dpf {
// message for dpf_last_error(NULL) from entry points that have no handle
void set_global_error(const std::string &msg) { g_create_error = msg; }

// allocation accounting and the one-shot injected failure (k-th following allocation)
static std::atomic<long long> g_fail_in{-1}, g_made{0}, g_live{0};

static bool injected_failure() {
    long long k = g_fail_in.load();
    while (k >= 0)
        if (g_fail_in.compare_exchange_weak(k, k - 1)) return k == 0;
    return false;
}

cudaError_t dev_malloc(void **p, size_t bytes) {
    *p = nullptr;
    if (injected_failure()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) { g_made++; g_live++; }
    return e;
}

cudaError_t host_malloc(void **p, size_t bytes) {
    *p = nullptr;
    if (injected_failure()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMallocHost(p, bytes);
    if (e == cudaSuccess) { g_made++; g_live++; }
    return e;
}

void dev_free(void *p) {
    if (!p) return;
    cudaFree(p);
    g_live--;
}

void host_free(void *p) {
    if (!p) return;
    cudaFreeHost(p);
    g_live--;
}
}  // namespace dpf

namespace dpf {
static std::vector<CheckReader> &check_readers() {
    static std::vector<CheckReader> r;
    return r;
}
void register_check_reader(CheckReader f) { check_readers().push_back(f); }
}  // namespace dpf

extern "C" int dpf_debug_check_report(int64_t *violations, int64_t *first) {
#if DPF_CHECKED
    long long total = 0, f0[3] = {0, 0, 0};
    bool have = false;
    for (dpf::CheckReader rd : dpf::check_readers()) {
        long long c = 0, f[3] = {0, 0, 0};
        if (rd(&c, f) != 0) {
            dpf::set_global_error("reading the check words failed");
            return DPF_CUDA;
        }
        if (c > 0 && !have) {
            have = true;
            for (int k = 0; k < 3; k++) f0[k] = f[k];
        }
        total += c;
    }
    if (violations) *violations = total;
    if (first)
        for (int k = 0; k < 3; k++) first[k] = f0[k];
    return DPF_OK;
#else
    (void)violations;
    (void)first;
    dpf::set_global_error("the library was built without DPF_CHECK");
    return DPF_UNSUPPORTED;
#endif
}

extern "C" void dpf_debug_fail_alloc(int64_t k) { dpf::g_fail_in.store(k < 0 ? -1 : (long long)k); }

extern "C" void dpf_debug_alloc_stats(int64_t *made, int64_t *live) {
    if (made) *made = dpf::g_made.load();
    if (live) *live = dpf::g_live.load();
}

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) { prev = -1; cudaGetLastError(); return; }
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e), e);
    }
}

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// copy n elements into the device buffer dst unless src already is device memory
template <typename T>
const T *stage_in(dpf_problem *P, const T *src, size_t n, T *dst) {
    if (!src) return nullptr;
    if (is_device_ptr(src)) {
        if (dst && dst != src) ck(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, P->stream),
                                  "copy in");
        return dst ? dst : src;
    }
    ck(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, P->stream), "host to device");
    return dst;
}

template <typename T>
void stage_out(dpf_problem *P, T *dst, const T *src, size_t n) {
    if (!dst) return;
    ck(cudaMemcpyAsync(dst, src, n * sizeof(T),
                       is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream),
       "copy out");
}

// n indices from a host or device array; a device array is read with one copy on the handle's
// stream, so it is ordered after the work the caller issued there
std::vector<int64_t> read_indices(dpf_problem *P, const int64_t *idx, int64_t n) {
    std::vector<int64_t> out(n > 0 ? n : 0);
    if (n <= 0) return out;
    if (is_device_ptr(idx)) {
        ck(cudaMemcpyAsync(out.data(), idx, n * sizeof(int64_t), cudaMemcpyDeviceToHost, P->stream), "indices");
        ck(cudaStreamSynchronize(P->stream), "indices");
    } else {
        std::memcpy(out.data(), idx, n * sizeof(int64_t));
    }
    return out;
}

template <typename T>
T *scratch(dpf_problem *P, size_t n) {
    void *p = nullptr;
    if (dev_malloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        throw OomError("device allocation failed");
    }
    P->scratch.push_back(p);
    return (T *)p;
}

void release(dpf_problem *P, void *p) {
    auto it = std::find(P->scratch.begin(), P->scratch.end(), p);
    if (it != P->scratch.end()) {
        dev_free(p);
        P->scratch.erase(it);
    }
}

int check_device() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return DPF_NO_DEVICE;
    }
    return DPF_OK;
}

template <typename F>
int guarded(dpf_problem *P, const char *name, F &&f) {
    if (!P) return DPF_BAD_INPUT;
    if (!P->parts.empty()) {
        P->err = std::string(name) + " is not available on a batch handle split into concurrent parts "
                                     "(create it with streams = 1)";
        return DPF_UNSUPPORTED;
    }
    NvtxRange range(name);
    DeviceGuard g(P->device);
    try {
        int rc = f();
        if (rc == DPF_OK) ck(cudaStreamSynchronize(P->stream), "stream synchronize");
        return rc;
    } catch (const DpfError &e) {
        P->err = e.what();
        return e.code;
    } catch (const std::exception &e) {
        P->err = e.what();
        return DPF_CUDA;
    }
}

int gs_status(dpf_problem *P, int rc) {
    if (rc != DPF_OK) P->err = P->gs->last_message.empty() ? "general-topology solve failed" : P->gs->last_message;
    return rc;
}

int solver_status(dpf_problem *P, StructBatch &S) {
    if (S.last_status != DPF_OK) {
        P->err = S.last_message.empty() ? (S.last_status == DPF_NOT_CONVERGED ? "CG did not converge within maxiter"
                                                                               : "non-finite residual")
                                        : S.last_message;
    }
    return S.last_status;
}

bool regular_faces_match(int64_t N, int64_t F, const int64_t *a, const int64_t *b, const double *aol, int nx, int ny,
                         int nz, double *aol3) {
    if ((int64_t)nx * ny * nz != N) return false;
    int64_t Fexp = 3LL * nx * ny * nz - (int64_t)nx * ny - (int64_t)nx * nz - (int64_t)ny * nz;
    if (Fexp != F) return false;
    const int64_t st[3] = {(int64_t)ny * nz, nz, 1};
    bool seen[3] = {false, false, false};
    int64_t f = 0;
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++)
            for (int iz = 0; iz < nz; iz++) {
                int64_t i = ((int64_t)ix * ny + iy) * nz + iz;
                const int co[3] = {ix, iy, iz};
                const int nn[3] = {nx, ny, nz};
                for (int d = 0; d < 3; d++) {
                    if (co[d] + 1 >= nn[d]) continue;
                    if (f >= F || a[f] != i || b[f] != i + st[d]) return false;
                    if (!seen[d]) { aol3[d] = aol[f]; seen[d] = true; }
                    else if (aol[f] != aol3[d]) return false;
                    f++;
                }
            }
    for (int d = 0; d < 3; d++) if (!seen[d]) aol3[d] = 1.0;
    return f == F;
}

dpf_options fill_options(const dpf_options *o) {
    dpf_options d;
    dpf_default_options(&d);
    if (!o) return d;
    dpf_options r = *o;
    if (!(r.reltol > 0)) r.reltol = d.reltol;
    if (r.maxiter <= 0) r.maxiter = d.maxiter;
    if (r.cheb_degree < 0) r.cheb_degree = d.cheb_degree;  // 0: the path's own default
    if (!(r.cheb_lo > 0 && r.cheb_lo < 1)) r.cheb_lo = d.cheb_lo;
    if (!(r.coarse_scale >= 0)) r.coarse_scale = d.coarse_scale;  // 0: the path's own default
    if (r.max_coarse <= 0) r.max_coarse = d.max_coarse;
    if (r.max_outer <= 0) r.max_outer = d.max_outer;
    if (r.check_every <= 0) r.check_every = d.check_every;
    if (r.blocks_per_sm <= 0) r.blocks_per_sm = d.blocks_per_sm;
    if (r.tail_cells == 0) r.tail_cells = d.tail_cells;
    if (r.plane == 0) r.plane = d.plane;
    if (r.plane_cells <= 0) r.plane_cells = d.plane_cells;
    r.plane_cells = std::min(4, std::max(1, (r.plane_cells + 255) / 256)) * 256;
    if (r.plane_blocks_per_sm <= 0) r.plane_blocks_per_sm = d.plane_blocks_per_sm;
    if (r.df_plane_cells == 0) r.df_plane_cells = d.df_plane_cells;
    if (r.df_plane_cells > 0) r.df_plane_cells = 256;  // one cell per thread: the product's only slab size
    if (r.df_plane_blocks_per_sm <= 0) r.df_plane_blocks_per_sm = d.df_plane_blocks_per_sm;
    if (r.tail_cluster <= 0) r.tail_cluster = d.tail_cluster;
    r.tail_cluster = std::min(16, r.tail_cluster);
    if (r.plane_levels < 0) r.plane_levels = d.plane_levels;
    if (r.streams < 0) r.streams = d.streams;
    if (r.fuse == 0) r.fuse = d.fuse;
    if (r.solver != DPF_SOLVER_CHOLESKY) r.solver = DPF_SOLVER_CG;
    return r;
}

// The number of concurrent parts of a batch: `streams` parts (at most one per problem) when
// streams > 1, else one. Each part is a complete batch handle on its own non-blocking stream,
// driven by its own host thread, so one part's bandwidth-bound finest-level kernels run while
// another part is in its latency-bound small levels.
int batch_parts(int nprob, int streams) {
    if (streams <= 1) return 1;
    return std::min(streams, nprob);
}

int make_struct(const std::vector<GridSpec> &grids, const std::vector<std::vector<int64_t>> &dn,
                const dpf_options *opts, dpf_problem **out) {
    if (!out) return DPF_BAD_INPUT;
    *out = nullptr;
    int rc = check_device();
    if (rc) { g_create_error = "no CUDA device"; return rc; }
    NvtxRange range("dpf_create (regular grids)");
    auto P = new dpf_problem();
    try {
        ck(cudaGetDevice(&P->device), "cudaGetDevice");
        P->opt = fill_options(opts);
        const int nprob = (int)grids.size();
        const int k = batch_parts(nprob, P->opt.streams);
        if (k > 1) {
            // concurrent parts: runs of consecutive problems (sizes differing by at most one),
            // each its own handle and stream
            dpf_options po = P->opt;
            po.streams = 1;
            int first = 0;
            for (int i = 0; i < k; i++) {
                const int cnt = nprob / k + (i < nprob % k ? 1 : 0);
                auto Q = new dpf_problem();
                P->parts.push_back(Q);  // owned by P from here on (deleted with it on any error)
                Q->device = P->device;
                Q->opt = po;
                ck(cudaStreamCreateWithFlags(&Q->stream, cudaStreamNonBlocking), "part stream");
                Q->own_stream = true;
                std::vector<GridSpec> g(grids.begin() + first, grids.begin() + first + cnt);
                std::vector<std::vector<int64_t>> d(dn.begin() + first, dn.begin() + first + cnt);
                Q->sb.reset(new StructBatch(g, d, Q->opt, Q->stream));
                P->part_first.push_back(first);
                first += cnt;
            }
            P->part_first.push_back(nprob);
            for (int i = 0; i <= k; i++) {
                cudaEvent_t e;
                ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "part event");
                P->part_events.push_back(e);
            }
            for (int i = 0; i < k; i++) {
                cudaEvent_t e;
                ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "part event");
                P->input_events.push_back(e);
            }
            P->pool.reset(new PartPool(k, P->device));
        } else {
            P->sb.reset(new StructBatch(grids, dn, P->opt, P->stream));
        }
    } catch (const DpfError &e) {
        g_create_error = e.what();
        delete P;
        return e.code;
    } catch (const std::exception &e) {
        g_create_error = e.what();
        delete P;
        return DPF_CUDA;
    }
    *out = P;
    return DPF_OK;
}

}  // namespace

extern "C" {

void dpf_default_options(dpf_options *o) {
    if (!o) return;
    o->reltol = 1e-10;
    o->maxiter = 500;
    o->precision = DPF_PREC_FP64;
    o->cheb_degree = 0;
    o->cheb_lo = 0.2;
    o->coarse_scale = 0.0;
    o->max_coarse = 64;
    o->max_outer = 6;
    o->use_graphs = 1;
    o->check_every = 1;
    o->blocks_per_sm = 16;
    o->tail_cells = 4096;
    o->plane = 1;
    o->plane_cells = 1024;
    o->plane_blocks_per_sm = 2;
    o->df_plane_cells = 256;
    o->df_plane_blocks_per_sm = 8;
    o->tail_cluster = 1;
    o->plane_levels = 0;
    o->streams = 0;
    o->fuse = -1;
    o->solver = DPF_SOLVER_CG;
}

int dpf_detect_regular3d(int64_t N, int64_t F, const int64_t *a, const int64_t *b, const double *aol, int *dims,
                         double *aol3) {
    if (N <= 0 || F < 0 || (F > 0 && (!a || !b || !aol))) return 0;
    // candidate strides are the distinct values of b - a; z fastest, then y, then x
    std::vector<int64_t> offs;
    for (int64_t f = 0; f < F && offs.size() < 4; f++) {
        int64_t d = b[f] - a[f];
        if (std::find(offs.begin(), offs.end(), d) == offs.end()) offs.push_back(d);
    }
    if (offs.size() > 3) return 0;
    std::sort(offs.begin(), offs.end());
    // enumerate assignments of the observed strides to (sz=1, sy=nz, sx=ny*nz)
    std::vector<std::array<int, 3>> cands;
    auto try_dims = [&](int64_t nx, int64_t ny, int64_t nz) {
        if (nx < 1 || ny < 1 || nz < 1 || nx * ny * nz != N) return;
        if (nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30)) return;
        cands.push_back({(int)nx, (int)ny, (int)nz});
    };
    if (F == 0) {
        try_dims(N, 1, 1);
    }
    for (int64_t sy : {(int64_t)0, (int64_t)1}) (void)sy;
    // stride values tell nz (sy) and ny*nz (sx); a missing stride means that dimension is 1
    std::vector<int64_t> cand_nz = {1}, cand_nynz = {};
    for (int64_t d : offs) { if (d > 1) cand_nz.push_back(d); }
    for (int64_t nzv : cand_nz) {
        std::vector<int64_t> nyz = {nzv};
        for (int64_t d : offs) if (d > nzv && d % nzv == 0) nyz.push_back(d);
        for (int64_t nynz : nyz) {
            if (nynz % nzv) continue;
            int64_t ny = nynz / nzv;
            if (N % nynz) continue;
            try_dims(N / nynz, ny, nzv);
            // the y dimension may be absent while x spans the rest
        }
        if (N % nzv == 0) try_dims(1, N / nzv, nzv);
    }
    try_dims(1, 1, N);
    try_dims(1, N, 1);
    try_dims(N, 1, 1);
    for (auto &c : cands) {
        double a3[3];
        if (regular_faces_match(N, F, a, b, aol, c[0], c[1], c[2], a3)) {
            if (dims) { dims[0] = c[0]; dims[1] = c[1]; dims[2] = c[2]; }
            if (aol3) { aol3[0] = a3[0]; aol3[1] = a3[1]; aol3[2] = a3[2]; }
            return 1;
        }
    }
    return 0;
}

static int create_faces(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b, const double *aol,
                        const double *volumes, int64_t nd, const int64_t *dn, const dpf_options *opts,
                        dpf_problem **out, bool detect_regular);

int dpf_create(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b, const double *aol,
               const double *volumes, int64_t nd, const int64_t *dn, const dpf_options *opts, dpf_problem **out) {
    return create_faces(N, F, nbr_a, nbr_b, aol, volumes, nd, dn, opts, out, true);
}

int dpf_create_general(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b, const double *aol,
                       const double *volumes, int64_t nd, const int64_t *dn, const dpf_options *opts,
                       dpf_problem **out) {
    return create_faces(N, F, nbr_a, nbr_b, aol, volumes, nd, dn, opts, out, false);
}

static int create_faces(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b, const double *aol,
                        const double *volumes, int64_t nd, const int64_t *dn, const dpf_options *opts,
                        dpf_problem **out, bool detect_regular) {
    if (!out || N <= 0 || F < 0 || nd < 0 || (F > 0 && (!nbr_a || !nbr_b || !aol)) || (nd > 0 && !dn)) {
        g_create_error = "invalid arguments";
        return DPF_BAD_INPUT;
    }
    for (int64_t f = 0; f < F; f++)
        if (nbr_a[f] < 0 || nbr_a[f] >= N || nbr_b[f] < 0 || nbr_b[f] >= N || nbr_a[f] == nbr_b[f]) {
            g_create_error = "neighbor index out of range (indices are 0-based)";
            return DPF_BAD_INPUT;
        }
    for (int64_t k = 0; k < nd; k++)
        if (dn[k] < 0 || dn[k] >= N) {
            g_create_error = "Dirichlet node index out of range (indices are 0-based)";
            return DPF_BAD_INPUT;
        }
    int dims[3];
    double aol3[3];
    bool uniform_vol = true;
    if (volumes)
        for (int64_t i = 1; i < N; i++) if (volumes[i] != volumes[0]) { uniform_vol = false; break; }
    if (detect_regular && uniform_vol && dpf_detect_regular3d(N, F, nbr_a, nbr_b, aol, dims, aol3)) {
        GridSpec g;
        for (int k = 0; k < 3; k++) { g.n[k] = dims[k]; g.mins[k] = 0; g.maxs[k] = dims[k] - 1; g.aol[k] = aol3[k]; }
        g.aol_override = true;
        g.vol_override = true;
        g.vol = volumes ? volumes[0] : 1.0;
        std::vector<GridSpec> gs{g};
        std::vector<std::vector<int64_t>> d{std::vector<int64_t>(dn, dn + nd)};
        return make_struct(gs, d, opts, out);
    }
    // general (CSR) path
    *out = nullptr;
    int rc = check_device();
    if (rc) { g_create_error = "no CUDA device"; return rc; }
    NvtxRange range("dpf_create (face list)");
    auto P = new dpf_problem();
    try {
        ck(cudaGetDevice(&P->device), "cudaGetDevice");
        P->opt = fill_options(opts);
        P->gs.reset(new GeneralSolver(N, F, nbr_a, nbr_b, aol, volumes, nd, dn, P->opt, P->stream));
    } catch (const DpfError &e) {
        g_create_error = e.what();
        delete P;
        return e.code;
    } catch (const std::exception &e) {
        g_create_error = e.what();
        delete P;
        return DPF_CUDA;
    }
    *out = P;
    return DPF_OK;
}

int dpf_create_regular3d(int nx, int ny, int nz, const double *mins, const double *maxs, int64_t nd,
                         const int64_t *dn, const dpf_options *opts, dpf_problem **out) {
    if (!out || !mins || !maxs || nx < 1 || ny < 1 || nz < 1 || nd < 0 || (nd > 0 && !dn)) {
        g_create_error = "invalid arguments";
        return DPF_BAD_INPUT;
    }
    GridSpec g;
    g.n[0] = nx; g.n[1] = ny; g.n[2] = nz;
    for (int k = 0; k < 3; k++) { g.mins[k] = mins[k]; g.maxs[k] = maxs[k]; }
    std::vector<GridSpec> gs{g};
    std::vector<std::vector<int64_t>> d{std::vector<int64_t>(dn, dn + nd)};
    return make_struct(gs, d, opts, out);
}

int dpf_batch_create(int nprob, const int *dims, const double *mins, const double *maxs, const int64_t *nd,
                     const int64_t *dn, const dpf_options *opts, dpf_problem **out) {
    if (!out || nprob <= 0 || !dims || !mins || !maxs || !nd) {
        g_create_error = "invalid arguments";
        return DPF_BAD_INPUT;
    }
    std::vector<GridSpec> gs(nprob);
    std::vector<std::vector<int64_t>> d(nprob);
    int64_t k = 0;
    for (int p = 0; p < nprob; p++) {
        for (int j = 0; j < 3; j++) {
            gs[p].n[j] = dims[3 * p + j];
            gs[p].mins[j] = mins[3 * p + j];
            gs[p].maxs[j] = maxs[3 * p + j];
        }
        if (nd[p] < 0 || (nd[p] > 0 && !dn)) { g_create_error = "invalid Dirichlet counts"; return DPF_BAD_INPUT; }
        d[p].assign(dn + k, dn + k + nd[p]);
        k += nd[p];
    }
    return make_struct(gs, d, opts, out);
}

void dpf_destroy(dpf_problem *P) {
    if (!P) return;
    DeviceGuard g(P->device);
    cudaStreamSynchronize(P->stream);
    delete P;
}

const char *dpf_last_error(const dpf_problem *P) {
    if (!P) return g_create_error.c_str();
    return P->err.c_str();
}

int dpf_info(const dpf_problem *P, int64_t *N, int64_t *F, int64_t *nfree, int *structured, int *levels) {
    if (!P) return DPF_BAD_INPUT;
    if (!P->parts.empty()) {
        int64_t n = 0, f = 0, nf = 0;
        int lv = 0;
        for (const dpf_problem *Q : P->parts) {
            n += Q->sb->N;
            f += Q->sb->F;
            nf += Q->sb->nfree_total;
            lv = std::max(lv, Q->sb->nlev_max);
        }
        if (N) *N = n;
        if (F) *F = f;
        if (nfree) *nfree = nf;
        if (structured) *structured = 1;
        if (levels) *levels = lv;
        return DPF_OK;
    }
    if (P->sb) {
        if (N) *N = P->sb->N;
        if (F) *F = P->sb->F;
        if (nfree) *nfree = P->sb->nfree_total;
        if (structured) *structured = 1;
        if (levels) *levels = P->sb->nlev_max;
    } else {
        if (N) *N = P->gs->N;
        if (F) *F = P->gs->F;
        if (nfree) *nfree = P->gs->nfree;
        if (structured) *structured = 0;
        if (levels) *levels = P->gs->nlevels();
    }
    return DPF_OK;
}

int dpf_last_stats(const dpf_problem *P, int *iterations, int *outer, double *relres) {
    if (!P) return DPF_BAD_INPUT;
    if (!P->parts.empty()) {
        int it = 0, ou = 0;
        double rr = 0.0;
        for (const dpf_problem *Q : P->parts) {
            it = std::max(it, Q->sb->stats_iters);
            ou = std::max(ou, Q->sb->stats_outer);
            rr = std::max(rr, Q->sb->stats_relres);
        }
        if (iterations) *iterations = it;
        if (outer) *outer = ou;
        if (relres) *relres = rr;
        return DPF_OK;
    }
    if (P->sb) {
        if (iterations) *iterations = P->sb->stats_iters;
        if (outer) *outer = P->sb->stats_outer;
        if (relres) *relres = P->sb->stats_relres;
    } else {
        if (iterations) *iterations = P->gs->stats_iters;
        if (outer) *outer = P->gs->stats_outer;
        if (relres) *relres = P->gs->stats_relres;
    }
    return DPF_OK;
}

// ------------------------------------------------------------- steady state
int dpf_steady_forward(dpf_problem *P, const double *Ks, const double *dh, const double *Qs, double *h_out) {
    return guarded(P, __func__, [&]() -> int {
        if (!Ks || !dh || !Qs) throw BadInput("Ks, dirichleths and Qs are required");
        if (P->gs) return gs_status(P, P->gs->forward(Ks, nullptr, 0, dh, Qs, h_out));
        StructBatch &S = *P->sb;
        stage_in(P, Ks, S.F, S.in_Ks);
        stage_in(P, dh, S.N, S.in_dh);
        stage_in(P, Qs, S.N, S.in_Q);
        S.forward(S.in_Ks, nullptr, 0);
        stage_out(P, h_out, S.h, S.N);
        return solver_status(P, S);
    });
}

int dpf_steady_forward_logk(dpf_problem *P, const double *logK, int kind, const double *dh, const double *Qs,
                            double *h_out) {
    return guarded(P, __func__, [&]() -> int {
        if (!logK || !dh || !Qs) throw BadInput("logK, dirichleths and Qs are required");
        if (kind != DPF_MEAN_GEOMETRIC && kind != DPF_MEAN_HARMONIC) throw BadInput("unknown mean kind");
        if (P->gs) return gs_status(P, P->gs->forward(nullptr, logK, kind, dh, Qs, h_out));
        StructBatch &S = *P->sb;
        stage_in(P, logK, S.N, S.in_logK);
        stage_in(P, dh, S.N, S.in_dh);
        stage_in(P, Qs, S.N, S.in_Q);
        S.forward(nullptr, S.in_logK, kind);
        stage_out(P, h_out, S.h, S.N);
        return solver_status(P, S);
    });
}

int dpf_steady_adjoint(dpf_problem *P, const double *delta, double *dKs, double *ddh, double *dQs) {
    return guarded(P, __func__, [&]() -> int {
        if (!delta) throw BadInput("delta is required");
        if (P->gs) return gs_status(P, P->gs->adjoint(delta, dKs, nullptr, ddh, dQs));
        StructBatch &S = *P->sb;
        if (!S.have_forward) { P->err = "adjoint called before a forward solve"; return DPF_STATE; }
        stage_in(P, delta, S.N, S.delta);
        S.adjoint_solve();
        int rc = solver_status(P, S);
        if (dKs) {
            double *tmp = is_device_ptr(dKs) ? dKs : scratch<double>(P, S.F);
            S.grad_faces(S.h, S.lam, tmp, false);
            if (tmp != dKs) { stage_out(P, dKs, tmp, S.F); ck(cudaStreamSynchronize(P->stream), "sync"); release(P, tmp); }
        }
        if (ddh || dQs) {
            double *t1 = ddh ? (is_device_ptr(ddh) ? ddh : scratch<double>(P, S.N)) : nullptr;
            double *t2 = dQs ? (is_device_ptr(dQs) ? dQs : scratch<double>(P, S.N)) : nullptr;
            S.grad_dh_q(S.lam, t1, t2, true, false);
            if (t1 && t1 != ddh) stage_out(P, ddh, t1, S.N);
            if (t2 && t2 != dQs) stage_out(P, dQs, t2, S.N);
            ck(cudaStreamSynchronize(P->stream), "sync");
            if (t1 && t1 != ddh) release(P, t1);
            if (t2 && t2 != dQs) release(P, t2);
        }
        return rc;
    });
}

int dpf_steady_adjoint_logk(dpf_problem *P, const double *delta, double *dlogK, double *ddh, double *dQs) {
    return guarded(P, __func__, [&]() -> int {
        if (!delta) throw BadInput("delta is required");
        if (P->gs) return gs_status(P, P->gs->adjoint(delta, nullptr, dlogK, ddh, dQs));
        StructBatch &S = *P->sb;
        if (!S.have_forward || S.fwd_kind != 1) {
            P->err = "dpf_steady_adjoint_logk needs a preceding dpf_steady_forward_logk";
            return DPF_STATE;
        }
        stage_in(P, delta, S.N, S.delta);
        S.adjoint_solve();
        int rc = solver_status(P, S);
        if (dlogK) {
            double *tmp = is_device_ptr(dlogK) ? dlogK : S.r64;
            S.grad_logk(tmp);
            if (tmp != dlogK) stage_out(P, dlogK, tmp, S.N);
        }
        if (ddh || dQs) {
            double *t1 = ddh ? (is_device_ptr(ddh) ? ddh : scratch<double>(P, S.N)) : nullptr;
            double *t2 = dQs ? (is_device_ptr(dQs) ? dQs : scratch<double>(P, S.N)) : nullptr;
            S.grad_dh_q(S.lam, t1, t2, true, false);
            if (t1 && t1 != ddh) stage_out(P, ddh, t1, S.N);
            if (t2 && t2 != dQs) stage_out(P, dQs, t2, S.N);
            ck(cudaStreamSynchronize(P->stream), "sync");
            if (t1 && t1 != ddh) release(P, t1);
            if (t2 && t2 != dQs) release(P, t2);
        }
        return rc;
    });
}

int dpf_logk_to_faces(dpf_problem *P, const double *logK, int kind, double *Ks) {
    return guarded(P, __func__, [&]() -> int {
        if (!logK || !Ks) throw BadInput("logK and Ks are required");
        if (kind != DPF_MEAN_GEOMETRIC && kind != DPF_MEAN_HARMONIC) throw BadInput("unknown mean kind");
        if (P->gs) return gs_status(P, P->gs->logk_to_faces(logK, kind, Ks));
        StructBatch &S = *P->sb;
        stage_in(P, logK, S.N, S.in_logK);
        double *tmp = is_device_ptr(Ks) ? Ks : S.in_Ks;
        S.logk_to_faces(S.in_logK, kind, tmp);
        if (tmp != Ks) stage_out(P, Ks, tmp, S.F);
        return DPF_OK;
    });
}

int dpf_logk_to_faces_vjp(dpf_problem *P, const double *logK, int kind, const double *dKs, double *dlogK) {
    return guarded(P, __func__, [&]() -> int {
        if (!logK || !dKs || !dlogK) throw BadInput("logK, dKs and dlogK are required");
        if (kind != DPF_MEAN_GEOMETRIC && kind != DPF_MEAN_HARMONIC) throw BadInput("unknown mean kind");
        if (P->gs) return gs_status(P, P->gs->logk_vjp(logK, kind, dKs, dlogK));
        StructBatch &S = *P->sb;
        stage_in(P, logK, S.N, S.in_logK);
        double *dk = scratch<double>(P, S.F);
        stage_in(P, dKs, S.F, dk);
        double *tmp = is_device_ptr(dlogK) ? dlogK : S.r64;
        S.logk_vjp(S.in_logK, kind, dk, tmp);
        if (tmp != dlogK) stage_out(P, dlogK, tmp, S.N);
        ck(cudaStreamSynchronize(P->stream), "sync");
        release(P, dk);
        return DPF_OK;
    });
}

// forward + objective sum h[obs]^2 + adjoint to dlogK for every problem of the handle
static int solve_grad_common(dpf_problem *P, const double *logK, int kind, const double *dh, const double *Qs,
                             const std::vector<long long> &obs_global, double *h_out, double *dlogK) {
    StructBatch &S = *P->sb;
    stage_in(P, logK, S.N, S.in_logK);
    stage_in(P, dh, S.N, S.in_dh);
    stage_in(P, Qs, S.N, S.in_Q);
    S.forward(nullptr, S.in_logK, kind);
    int rc = solver_status(P, S);
    if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) return rc;
    long long *d_obs = S.obs_buffer(obs_global.size());
    if (!obs_global.empty())
        ck(cudaMemcpyAsync(d_obs, obs_global.data(), obs_global.size() * sizeof(long long), cudaMemcpyHostToDevice,
                           P->stream),
           "obs");
    S.obs_delta(d_obs, (long long)obs_global.size());
    // heads to a host buffer: copied on the handle's copy stream while the adjoint runs (the
    // adjoint and the gradient only read S.h); the handle's stream waits for the copy before
    // anything after this call can overwrite S.h, and the copy is complete when this returns
    struct CopyJoin {
        dpf_problem *P;
        bool pending = false;
        ~CopyJoin() {
            if (pending) cudaStreamSynchronize(P->copy_stream);  // an error path: the caller's buffer is settled
        }
    } join{P};
    if (h_out && !is_device_ptr(h_out)) {
        if (!P->copy_stream) {
            ck(cudaStreamCreateWithFlags(&P->copy_stream, cudaStreamNonBlocking), "copy stream");
            for (cudaEvent_t &e : P->copy_events) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event");
        }
        ck(cudaEventRecord(P->copy_events[0], P->stream), "event record");
        ck(cudaStreamWaitEvent(P->copy_stream, P->copy_events[0], 0), "stream wait");
        join.pending = true;
        ck(cudaMemcpyAsync(h_out, S.h, S.N * sizeof(double), cudaMemcpyDeviceToHost, P->copy_stream), "copy out");
        ck(cudaEventRecord(P->copy_events[1], P->copy_stream), "event record");
    } else {
        stage_out(P, h_out, S.h, S.N);
    }
    S.adjoint_solve();
    int rc2 = solver_status(P, S);
    if (dlogK) {
        double *tmp = is_device_ptr(dlogK) ? dlogK : S.r64;
        S.grad_logk(tmp);
        if (tmp != dlogK) stage_out(P, dlogK, tmp, S.N);
    }
    if (join.pending) {
        ck(cudaStreamWaitEvent(P->stream, P->copy_events[1], 0), "stream wait");
        join.pending = false;
    }
    ck(cudaStreamSynchronize(P->stream), "sync");
    return rc != DPF_OK ? rc : rc2;
}

int dpf_solve_grad_logk(dpf_problem *P, const double *logK, int kind, const double *dh, const double *Qs,
                        int64_t nobs, const int64_t *obs, double *h_out, double *dlogK) {
    return guarded(P, __func__, [&]() -> int {
        if (!logK || !dh || !Qs || nobs < 0 || (nobs > 0 && !obs)) throw BadInput("invalid arguments");
        if (kind != DPF_MEAN_GEOMETRIC && kind != DPF_MEAN_HARMONIC) throw BadInput("unknown mean kind");
        if (P->gs) return gs_status(P, P->gs->solve_grad_logk(logK, kind, dh, Qs, nobs, obs, h_out, dlogK));
        StructBatch &S = *P->sb;
        if (S.nprob != 1) throw BadInput("use dpf_batch_solve_grad_logk for a batch");
        std::vector<long long> og(nobs);
        const std::vector<int64_t> ho = read_indices(P, obs, nobs);
        for (int64_t k = 0; k < nobs; k++) {
            if (ho[k] < 0 || ho[k] >= S.N) throw BadInput("observation index out of range");
            og[k] = ho[k];
        }
        return solve_grad_common(P, logK, kind, dh, Qs, og, h_out, dlogK);
    });
}

// cells and faces of the problems before part i of a split batch
static void part_base(const dpf_problem *P, int i, int64_t &c0, int64_t &f0) {
    c0 = f0 = 0;
    for (int j = 0; j < i; j++) {
        c0 += P->parts[j]->sb->N;
        f0 += P->parts[j]->sb->F;
    }
}

int dpf_batch_offsets(const dpf_problem *P, int p, int64_t *cell_offset, int64_t *face_offset) {
    if (P && !P->parts.empty()) {
        const int k = (int)P->parts.size();
        if (p < 0 || p > P->part_first[k]) return DPF_BAD_INPUT;
        int i = 0;
        while (i + 1 < k && p >= P->part_first[i + 1]) i++;
        int64_t c0, f0;
        part_base(P, i, c0, f0);
        const StructBatch &S = *P->parts[i]->sb;
        if (cell_offset) *cell_offset = c0 + S.cell_off[p - P->part_first[i]];
        if (face_offset) *face_offset = f0 + S.face_off[p - P->part_first[i]];
        return DPF_OK;
    }
    if (!P || !P->sb || p < 0 || p > P->sb->nprob) return DPF_BAD_INPUT;
    if (cell_offset) *cell_offset = P->sb->cell_off[p];
    if (face_offset) *face_offset = P->sb->face_off[p];
    return DPF_OK;
}

// A split batch: every part solves its problems on its own stream from its own host thread.
// The parts start after the work already on the handle's stream and that stream continues
// after all of them; the status is the most severe of the parts' (its part's message).
static int split_solve_grad_logk(dpf_problem *P, const double *logK, int kind, const double *dh, const double *Qs,
                                 const int64_t *obs_offsets, const int64_t *obs, double *h_out, double *dlogK) {
    NvtxRange range("dpf_batch_solve_grad_logk (concurrent parts)");
    DeviceGuard g(P->device);
    const int k = (int)P->parts.size();
    const int nprob = P->part_first[k];
    if (!dh || !Qs || !obs_offsets) { P->err = "invalid arguments"; return DPF_BAD_INPUT; }
    for (int p = 0; p < nprob; p++)
        if (obs_offsets[p] < 0 || obs_offsets[p + 1] < obs_offsets[p]) {
            P->err = "obs_offsets must be non-decreasing";
            return DPF_BAD_INPUT;
        }
    if (cudaEventRecord(P->part_events[k], P->stream) != cudaSuccess) {
        P->err = std::string("event record: ") + cudaGetErrorString(cudaGetLastError());
        return DPF_CUDA;
    }
    std::vector<int> rcs(k, DPF_OK);
    std::vector<std::vector<int64_t>> offs(k);
    // Inputs in host memory are copied here, part after part (each part's copies wait for the
    // previous part's), so the first part computes while the later parts' inputs are still in
    // flight instead of every part waiting for the whole batch's copies.
    std::vector<const double *> in_lk(k), in_dh(k), in_q(k);
    const bool lk_host = logK && !is_device_ptr(logK), dh_host = !is_device_ptr(dh), q_host = !is_device_ptr(Qs);
    for (int i = 0; i < k; i++) {
        dpf_problem *Q = P->parts[i];
        StructBatch &S = *Q->sb;
        int64_t c0, f0;
        part_base(P, i, c0, f0);
        in_lk[i] = logK ? (lk_host ? S.in_logK : logK + c0) : nullptr;
        if (lk_host) S.have_sampled = false;  // the input is staged over the drawn fields
        in_dh[i] = dh_host ? S.in_dh : dh + c0;
        in_q[i] = q_host ? S.in_Q : Qs + c0;
        cudaError_t e = cudaStreamWaitEvent(Q->stream, P->part_events[k], 0);
        if (e == cudaSuccess && (lk_host || dh_host || q_host)) {
            if (i > 0) e = cudaStreamWaitEvent(Q->stream, P->input_events[i - 1], 0);
            if (e == cudaSuccess && lk_host)
                e = cudaMemcpyAsync(S.in_logK, logK + c0, S.N * sizeof(double), cudaMemcpyHostToDevice, Q->stream);
            if (e == cudaSuccess && dh_host)
                e = cudaMemcpyAsync(S.in_dh, dh + c0, S.N * sizeof(double), cudaMemcpyHostToDevice, Q->stream);
            if (e == cudaSuccess && q_host)
                e = cudaMemcpyAsync(S.in_Q, Qs + c0, S.N * sizeof(double), cudaMemcpyHostToDevice, Q->stream);
            if (e == cudaSuccess) e = cudaEventRecord(P->input_events[i], Q->stream);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            P->err = std::string("part inputs: ") + cudaGetErrorString(e);
            // parts already started are drained before the caller may reuse its buffers
            for (int j = 0; j <= i; j++) cudaStreamSynchronize(P->parts[j]->stream);
            return DPF_CUDA;
        }
    }
    P->pool->run([&](int i) {
        dpf_problem *Q = P->parts[i];
        const int p0 = P->part_first[i], p1 = P->part_first[i + 1];
        int64_t c0, f0;
        part_base(P, i, c0, f0);
        offs[i].resize(p1 - p0 + 1);
        for (int p = p0; p <= p1; p++) offs[i][p - p0] = obs_offsets[p] - obs_offsets[p0];
        rcs[i] = dpf_batch_solve_grad_logk(Q, in_lk[i], kind, in_dh[i], in_q[i], offs[i].data(),
                                           obs ? obs + obs_offsets[p0] : nullptr, h_out ? h_out + c0 : nullptr,
                                           dlogK ? dlogK + c0 : nullptr);
        if (cudaEventRecord(P->part_events[i], Q->stream) != cudaSuccess) {
            Q->err = std::string("event record: ") + cudaGetErrorString(cudaGetLastError());
            if (rcs[i] == DPF_OK || rcs[i] == DPF_NOT_CONVERGED) rcs[i] = DPF_CUDA;
        }
    });
    int rc = DPF_OK;
    for (int i = 0; i < k; i++) {
        if (cudaStreamWaitEvent(P->stream, P->part_events[i], 0) != cudaSuccess) {
            P->err = std::string("stream wait: ") + cudaGetErrorString(cudaGetLastError());
            rc = DPF_CUDA;
        }
        if (rcs[i] != DPF_OK && (rc == DPF_OK || rc == DPF_NOT_CONVERGED)) {
            rc = rcs[i];
            P->err = P->parts[i]->err;
        }
    }
    return rc;
}

// Draws into part or handle Q's own field buffer, and copies to out (host or device) when given.
static int sample_into(dpf_problem *Q, int nmodes, const uint64_t *seeds, const double *ell, const double *sigma,
                       const double *mean, double *out) {
    return guarded(Q, "dpf_batch_sample_logk", [&]() -> int {
        StructBatch &S = *Q->sb;
        static_assert(sizeof(uint64_t) == sizeof(unsigned long long), "seed width");
        const bool direct = out && is_device_ptr(out);
        S.have_sampled = false;
        S.sample_logk(nmodes, (const unsigned long long *)seeds, ell, sigma, mean, direct ? out : S.in_logK);
        if (!direct) {
            S.have_sampled = true;
            if (out) stage_out(Q, out, S.in_logK, S.N);
        }
        return DPF_OK;
    });
}

int dpf_batch_sample_logk(dpf_problem *P, int nmodes, const uint64_t *seeds, const double *ell, const double *sigma,
                          const double *mean, double *logK) {
    if (!P) return DPF_BAD_INPUT;
    if (!seeds || !ell || !sigma || !mean) {
        P->err = "seeds, ell, sigma and mean are required (one per problem)";
        return DPF_BAD_INPUT;
    }
    if (P->gs) {
        P->err = "the sampler needs a regular-grid handle";
        return DPF_UNSUPPORTED;
    }
    if (P->parts.empty()) return sample_into(P, nmodes, seeds, ell, sigma, mean, logK);
    DeviceGuard g(P->device);
    for (size_t i = 0; i < P->parts.size(); i++) {
        const int p0 = P->part_first[i];
        int64_t c0, f0;
        part_base(P, (int)i, c0, f0);
        const int rc = sample_into(P->parts[i], nmodes, seeds + p0, ell + p0, sigma + p0, mean + p0,
                                   logK ? logK + c0 : nullptr);
        if (rc != DPF_OK) {
            P->err = P->parts[i]->err;
            return rc;
        }
    }
    return DPF_OK;
}

int dpf_batch_solve_grad_logk(dpf_problem *P, const double *logK, int kind, const double *dh, const double *Qs,
                              const int64_t *obs_offsets, const int64_t *obs, double *h_out, double *dlogK) {
    if (P && !P->parts.empty()) return split_solve_grad_logk(P, logK, kind, dh, Qs, obs_offsets, obs, h_out, dlogK);
    return guarded(P, __func__, [&]() -> int {
        if (!P->sb) throw BadInput("not a batch handle");
        if (!dh || !Qs || !obs_offsets) throw BadInput("invalid arguments");
        if (kind != DPF_MEAN_GEOMETRIC && kind != DPF_MEAN_HARMONIC) throw BadInput("unknown mean kind");
        StructBatch &S = *P->sb;
        if (!logK) {
            // the fields last drawn into the handle by dpf_batch_sample_logk
            if (!S.have_sampled) {
                P->err = "logK is NULL but no fields were drawn into the handle (dpf_batch_sample_logk)";
                return DPF_STATE;
            }
            logK = S.in_logK;
        } else if (logK != S.in_logK) {
            S.have_sampled = false;  // the input is staged over the drawn fields
        }
        std::vector<long long> og;
        for (int p = 0; p < S.nprob; p++) {
            int64_t a = obs_offsets[p], b = obs_offsets[p + 1];
            if (a < 0 || b < a) throw BadInput("obs_offsets must be non-decreasing");
            for (int64_t k = a; k < b; k++) {
                int64_t loc = obs[k];
                if (loc < 0 || loc >= S.cell_off[p + 1] - S.cell_off[p]) throw BadInput("observation index out of range");
                og.push_back(S.cell_off[p] + loc);
            }
        }
        return solve_grad_common(P, logK, kind, dh, Qs, og, h_out, dlogK);
    });
}

int dpf_apply_operator(dpf_problem *P, const double *x, double *y) {
    return guarded(P, __func__, [&]() -> int {
        if (!x || !y) throw BadInput("x and y are required");
        if (P->gs) return gs_status(P, P->gs->apply(x, y));
        StructBatch &S = *P->sb;
        if (!S.have_operator) { P->err = "no operator assembled yet"; return DPF_STATE; }
        stage_in(P, x, S.N, S.r64);
        S.apply(S.r64, S.arhs);
        stage_out(P, y, S.arhs, S.N);
        return DPF_OK;
    });
}

// ---------------------------------------------------------------- transient
int dpf_transient_forward(dpf_problem *P, const double *Ks, const double *dh, const double *Qs, const double *Ss,
                          double dt, int nsteps, const double *h0, int checkpoint_every, double *states,
                          double *hT) {
    return guarded(P, __func__, [&]() -> int {
        if (!Ks || !dh || !Qs || !Ss || !h0 || nsteps <= 0 || !(dt > 0)) throw BadInput("invalid arguments");
        if (P->gs) return gs_status(P, P->gs->transient_forward(Ks, dh, Qs, Ss, dt, nsteps, h0, states, hT));
        StructBatch &S = *P->sb;
        int ck_every = checkpoint_every <= 0 ? 1 : std::min(checkpoint_every, nsteps);
        int nck = nsteps / ck_every + 1;
        // (re)allocate transient buffers
        for (double *&b : {std::ref(P->tr_b0), std::ref(P->tr_ck_states), std::ref(P->tr_seg), std::ref(P->tr_Ss)}) {
            if (b) { release(P, b); b = nullptr; }
        }
        P->tr_b0 = scratch<double>(P, S.N);
        P->tr_Ss = scratch<double>(P, S.N);
        P->tr_ck_states = scratch<double>(P, (size_t)nck * S.N);
        P->tr_seg = scratch<double>(P, (size_t)ck_every * S.N);
        P->tr_nsteps = nsteps;
        P->tr_ck = ck_every;
        P->tr_dt = dt;
        stage_in(P, Ks, S.F, S.in_Ks);
        stage_in(P, dh, S.N, S.in_dh);
        stage_in(P, Qs, S.N, S.in_Q);
        stage_in(P, Ss, S.N, P->tr_Ss);
        stage_in(P, h0, S.N, S.h);
        S.set_shift(P->tr_Ss, dt);
        S.assemble(S.in_Ks, nullptr, 0, S.shift, false);
        S.fwd_kind = 0;
        S.mean_kind = 0;
        ck(cudaMemcpyAsync(P->tr_b0, S.b64, S.N * sizeof(double), cudaMemcpyDeviceToDevice, P->stream), "b0");
        ck(cudaMemcpyAsync(P->tr_ck_states, S.h, S.N * sizeof(double), cudaMemcpyDeviceToDevice, P->stream), "ck0");
        bool states_dev = states && is_device_ptr(states);
        int worst = DPF_OK;
        long long tot_iters = 0;
        for (int n = 1; n <= nsteps; n++) {
            S.transient_step(P->tr_b0, S.h);
            tot_iters += S.stats_iters;
            if (S.last_status != DPF_OK && worst == DPF_OK) worst = solver_status(P, S);
            if (n % ck_every == 0)
                ck(cudaMemcpyAsync(P->tr_ck_states + (size_t)(n / ck_every) * S.N, S.h, S.N * sizeof(double),
                                   cudaMemcpyDeviceToDevice, P->stream),
                   "checkpoint");
            if (states)
                ck(cudaMemcpyAsync(states + (size_t)(n - 1) * S.N, S.h, S.N * sizeof(double),
                                   states_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream),
                   "states");
        }
        S.stats_iters = (int)std::min<long long>(tot_iters, 1 << 30);
        stage_out(P, hT, S.h, S.N);
        S.have_forward = false;  // the steady adjoint does not apply to this state
        return worst;
    });
}

// rhs = 2 w_k h[obs_k] (+ gT on the last step) + shift * mu at free cells, 0 at Dirichlet cells
__global__ void k_trans_adj_rhs(long long N, const uint8_t *__restrict__ dir, const double *__restrict__ shift,
                                const double *__restrict__ mu, const double *__restrict__ gT, double *__restrict__ rhs) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double v = shift[i] * mu[i];
    if (gT) v += gT[i];
    rhs[i] = dir[i] ? 0.0 : v;
}
__global__ void k_trans_obs(long long nobs, const long long *__restrict__ obs, const double *__restrict__ w,
                            const uint8_t *__restrict__ dir, const double *__restrict__ h, double *__restrict__ rhs) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nobs) return;
    long long i = obs[k];
    if (!dir[i]) atomicAdd(&rhs[i], 2.0 * (w ? w[k] : 1.0) * h[i]);
}
__global__ void k_dh0(long long N, const uint8_t *__restrict__ dir, const double *__restrict__ shift,
                      const double *__restrict__ mu, double *__restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    out[i] = dir[i] ? 0.0 : shift[i] * mu[i];
}

int dpf_transient_adjoint(dpf_problem *P, int64_t nobs, const int64_t *obs, const double *w, const double *gT,
                          double *dKs, double *ddh, double *dQs, double *dh0) {
    return guarded(P, __func__, [&]() -> int {
        if (nobs < 0 || (nobs > 0 && !obs)) throw BadInput("invalid arguments");
        if (P->gs) return gs_status(P, P->gs->transient_adjoint(nobs, obs, w, gT, dKs, ddh, dQs, dh0));
        StructBatch &S = *P->sb;
        if (P->tr_nsteps <= 0) { P->err = "transient adjoint needs a preceding transient forward"; return DPF_STATE; }
        const long long N = S.N;
        const int nsteps = P->tr_nsteps, ck_every = P->tr_ck;
        std::vector<long long> ho(nobs);
        const std::vector<int64_t> hv = read_indices(P, obs, nobs);
        for (int64_t k = 0; k < nobs; k++) {
            if (hv[k] < 0 || hv[k] >= N) throw BadInput("observation index out of range");
            ho[k] = hv[k];
        }
        long long *d_obs = scratch<long long>(P, nobs);
        if (nobs) ck(cudaMemcpyAsync(d_obs, ho.data(), nobs * sizeof(long long), cudaMemcpyHostToDevice, P->stream), "obs");
        double *d_w = nullptr, *d_gT = nullptr;
        if (w) { d_w = scratch<double>(P, nobs); stage_in(P, w, nobs, d_w); }
        if (gT) { d_gT = scratch<double>(P, N); stage_in(P, gT, N, d_gT); }
        double *acc_K = scratch<double>(P, S.F), *acc_dh = scratch<double>(P, N), *acc_Q = scratch<double>(P, N);
        double *mu = S.lam;
        ck(cudaMemsetAsync(acc_K, 0, S.F * sizeof(double), P->stream), "zero");
        ck(cudaMemsetAsync(acc_dh, 0, N * sizeof(double), P->stream), "zero");
        ck(cudaMemsetAsync(acc_Q, 0, N * sizeof(double), P->stream), "zero");
        ck(cudaMemsetAsync(mu, 0, N * sizeof(double), P->stream), "zero");
        const unsigned gN = (unsigned)((N + 255) / 256), gO = (unsigned)((nobs + 255) / 256);
        int worst = DPF_OK;
        const int nseg = (nsteps + ck_every - 1) / ck_every;
        for (int sgi = nseg - 1; sgi >= 0; sgi--) {
            int n0 = sgi * ck_every;                      // checkpointed state index
            int n1 = std::min(nsteps, n0 + ck_every);     // last state of the segment
            // recompute states n0+1..n1 from the checkpoint into tr_seg
            ck(cudaMemcpyAsync(S.h, P->tr_ck_states + (size_t)sgi * N, N * sizeof(double), cudaMemcpyDeviceToDevice,
                               P->stream), "restore");
            for (int n = n0 + 1; n <= n1; n++) {
                S.transient_step(P->tr_b0, S.h);
                if (S.last_status != DPF_OK && worst == DPF_OK) worst = solver_status(P, S);
                ck(cudaMemcpyAsync(P->tr_seg + (size_t)(n - n0 - 1) * N, S.h, N * sizeof(double),
                                   cudaMemcpyDeviceToDevice, P->stream), "segment");
            }
            for (int n = n1; n > n0; n--) {
                const double *hn = P->tr_seg + (size_t)(n - n0 - 1) * N;
                k_trans_adj_rhs<<<gN, 256, 0, P->stream>>>(N, S.lv[0].dir, S.shift, mu, n == nsteps ? d_gT : nullptr,
                                                           S.arhs);
                if (nobs) k_trans_obs<<<gO, 256, 0, P->stream>>>(nobs, d_obs, d_w, S.lv[0].dir, hn, S.arhs);
                ck(cudaGetLastError(), "adjoint rhs");
                S.solve(S.arhs, mu, S.opt.reltol);
                if (S.last_status != DPF_OK && worst == DPF_OK) worst = solver_status(P, S);
                S.grad_faces(hn, mu, acc_K, true);
                S.grad_dh_q(mu, acc_dh, acc_Q, false, true);
            }
        }
        if (dh0) {
            double *t = scratch<double>(P, N);
            k_dh0<<<gN, 256, 0, P->stream>>>(N, S.lv[0].dir, S.shift, mu, t);
            ck(cudaGetLastError(), "dh0");
            stage_out(P, dh0, t, N);
            ck(cudaStreamSynchronize(P->stream), "sync");
            release(P, t);
        }
        stage_out(P, dKs, acc_K, S.F);
        stage_out(P, ddh, acc_dh, N);
        stage_out(P, dQs, acc_Q, N);
        ck(cudaStreamSynchronize(P->stream), "sync");
        for (void *p : {(void *)d_obs, (void *)d_w, (void *)d_gT, (void *)acc_K, (void *)acc_dh, (void *)acc_Q})
            if (p) release(P, p);
        return worst;
    });
}

int dpf_profile(dpf_problem *P, int enable) {
    if (!P) return DPF_BAD_INPUT;
    DeviceGuard g(P->device);
    for (dpf_problem *Q : P->parts) Q->sb->profile(enable != 0);
    if (!P->parts.empty()) return DPF_OK;
    if (P->sb) P->sb->profile(enable != 0);
    else P->gs->profile(enable != 0);
    return DPF_OK;
}

int dpf_profile_report(dpf_problem *P, int cap, const char **names, long long *launches, double *ms,
                       long long *cells) {
    if (!P) return -DPF_BAD_INPUT;
    DeviceGuard g(P->device);
    try {
        if (!P->parts.empty()) {
            // the parts' reports merged by kernel name
            std::vector<const char *> nm;
            std::vector<long long> cnt, cl;
            std::vector<double> tot;
            for (dpf_problem *Q : P->parts) {
                const int n = Q->sb->profile_report(0, nullptr, nullptr, nullptr, nullptr);
                std::vector<const char *> qn(n);
                std::vector<long long> qc(n), qcl(n);
                std::vector<double> qm(n);
                Q->sb->profile_report(n, qn.data(), qc.data(), qm.data(), qcl.data());
                for (int j = 0; j < n; j++) {
                    size_t t = 0;
                    while (t < nm.size() && std::strcmp(nm[t], qn[j]) != 0) t++;
                    if (t == nm.size()) { nm.push_back(qn[j]); cnt.push_back(0); tot.push_back(0.0); cl.push_back(0); }
                    cnt[t] += qc[j];
                    tot[t] += qm[j];
                    cl[t] += qcl[j];
                }
            }
            for (size_t t = 0; t < nm.size() && (int)t < cap; t++) {
                if (names) names[t] = nm[t];
                if (launches) launches[t] = cnt[t];
                if (ms) ms[t] = tot[t];
                if (cells) cells[t] = cl[t];
            }
            return (int)nm.size();
        }
        if (P->sb) return P->sb->profile_report(cap, names, launches, ms, cells);
        return P->gs->profile_report(cap, names, launches, ms, cells);
    } catch (const DpfError &e) {
        P->err = e.what();
        return -e.code;
    }
}

// ------------------------------------------------------------- Richards (face-list handles)
int dpf_richards_steady(dpf_problem *P, const double *psi0, const double *Ks, const double *dirichletpsis,
                        const double *z, const double *alphas, const double *Ns, const double *Qs, double tol,
                        int maxiter, double *psi_out) {
    return guarded(P, __func__, [&]() -> int {
        if (!P->gs) {
            P->err = "the Richards solver runs on face-list handles (dpf_create_general)";
            return DPF_UNSUPPORTED;
        }
        if (!psi0 || !Ks || !dirichletpsis || !z || !alphas || !Ns || !Qs || !psi_out) throw BadInput("invalid arguments");
        if (!(tol > 0)) tol = 1e-10;
        if (maxiter <= 0) maxiter = 200;
        return gs_status(P, P->gs->richards_steady(psi0, Ks, dirichletpsis, z, alphas, Ns, Qs, tol, maxiter, psi_out));
    });
}

int dpf_richards_adjoint(dpf_problem *P, const double *delta, double tol, int maxiter, double *dKs, double *ddpsi,
                         double *dalphas, double *dNs, double *dQs) {
    return guarded(P, __func__, [&]() -> int {
        if (!P->gs) {
            P->err = "the Richards solver runs on face-list handles (dpf_create_general)";
            return DPF_UNSUPPORTED;
        }
        if (!delta) throw BadInput("delta is required");
        if (!(tol > 0)) tol = 1e-10;
        if (maxiter <= 0) maxiter = 200;
        return gs_status(P, P->gs->richards_adjoint(delta, tol, maxiter, dKs, ddpsi, dalphas, dNs, dQs));
    });
}

int dpf_richards_transient_forward(dpf_problem *P, const double *psi0, const double *Ks, const double *dirichletpsis,
                                   const double *z, const double *alphas, const double *Ns, const double *Qs,
                                   const double *specificstorage, double dt, int nsteps, double tol, int maxiter,
                                   double *states, double *psiT) {
    return guarded(P, __func__, [&]() -> int {
        if (!P->gs) {
            P->err = "the Richards solver runs on face-list handles (dpf_create_general)";
            return DPF_UNSUPPORTED;
        }
        if (!psi0 || !Ks || !dirichletpsis || !z || !alphas || !Ns || !Qs || !specificstorage)
            throw BadInput("invalid arguments");
        if (!(tol > 0)) tol = 1e-10;
        if (maxiter <= 0) maxiter = 200;
        return gs_status(P, P->gs->richards_transient_forward(psi0, Ks, dirichletpsis, z, alphas, Ns, Qs,
                                                              specificstorage, dt, nsteps, tol, maxiter, states,
                                                              psiT));
    });
}

int dpf_richards_transient_adjoint(dpf_problem *P, int64_t nobs, const int64_t *obs, const double *w,
                                   const double *gT, double tol, int maxiter, double *dKs, double *ddpsi,
                                   double *dalphas, double *dNs, double *dQs, double *dpsi0) {
    return guarded(P, __func__, [&]() -> int {
        if (!P->gs) {
            P->err = "the Richards solver runs on face-list handles (dpf_create_general)";
            return DPF_UNSUPPORTED;
        }
        if (nobs < 0 || (nobs > 0 && !obs)) throw BadInput("invalid observations");
        if (!(tol > 0)) tol = 1e-10;
        if (maxiter <= 0) maxiter = 200;
        return gs_status(P, P->gs->richards_transient_adjoint(nobs, obs, w, gT, tol, maxiter, dKs, ddpsi, dalphas,
                                                              dNs, dQs, dpsi0));
    });
}

int dpf_richards_stats(const dpf_problem *P, int *iterations, int *adjoint_iterations, double *relres) {
    if (!P || !P->gs) return DPF_BAD_INPUT;
    if (iterations) *iterations = P->gs->rich_iters;
    if (adjoint_iterations) *adjoint_iterations = P->gs->rich_adj_iters;
    if (relres) *relres = P->gs->rich_relres;
    return DPF_OK;
}

int dpf_set_stream(dpf_problem *P, void *stream) {
    if (!P) return DPF_BAD_INPUT;
    DeviceGuard g(P->device);
    if (cudaStreamSynchronize(P->stream) != cudaSuccess) {
        P->err = std::string("stream synchronize: ") + cudaGetErrorString(cudaGetLastError());
        return DPF_CUDA;
    }
    P->stream = (cudaStream_t)stream;
    if (P->sb) P->sb->stream = P->stream;
    if (P->gs) P->gs->set_stream(P->stream);
    return DPF_OK;
}

long long dpf_launch_count(const dpf_problem *P) {
    if (!P) return -1;
    if (!P->parts.empty()) {
        long long n = 0;
        for (const dpf_problem *Q : P->parts) n += Q->sb->launches;
        return n;
    }
    if (P->sb) return P->sb->launches;
    return P->gs ? P->gs->launches : 0;
}

}  // extern "C"
