// dpf_noalloc.cu -- face conductances of a regular grid from cell log-conductivities,
// without any device allocation.
//
// Who needs this: callers that must not have this library allocate device memory.
// A host application that owns all device memory through its own pool (Julia's
// CUDA.jl or PyTorch's caching allocator, or a simulator running inside a fixed
// memory budget) cannot let a third-party library call cudaMalloc/cudaFree behind
// its back: those calls synchronize the device, fragment the pool, and can fail
// when the application has reserved the memory for itself. Such a caller passes its
// own device buffers for the input and the output; the only working memory of this
// path is the fixed array below.
//
// Scratch: g_noalloc_kc holds one value per cell (exp(logK/2) for the geometric
// mean, exp(logK) for the harmonic mean), at most kNoAllocMaxCells cells
// (16 MiB). It is a module global, so every GPU that loads the library holds it
// until the process exits. Every call overwrites the cells it uses before reading
// them, so nothing needs to start at zero; the array keeps the last call's values.
// All calls share the one array: calls that overlap on the GPU (for example the
// same entry point called concurrently from two host threads) race on it and must
// be serialized by the caller.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address with cudaGetSymbolAddress (the host-side name of a
// __device__ array is only a host stand-in, not a device address). Make that first
// call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "dpf_internal.h"

namespace {

constexpr long long kNoAllocMaxCells = 1LL << 21;  // 2,097,152 cells -> 16 MiB of scratch
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_kc[kNoAllocMaxCells];

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Same index as the face list of regulargrid3d (src/grid.jl:163-185): faces are
// emitted per cell in the order +x, +y, +z when the neighbour exists.
__device__ __forceinline__ long long na_face_index(int nx, int ny, int nz, int ix, int iy, int iz, int d) {
    long long ex = ix < nx - 1, ey = iy < ny - 1;
    long long base = (long long)ix * (3LL * ny * nz - nz - ny) + (long long)iy * (ex * nz + nz + nz - 1) +
                     (long long)iz * (ex + ey + 1);
    if (d == 0) return base;
    if (d == 1) return base + ex;
    return base + ex + ey;
}

__global__ void k_na_cell(long long n, const double *__restrict__ logK, int kind, double *__restrict__ kc) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = logK[i];
    kc[i] = exp(kind == DPF_MEAN_GEOMETRIC ? 0.5 * v : v);
}

__global__ void k_na_faces(int nx, int ny, int nz, unsigned mag_nz, int sh_nz, unsigned mag_ny, int sh_ny,
                           const double *__restrict__ kc, int kind, double *__restrict__ Ks) {
    long long n = (long long)nx * ny * nz;
    long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    unsigned u = (unsigned)li;
    unsigned q = (__umulhi(u, mag_nz) + u) >> sh_nz;
    int iz = (int)(u - q * (unsigned)nz);
    unsigned x = (__umulhi(q, mag_ny) + q) >> sh_ny;
    int iy = (int)(q - x * (unsigned)ny), ix = (int)x;
    const long long st[3] = {(long long)ny * nz, (long long)nz, 1};
    const int co[3] = {ix, iy, iz};
    const int nn[3] = {nx, ny, nz};
    const double ka = kc[li];
    for (int d = 0; d < 3; d++) {
        if (co[d] + 1 >= nn[d]) continue;
        double kb = kc[li + st[d]];
        double K = kind == DPF_MEAN_GEOMETRIC ? ka * kb : 2.0 * ka * kb / (ka + kb);
        Ks[na_face_index(nx, ny, nz, ix, iy, iz, d)] = K;
    }
}

// device (or managed) memory of the current device: the kernels read and write it without
// peer access, so a pointer into another GPU's memory is rejected here, on the host
bool on_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice) return a.device == cur;
    return a.type == cudaMemoryTypeManaged;
}

// device address of the scratch array on the current device (looked up once per device)
int scratch_address(double **out, std::string &err) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        err = "no CUDA device";
        return DPF_NO_DEVICE;
    }
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        err = "device index out of the supported range";
        return DPF_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_kc);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            err = std::string("cudaGetSymbolAddress of the scratch array failed: ") + cudaGetErrorString(e);
            return DPF_CUDA;
        }
        g_noalloc_ptr[dev] = (double *)p;
    }
    *out = g_noalloc_ptr[dev];
    return DPF_OK;
}

}  // namespace

namespace dpf {
void set_global_error(const std::string &msg);
}

extern "C" int dpf_logk_to_faces_regular_noalloc(int nx, int ny, int nz, const double *logK, int mean_kind,
                                                 double *Ks) {
    if (nx < 1 || ny < 1 || nz < 1 || !logK || !Ks) {
        dpf::set_global_error("invalid arguments");
        return DPF_BAD_INPUT;
    }
    if (mean_kind != DPF_MEAN_GEOMETRIC && mean_kind != DPF_MEAN_HARMONIC) {
        dpf::set_global_error("unknown mean kind");
        return DPF_BAD_INPUT;
    }
    long long n = (long long)nx * ny * nz;
    if (n > kNoAllocMaxCells) {
        dpf::set_global_error("grid has " + std::to_string(n) + " cells; the allocation-free path handles at most " +
                              std::to_string(kNoAllocMaxCells));
        return DPF_BAD_INPUT;
    }
    if (!on_device(logK) || !on_device(Ks)) {
        dpf::set_global_error("the allocation-free path needs device pointers of the current device for logK and Ks");
        return DPF_BAD_INPUT;
    }
    std::string err;
    double *kc = nullptr;
    int rc = scratch_address(&kc, err);
    if (rc != DPF_OK) {
        dpf::set_global_error(err);
        return rc;
    }
    unsigned mz, my;
    int sz, sy;
    dpf::fast_div_magic((unsigned)nz, mz, sz);
    dpf::fast_div_magic((unsigned)ny, my, sy);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_na_cell<<<blocks, 256, 0, 0>>>(n, logK, mean_kind, kc);
    k_na_faces<<<blocks, 256, 0, 0>>>(nx, ny, nz, mz, sz, my, sy, kc, mean_kind, Ks);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
        dpf::set_global_error(std::string("kernel failed: ") + cudaGetErrorString(e));
        return DPF_CUDA;
    }
    return DPF_OK;
}
