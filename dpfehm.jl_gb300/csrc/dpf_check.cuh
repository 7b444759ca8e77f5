// dpf_check.cuh -- the checked build (-DDPF_CHECK): device-side bounds and alignment checks.
//
// Without a memory checker on the devices these kernels run on, a library built with
// DPF_CHECK defined checks the indices every kernel's memory accesses are derived from:
// the cell decode (cell_at), the stencil neighbours (apply7), the aggregate of a fine cell,
// the ranges, slots and alignment of the staged bulk copies of the plane kernels, and the
// column indices of the CSR operator. A violation is counted in a per-translation-unit
// device word, the first one keeps its site code, index and bound, and the access is
// clamped or skipped (never a trap); dpf_debug_check_report reads and clears the words.
// Without DPF_CHECK the checks compile to nothing.
#pragma once
#include <cuda_runtime.h>

namespace dpf {

enum CheckSite : int {
    CK_CELL = 1,         // cell decode: linear index or coordinates outside the grid
    CK_NEIGHBOUR = 2,    // stencil neighbour outside the problem's cells
    CK_AGGREGATE = 3,    // aggregate of a fine cell outside the coarse grid
    CK_STAGE_SRC = 4,    // staged copy: source elements outside the problem's cells
    CK_STAGE_DST = 5,    // staged copy: destination outside its shared-memory slot
    CK_STAGE_ALIGN = 6,  // staged copy: address or size not on a 16-byte boundary
    CK_CSR_COL = 7,      // CSR column index outside the level
};

// Reads (and clears) one translation unit's check words: violations and the first one's
// {site, index, bound}. Every translation unit that includes this header in a checked
// build registers one at load time.
using CheckReader = int (*)(long long *count, long long first[3]);
void register_check_reader(CheckReader f);

#ifdef DPF_CHECK
static __device__ unsigned long long g_check_count;
static __device__ long long g_check_first[3];

static __device__ __noinline__ bool check_fail(int site, long long v, long long bound) {
    if (atomicAdd(&g_check_count, 1ull) == 0ull) {
        g_check_first[0] = site;
        g_check_first[1] = v;
        g_check_first[2] = bound;
    }
    return false;
}

static int read_check_words(long long *count, long long first[3]) {
    unsigned long long c = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&c, g_check_count, sizeof(c)) != cudaSuccess ||
        cudaMemcpyFromSymbol(first, g_check_first, 3 * sizeof(long long)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_check_count, &zero, sizeof(zero)) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    *count = (long long)c;
    return 0;
}

static const bool g_check_registered = (register_check_reader(&read_check_words), true);

// true when lo <= v < hi; otherwise the violation is recorded and the result is false
#define DPF_INSIDE(site, v, lo, hi)                                                        \
    (((long long)(v) >= (long long)(lo) && (long long)(v) < (long long)(hi))              \
         ? true                                                                            \
         : ::dpf::check_fail((site), (long long)(v), (long long)(hi)))
#define DPF_CHECKED 1
#else
#define DPF_INSIDE(site, v, lo, hi) true
#define DPF_CHECKED 0
#endif

}  // namespace dpf
