// dpf_internal.h -- shared declarations of the GB300 groundwater library.
//
// Data layout in HBM (structured path). A batch of nprob regular grids is
// stored level by level; at every multigrid level the cells of all problems
// that have that level are concatenated (problem order), each grid in the
// reference's order (z fastest, then y, then x; src/grid.jl:151). Per cell and
// level the operator is four structure-of-arrays values:
//   cx, cy, cz : conductance K*aol of the +x/+y/+z face (0 when the face does
//                not exist or touches a Dirichlet cell)
//   leak       : the part of the diagonal not carried by cx/cy/cz (faces to
//                Dirichlet cells, storage/dt in transient runs); 1 for a
//                Dirichlet cell, whose row is the identity.
// The operator is applied in flux form, y_i = leak_i x_i + sum_f c_f (x_i - x_j),
// which avoids the cancellation of diag*x - sum c*x for smooth x.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/dpfehm_gpu.h"

namespace dpf {

constexpr int kBlock = 256;        // threads per block of every cell-parallel kernel
constexpr int kMaxCoarse = 64;     // largest dense coarsest level (cells)
constexpr int kMinBlocks = 6;      // resident blocks per SM the CG stencils are compiled for
// Mixed precision: a round of double-float CG also ends once its recursive residual has dropped
// by 1e-12 from the round's start (|r|^2 <= 1e-24 in the round's units, where |r| starts at 1).
// A double-float recurrence carries about 48 bits, so a deeper drop within one round would not
// be reflected in the true residual; the FP64 check that follows then continues from the true
// residual or, at the system's FP64 rounding floor, accepts. This lets a tolerance below that
// floor (reltol 0) end at the floor with status OK instead of at the iteration cap.
constexpr double kRoundDrop2 = 1e-24;

struct LevelDesc {                 // one problem at one level
    int nx, ny, nz, pad;
    long long n;                   // cells
    long long off;                 // offset of the problem's cells in the level arrays
    unsigned mag_nz, mag_ny;       // invariant-integer division by nz and ny (see fast_div)
    int sh_nz, sh_ny;
};

// Division by an invariant integer d >= 1 for numerators n < 2^31 (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, q = (mulhi(n, m) + n) >> l.
inline void fast_div_magic(unsigned d, unsigned &m, int &l) {
    l = 0;
    while ((1ull << l) < d) l++;
    m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
}

struct BlockMap {                  // launch map: block -> (problem, block within problem, blocks of problem)
    int4 *d_map = nullptr;         // [nblocks]
    int2 *d_pinfo = nullptr;       // [nprob] {first block, number of blocks} (0,0 if absent)
    int nblocks = 0;
};

// Per-problem CG state, device resident. Scalars are FP64 whatever the vector type.
struct CgState {
    double rz, rz_old, pq, rr, bb, tol2;
    double alpha, beta;
    double scale;                  // mixed precision: normalisation of the double-float residual
    double floor2;                 // mixed precision: FP64 rounding floor of |b - A x|^2 at the last check
    double cont;                   // mixed precision: factor of the next beta after a residual replacement
    double orr, obb;               // mixed precision: true (FP64) residual and rhs norms squared
    double orr_prev;               // mixed precision: true residual norm squared after the previous round
    int iters, active, status, outer;  // outer: rounds so far
    int ru_flag, total_iters, stall, pad2;  // ru_flag: problem takes part in the current round
};

// Double-float copies of the finest operator's coefficients (hi, lo per entry).
struct CoeffsDF {
    const float2 *cx, *cy, *cz, *leak;
};

// Reduction scratch: one double2 partial per block of the widest launch, one
// ticket counter per problem; the last block of each problem sums the partials
// in a fixed order (deterministic) and finalises that problem's scalars.
struct ReduceScratch {
    double2 *partials = nullptr;
    unsigned *tickets = nullptr;
    int capacity = 0;
};

struct ProbParam {                 // per-problem constants of a regular grid
    double aol[3];                 // areas over lengths of +x, +y, +z faces
    double vol;                    // cell volume (transient storage term)
    long long face_off;            // offset of the problem's faces in concatenated face arrays
    long long F;                   // faces of the problem
    double x0[3], dx[3];           // node coordinates: x0 + i dx per axis (regulargrid3d's)
};

// Storage type of the operator coefficients of a level whose vectors are T. FP64 levels
// keep FP64. The FP32 V-cycle (a preconditioner: CG's own operator products are FP64 or
// double-float) reads bf16 coefficients, 8 significant bits with FP32's exponent range,
// which halves its coefficient traffic; its diagonals are formed from the same rounded
// values, so every smoother step and the Galerkin levels see one consistent operator.
template <typename T>
struct CoefStore {
    using type = T;
};
template <>
struct CoefStore<float> {
    using type = __nv_bfloat16;
};
template <typename T>
using coef_t = typename CoefStore<T>::type;

template <typename T>
struct Coeffs {
    const coef_t<T> *cx, *cy, *cz, *leak;
    const T *idg;                  // inverse diagonal
};

// Per-level pointers and the Chebyshev parameters of the fused small-level tail kernel.
template <typename T>
struct TailLevel {
    const LevelDesc *desc;
    Coeffs<T> C;
    T *xa, *xb, *b, *d;
    const uint8_t *dir;
};

template <typename T>
struct TailParams {
    T c1[8], c2[8];  // Chebyshev recurrence coefficients, steps 0..deg-1
    T invtheta, coarse_scale;
    int deg;
};

constexpr int kTailThreads = 1024;

// Every device and pinned-host allocation of the library goes through these calls: they keep
// the process-wide counts that dpf_debug_alloc_stats reports and fail the allocation that
// dpf_debug_fail_alloc selects (cudaErrorMemoryAllocation, nothing allocated). The frees
// accept nullptr.
cudaError_t dev_malloc(void **p, size_t bytes);
cudaError_t host_malloc(void **p, size_t bytes);
void dev_free(void *p);
void host_free(void *p);

// An NVTX range over a scope (entry points and solver phases) for profilers that record
// NVTX; without one attached the push and pop return at once.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// The device (DevList) and pinned-host (HostList) allocations a solver object owns. As
// members they free what they hold when the object is destroyed, and also when its
// constructor throws part-way through (members already built are destroyed then; the
// object's own destructor is not run).
struct DevList : std::vector<void *> {
    DevList() = default;
    DevList(const DevList &) = delete;
    DevList &operator=(const DevList &) = delete;
    ~DevList() {
        for (void *p : *this) dev_free(p);
    }
};
struct HostList : std::vector<void *> {
    HostList() = default;
    HostList(const HostList &) = delete;
    HostList &operator=(const HostList &) = delete;
    // a pinned buffer of the given size that the list owns; nullptr on failure
    void *alloc(size_t bytes) {
        void *p = nullptr;
        if (host_malloc(&p, bytes) != cudaSuccess) return nullptr;
        push_back(p);
        return p;
    }
    ~HostList() {
        for (void *p : *this) host_free(p);
    }
};

}  // namespace dpf
