// dpf_direct.h -- banded Cholesky factorisation of the FP64 groundwater operator: the direct
// solver behind `linear_solver = cholesky_solver` (src/groundwater.jl:56-60, which calls
// LinearAlgebra.cholesky on the assembled sparse matrix).
//
// The operator is SPD (every problem has a Dirichlet cell; Dirichlet cells are identity rows).
// Its rows are renumbered so that every coupling lies within a narrow band (regular grids: the
// two shortest axes fastest; other meshes: reverse Cuthill-McKee), and A = L L^T is factored in
// that band. Cholesky creates no fill outside the band, so the factor needs n (w + 1) values
// for a half-bandwidth w, and n w^2 multiply-adds. That makes it a direct solve for 2-D grids,
// thin 3-D grids and moderate meshes; wider bands are refused (fits() false) and the caller
// takes its iterative solve to the rounding floor instead.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <vector>

namespace dpf {

// A band ordering: perm[k] = original row of band row k, and the half-bandwidth w = the largest
// |k_i - k_j| over the couplings (i, j).
struct BandOrder {
    std::vector<long long> perm;
    long long w = 0;
};

// The cells of a batch of regular grids (problem p: dims[p] = {nx, ny, nz}, z fastest, its
// cells from off[p]): per problem the axes re-nested by extent (the longest slowest), problems
// one after another; w = the largest product of a problem's two shorter extents.
BandOrder band_order_regular(const std::vector<std::array<int, 3>> &dims, const std::vector<long long> &off);

// A symmetric graph in CSR form (rp[n + 1], ci; no diagonal): reverse Cuthill-McKee, each
// connected component started from a pseudo-peripheral vertex (the last one reached by a
// breadth-first search from its lowest-degree vertex).
BandOrder band_order_rcm(long long n, const std::vector<int> &rp, const std::vector<int> &ci);

class BandCholesky {
public:
    // the largest band the direct solver takes: n (w + 1) doubles within `mem_bytes`, and at most
    // about 2e13 multiply-adds (a few tens of seconds on GB300's FP64 pipe)
    static bool fits(long long n, long long w, size_t mem_bytes);

    BandCholesky(const BandOrder &ord, cudaStream_t stream);
    ~BandCholesky();
    BandCholesky(const BandCholesky &) = delete;
    BandCholesky &operator=(const BandCholesky &) = delete;

    // column-major lower band: entry (r, c), 0 <= r - c <= w, at band()[c (w + 1) + r - c], in band
    // row numbers; clear() zeroes it before a caller's kernel fills it
    double *band() { return B; }
    const long long *iperm() const { return d_iperm; }  // original row -> band row (device)
    void clear();
    // factor in place; false when a pivot is not positive (the matrix is not positive definite)
    bool factor();
    // x = A^-1 b for vectors in the original numbering (device; x and b may be the same array)
    void solve(const double *b, double *x);
    void set_stream(cudaStream_t s) { stream = s; }
    // sqrt(sum (b - Ax)^2 / sum b^2) over the rows with dir[i] == 0 (a diagnostic of a solve; acc:
    // two device doubles of scratch; FP64 atomics, so the last bits may vary from run to run)
    static double relres(cudaStream_t s, long long n, const uint8_t *dir, const double *b, const double *Ax,
                         double *acc);

    long long n = 0, w = 0;
    long long launches = 0;

private:
    cudaStream_t stream;
    double *B = nullptr;
    double *y = nullptr;           // the permuted right-hand side / solution
    long long *d_perm = nullptr, *d_iperm = nullptr;
    int *d_err = nullptr;
};

}  // namespace dpf
