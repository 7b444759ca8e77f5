/*
 * dpfehm_gpu.h -- C ABI of the GB300 groundwater solve library (libdpfehm_gpu.so).
 *
 * Drop-in boundary for DPFEHM.jl's steady-state groundwater solve and its
 * ChainRules rrule, plus the transient backward-Euler solve built from the same
 * residual. Every entry point replaces a piece of the reference named beside it
 * (paths relative to the DPFEHM.jl project):
 *
 *   dpf_create / dpf_create_regular3d   getfreenodes + problem topology
 *                                       (src/utilities.jl:10-24, src/grid.jl:150-188)
 *   dpf_steady_forward                  groundwater_steadystate (src/groundwater.jl:75-83)
 *   dpf_steady_adjoint                  rrule pullback (src/groundwater.jl:85-107)
 *   dpf_logk_to_faces(_vjp)             caller-side logKs2Ks_neighbors and its Zygote VJP
 *                                       (examples/gw_steadystate_3d/inputdeck.jl:51;
 *                                        harmonic mean: src/richards.jl:50-52)
 *   dpf_transient_forward/_adjoint      backward-Euler stepping of -groundwater_residuals
 *                                       (src/groundwater.jl:1-21 with specificstorage,
 *                                        volumes; examples/gw_transient_3d/inputdeck.jl:60-92)
 *   dpf_batch_*                         many independent problems in one set of launches
 *                                       (replaces Distributed.pmap replicas,
 *                                        examples/scott_example/ex.jl:10)
 *
 * Conventions
 *   - Indices are 0-based (the Julia shim subtracts 1).
 *   - Array arguments may be host or device pointers; the library detects which
 *     with cudaPointerGetAttributes. Host arrays are copied with cudaMemcpyAsync
 *     (page-locked host memory gives asynchronous DMA); device arrays are read
 *     in place.
 *   - Every call is ordered on the handle's CUDA stream and returns when its
 *     outputs are complete.
 *   - A handle is not thread-safe; distinct handles may be used from distinct
 *     threads.
 *   - Every function returns a dpf_status; dpf_last_error(h) describes the last
 *     failure on h (or the last create failure when h is NULL).
 *   - Nothing falls back to the CPU: without a usable CUDA device every call
 *     fails with DPF_NO_DEVICE.
 */
#ifndef DPFEHM_GPU_H
#define DPFEHM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DPF_OK = 0,
    DPF_BAD_INPUT = 1,      /* invalid sizes, indices or options */
    DPF_NOT_CONVERGED = 2,  /* iteration cap reached; outputs hold the last iterate */
    DPF_NAN = 3,            /* a residual became NaN/Inf */
    DPF_OOM = 4,            /* device or pinned allocation failed */
    DPF_CUDA = 5,           /* a CUDA runtime call failed */
    DPF_NO_DEVICE = 6,      /* no CUDA device */
    DPF_STATE = 7,          /* call out of order (e.g. adjoint before forward) */
    DPF_UNSUPPORTED = 8,    /* option not available for this problem kind */
    DPF_TIMEOUT = 9         /* a bounded device-side wait expired; the handle stays usable */
} dpf_status;

typedef enum { DPF_MEAN_GEOMETRIC = 0, DPF_MEAN_HARMONIC = 1 } dpf_mean_kind;

typedef enum {
    DPF_PREC_FP64 = 0,  /* FP64 CG with an FP64 V-cycle */
    DPF_PREC_MIXED = 1  /* FP32 V-cycle; CG recurrence and finest-level SpMV in double-float (pairs of
                           floats, FP32 arithmetic); FP64 solution, FP64 true residual check per round,
                           FP64 CG scalars */
} dpf_precision;

typedef enum {
    DPF_SOLVER_CG = 0,       /* AMG-preconditioned CG to reltol (the reference's amg_solver) */
    DPF_SOLVER_CHOLESKY = 1  /* banded Cholesky factorisation of the FP64 operator (the reference's
                                cholesky_solver, src/groundwater.jl:56-60): the rows renumbered into a
                                narrow band (regular grids: the two shortest axes fastest; other meshes:
                                reverse Cuthill-McKee), factored once per assembly, two triangular solves
                                per solve; a band too wide for the device (more than half its free memory,
                                or above about 2e13 multiply-adds) falls back to the CG solve */
} dpf_solver;

typedef struct dpf_options {
    double reltol;       /* stop when ||b - A h|| <= reltol * ||b||            (default 1e-10) */
    int maxiter;         /* CG iteration cap per solve                        (default 500)   */
    int precision;       /* dpf_precision                                     (default FP64)  */
    int cheb_degree;     /* Chebyshev smoother degree per pre/post sweep (default 0: 2 on regular
                            grids, 3 on the general path) */
    double cheb_lo;      /* lower end of the Chebyshev interval / upper end   (default 0.2)   */
    double coarse_scale; /* scaling of the coarse-grid correction (default 0: 2.0 on regular grids,
                            3.5 on the general path, whose graph aggregates are larger) */
    int max_coarse;      /* coarsen until a level has at most this many cells (default 64, <= 64) */
    int max_outer;       /* MIXED: cap on rounds, each restarted from the true FP64 residual (default 6) */
    int use_graphs;      /* capture each solve's iteration in a CUDA graph    (default 1)     */
    int check_every;     /* host-driven CG loops (use_graphs = 0, and the general path): convergence is
                            read back every this many iterations (default 1); the general path reads
                            only every eighth until two iterations before the handle's previous solve
                            stopped */
    int blocks_per_sm;   /* launch shape: grids hold SMs x this many 256-thread blocks (default 16) */
    int tail_cells;      /* regular grids: the multigrid levels of a problem with at most this many cells
                            run as one fused kernel per problem (default 4096; negative: off) */
    int plane;           /* regular grids, MIXED: plane-marching smoother kernels with shared-memory
                            staging (default 1: where the finest level of the handle holds at least
                            2^21 cells; 2: at every size; negative: grid-stride kernels) */
    int plane_cells;     /* plane-marching slab capacity in cells: 256, 512, 768 or 1024 (default 1024) */
    int plane_blocks_per_sm; /* plane-marching work items per SM (default 2) */
    int df_plane_cells;  /* MIXED: positive: the double-float CG product marches along x over slabs of
                            whole rows of at most 256 cells, every face flux computed once (default
                            256); negative: the grid-stride product; an autotuner choice */
    int df_plane_blocks_per_sm; /* the marching product's work runs per SM (default 8) */
    int tail_cluster;    /* blocks (a thread-block cluster, 2..16) per problem for the fused tail
                            (default 1: one block) */
    int plane_levels;    /* regular grids, MIXED: the plane-marching kernels run on this many of the
                            finest levels, grid-stride kernels below (default 0: every level whose
                            rows fit a slab) */
    int streams;         /* batches: split into this many concurrent parts (consecutive problems, each
                            on its own non-blocking stream and host thread), so that one part's
                            finest-level kernels overlap another's small levels (default 0: one
                            stream; an autotuner choice) */
    int fuse;            /* regular grids, MIXED, Chebyshev degree 2: the plane-marching pre-smoothing and
                            restriction of a level run as one pass, and so do the prolongation and
                            post-smoothing (the intermediate iterate stays in shared memory); half
                            the bytes, but more instructions per cell, and slower on GB300 at the
                            benchmark sizes (default -1: separate passes; an autotuner choice) */
    int solver;          /* dpf_solver: steady and transient solves of single problems and batches
                            (default DPF_SOLVER_CG) */
} dpf_options;

typedef struct dpf_problem dpf_problem;

/* Fill *opts with the defaults listed above. */
void dpf_default_options(dpf_options *opts);

/* ---------------------------------------------------------------- topology */

/* General topology from the reference's arrays (src/groundwater.jl:75 argument
 * list): N cells, F faces (nbr_a[f], nbr_b[f], 0-based), areasoverlengths[F],
 * nd Dirichlet cells. When the faces are exactly those of regulargrid3d
 * (src/grid.jl:150-188) the matrix-free 7-point path is used, otherwise the CSR
 * path. volumes may be NULL (unit volumes). opts may be NULL (defaults). */
int dpf_create(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b, const double *areasoverlengths,
               const double *volumes, int64_t nd, const int64_t *dirichletnodes, const dpf_options *opts,
               dpf_problem **out);

/* Regular grid straight from regulargrid3d's arguments (mins, maxs: 3 each; ns = nx, ny, nz). */
int dpf_create_regular3d(int nx, int ny, int nz, const double *mins, const double *maxs, int64_t nd,
                         const int64_t *dirichletnodes, const dpf_options *opts, dpf_problem **out);

/* Host-only check (no GPU needed): if the faces/areas are those of regulargrid3d
 * for some (nx, ny, nz), write them to dims[3] and the three areas-over-lengths
 * to aol3[3] and return 1; otherwise return 0. */
int dpf_detect_regular3d(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b,
                         const double *areasoverlengths, int *dims, double *aol3);

void dpf_destroy(dpf_problem *h);
const char *dpf_last_error(const dpf_problem *h);

/* Sizes: N, F, number of free cells, 1 if the structured path is in use, number of AMG levels. */
int dpf_info(const dpf_problem *h, int64_t *N, int64_t *F, int64_t *nfree, int *structured, int *levels);

/* Statistics of the last solve: iterations (CG, summed over refinement steps),
 * refinement steps, final relative residual ||b - A h|| / ||b|| (FP64). */
int dpf_last_stats(const dpf_problem *h, int *iterations, int *outer, double *relres);

/* ---------------------------------------------------- steady state + rrule */

/* groundwater_steadystate: Ks[F], dirichleths[N], Qs[N] -> h[N]
 * (dirichleths copied to the Dirichlet cells). Keeps h on the device for the adjoint. */
int dpf_steady_forward(dpf_problem *h, const double *Ks, const double *dirichleths, const double *Qs, double *h_out);

/* rrule pullback for cotangent delta[N] of the last forward solve:
 * dKs[F], ddirichleths[N], dQs[N] (any output may be NULL). The forward
 * hierarchy is reused (the operator is symmetric). */
int dpf_steady_adjoint(dpf_problem *h, const double *delta, double *dKs, double *ddirichleths, double *dQs);

/* Face conductances from cell log-conductivities (structured or general). */
int dpf_logk_to_faces(dpf_problem *h, const double *logK, int mean_kind, double *Ks);
/* dlogK[N] = (dKs/dlogK)^T dKs */
int dpf_logk_to_faces_vjp(dpf_problem *h, const double *logK, int mean_kind, const double *dKs, double *dlogK);

/* Fused forward from logK (face means computed on the device, no Ks round trip). */
int dpf_steady_forward_logk(dpf_problem *h, const double *logK, int mean_kind, const double *dirichleths,
                            const double *Qs, double *h_out);
/* Fused adjoint straight to dlogK[N] (and optionally ddirichleths, dQs). Requires
 * the last forward to have been dpf_steady_forward_logk. */
int dpf_steady_adjoint_logk(dpf_problem *h, const double *delta, double *dlogK, double *ddirichleths, double *dQs);

/* --------------------------------------------------------------- transient */

/* Fixed-step backward Euler of S_i V_i dh_i/dt = Q_i - sum_f K_f aol_f (h_i - h_nb)
 * (the scaling of src/groundwater.jl:7,15,17): nsteps steps of dt from h0[N]
 * (values at Dirichlet cells ignored). Writes h at the final step to hT[N] and,
 * if states != NULL, every step to states[nsteps*N]. Heads of every
 * checkpoint_every-th step are kept on the device for the adjoint, which
 * recomputes the others segment by segment (checkpoint_every = 1 keeps all). */
int dpf_transient_forward(dpf_problem *h, const double *Ks, const double *dirichleths, const double *Qs,
                          const double *specificstorage, double dt, int nsteps, const double *h0,
                          int checkpoint_every, double *states, double *hT);

/* Adjoint of the last transient forward for
 *   J = sum_{n=1..nsteps} sum_k w_k h^n[obs_k]^2  +  gT . h^nsteps
 * (w may be NULL for unit weights, gT may be NULL). Outputs dKs[F],
 * ddirichleths[N], dQs[N], dh0[N] (any may be NULL). */
int dpf_transient_adjoint(dpf_problem *h, int64_t nobs, const int64_t *obs, const double *w, const double *gT,
                          double *dKs, double *ddirichleths, double *dQs, double *dh0);

/* ------------------------------------------------------------------- batch */

/* nprob independent regular grids (dims[3*p..], mins/maxs[3*p..]) in one handle;
 * nd[p] Dirichlet cells each, concatenated in dirichletnodes (indices local to
 * each problem). Per-problem arrays passed to the batch calls are concatenated in
 * problem order. */
int dpf_batch_create(int nprob, const int *dims, const double *mins, const double *maxs, const int64_t *nd,
                     const int64_t *dirichletnodes, const dpf_options *opts, dpf_problem **out);

/* Offsets of problem p's cells / faces in concatenated arrays (p = nprob gives totals). */
int dpf_batch_offsets(const dpf_problem *h, int p, int64_t *cell_offset, int64_t *face_offset);

/* Forward + adjoint of every problem from concatenated logK; delta for the
 * adjoint is J_p = sum_k h_p[obs]^2 over each problem's observation cells
 * (obs_offsets[nprob+1] into obs, local indices). Outputs h[N_total] and
 * dlogK[N_total] (either may be NULL). logK NULL: the fields last drawn into the
 * handle by dpf_batch_sample_logk (DPF_STATE if there are none). */
int dpf_batch_solve_grad_logk(dpf_problem *h, const double *logK, int mean_kind, const double *dirichleths,
                              const double *Qs, const int64_t *obs_offsets, const int64_t *obs, double *h_out,
                              double *dlogK);

/* Seeded Gaussian log-conductivity fields with Matern (nu = 1) covariance for every problem of a
 * regular-grid batch, drawn on the GPU (the inverse and uncertainty-quantification drivers' field
 * step, examples/gw_multigrid_inverse/inputdeck.jl:58-105, where the reference samples on the host):
 * logK_p(x) = mean[p] + sigma[p] sqrt(2/M) sum_k cos(w_k . x + phi_k) over M = nmodes modes, with the
 * frequencies drawn from the Matern spectral density for correlation length ell[p] (the convention
 * (2/ell^2 + |w|^2)^-(5/2) of the package's FFT sampler) and the phases uniform, from the
 * counter-based Philox4x32-10 generator keyed by seeds[p]: a field depends only on its seed, grid
 * and nmodes (1..65536), and repeats bit for bit. Cells sit at the grid's node coordinates (integer
 * indices for a grid detected from a face list). logK[N_total] (host or device) receives the
 * fields; with logK NULL they stay in the handle, and dpf_batch_solve_grad_logk with a NULL logK
 * solves on them, so a draw-solve-differentiate loop has no host step for the fields. */
int dpf_batch_sample_logk(dpf_problem *h, int nmodes, const uint64_t *seeds, const double *ell, const double *sigma,
                          const double *mean, double *logK);

/* Autotuner for a batch (same arguments as dpf_batch_create and dpf_batch_solve_grad_logk):
 * coordinate descent over the Chebyshev degree, plane_cells, plane_blocks_per_sm,
 * tail_cells, blocks_per_sm, df_plane_cells and tail_cluster, starting from *base (NULL: defaults), each candidate timed
 * over `repeats` forward + adjoint solves of the given inputs (host or device buffers)
 * after one untimed solve; a candidate is kept if it converges and is >= 2 % faster.
 * Writes the chosen options to *best and their time per solve call to *best_ms.
 * Launch shapes and smoother degree are this library's own; no reference counterpart. */
int dpf_batch_autotune(int nprob, const int *dims, const double *mins, const double *maxs, const int64_t *nd,
                       const int64_t *dn, const dpf_options *base, const double *logK, int kind, const double *dh,
                       const double *Qs, const int64_t *obs_offsets, const int64_t *obs, int repeats,
                       dpf_options *best, double *best_ms);

/* Same as dpf_batch_solve_grad_logk for a single problem (nprob = 1 handles of
 * any kind): forward, objective sum_k h[obs_k]^2, adjoint to dlogK. */
int dpf_solve_grad_logk(dpf_problem *h, const double *logK, int mean_kind, const double *dirichleths,
                        const double *Qs, int64_t nobs, const int64_t *obs, double *h_out, double *dlogK);

/* ----------------------------------------------------------- diagnostics */

/* Apply the assembled operator (last forward) to x[N]: y = A x, Dirichlet rows identity. */
int dpf_apply_operator(dpf_problem *h, const double *x, double *y);

/* ------------------------------------------------------------ diagnostics */

/* Start (enable != 0) or stop per-kernel timing: while on, every kernel launch on
 * the handle's stream is bracketed by CUDA events. Enabling clears earlier records. */
int dpf_profile(dpf_problem *h, int enable);

/* Per-kernel totals of the records since dpf_profile(h, 1): up to cap entries of
 * kernel name ("kernel<f64|f32>/L<multigrid level>"), launches, summed device
 * milliseconds and summed cells the launches were scheduled over (any output
 * array may be NULL). Returns the number of distinct kernels (negative
 * dpf_status on error). Names stay valid for the lifetime of the library. */
int dpf_profile_report(dpf_problem *h, int cap, const char **names, long long *launches, double *ms,
                       long long *cells);

/* Kernel launches issued by the handle since it was created. */
long long dpf_launch_count(const dpf_problem *h);

/* No counterpart in the reference. Issue the handle's work on `stream`, a cudaStream_t of
 * the handle's device (NULL: the legacy default stream, the default). Work already issued
 * is completed first. Every entry point still returns when its results are complete;
 * handles on different streams, driven from different host threads, run concurrently. */
int dpf_set_stream(dpf_problem *h, void *stream);

/* ------------------------------------------------------ allocation-free path */

/* No counterpart in the reference. The same face conductances as
 * dpf_logk_to_faces on a regulargrid3d handle, for callers that must not have the
 * library allocate device memory (an application that owns all device memory
 * through its own pool): no handle, no cudaMalloc/cudaFree. logK[nx*ny*nz] and
 * Ks[F] must be device pointers on the current device. The working memory is a
 * fixed 16 MiB module array, so grids are limited to 2,097,152 cells (larger ones
 * get DPF_BAD_INPUT). The first call on a device looks up that array's address;
 * make it before any stream capture. All calls share the array: calls that
 * overlap on the GPU race and must be serialized by the caller. Runs on the
 * legacy default stream and returns when Ks is complete; errors are described by
 * dpf_last_error(NULL). */
int dpf_logk_to_faces_regular_noalloc(int nx, int ny, int nz, const double *logK, int mean_kind, double *Ks);

/* --------------------------------------------------------------- Richards */

/* dpf_create on the CSR path even when the face list is a regular grid (the Richards solver
 * and any caller that wants the general path). Same arguments and errors as dpf_create. */
int dpf_create_general(int64_t N, int64_t F, const int64_t *nbr_a, const int64_t *nbr_b,
                       const double *areasoverlengths, const double *volumes_or_null, int64_t nd,
                       const int64_t *dirichletnodes, const dpf_options *opts, dpf_problem **out);

/* DPFEHM.richards_steadystate (src/richards.jl:148-167) on a dpf_create_general handle: the
 * steady Richards equation with van Genuchten relative permeability (per-face alphas[F] and
 * Ns[F]), harmonic face means of kr and gravity through the cell elevations z[N] (the
 * reference's coords[3, :]). psi0[N] is the initial guess; psi_out[N] carries dirichletpsis at
 * Dirichlet cells. Solved by a Picard iteration with the handle's CG + AMG until the residual is
 * tol (default 1e-10 when <= 0) times max(|R(psi0)|, |Qs|) or maxiter (default 200) steps
 * (DPF_NOT_CONVERGED then). Any argument may be a host or a device pointer. */
int dpf_richards_steady(dpf_problem *h, const double *psi0, const double *Ks, const double *dirichletpsis,
                        const double *z, const double *alphas, const double *Ns, const double *Qs, double tol,
                        int maxiter, double *psi_out);

/* The rrule pullback of richards_steadystate (src/richards.jl:168-190) at the last solve:
 * lambda = J^-T delta by restarted GMRES(30) preconditioned with the Picard operator (each step
 * one CG + AMG solve; to relative residual tol, at most maxiter steps), then dKs[F],
 * ddirichletpsis[N], dalphas[F], dNs[F], dQs[N] (any output may be NULL; the psi0 tangent is
 * zero). */
int dpf_richards_adjoint(dpf_problem *h, const double *delta, double tol, int maxiter, double *dKs,
                         double *ddirichletpsis, double *dalphas, double *dNs, double *dQs);

/* Fixed-step backward Euler of S_i V_i dpsi_i/dt = R_i(psi), R the steady Richards residual
 * above (the reference's richards_residuals with specificstorage and volumes, stepped by
 * DifferentiableBackwardEuler in examples/richards_transient_3d/inputdeck.jl): nsteps steps of dt
 * from psi0[N], each a Picard iteration on S V/dt + A(psi) to tol. Writes psi at the final step
 * to psiT[N] and, if states != NULL, every step to states[nsteps*N]. */
int dpf_richards_transient_forward(dpf_problem *h, const double *psi0, const double *Ks,
                                   const double *dirichletpsis, const double *z, const double *alphas,
                                   const double *Ns, const double *Qs, const double *specificstorage, double dt,
                                   int nsteps, double tol, int maxiter, double *states, double *psiT);

/* Adjoint of the last transient Richards run for
 *   J = sum_{n=1..nsteps} sum_k w_k psi^n[obs_k]^2  +  gT . psi^nsteps
 * (w may be NULL for unit weights, gT may be NULL): backward in time, each step one GMRES solve
 * with the transposed Jacobian (tolerance tol, at most maxiter steps). Outputs dKs[F],
 * ddirichletpsis[N], dalphas[F], dNs[F], dQs[N], dpsi0[N] (any may be NULL). */
int dpf_richards_transient_adjoint(dpf_problem *h, int64_t nobs, const int64_t *obs, const double *w,
                                   const double *gT, double tol, int maxiter, double *dKs,
                                   double *ddirichletpsis, double *dalphas, double *dNs, double *dQs,
                                   double *dpsi0);

/* Picard steps of the last Richards solve (summed over the steps of a transient run), GMRES
 * steps of the last adjoint, and the final relative residual (the largest over the steps). */
int dpf_richards_stats(const dpf_problem *h, int *iterations, int *adjoint_iterations, double *relres);

/* ------------------------------------------------------------ test hooks */

/* No counterpart in the reference. Every device and pinned-host allocation of the
 * library is counted; dpf_debug_fail_alloc(k) makes the k-th following one fail
 * as if the device were out of memory (k = 0: the next one; k < 0: none), once,
 * so that a test can walk each allocation's error path on a healthy device.
 * dpf_debug_alloc_stats reports the allocations made since the library was
 * loaded and those still live (either pointer may be NULL). Process-wide. */
void dpf_debug_fail_alloc(int64_t k);
void dpf_debug_alloc_stats(int64_t *made, int64_t *live);

/* No counterpart in the reference. Runs one block whose threads wait on a
 * shared-memory barrier that nothing arrives on, through the bounded wait every
 * staging kernel uses (one second by the device's global timer). Returns DPF_TIMEOUT when
 * the bound ended the wait as designed, with the milliseconds it took in
 * *waited_ms (may be NULL); any other status is a defect. The device stays usable. */
int dpf_debug_expired_wait(double *waited_ms);

/* No counterpart in the reference. For n doubles v (device memory) the split that the
 * mixed-precision assembly and round start use: v48 = v rounded to 48 significant bits
 * (to nearest, ties away from zero), hi + lo = v48 exactly (two floats), formed with integer
 * operations only; ok[i] = 1 where the split applies (zero, 2^-79 <= |v48| < 2^128), 0 where
 * the FP64 route is taken
 * (outputs then unspecified). All outputs are device arrays of n entries. */
int dpf_debug_split48(int64_t n, const double *v, float *hi, float *lo, double *v48, int *ok);

/* No counterpart in the reference. The band orderings of the direct solver, run on the host (no
 * device needed): for a symmetric graph in CSR form (rp[n + 1], ci, host arrays) the reverse
 * Cuthill-McKee order; for nprob regular grids (dims[3 p .. 3 p + 2] = nx, ny, nz, cells z fastest,
 * problems one after another) the order with each grid's two shortest axes fastest. perm[k] (n
 * entries, host) is the original row of band row k and *w the half-bandwidth the order gives.
 * DPF_BAD_INPUT for malformed arrays or extents. */
int dpf_debug_band_order_graph(int64_t n, const int32_t *rp, const int32_t *ci, int64_t *perm, int64_t *w);
int dpf_debug_band_order_grids(int nprob, const int32_t *dims, int64_t *perm, int64_t *w);

/* No counterpart in the reference. In a library built with DPF_CHECK defined
 * (device-side bounds and alignment checks on cell decodes, stencil neighbours,
 * aggregates, staged copies and CSR columns; a violating access is clamped or
 * skipped, never trapped): the violations recorded since the last call, which are
 * then cleared, and the first one's {site code, index, bound} in first[3] (either
 * pointer may be NULL). Returns DPF_UNSUPPORTED in a library built without them. */
int dpf_debug_check_report(int64_t *violations, int64_t *first);

#ifdef __cplusplus
}
#endif
#endif
