// dpf_struct.h -- host-side class of the structured (regular-grid) batch solver.
#pragma once
#include <array>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "dpf_internal.h"

namespace dpf {

struct DpfError : std::runtime_error {
    int code;
    DpfError(const std::string &m, int c) : std::runtime_error(m), code(c) {}
};
struct BadInput : DpfError {
    explicit BadInput(const std::string &m) : DpfError(m, DPF_BAD_INPUT) {}
};
struct OomError : DpfError {
    explicit OomError(const std::string &m) : DpfError(m, DPF_OOM) {}
};
struct CudaError : DpfError {
    CudaError(const std::string &m, cudaError_t) : DpfError(m, DPF_CUDA) {}
};

struct GridSpec {
    int n[3];                 // nx, ny, nz
    double mins[3], maxs[3];
    bool aol_override = false;
    double aol[3] = {0, 0, 0};
    bool vol_override = false;
    double vol = 0;
};

class StructBatch;
class BandCholesky;

// Counts every kernel launch and, while profiling is on, brackets it with a pair
// of CUDA events on the launching stream (per-kernel device time).
struct KTimer {
    StructBatch *S;
    int slot = -1;
    KTimer(StructBatch *s, const char *name, long long cells);
    ~KTimer();
};

struct ProfRec {
    const char *name;
    int ev;           // index of the first of two events in the pool
    long long cells;  // cells the launch was scheduled over (all problems of its launch map)
};

const char *kname(const char *base, int level, bool fp32);

class StructBatch {
public:
    // Plane-marching work items {p, y0, x0, x1} (slab of rows y0.. of planes x0..x1-1), each
    // block's contiguous range of items (first[b] .. first[b+1]-1), per-problem item ranges (an
    // item's reduction slot is its index), and the largest stage regions (elements)
    struct PlaneItems {
        int4 *items = nullptr;
        int *first = nullptr;
        int2 *pinfo = nullptr;
        int n = 0;   // items
        int nb = 0;  // blocks of a launch
        bool ok = false;
        int cells = 0;  // slab capacity: Ty = cells / nz whole rows
        int halo = 0, cy = 0, slab = 0, coarse = 0;
        int halo2 = 0, cy2 = 0, coarse2 = 0;  // regions of the fused kernels (two halo rows)
    };
    struct Level {
        long long ntot = 0;
        long long all_cells = 0, smooth_cells = 0, coarse_cells = 0;
        std::vector<LevelDesc> h_desc;
        LevelDesc *d_desc = nullptr;
        BlockMap all, smooth;          // every problem with this level / those smoothed by per-level kernels
        BlockMap restr;                // problems whose residual is restricted into this level by a per-level kernel
        long long restr_cells = 0;
        std::vector<int> coarse_list;  // problems whose coarsest level this is
        int *d_coarse = nullptr;
        PlaneItems pm;  // plane-marching launches over the smoothed problems
        PlaneItems pa;  // finest level: plane-marching CG product over all problems
        std::vector<int> csolve_list;  // ... of those, the ones solved by a per-level launch (no fused tail)
        int *d_csolve = nullptr;
        long long csolve_cells = 0;
        uint8_t *dir = nullptr;        // identity (Dirichlet) rows
        double *c64[4] = {nullptr, nullptr, nullptr, nullptr};  // cx, cy, cz, leak
        double *idg64 = nullptr;       // inverse diagonal (FP64 solves)
        __nv_bfloat16 *c16[4] = {nullptr, nullptr, nullptr, nullptr};  // FP32 V-cycle (bf16)
        float *idg32 = nullptr;        // inverse diagonal (FP32 V-cycle)
        void *work[4] = {nullptr, nullptr, nullptr, nullptr};   // xa, xb, b, d (V-cycle precision)
    };

    StructBatch(const std::vector<GridSpec> &grids, const std::vector<std::vector<int64_t>> &dnodes,
                const dpf_options &opt, cudaStream_t stream);
    ~StructBatch();
    StructBatch(const StructBatch &) = delete;
    StructBatch &operator=(const StructBatch &) = delete;

    // operations (device pointers, all ordered on `stream`)
    void assemble(const double *Ks, const double *kc, int kind, const double *shift, bool init_x);
    void cell_k(const double *logK, int kind, double *kc);
    void solve(const double *b, double *x, double reltol);
    void forward(const double *Ks, const double *logK, int kind);
    void adjoint_solve();  // lam = A^-1 delta (Dirichlet rows 0)
    void obs_delta(const long long *d_obs, long long nobs);
    void grad_faces(const double *hv, const double *lv_, double *dKs, bool accumulate);
    void grad_logk(double *g);
    void grad_dh_q(const double *lv_, double *ddh, double *dQs, bool with_delta, bool accumulate);
    void logk_to_faces(const double *logK, int kind, double *Ks);
    void logk_vjp(const double *logK, int kind, const double *dKs, double *g);
    void apply(const double *x, double *y);
    void set_shift(const double *Ss, double dt);
    void transient_step(const double *b0, const double *hprev);

    template <typename T>
    void vcycle(const T *r, T *z);
    void build_plane_items(PlaneItems &P, const Level &L, const std::vector<int> &take, int sms, int cells,
                           int blocks_per_sm, const std::vector<std::vector<std::array<int, 3>>> *shapes, int l);
    template <typename T>
    void launch_tail(const TailParams<T> &tp);
    void write_tail_table();
    // Matern(nu = 1) log-conductivity fields of every problem, drawn on the device (dpf_sampler.cu)
    void sample_logk(int nmodes, const unsigned long long *seeds, const double *ell, const double *sigma,
                     const double *mean, double *out);
    void *dalloc_bytes(size_t bytes);  // a device allocation owned by the batch
    template <typename T>
    void pm_restrict(int l, const T *b, const T *x, T *bc);
    template <typename T>
    void pm_pre2r(int l, const T *b, T *xout, T *bc, T c1, T c2, T invth);
    template <typename T>
    void pm_post2(int l, const T *b, const T *xin, T *xout, const T *e, T c2a, T c1b, T c2b, T sc);
    void pm_df_spmv(const CoeffsDF &C);
    template <typename T>
    void pm_launch(int mode, int l, const T *b, const T *xin, T *xout, T *d, const T *e, T c1, T c2, T invth, T sc);
    template <typename T>
    void pcg(const T *b, T *x, double tol2);
    void df_pcg(const double *b64, double *x64, double tol2);
    template <typename T>
    void pcg_iteration(T *x);
    void df_iteration(double *x64);
    // options.solver = DPF_SOLVER_CHOLESKY: x = A^-1 b by the banded Cholesky factor of the FP64
    // operator (factored again after each assembly); false when the band is too wide for the device
    // (the iterative solve then runs instead)
    bool direct_solve(const double *b, double *x);
    std::unique_ptr<BandCholesky> direct;
    bool direct_tried = false, direct_stale = true, direct_ok = false;
    double *d_direct_acc = nullptr;  // the direct solve's residual sums
    cudaGraphExec_t loop_graph(int kind, void *x);
    void run_loop(int kind, void *x);
    int read_count(int which);
    // the problems' states, the error words, the loop passes and the active count in one
    // synchronisation; returns the active count
    int read_stats();
    bool stats_fresh = false;        // the host copies hold the solve's final statistics

    // configuration and sizes
    dpf_options opt;
    cudaStream_t stream;
    bool mixed = false;
    int nprob = 0, nlev_max = 0;
    std::vector<int> nlev;
    std::vector<long long> ndir;   // distinct Dirichlet cells per problem
    std::vector<Level> lv;
    long long N = 0, F = 0, nfree_total = 0;
    std::vector<long long> cell_off, face_off;
    std::vector<ProbParam> prm;
    ProbParam *d_prm = nullptr;

    // fine-level FP64 vectors
    double *h = nullptr, *b64 = nullptr, *r64 = nullptr, *lam = nullptr, *delta = nullptr, *arhs = nullptr;
    double *in_dh = nullptr, *in_Q = nullptr, *in_logK = nullptr, *in_Ks = nullptr, *shift = nullptr;
    double *in_kc = nullptr, *aux_kc = nullptr;  // per-cell face-mean values of the forward / standalone calls
    void *cgv[4] = {nullptr, nullptr, nullptr, nullptr};  // FP64: r, z, p, q; mixed: r32, z32
    float2 *dfv[4] = {nullptr, nullptr, nullptr, nullptr};  // mixed: -, r, p, q in double-float
    float2 *cdf[4] = {nullptr, nullptr, nullptr, nullptr};  // mixed: finest cx, cy, cz, leak in double-float

    // device state
    CgState *d_state = nullptr;
    int *d_count = nullptr;       // [0] active CG problems, [2] loop passes
    int *d_factor_status = nullptr;  // [0] coarsest factorisation failed, [1] an async-copy wait expired
    ReduceScratch rs;
    double *d_coarseL = nullptr;
    // fused tail: per problem {p, first tail level, coarsest level, 0}; per-level pointer table
    // (TailLevel of the V-cycle precision) written at construction by write_tail_table
    bool zero_guess = false;  // the next solve starts from 0 (Dirichlet values on identity rows)
    // sampler state: per-problem parameters (device and pinned staging) and the modes of the last draw
    void *d_sample = nullptr, *h_sample = nullptr, *d_modes = nullptr;
    long long modes_cap = 0;
    bool have_sampled = false;  // in_logK holds fields drawn by sample_logk
    // device buffer for observation indices, kept between calls (no allocation per call)
    long long *obs_buffer(size_t n);
    long long *d_obs_buf = nullptr;
    size_t obs_cap = 0;
    std::vector<int4> tails;
    int4 *d_tails = nullptr;
    void *d_tail_lv = nullptr;
    long long tail_cells_total = 0;
    int tail_cs = 0;  // cluster size actually used for the tail (0: not yet chosen)
    int *h_misc = nullptr;           // pinned: error words and graph passes read with the statistics
    long long graph_body_kernels = 0;  // kernels per pass of the loop graph used by the current solve
    int tail_first_level = 0;
    int *h_count = nullptr;
    void *h_state_buf = nullptr;
    struct GraphRec {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        long long body_kernels = 0;
    };
    struct GraphKey {
        int kind;
        void *x;
        bool operator<(const GraphKey &o) const { return kind != o.kind ? kind < o.kind : x < o.x; }
    };
    std::map<GraphKey, GraphRec> graphs;  // CG loop graphs per (vector size, buffers)
    cudaStream_t cap_stream = nullptr;    // streams used only to capture graphs

    // Chebyshev
    double inv_theta = 1.0;
    std::vector<double> cheb_c1, cheb_c2;

    // last-call bookkeeping
    bool have_operator = false, have_forward = false;
    int fwd_kind = 0, mean_kind = 0;
    int last_status = DPF_OK, stats_iters = 0, stats_outer = 0;
    double stats_relres = 0.0;
    std::string last_message;

    // launch counting / per-kernel timing
    long long launches = 0;
    bool prof_on = false;
    std::vector<ProfRec> prof_recs;
    std::vector<cudaEvent_t> ev_pool;
    void profile(bool on);
    int profile_report(int cap, const char **names, long long *counts, double *ms, long long *cells);

    DevList owned;                   // every device allocation of the batch
    HostList pinned;                 // h_count, h_misc, h_state_buf
};

}  // namespace dpf
