// dpf_general.h -- CSR (general topology) groundwater solver.
//
// For face lists that are not a regulargrid3d (unstructured meshes read by
// load_uge, graphs with extra or duplicated faces). Same formulation as the
// structured path: all N cells, Dirichlet cells as identity rows with decoupled
// faces, operator applied in flux form y_i = leak_i x_i + sum_e c_e (x_i - x_j)
// over the CSR couplings of row i. Multigrid by greedy graph aggregation (set up
// once per topology on the host; the numeric Galerkin rebuild each forward is a
// deterministic gather on the device).
#pragma once
#include <memory>
#include <vector>

#include "dpf_struct.h"

namespace dpf {

struct GLevel {
    int n = 0, nnz = 0;
    int *rp = nullptr, *ci = nullptr;        // couplings (no diagonal)
    double *v64 = nullptr, *leak64 = nullptr, *idg64 = nullptr;
    float *v32 = nullptr, *leak32 = nullptr, *idg32 = nullptr;
    uint8_t *dir = nullptr;                   // identity rows
    // transfer to the next coarser level
    int *agg = nullptr;                       // fine cell -> aggregate (-1: none)
    int *mrp = nullptr, *mci = nullptr;       // aggregate -> member cells (next level's row order)
    int *crp = nullptr, *cci = nullptr;       // coarse coupling -> contributing fine couplings
    void *work[4] = {nullptr, nullptr, nullptr, nullptr};  // xa, xb, b, d
    bool dense = false;                       // coarsest level solved by its dense inverse
};

class GeneralSolver {
public:
    GeneralSolver(long long N, long long F, const int64_t *a, const int64_t *b, const double *aol,
                  const double *volumes, long long nd, const int64_t *dn, const dpf_options &opt,
                  cudaStream_t stream);
    ~GeneralSolver();
    GeneralSolver(const GeneralSolver &) = delete;
    GeneralSolver &operator=(const GeneralSolver &) = delete;

    int forward(const double *Ks, const double *logK, int kind, const double *dh, const double *Qs, double *h_out);
    void set_stream(cudaStream_t s) { stream = s; }
    int adjoint(const double *delta, double *dKs, double *dlogK, double *ddh, double *dQs);
    int logk_to_faces(const double *logK, int kind, double *Ks);
    int logk_vjp(const double *logK, int kind, const double *dKs, double *dlogK);
    int solve_grad_logk(const double *logK, int kind, const double *dh, const double *Qs, long long nobs,
                        const int64_t *obs, double *h_out, double *dlogK);
    int apply(const double *x, double *y);
    int transient_forward(const double *Ks, const double *dh, const double *Qs, const double *Ss, double dt,
                          int nsteps, const double *h0, double *states, double *hT);
    int transient_adjoint(long long nobs, const int64_t *obs, const double *w, const double *gT, double *dKs,
                          double *ddh, double *dQs, double *dh0);
    int nlevels() const { return (int)lv.size(); }
    // steady Richards equation (dpf_richards.cu): Picard iteration to `tol` (relative residual),
    // and the adjoint fixed point for the reference rrule's tangents
    int richards_steady(const double *psi0, const double *Ks, const double *dpsi, const double *z,
                        const double *alphas, const double *Ns, const double *Qs, double tol, int maxit,
                        double *psi_out);
    int richards_adjoint(const double *delta, double tol, int maxit, double *dKs, double *ddpsi, double *dalphas,
                         double *dNs, double *dQs);
    int richards_transient_forward(const double *psi0, const double *Ks, const double *dpsi, const double *z,
                                   const double *alphas, const double *Ns, const double *Qs, const double *Ss,
                                   double dt, int nsteps, double tol, int maxit, double *states, double *psiT);
    int richards_transient_adjoint(long long nobs, const int64_t *obs, const double *w, const double *gT, double tol,
                                   int maxit, double *dKs, double *ddpsi, double *dalphas, double *dNs, double *dQs,
                                   double *dpsi0);
    int rich_iters = 0, rich_adj_iters = 0;
    double rich_relres = 0.0;

    long long N = 0, F = 0, nfree = 0;
    int stats_iters = 0, stats_outer = 0;
    double stats_relres = 0.0;
    long long launches = 0;
    // per-kernel timing (dpf_profile): event pairs around the iteration kernels while on
    bool prof_on = false;
    std::vector<ProfRec> prof_recs;
    std::vector<cudaEvent_t> ev_pool;
    void profile(bool on);
    int profile_report(int cap, const char **names, long long *counts, double *ms, long long *cells);
    std::string last_message;

private:
    friend struct GTimer;
    void setup_topology(const int64_t *a, const int64_t *b, const double *aol, const double *volumes, long long nd,
                        const int64_t *dn);
    void build_hierarchy();
    void assemble(const double *Ks, const double *kc, int kind, const double *shift, bool init_x);
    void solve(const double *b, double *x);
    // options.solver = DPF_SOLVER_CHOLESKY: x = A^-1 b by the banded Cholesky factor of the FP64
    // operator in reverse Cuthill-McKee order (factored again after each assembly); false when the
    // band is too wide for the device (the iterative solve then runs instead)
    bool direct_solve(const double *b, double *x);
    std::unique_ptr<BandCholesky> direct;
    bool direct_tried = false, direct_stale = true, direct_ok = false;
    double *d_direct_acc = nullptr;
    template <typename T>
    void vcycle(const T *r, T *z);
    template <typename T>
    void pcg(const T *b, T *x, double tol2);
    void df_pcg(const double *b64, double *x64, double tol2);
    void adjoint_solve(const double *delta_dev);
    int finish_status();
    int read_active();
    // whether the CG loop reads its convergence after iteration `it`: every check_every
    // iterations, but up to two iterations before the one at which the previous solve's first
    // round stopped (loop_hint) only every eighth, since each read is a host synchronisation
    bool check_due(int it) const;
    int loop_hint = 0;
    template <typename T>
    T *dev(size_t n);
    void drop(void *p);            // free an allocation made by dev() (nullptr: nothing)
    void to_dev(void *dst, const void *src, size_t bytes);
    void from_dev(void *dst, const void *src, size_t bytes);
    std::vector<long long> read_indices(const int64_t *idx, long long n);
    const double *stage(const double *src, size_t n, double *dst);
    void richards_buffers();
    void richards_stage(const double *Ks, const double *dpsi, const double *z, const double *alphas,
                        const double *Ns, const double *Qs, const double *psi0);
    int richards_spd_solve(const double *rhs_dev, double *x_dev, const double *shift_dev);
    int richards_nonlinear(const double *shift_dev, const double *psi_old, double tol, int maxit, int &iters,
                           double &relres);
    int richards_gmres(const double *rhs_dev, double *x_dev, const double *shift_dev, double tol, int maxit,
                       int &iters, double &rel);

    dpf_options opt;
    cudaStream_t stream;
    bool mixed = false;
    int nblocks = 0;                         // grid of every cell- or entry-parallel launch
    std::vector<GLevel> lv;
    DevList owned;                 // every device allocation of the solver
    HostList pinned;               // h_count, h_state

    // topology (device)
    int *fa = nullptr, *fb = nullptr;        // face ends
    double *faol = nullptr;                  // areas over lengths
    int *e_face = nullptr;                   // fine coupling -> face
    int *irp = nullptr, *ifc = nullptr;      // cell -> incident faces
    double *vol = nullptr;                   // cell volumes
    // vectors
    double *h = nullptr, *b64 = nullptr, *r64 = nullptr, *lam = nullptr, *delta = nullptr, *arhs = nullptr;
    double *in_Ks = nullptr, *in_kc = nullptr, *aux_kc = nullptr, *in_dh = nullptr, *in_Q = nullptr;
    double *shift = nullptr, *tmpN = nullptr, *tmpF = nullptr;
    void *cgv[4] = {nullptr, nullptr, nullptr, nullptr};
    float2 *dfv[4] = {nullptr, nullptr, nullptr, nullptr};
    float2 *vdf = nullptr, *leakdf = nullptr;
    double *dense_inv = nullptr;
    // CG state
    CgState *d_state = nullptr;
    int *d_count = nullptr;
    int *d_status = nullptr;
    int *h_count = nullptr;
    CgState *h_state = nullptr;
    ReduceScratch rs;
    int2 *d_pinfo = nullptr;
    double inv_theta = 1.0;
    std::vector<double> cheb_c1, cheb_c2;
    std::vector<double> cheb8_c1, cheb8_c2;  // degree-8 sweep standing in for a coarsest solve
    std::vector<int> hrp_, hci_;             // finest couplings on the host (hierarchy set-up)
    // Richards: psi, residual, step, adjoint mu, z, Dirichlet psi, zeros, sources, delta (N);
    // Ks, alphas, Ns, Picard conductances, Jacobian parts, gradients (F); reduction partials
    double *rc_psi = nullptr, *rc_R = nullptr, *rc_d = nullptr, *rc_mu = nullptr, *rc_z = nullptr;
    double *rc_dpsi = nullptr, *rc_zero = nullptr, *rc_Q = nullptr, *rc_delta = nullptr;
    double *rc_Ks = nullptr, *rc_al = nullptr, *rc_N = nullptr, *rc_Kh = nullptr, *rc_na = nullptr, *rc_nb = nullptr;
    double *rc_gK = nullptr, *rc_ga = nullptr, *rc_gN = nullptr;
    double2 *rc_part = nullptr;
    std::vector<double *> rc_V;    // GMRES basis of the Richards adjoint
    double *rc_c = nullptr;        // its preconditioned right-hand side
    // transient Richards: states psi^0..psi^n, storage shift S V / dt, adjoint buffers
    double *rt_states = nullptr, *rt_shift = nullptr, *rt_gQ = nullptr, *rt_gD = nullptr, *rt_lam = nullptr;
    int rt_cap = 0, rt_nsteps = 0;
    bool have_richards = false;
    // bookkeeping
    bool have_forward = false;
    int fwd_kind = 0, mean_kind = 0;
    int tr_nsteps = 0;
    double *tr_b0 = nullptr, *tr_states = nullptr;
    std::vector<int> h_dir;
};

}  // namespace dpf
