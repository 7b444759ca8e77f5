// dpf_richards.cu -- steady Richards equation on a face-list (CSR) handle, and its adjoint.
//
// Residual at the free cells (DPFEHM src/richards.jl:98-118, steady: S = V = 1):
//   R_j = Q_j + sum_{f = (j, k)} hm(kr(psi_j), kr(psi_k)) K_f aol_f (psi_k + z_k - psi_j - z_j)
// with the van Genuchten relative permeability kr(psi; alpha_f, N_f) of the face's parameters
// (src/richards.jl:18-27), hm(x, y) = 2 / (1/x + 1/y) (:50-52), and psi_k = dirichletpsis[k] at a
// Dirichlet neighbour. The reference solves R = 0 by Newton (NLsolve, :148-166) and its rrule solves
// the transposed Jacobian system (:168-190).
//
// Here the nonlinear solve is a Picard iteration: A(psi) d = R(psi), psi += d, where A(psi) is the
// groundwater operator with face conductances K_f hm(kr_j, kr_k) (symmetric positive definite,
// solved by the handle's CG + AMG), with step halving while the residual does not drop. Writing
// the Jacobian as J = -A + N (N: the terms of the derivatives of kr), the adjoint
// J^T lambda = delta becomes, with mu = -lambda, (I - A^-1 N^T) mu = A^-1 delta, solved by
// restarted GMRES(30) whose every step is one N^T product and one CG + AMG solve (the plain
// fixed point mu = A^-1 (delta + N^T mu) can diverge: an eigenvalue of A^-1 N^T below -1 is what
// the forward iteration's step halving damps). Both reach the roots of the reference's
// equations; only the iteration differs. Transient runs take fixed backward-Euler steps of
// S V dpsi/dt = R(psi) on the shifted operator S V / dt + A(psi), and the adjoint runs backward
// in time over the stored states.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <vector>

#include "dpf_general.h"
#include "dpf_struct_kernels.cuh"

namespace dpf {

namespace {

constexpr int kRBlock = 256;

#define RSTRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// van Genuchten kr(psi; alpha, N) and its derivatives by psi, alpha and N (psi >= 0: kr = 1)
struct Kr {
    double v, dpsi, dalpha, dN;
};

__device__ Kr kr_vg(double psi, double alpha, double N) {
    Kr k{1.0, 0.0, 0.0, 0.0};
    if (!(psi < 0.0)) return k;
    const double m = (N - 1.0) / N;
    const double ap = fabs(alpha * psi);                 // u
    const double uN = pow(ap, N), uN1 = pow(ap, N - 1.0);
    const double A = 1.0 + uN;
    const double Am = pow(A, -m);
    const double numer = 1.0 - uN1 * Am;
    const double Amh = pow(A, -0.5 * m);
    k.v = numer * numer * Amh;
    // by u: d numer = -(N-1) u^(N-2) A^-m + m N u^(2N-2) A^(-m-1); d A = N u^(N-1)
    const double uN2 = ap > 0.0 ? uN1 / ap : 0.0;
    const double dnum_du = -(N - 1.0) * uN2 * Am + m * N * uN1 * uN1 * Am / A;
    const double dkr_du = 2.0 * numer * dnum_du * Amh - 0.5 * m * numer * numer * Amh / A * N * uN1;
    k.dpsi = dkr_du * (-alpha);   // u = -alpha psi for psi < 0, alpha > 0
    k.dalpha = dkr_du * fabs(psi);
    // by N (m = 1 - 1/N, dm/dN = 1/N^2); u^N and u^(N-1) gain a factor ln u
    if (ap > 0.0) {
        const double lu = log(ap), lA = log(A), dm = 1.0 / (N * N);
        const double dA = uN * lu;
        const double dAm = Am * (-dm * lA - m * dA / A);
        const double dnum = -(uN1 * lu * Am + uN1 * dAm);
        const double dAmh = Amh * (-0.5 * dm * lA - 0.5 * m * dA / A);
        k.dN = 2.0 * numer * dnum * Amh + numer * numer * dAmh;
    }
    return k;
}

// Per face: Picard conductance K hm (kr_a, kr_b), the flux-derivative parts of the Jacobian
// (na, nb) and the face difference of the total head.
__global__ void kr_faces(int F, const int *__restrict__ fa, const int *__restrict__ fb,
                         const double *__restrict__ aol, const double *__restrict__ Ks,
                         const double *__restrict__ alphas, const double *__restrict__ Ns,
                         const double *__restrict__ psi, const double *__restrict__ z, double *__restrict__ Kh,
                         double *__restrict__ na, double *__restrict__ nb) {
    RSTRIDE(f, F) {
        const int a = fa[f], b = fb[f];
        const Kr ka = kr_vg(psi[a], alphas[f], Ns[f]), kb = kr_vg(psi[b], alphas[f], Ns[f]);
        const double s = ka.v + kb.v;
        const double is = s > 0.0 ? 1.0 / s : 0.0;  // both kr zero: no conductance
        const double H = 2.0 * ka.v * kb.v * is;
        const double dHa = 2.0 * kb.v * kb.v * is * is * ka.dpsi, dHb = 2.0 * ka.v * ka.v * is * is * kb.dpsi;
        const double D = psi[b] + z[b] - psi[a] - z[a];
        const double Ka = Ks[f] * aol[f];
        Kh[f] = Ks[f] * H;
        if (na) {
            na[f] = Ka * dHa * D;
            nb[f] = -Ka * dHb * D;
        }
    }
}

// R_j = Q_j + sum_f Kh_f aol_f (psi_k + z_k - psi_j - z_j) at free cells, 0 at Dirichlet
// cells, minus shift_j (psi_j - psi_old_j) in a backward-Euler step (shift = S V / dt, null
// when steady); per-block partial sums of R^2 and Q^2 (fixed order: deterministic)
__global__ void richards_residual(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                                  const int *__restrict__ fa, const int *__restrict__ fb,
                                  const double *__restrict__ aol, const double *__restrict__ Kh,
                                  const uint8_t *__restrict__ dir, const double *__restrict__ psi,
                                  const double *__restrict__ z, const double *__restrict__ Qs,
                                  const double *__restrict__ shift, const double *__restrict__ psi_old,
                                  double *__restrict__ R, double2 *__restrict__ part) {
    // part[b] = (|R|^2, |Q|^2) and part[gridDim.x + b] = (floor^2, 0) of this block's cells, where
    // the floor of a cell is twice the FP64 rounding bound of its residual: u (|Q| + the storage
    // term's operands + per face K aol (|psi_j + z_j| + |h_i| + |flux difference|)), u = 2^-53
    double rr = 0.0, qq = 0.0, ff = 0.0;
    RSTRIDE(i, n) {
        double r = 0.0;
        if (!dir[i]) {
            r = Qs[i];
            double fl = fabs(Qs[i]);
            if (shift) {
                r -= shift[i] * (psi[i] - psi_old[i]);
                fl += shift[i] * (fabs(psi[i]) + fabs(psi_old[i]));
            }
            const double hi = psi[i] + z[i];
            for (int k = irp[i]; k < irp[i + 1]; k++) {
                const int f = ifc[k];
                const int j = fa[f] == i ? fb[f] : fa[f];
                if (!DPF_INSIDE(CK_NEIGHBOUR, j, 0, n)) continue;
                const double hj = psi[j] + z[j], c = Kh[f] * aol[f];
                r += c * (hj - hi);
                fl += c * (fabs(hj) + fabs(hi) + fabs(hj - hi));
            }
            qq += Qs[i] * Qs[i];
            const double f2 = 0x1p-52 * fl;
            ff += f2 * f2;
        }
        R[i] = r;
        rr += r * r;
    }
    __shared__ double sr[kRBlock], sq[kRBlock], sf[kRBlock];
    sr[threadIdx.x] = rr;
    sq[threadIdx.x] = qq;
    sf[threadIdx.x] = ff;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sr[threadIdx.x] += sr[threadIdx.x + s];
            sq[threadIdx.x] += sq[threadIdx.x + s];
            sf[threadIdx.x] += sf[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = make_double2(sr[0], sq[0]);
        part[gridDim.x + blockIdx.x] = make_double2(sf[0], 0.0);
    }
}

// psi += w d at free cells; per-block sums of (w d)^2 and psi^2
__global__ void richards_update(int n, const uint8_t *__restrict__ dir, double w, const double *__restrict__ d,
                                double *__restrict__ psi, double2 *__restrict__ part) {
    double dd = 0.0, pp = 0.0;
    RSTRIDE(i, n) {
        if (!dir[i]) {
            const double s = w * d[i];
            psi[i] += s;
            dd += s * s;
        }
        pp += psi[i] * psi[i];
    }
    __shared__ double sd[kRBlock], sp[kRBlock];
    sd[threadIdx.x] = dd;
    sp[threadIdx.x] = pp;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sd[threadIdx.x] += sd[threadIdx.x + s];
            sp[threadIdx.x] += sp[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sd[0], sp[0]);
}

// psi = dirichletpsis at Dirichlet cells, psi0 elsewhere
__global__ void richards_init(int n, const uint8_t *__restrict__ dir, const double *__restrict__ psi0,
                              const double *__restrict__ dpsi, double *__restrict__ psi) {
    RSTRIDE(i, n) psi[i] = dir[i] ? dpsi[i] : psi0[i];
}

// rhs_i = delta_i + (N^T mu)_i at free cells, 0 at Dirichlet cells;
// (N^T mu)_a = sum_f na_f (mu_a - mu_b), (N^T mu)_b = sum_f nb_f (mu_b - mu_a), mu = 0 at Dirichlet cells
__global__ void richards_adjoint_rhs(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                                     const int *__restrict__ fa, const int *__restrict__ fb,
                                     const double *__restrict__ na, const double *__restrict__ nb,
                                     const uint8_t *__restrict__ dir, const double *__restrict__ delta,
                                     const double *__restrict__ mu, double *__restrict__ rhs) {
    RSTRIDE(i, n) {
        double r = 0.0;
        if (!dir[i]) {
            r = delta[i];
            if (mu) {
                const double mi = mu[i];
                for (int k = irp[i]; k < irp[i + 1]; k++) {
                    const int f = ifc[k];
                    const bool isa = fa[f] == i;
                    const int j = isa ? fb[f] : fa[f];
                    if (!DPF_INSIDE(CK_NEIGHBOUR, j, 0, n)) continue;
                    const double mj = dir[j] ? 0.0 : mu[j];
                    r += (isa ? na[f] : nb[f]) * (mi - mj);
                }
            }
        }
        rhs[i] = r;
    }
}

// per-block sums of (mu_new - mu)^2 and mu_new^2; mu = mu_new
__global__ void richards_mu_step(int n, const double *__restrict__ mnew, double *__restrict__ mu,
                                 double2 *__restrict__ part) {
    double dd = 0.0, mm = 0.0;
    RSTRIDE(i, n) {
        const double d = mnew[i] - mu[i];
        dd += d * d;
        mm += mnew[i] * mnew[i];
        mu[i] = mnew[i];
    }
    __shared__ double sd[kRBlock], sm[kRBlock];
    sd[threadIdx.x] = dd;
    sm[threadIdx.x] = mm;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sd[threadIdx.x] += sd[threadIdx.x + s];
            sm[threadIdx.x] += sm[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sd[0], sm[0]);
}

// Face gradients with mu = -lambda (0 at Dirichlet cells): dK_f = H aol D (mu_a - mu_b);
// dalpha_f, dN_f = K aol D (mu_a - mu_b) dH/d(.)
__global__ void richards_face_grads(int F, const int *__restrict__ fa, const int *__restrict__ fb,
                                    const double *__restrict__ aol, const double *__restrict__ Ks,
                                    const double *__restrict__ alphas, const double *__restrict__ Ns,
                                    const double *__restrict__ psi, const double *__restrict__ z,
                                    const uint8_t *__restrict__ dir, const double *__restrict__ mu,
                                    double *__restrict__ dK, double *__restrict__ dal, double *__restrict__ dN,
                                    int accumulate) {
    RSTRIDE(f, F) {
        const int a = fa[f], b = fb[f];
        const Kr ka = kr_vg(psi[a], alphas[f], Ns[f]), kb = kr_vg(psi[b], alphas[f], Ns[f]);
        const double s = ka.v + kb.v;
        const double is = s > 0.0 ? 1.0 / s : 0.0;
        const double H = 2.0 * ka.v * kb.v * is;
        const double wa = 2.0 * kb.v * kb.v * is * is, wb = 2.0 * ka.v * ka.v * is * is;
        const double D = psi[b] + z[b] - psi[a] - z[a];
        const double dm = (dir[a] ? 0.0 : mu[a]) - (dir[b] ? 0.0 : mu[b]);
        const double c = Ks[f] * aol[f] * D * dm;
        if (dK) dK[f] = (accumulate ? dK[f] : 0.0) + H * aol[f] * D * dm;
        if (dal) dal[f] = (accumulate ? dal[f] : 0.0) + c * (wa * ka.dalpha + wb * kb.dalpha);
        if (dN) dN[f] = (accumulate ? dN[f] : 0.0) + c * (wa * ka.dN + wb * kb.dN);
    }
}

// dQ_j = mu_j at free cells; ddirichletpsis_k = delta_k + sum_{f=(j,k), j free} mu_j dF_jk/dpsi_k
// at Dirichlet cells (dF_jk/dpsi_k = K aol (dH/dpsi_k D_jk + H))
__global__ void richards_cell_grads(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                                    const int *__restrict__ fa, const int *__restrict__ fb,
                                    const double *__restrict__ aol, const double *__restrict__ Ks,
                                    const double *__restrict__ alphas, const double *__restrict__ Ns,
                                    const double *__restrict__ psi, const double *__restrict__ z,
                                    const uint8_t *__restrict__ dir, const double *__restrict__ mu,
                                    const double *__restrict__ delta, double *__restrict__ dQ,
                                    double *__restrict__ ddp, int accumulate) {
    RSTRIDE(k, n) {
        if (dQ) dQ[k] = (accumulate ? dQ[k] : 0.0) + (dir[k] ? 0.0 : mu[k]);
        if (!ddp) continue;
        if (!dir[k]) {
            if (!accumulate) ddp[k] = 0.0;
            continue;
        }
        double g = (accumulate ? ddp[k] : 0.0) + delta[k];
        for (int e = irp[k]; e < irp[k + 1]; e++) {
            const int f = ifc[e];
            const int j = fa[f] == k ? fb[f] : fa[f];
            if (!DPF_INSIDE(CK_NEIGHBOUR, j, 0, n)) continue;
            if (dir[j]) continue;
            const Kr kk = kr_vg(psi[k], alphas[f], Ns[f]), kj = kr_vg(psi[j], alphas[f], Ns[f]);
            const double s = kk.v + kj.v;
            const double is = s > 0.0 ? 1.0 / s : 0.0;
            const double H = 2.0 * kk.v * kj.v * is;
            const double dHk = 2.0 * kj.v * kj.v * is * is * kk.dpsi;
            const double Djk = psi[k] + z[k] - psi[j] - z[j];
            g += mu[j] * Ks[f] * aol[f] * (dHk * Djk + H);
        }
        ddp[k] = g;
    }
}

// shift = S V / dt per cell (the backward-Euler storage term)
__global__ void richards_shift(int n, const double *__restrict__ Ss, const double *__restrict__ vol, double rdt,
                               double *__restrict__ shift) {
    RSTRIDE(i, n) shift[i] = Ss[i] * vol[i] * rdt;
}

// transient adjoint seed: s_i = 2 w_k psi_i at observation cells (+ gT_i at the last step)
__global__ void richards_seed(int nobs, const long long *__restrict__ obs, const double *__restrict__ w,
                              const double *__restrict__ psi, double *__restrict__ seed) {
    RSTRIDE(k, nobs) {
        const long long i = obs[k];
        atomicAdd(&seed[i], 2.0 * (w ? w[k] : 1.0) * psi[i]);  // a cell observed twice gets both terms
    }
}

// rhs = seed + shift lam_next at free cells, 0 at Dirichlet cells
__global__ void richards_trans_rhs(int n, const uint8_t *__restrict__ dir, const double *__restrict__ seed,
                                   const double *__restrict__ shift, const double *__restrict__ lam_next,
                                   double *__restrict__ rhs) {
    RSTRIDE(i, n) rhs[i] = dir[i] ? 0.0 : seed[i] + shift[i] * lam_next[i];
}

// per-block partial sums of x . y
__global__ void vec_dot(int n, const double *__restrict__ x, const double *__restrict__ y, double2 *__restrict__ part) {
    double s = 0.0;
    RSTRIDE(i, n) s += x[i] * y[i];
    __shared__ double sh[kRBlock];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sh[0], 0.0);
}

// y = a x + b y
__global__ void vec_axpby(int n, double a, const double *__restrict__ x, double b, double *__restrict__ y) {
    RSTRIDE(i, n) y[i] = a * x[i] + b * y[i];
}

#undef RSTRIDE

}  // namespace

static void rck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e), e);
    }
}
#define GLAUNCH_CHECK()                      \
    do {                                     \
        launches++;                          \
        rck(cudaGetLastError(), "kernel launch"); \
    } while (0)

static bool r_is_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static void rcopy_out(double *dst, const double *src, size_t n, cudaStream_t s) {
    if (!dst) return;
    rck(cudaMemcpyAsync(dst, src, n * sizeof(double), r_is_device(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                        s),
        "copy out");
}

static unsigned rblocks(long long n, int cap) {
    return (unsigned)std::max(1LL, std::min((n + kRBlock - 1) / kRBlock, (long long)cap));
}

// sums of the per-block partials, in block order
static double2 sum_parts(const double2 *d_part, int nb, cudaStream_t s) {
    std::vector<double2> h(nb);
    if (cudaMemcpyAsync(h.data(), d_part, nb * sizeof(double2), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        const cudaError_t e = cudaGetLastError();
        throw CudaError(std::string("reduction read-back: ") + cudaGetErrorString(e), e);
    }
    double2 t = make_double2(0.0, 0.0);
    for (const double2 &v : h) {
        t.x += v.x;
        t.y += v.y;
    }
    return t;
}

void GeneralSolver::richards_buffers() {
    if (rc_psi) return;
    rc_psi = dev<double>(N);
    rc_R = dev<double>(N);
    rc_d = dev<double>(N);
    rc_mu = dev<double>(N);
    rc_z = dev<double>(N);
    rc_dpsi = dev<double>(N);
    rc_zero = dev<double>(N);
    rc_Ks = dev<double>(F);
    rc_al = dev<double>(F);
    rc_N = dev<double>(F);
    rc_Kh = dev<double>(F);
    rc_na = dev<double>(F);
    rc_nb = dev<double>(F);
    rc_Q = dev<double>(N);
    rc_delta = dev<double>(N);
    rc_gK = dev<double>(F);
    rc_ga = dev<double>(F);
    rc_gN = dev<double>(F);
    rc_part = dev<double2>(2 * (size_t)nblocks);  // the residual kernel's sums and rounding floors
    rck(cudaMemsetAsync(rc_zero, 0, N * sizeof(double), stream), "zero");
}

// One SPD solve (shift + A(Kh)) x = rhs (x = 0 at Dirichlet cells) with the handle's CG + AMG;
// shift = S V / dt in a backward-Euler step, null when steady.
int GeneralSolver::richards_spd_solve(const double *rhs_dev, double *x_dev, const double *shift_dev) {
    rck(cudaMemcpyAsync(in_Q, rhs_dev, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "rhs");
    rck(cudaMemcpyAsync(in_dh, rc_zero, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "dh");
    assemble(rc_Kh, nullptr, 0, shift_dev, true);
    solve(b64, h);
    rck(cudaMemcpyAsync(x_dev, h, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "solution");
    rck(cudaStreamSynchronize(stream), "sync");
    return finish_status();
}

// Nonlinear solve of one steady or backward-Euler Richards system from the current rc_psi:
// Picard steps (shift + A(psi)) d = G(psi), G = R(psi) - shift (psi - psi_old), halved while the
// residual does not drop, until |G| <= tol max(|G(psi_0)|, |Q|) or maxit steps. The iteration
// also ends, converged, at the FP64 rounding floor of G: when |G| is within the floor's bound,
// or when a step (with all its halvings) no longer lowers |G| and |G| is within 100 times the
// bound. No further accuracy exists in FP64 there (heads of 1000 m leave a floor above a
// tolerance of 1e-12 times |Q|). Leaves the Picard conductances and the Jacobian parts at the
// result in rc_Kh, rc_na, rc_nb.
int GeneralSolver::richards_nonlinear(const double *shift_dev, const double *psi_old, double tol, int maxit,
                                      int &iters, double &relres) {
    const unsigned nbF = rblocks(F, nblocks), nbN = rblocks(N, nblocks);
    double floor2 = 0.0;  // squared rounding floor of the last residual evaluated
    auto residual = [&]() -> double2 {
        kr_faces<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z, rc_Kh,
                                              nullptr, nullptr);
        GLAUNCH_CHECK();
        richards_residual<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, faol, rc_Kh, lv[0].dir, rc_psi,
                                                       rc_z, rc_Q, shift_dev, psi_old, rc_R, rc_part);
        GLAUNCH_CHECK();
        floor2 = sum_parts(rc_part + nbN, (int)nbN, stream).x;
        return sum_parts(rc_part, (int)nbN, stream);
    };
    const double2 rq = residual();
    const double r0 = std::sqrt(rq.x), scale = std::max(r0, std::sqrt(rq.y));
    double rn = r0;
    int it = 0;
    bool at_floor = rn * rn <= floor2;
    while (rn > tol * scale && !at_floor && it < maxit) {
        const int src = richards_spd_solve(rc_R, rc_d, shift_dev);
        if (src != DPF_OK && src != DPF_NOT_CONVERGED) return src;
        double w = 1.0, applied = 0.0;
        for (int k = 0; k < 6; k++) {
            richards_update<<<nbN, kRBlock, 0, stream>>>((int)N, lv[0].dir, w - applied, rc_d, rc_psi, rc_part);
            GLAUNCH_CHECK();
            applied = w;
            const double rnew = std::sqrt(residual().x);
            if (rnew < rn || k == 5) {
                if (rnew >= rn && rnew * rnew <= 1e4 * floor2) at_floor = true;  // stalled at the floor
                rn = rnew;
                break;
            }
            w *= 0.5;
        }
        if (rn * rn <= floor2) at_floor = true;
        it++;
    }
    iters = it;
    relres = scale > 0 ? rn / scale : 0.0;
    kr_faces<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z, rc_Kh, rc_na,
                                          rc_nb);
    GLAUNCH_CHECK();
    rck(cudaStreamSynchronize(stream), "sync");
    if (!std::isfinite(rn)) return DPF_NAN;
    return (rn > tol * scale && !at_floor) ? DPF_NOT_CONVERGED : DPF_OK;
}

// (shift + A - N^T) x = rhs at the Jacobian parts in rc_Kh, rc_na, rc_nb: with M = shift + A
// (the Picard operator, solved by CG + AMG), (I - M^-1 N^T) x = M^-1 rhs by restarted GMRES(30).
// x = 0 at Dirichlet cells; iters and the final relative residual are returned.
int GeneralSolver::richards_gmres(const double *rhs_dev, double *x_dev, const double *shift_dev, double tol,
                                  int maxit, int &iters, double &rel) {
    const unsigned nbN = rblocks(N, nblocks);
    const int m = 30;
    if (rc_V.empty()) {
        for (int k = 0; k <= m; k++) rc_V.push_back(dev<double>(N));
        rc_c = dev<double>(N);
    }
    auto dot = [&](const double *x, const double *y) {
        vec_dot<<<nbN, kRBlock, 0, stream>>>((int)N, x, y, rc_part);
        GLAUNCH_CHECK();
        return sum_parts(rc_part, (int)nbN, stream).x;
    };
    auto axpby = [&](double a, const double *x, double b, double *y) {
        vec_axpby<<<nbN, kRBlock, 0, stream>>>((int)N, a, x, b, y);
        GLAUNCH_CHECK();
    };
    auto apply = [&](const double *v, double *out) -> int {  // out = v - M^-1 N^T v
        richards_adjoint_rhs<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, rc_na, rc_nb, lv[0].dir, rc_zero,
                                                          v, rc_R);
        GLAUNCH_CHECK();
        const int src = richards_spd_solve(rc_R, out, shift_dev);
        if (src != DPF_OK && src != DPF_NOT_CONVERGED) return src;
        axpby(1.0, v, -1.0, out);
        return DPF_OK;
    };
    int rc = richards_spd_solve(rhs_dev, rc_c, shift_dev);  // c = M^-1 rhs
    if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) return rc;
    const double cnorm = std::sqrt(dot(rc_c, rc_c));
    rck(cudaMemsetAsync(x_dev, 0, N * sizeof(double), stream), "zero");
    int it = 0;
    rel = cnorm > 0 ? 1.0 : 0.0;
    std::vector<double> Hm((m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    while (rel > tol && it < maxit) {
        int r2 = apply(x_dev, rc_V[0]);  // r = c - (I - M^-1 N^T) x
        if (r2 != DPF_OK) return r2;
        axpby(1.0, rc_c, -1.0, rc_V[0]);
        const double beta = std::sqrt(dot(rc_V[0], rc_V[0]));
        if (!std::isfinite(beta)) return DPF_NAN;
        rel = cnorm > 0 ? beta / cnorm : 0.0;
        if (rel <= tol) break;
        axpby(0.0, rc_V[0], 1.0 / beta, rc_V[0]);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (; k < m && it < maxit; k++, it++) {
            r2 = apply(rc_V[k], rc_V[k + 1]);
            if (r2 != DPF_OK) return r2;
            for (int i2 = 0; i2 <= k; i2++) {  // modified Gram-Schmidt
                const double h2 = dot(rc_V[k + 1], rc_V[i2]);
                Hm[i2 * m + k] = h2;
                axpby(-h2, rc_V[i2], 1.0, rc_V[k + 1]);
            }
            const double hn = std::sqrt(dot(rc_V[k + 1], rc_V[k + 1]));
            Hm[(k + 1) * m + k] = hn;
            if (hn > 0) axpby(0.0, rc_V[k + 1], 1.0 / hn, rc_V[k + 1]);
            for (int i2 = 0; i2 < k; i2++) {  // the earlier Givens rotations
                const double a = Hm[i2 * m + k], b = Hm[(i2 + 1) * m + k];
                Hm[i2 * m + k] = cs[i2] * a + sn[i2] * b;
                Hm[(i2 + 1) * m + k] = -sn[i2] * a + cs[i2] * b;
            }
            const double a = Hm[k * m + k], b = Hm[(k + 1) * m + k];
            const double r = std::hypot(a, b);
            cs[k] = r > 0 ? a / r : 1.0;
            sn[k] = r > 0 ? b / r : 0.0;
            Hm[k * m + k] = r;
            Hm[(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            rel = cnorm > 0 ? std::fabs(g[k + 1]) / cnorm : 0.0;
            if (!std::isfinite(rel)) return DPF_NAN;
            if (rel <= tol || hn == 0) {
                k++;
                it++;
                break;
            }
        }
        for (int i2 = k - 1; i2 >= 0; i2--) {  // x += V y with H y = g
            double s2 = g[i2];
            for (int j2 = i2 + 1; j2 < k; j2++) s2 -= Hm[i2 * m + j2] * y[j2];
            y[i2] = s2 / Hm[i2 * m + i2];
        }
        for (int i2 = 0; i2 < k; i2++) axpby(y[i2], rc_V[i2], 1.0, x_dev);
    }
    iters = it;
    return rc;
}

void GeneralSolver::richards_stage(const double *Ks, const double *dpsi, const double *z, const double *alphas,
                                   const double *Ns, const double *Qs, const double *psi0) {
    richards_buffers();
    stage(Ks, F, rc_Ks);
    stage(alphas, F, rc_al);
    stage(Ns, F, rc_N);
    stage(z, N, rc_z);
    stage(dpsi, N, rc_dpsi);
    stage(Qs, N, rc_Q);
    stage(psi0, N, rc_d);
    richards_init<<<rblocks(N, nblocks), kRBlock, 0, stream>>>((int)N, lv[0].dir, rc_d, rc_dpsi, rc_psi);
    GLAUNCH_CHECK();
}

int GeneralSolver::richards_steady(const double *psi0, const double *Ks, const double *dpsi, const double *z,
                                   const double *alphas, const double *Ns, const double *Qs, double tol, int maxit,
                                   double *psi_out) {
    if (nfree == N) throw BadInput("the problem has no Dirichlet cell: the steady-state operator is singular");
    richards_stage(Ks, dpsi, z, alphas, Ns, Qs, psi0);
    have_richards = false;
    const int rc = richards_nonlinear(nullptr, nullptr, tol, maxit, rich_iters, rich_relres);
    rcopy_out(psi_out, rc_psi, N, stream);
    rck(cudaStreamSynchronize(stream), "sync");
    have_richards = rc == DPF_OK || rc == DPF_NOT_CONVERGED;
    if (rc == DPF_NOT_CONVERGED) last_message = "the Richards iteration did not reach its tolerance";
    else if (rc == DPF_NAN) last_message = "non-finite Richards residual";
    return rc;
}

int GeneralSolver::richards_adjoint(const double *delta_in, double tol, int maxit, double *dKs, double *ddpsi,
                                    double *dalphas, double *dNs, double *dQs) {
    if (!have_richards) throw DpfError("richards adjoint called before a Richards solve", DPF_STATE);
    stage(delta_in, N, rc_delta);
    const unsigned nbF = rblocks(F, nblocks), nbN = rblocks(N, nblocks);
    // mu = -lambda: (A - N^T) mu = delta at the free cells
    richards_adjoint_rhs<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, rc_na, rc_nb, lv[0].dir, rc_delta,
                                                      nullptr, rc_d);
    GLAUNCH_CHECK();
    double rel = 0.0;
    const int rc = richards_gmres(rc_d, rc_mu, nullptr, tol, maxit, rich_adj_iters, rel);
    if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) return rc;
    richards_face_grads<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z,
                                                     lv[0].dir, rc_mu, dKs ? rc_gK : nullptr,
                                                     dalphas ? rc_ga : nullptr, dNs ? rc_gN : nullptr, 0);
    GLAUNCH_CHECK();
    richards_cell_grads<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi,
                                                     rc_z, lv[0].dir, rc_mu, rc_delta, dQs ? rc_d : nullptr,
                                                     ddpsi ? rc_R : nullptr, 0);
    GLAUNCH_CHECK();
    rcopy_out(dKs, rc_gK, F, stream);
    rcopy_out(dalphas, rc_ga, F, stream);
    rcopy_out(dNs, rc_gN, F, stream);
    rcopy_out(dQs, rc_d, N, stream);
    rcopy_out(ddpsi, rc_R, N, stream);
    rck(cudaStreamSynchronize(stream), "sync");
    if (rel > tol) {
        last_message = "the Richards adjoint iteration did not reach its tolerance";
        return DPF_NOT_CONVERGED;
    }
    return DPF_OK;
}

// ---- transient: fixed-step backward Euler of S_i V_i dpsi_i/dt = R_i(psi) (the reference's
// richards_residuals with specific storage and volumes, stepped by an external integrator)
int GeneralSolver::richards_transient_forward(const double *psi0, const double *Ks, const double *dpsi,
                                              const double *z, const double *alphas, const double *Ns,
                                              const double *Qs, const double *Ss, double dt, int nsteps, double tol,
                                              int maxit, double *states, double *psiT) {
    if (!(dt > 0) || nsteps < 1) throw BadInput("dt must be positive and nsteps at least 1");
    richards_stage(Ks, dpsi, z, alphas, Ns, Qs, psi0);
    have_richards = false;
    rt_nsteps = 0;
    if (!rt_shift) rt_shift = dev<double>(N);
    if (rt_cap < nsteps) {
        drop(rt_states);
        rt_states = dev<double>((size_t)(nsteps + 1) * N);  // psi^0 .. psi^nsteps
        rt_cap = nsteps;
    }
    stage(Ss, N, rc_d);
    richards_shift<<<rblocks(N, nblocks), kRBlock, 0, stream>>>((int)N, rc_d, vol, 1.0 / dt, rt_shift);
    GLAUNCH_CHECK();
    rck(cudaMemcpyAsync(rt_states, rc_psi, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "state");
    int worst = DPF_OK, total = 0;
    double rr = 0.0;
    for (int n = 1; n <= nsteps; n++) {
        int it = 0;
        double rel = 0.0;
        const int rc = richards_nonlinear(rt_shift, rt_states + (size_t)(n - 1) * N, tol, maxit, it, rel);
        if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) {
            last_message = rc == DPF_NAN ? "non-finite Richards residual" : last_message;
            return rc;
        }
        if (rc == DPF_NOT_CONVERGED) worst = rc;
        total += it;
        rr = std::max(rr, rel);
        rck(cudaMemcpyAsync(rt_states + (size_t)n * N, rc_psi, N * sizeof(double), cudaMemcpyDeviceToDevice, stream),
            "state");
        if (states)
            rck(cudaMemcpyAsync(states + (size_t)(n - 1) * N, rc_psi, N * sizeof(double),
                                r_is_device(states) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream),
                "states");
    }
    rcopy_out(psiT, rc_psi, N, stream);
    rck(cudaStreamSynchronize(stream), "sync");
    rich_iters = total;
    rich_relres = rr;
    rt_nsteps = nsteps;
    if (worst == DPF_NOT_CONVERGED) last_message = "a Richards step did not reach its tolerance";
    return worst;
}

// Adjoint of the last transient run for J = sum_{n=1..nsteps} sum_k w_k psi^n[obs_k]^2 + gT . psi^nsteps:
// backward in time (shift + A - N^T)(psi^n) lam^n = dJ/dpsi^n + shift lam^(n+1), the tangents
// sum_n (dR(psi^n)/dp)^T lam^n, and dpsi0 = shift lam^1.
int GeneralSolver::richards_transient_adjoint(long long nobs, const int64_t *obs, const double *w, const double *gT,
                                              double tol, int maxit, double *dKs, double *ddpsi, double *dalphas,
                                              double *dNs, double *dQs, double *dpsi0) {
    if (rt_nsteps < 1) throw DpfError("transient Richards adjoint called before a transient Richards run", DPF_STATE);
    const unsigned nbF = rblocks(F, nblocks), nbN = rblocks(N, nblocks);
    std::vector<long long> ho(nobs);
    if (nobs && r_is_device(obs)) {
        rck(cudaMemcpyAsync(ho.data(), obs, nobs * sizeof(int64_t), cudaMemcpyDeviceToHost, stream), "obs");
        rck(cudaStreamSynchronize(stream), "obs");
    } else if (nobs) {
        std::memcpy(ho.data(), obs, nobs * sizeof(int64_t));
    }
    for (long long k = 0; k < nobs; k++)
        if (ho[k] < 0 || ho[k] >= N) throw BadInput("observation index out of range");
    long long *d_obs = dev<long long>(std::max(nobs, 1LL));
    double *d_w = w ? dev<double>(std::max(nobs, 1LL)) : nullptr;
    double *d_gT = gT ? dev<double>(N) : nullptr;
    if (nobs) rck(cudaMemcpyAsync(d_obs, ho.data(), nobs * sizeof(long long), cudaMemcpyHostToDevice, stream), "obs");
    if (w) stage(w, nobs, d_w);
    if (gT) stage(gT, N, d_gT);
    if (!rt_gQ) {
        rt_gQ = dev<double>(N);
        rt_gD = dev<double>(N);
        rt_lam = dev<double>(N);
    }
    double *lam = rc_mu, *seed = rc_delta, *lam_hold = rt_lam;
    rck(cudaMemsetAsync(lam_hold, 0, N * sizeof(double), stream), "zero");  // lam^(nsteps+1) = 0
    int worst = DPF_OK, total = 0;
    const int nsteps = rt_nsteps;
    for (int n = nsteps; n >= 1; n--) {
        const double *psi_n = rt_states + (size_t)n * N;
        rck(cudaMemcpyAsync(rc_psi, psi_n, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "state");
        kr_faces<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z, rc_Kh, rc_na,
                                              rc_nb);
        GLAUNCH_CHECK();
        // seed = dJ/dpsi^n
        if (n == nsteps && d_gT)
            rck(cudaMemcpyAsync(seed, d_gT, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "gT");
        else
            rck(cudaMemsetAsync(seed, 0, N * sizeof(double), stream), "seed");
        if (nobs) {
            richards_seed<<<rblocks(nobs, nblocks), kRBlock, 0, stream>>>((int)nobs, d_obs, d_w, rc_psi, seed);
            GLAUNCH_CHECK();
        }
        richards_trans_rhs<<<nbN, kRBlock, 0, stream>>>((int)N, lv[0].dir, seed, rt_shift, lam_hold, rc_R);
        GLAUNCH_CHECK();
        rck(cudaMemcpyAsync(rc_d, rc_R, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "rhs");
        int it = 0;
        double rel = 0.0;
        const int rc = richards_gmres(rc_d, lam, rt_shift, tol, maxit, it, rel);
        if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) return rc;
        if (rel > tol) worst = DPF_NOT_CONVERGED;
        total += it;
        const int acc = n == nsteps ? 0 : 1;
        richards_face_grads<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z,
                                                         lv[0].dir, lam, dKs ? rc_gK : nullptr,
                                                         dalphas ? rc_ga : nullptr, dNs ? rc_gN : nullptr, acc);
        GLAUNCH_CHECK();
        richards_cell_grads<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi,
                                                         rc_z, lv[0].dir, lam, seed, dQs ? rt_gQ : nullptr,
                                                         ddpsi ? rt_gD : nullptr, acc);
        GLAUNCH_CHECK();
        rck(cudaMemcpyAsync(lam_hold, lam, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "lam");
    }
    // dpsi0 = shift lam^1 at the free cells
    if (dpsi0) {
        richards_trans_rhs<<<nbN, kRBlock, 0, stream>>>((int)N, lv[0].dir, rc_zero, rt_shift, lam_hold, rc_R);
        GLAUNCH_CHECK();
    }
    rcopy_out(dKs, rc_gK, F, stream);
    rcopy_out(dalphas, rc_ga, F, stream);
    rcopy_out(dNs, rc_gN, F, stream);
    rcopy_out(dQs, rt_gQ, N, stream);
    rcopy_out(ddpsi, rt_gD, N, stream);
    rcopy_out(dpsi0, rc_R, N, stream);
    rck(cudaStreamSynchronize(stream), "sync");
    drop(d_obs);
    drop(d_w);
    drop(d_gT);
    rich_adj_iters = total;
    if (worst == DPF_NOT_CONVERGED) last_message = "a Richards adjoint step did not reach its tolerance";
    return worst;
}

}  // namespace dpf
