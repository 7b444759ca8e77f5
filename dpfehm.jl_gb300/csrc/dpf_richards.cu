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
// solved by the handle's CG + AMG). Writing the Jacobian as J = -A + N (N: the terms of the
// derivatives of kr), the adjoint J^T lambda = delta becomes, with mu = -lambda, the fixed point
// mu = A^-1 (delta + N^T mu); its contraction factor is that of the Picard iteration at the
// solution, so it converges wherever the forward iteration does. Both reach the roots of the
// reference's equations; only the iteration differs.
#include <algorithm>
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
// cells; per-block partial sums of R^2 and Q^2 (fixed order: deterministic)
__global__ void richards_residual(int n, const int *__restrict__ irp, const int *__restrict__ ifc,
                                  const int *__restrict__ fa, const int *__restrict__ fb,
                                  const double *__restrict__ aol, const double *__restrict__ Kh,
                                  const uint8_t *__restrict__ dir, const double *__restrict__ psi,
                                  const double *__restrict__ z, const double *__restrict__ Qs, double *__restrict__ R,
                                  double2 *__restrict__ part) {
    double rr = 0.0, qq = 0.0;
    RSTRIDE(i, n) {
        double r = 0.0;
        if (!dir[i]) {
            r = Qs[i];
            const double hi = psi[i] + z[i];
            for (int k = irp[i]; k < irp[i + 1]; k++) {
                const int f = ifc[k];
                const int j = fa[f] == i ? fb[f] : fa[f];
                r += Kh[f] * aol[f] * (psi[j] + z[j] - hi);
            }
            qq += Qs[i] * Qs[i];
        }
        R[i] = r;
        rr += r * r;
    }
    __shared__ double sr[kRBlock], sq[kRBlock];
    sr[threadIdx.x] = rr;
    sq[threadIdx.x] = qq;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            sr[threadIdx.x] += sr[threadIdx.x + s];
            sq[threadIdx.x] += sq[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sr[0], sq[0]);
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
                                    double *__restrict__ dK, double *__restrict__ dal, double *__restrict__ dN) {
    RSTRIDE(f, F) {
        const int a = fa[f], b = fb[f];
        const Kr ka = kr_vg(psi[a], alphas[f], Ns[f]), kb = kr_vg(psi[b], alphas[f], Ns[f]);
        const double s = ka.v + kb.v;
        const double is = s > 0.0 ? 1.0 / s : 0.0;
        const double H = 2.0 * ka.v * kb.v * is;
        const double wa = 2.0 * kb.v * kb.v * is * is, wb = 2.0 * ka.v * ka.v * is * is;
        const double D = psi[b] + z[b] - psi[a] - z[a];
        const double dm = (dir[a] ? 0.0 : mu[a]) - (dir[b] ? 0.0 : mu[b]);
        if (dK) dK[f] = H * aol[f] * D * dm;
        const double c = Ks[f] * aol[f] * D * dm;
        if (dal) dal[f] = c * (wa * ka.dalpha + wb * kb.dalpha);
        if (dN) dN[f] = c * (wa * ka.dN + wb * kb.dN);
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
                                    double *__restrict__ ddp) {
    RSTRIDE(k, n) {
        if (dQ) dQ[k] = dir[k] ? 0.0 : mu[k];
        if (!ddp) continue;
        if (!dir[k]) {
            ddp[k] = 0.0;
            continue;
        }
        double g = delta[k];
        for (int e = irp[k]; e < irp[k + 1]; e++) {
            const int f = ifc[e];
            const int j = fa[f] == k ? fb[f] : fa[f];
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
    rc_part = dev<double2>(nblocks);
    rck(cudaMemsetAsync(rc_zero, 0, N * sizeof(double), stream), "zero");
}

// One SPD solve A(Kh) x = rhs (x = 0 at Dirichlet cells) with the handle's CG + AMG.
int GeneralSolver::richards_spd_solve(const double *rhs_dev, double *x_dev) {
    rck(cudaMemcpyAsync(in_Q, rhs_dev, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "rhs");
    rck(cudaMemcpyAsync(in_dh, rc_zero, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "dh");
    assemble(rc_Kh, nullptr, 0, nullptr, true);
    solve(b64, h);
    rck(cudaMemcpyAsync(x_dev, h, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "solution");
    rck(cudaStreamSynchronize(stream), "sync");
    return finish_status();
}

int GeneralSolver::richards_steady(const double *psi0, const double *Ks, const double *dpsi, const double *z,
                                   const double *alphas, const double *Ns, const double *Qs, double tol, int maxit,
                                   double *psi_out) {
    if (nfree == N) throw BadInput("the problem has no Dirichlet cell: the steady-state operator is singular");
    richards_buffers();
    stage(Ks, F, rc_Ks);
    stage(alphas, F, rc_al);
    stage(Ns, F, rc_N);
    stage(z, N, rc_z);
    stage(dpsi, N, rc_dpsi);
    stage(Qs, N, rc_Q);
    const double *Qd = rc_Q;
    stage(psi0, N, rc_d);
    const unsigned nbF = rblocks(F, nblocks), nbN = rblocks(N, nblocks);
    richards_init<<<nbN, kRBlock, 0, stream>>>((int)N, lv[0].dir, rc_d, rc_dpsi, rc_psi);
    GLAUNCH_CHECK();
    auto residual = [&]() -> double2 {
        kr_faces<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z, rc_Kh,
                                              nullptr, nullptr);
        GLAUNCH_CHECK();
        richards_residual<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, faol, rc_Kh, lv[0].dir, rc_psi,
                                                       rc_z, Qd, rc_R, rc_part);
        GLAUNCH_CHECK();
        return sum_parts(rc_part, (int)nbN, stream);
    };
    double2 rq = residual();
    const double r0 = std::sqrt(rq.x), scale = std::max(r0, std::sqrt(rq.y));
    double rn = r0;
    int it = 0, rc = DPF_OK;
    rich_iters = 0;
    while (rn > tol * scale && it < maxit) {
        // Picard step d = A(psi)^-1 R(psi), halved while it does not reduce the residual
        const int src = richards_spd_solve(rc_R, rc_d);
        if (src != DPF_OK && src != DPF_NOT_CONVERGED) return src;
        double w = 1.0, applied = 0.0;
        for (int k = 0; k < 6; k++) {
            richards_update<<<nbN, kRBlock, 0, stream>>>((int)N, lv[0].dir, w - applied, rc_d, rc_psi, rc_part);
            GLAUNCH_CHECK();
            applied = w;
            const double2 r = residual();
            const double rnew = std::sqrt(r.x);
            if (rnew < rn || k == 5) {
                rn = rnew;
                break;
            }
            w *= 0.5;
        }
        it++;
    }
    rich_iters = it;
    rich_relres = scale > 0 ? rn / scale : 0.0;
    if (!std::isfinite(rn)) rc = DPF_NAN;
    else if (rn > tol * scale) rc = DPF_NOT_CONVERGED;
    // the solution (Dirichlet values included) and the face terms at it, for the adjoint
    rcopy_out(psi_out, rc_psi, N, stream);
    kr_faces<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z, rc_Kh, rc_na,
                                          rc_nb);
    GLAUNCH_CHECK();
    rck(cudaStreamSynchronize(stream), "sync");
    have_richards = rc == DPF_OK || rc == DPF_NOT_CONVERGED;
    if (rc == DPF_NOT_CONVERGED) last_message = "the Richards iteration did not reach its tolerance";
    else if (rc == DPF_NAN) last_message = "non-finite Richards residual";
    return rc;
}

int GeneralSolver::richards_adjoint(const double *delta_in, double tol, int maxit, double *dKs, double *ddpsi,
                                    double *dalphas, double *dNs, double *dQs) {
    if (!have_richards) throw DpfError("richards adjoint called before a Richards solve", DPF_STATE);
    double *dl = rc_delta;
    stage(delta_in, N, dl);
    const unsigned nbF = rblocks(F, nblocks), nbN = rblocks(N, nblocks);
    // (I - A^-1 N^T) mu = A^-1 delta by restarted GMRES (the Picard operator A preconditions the
    // transposed Jacobian -J^T = A - N^T); mu = 0 at Dirichlet cells throughout
    const int m = 30;
    if (rc_V.empty()) {
        for (int k = 0; k <= m; k++) rc_V.push_back(dev<double>(N));
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
    int rc = DPF_OK;
    auto apply = [&](const double *v, double *out) -> int {  // out = v - A^-1 N^T v
        richards_adjoint_rhs<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, rc_na, rc_nb, lv[0].dir, rc_zero,
                                                          v, rc_R);
        GLAUNCH_CHECK();
        const int src = richards_spd_solve(rc_R, out);
        if (src != DPF_OK && src != DPF_NOT_CONVERGED) return src;
        axpby(1.0, v, -1.0, out);
        return DPF_OK;
    };
    // c = A^-1 delta (free cells)
    richards_adjoint_rhs<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, rc_na, rc_nb, lv[0].dir, dl, nullptr,
                                                      rc_R);
    GLAUNCH_CHECK();
    rc = richards_spd_solve(rc_R, rc_d);
    if (rc != DPF_OK && rc != DPF_NOT_CONVERGED) return rc;
    const double cnorm = std::sqrt(dot(rc_d, rc_d));
    rck(cudaMemsetAsync(rc_mu, 0, N * sizeof(double), stream), "zero");
    int it = 0;
    double rel = cnorm > 0 ? 1.0 : 0.0;
    std::vector<double> Hm((m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    while (rel > tol && it < maxit) {
        // r = c - M mu into V0
        int r2 = apply(rc_mu, rc_V[0]);
        if (r2 != DPF_OK) return r2;
        axpby(1.0, rc_d, -1.0, rc_V[0]);
        double beta = std::sqrt(dot(rc_V[0], rc_V[0]));
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
            for (int i2 = 0; i2 < k; i2++) {  // earlier Givens rotations
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
        // mu += V y, H y = g
        for (int i2 = k - 1; i2 >= 0; i2--) {
            double s2 = g[i2];
            for (int j2 = i2 + 1; j2 < k; j2++) s2 -= Hm[i2 * m + j2] * y[j2];
            y[i2] = s2 / Hm[i2 * m + i2];
        }
        for (int i2 = 0; i2 < k; i2++) axpby(y[i2], rc_V[i2], 1.0, rc_mu);
    }
    rich_adj_iters = it;
    // gradients at the solution
    double *gK = dKs ? rc_gK : nullptr;
    double *ga = dalphas ? rc_ga : nullptr;
    double *gN = dNs ? rc_gN : nullptr;
    richards_face_grads<<<nbF, kRBlock, 0, stream>>>((int)F, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi, rc_z,
                                                     lv[0].dir, rc_mu, gK, ga, gN);
    GLAUNCH_CHECK();
    double *gQ = dQs ? rc_d : nullptr;
    double *gD = ddpsi ? rc_R : nullptr;
    richards_cell_grads<<<nbN, kRBlock, 0, stream>>>((int)N, irp, ifc, fa, fb, faol, rc_Ks, rc_al, rc_N, rc_psi,
                                                     rc_z, lv[0].dir, rc_mu, dl, gQ, gD);
    GLAUNCH_CHECK();
    if (dKs) rcopy_out(dKs, gK, F, stream);
    if (dalphas) rcopy_out(dalphas, ga, F, stream);
    if (dNs) rcopy_out(dNs, gN, F, stream);
    if (dQs) rcopy_out(dQs, gQ, N, stream);
    if (ddpsi) rcopy_out(ddpsi, gD, N, stream);
    rck(cudaStreamSynchronize(stream), "sync");
    if (rel > tol) {
        last_message = "the Richards adjoint iteration did not reach its tolerance";
        return DPF_NOT_CONVERGED;
    }
    return rc;
}

}  // namespace dpf
