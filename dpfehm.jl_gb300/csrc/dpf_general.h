// dpf_general.h -- CSR (general topology) groundwater solver.
#pragma once
#include <vector>

#include "dpf_struct.h"

namespace dpf {

class GeneralSolver {
public:
    GeneralSolver(long long N, long long F, const int64_t *a, const int64_t *b, const double *aol,
                  const double *volumes, long long nd, const int64_t *dn, const dpf_options &opt,
                  cudaStream_t stream);
    ~GeneralSolver();
    int forward(const double *Ks, const double *logK, int kind, const double *dh, const double *Qs, double *h_out);
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
    int nlevels() const;

    long long N = 0, F = 0, nfree = 0;
    int stats_iters = 0, stats_outer = 0;
    long long launches = 0;
    double stats_relres = 0.0;
};

}  // namespace dpf
