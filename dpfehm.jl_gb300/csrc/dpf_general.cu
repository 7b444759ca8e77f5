// dpf_general.cu -- CSR (general topology) groundwater solver (placeholder until the CSR kernels land).
#include "dpf_general.h"

namespace dpf {

GeneralSolver::GeneralSolver(long long, long long, const int64_t *, const int64_t *, const double *, const double *,
                             long long, const int64_t *, const dpf_options &, cudaStream_t) {
    throw DpfError("general (non-regular) topologies are not supported yet", DPF_UNSUPPORTED);
}
GeneralSolver::~GeneralSolver() {}
int GeneralSolver::forward(const double *, const double *, int, const double *, const double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::adjoint(const double *, double *, double *, double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::logk_to_faces(const double *, int, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::logk_vjp(const double *, int, const double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::solve_grad_logk(const double *, int, const double *, const double *, long long, const int64_t *,
                                   double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::apply(const double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::transient_forward(const double *, const double *, const double *, const double *, double, int,
                                     const double *, double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::transient_adjoint(long long, const int64_t *, const double *, const double *, double *, double *,
                                     double *, double *) { return DPF_UNSUPPORTED; }
int GeneralSolver::nlevels() const { return 0; }

}  // namespace dpf
