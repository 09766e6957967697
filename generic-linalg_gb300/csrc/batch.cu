// batch.cu -- entry points for many independent systems (no reference counterpart: the
// reference solves one system per call, e.g. tests/multishift/multishift.cpp:446-489).
//
// glinalg_cg_m_multi: multishift CG for n_rhs sources of one operator (all sources in one
//                     CUDA graph, cgm_batch.cu, for the staggered-normal and Laplace kinds).
// glinalg_cg_batch:   CG on n_sys independent Hermitian systems of any sizes (mixed precision:
//                     all systems advanced by the same kernels, cg_batch.cu).

#include <vector>

#include "solvers.h"

using namespace glinalg;

static glinalg_status cg_m_each_impl(const glinalg_operator_s *op, double2 *X, const double2 *B, int n_rhs,
                                     int n_shift, int resid_freq_check, int max_iter, double eps,
                                     const double *shifts, glinalg_info *infos, cudaStream_t st);

extern "C" glinalg_status glinalg_cg_m_multi(glinalg_operator op, double *phi, const double *phi0,
                                             int n_rhs, int n_shift, int size, int resid_freq_check,
                                             int max_iter, double eps, const double *shifts,
                                             const glinalg_solver_params *params,
                                             glinalg_info *infos)
{
    if (!op || !phi || !phi0 || !shifts || !infos || n_rhs <= 0 || n_shift <= 0)
        return GLINALG_ERROR_INVALID_VALUE;
    if ((long)size != op->size || resid_freq_check <= 0)
        return invalid_arg("(long)size != op->size || resid_freq_check <= 0");
    GL_TRY(ensure_device());
    const bool dev = params && (params->flags & GLINALG_PTR_DEVICE);
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long n = op->size;
    double2 *X = (double2 *)phi;
    const double2 *B = (const double2 *)phi0;
    if (!dev) {
        double2 *tx, *tb;
        GL_TRY(sc.alloc(&tx, (size_t)n * n_rhs * n_shift));
        GL_TRY(sc.alloc(&tb, (size_t)n * n_rhs));
        GL_CUDA(cudaMemcpyAsync(tb, phi0, sizeof(double2) * n * n_rhs, cudaMemcpyHostToDevice, st));
        X = tx;
        B = tb;
    }
    const int prec = params ? params->precision : GLINALG_PREC_DOUBLE;
    if (prec != GLINALG_PREC_DOUBLE) {
        if (prec != GLINALG_PREC_SINGLE || !cg_m_batch_mixed_supported(op, n_shift)) {
            set_last_error("mixed-precision multishift needs precision SINGLE, the staggered normal operator "
                           "and at most 32 shifts");
            return GLINALG_ERROR_UNSUPPORTED_OP;
        }
        GL_TRY(cg_m_batch_mixed(op, X, B, n_rhs, n_shift, resid_freq_check, max_iter, eps, shifts, infos, st));
    } else if (cg_m_batch_supported(op, n_shift)) {
        GL_TRY(cg_m_batch(op, X, B, n_rhs, n_shift, resid_freq_check, max_iter, eps, shifts, infos, st));
    } else {
        // other operator kinds: one source after another
        GL_TRY(cg_m_each_impl(op, X, B, n_rhs, n_shift, resid_freq_check, max_iter, eps, shifts, infos, st));
    }
    if (!dev)
        GL_CUDA(cudaMemcpyAsync(phi, X, sizeof(double2) * n * n_rhs * n_shift, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

static glinalg_status cg_m_each_impl(const glinalg_operator_s *op, double2 *X, const double2 *B, int n_rhs,
                                     int n_shift, int resid_freq_check, int max_iter, double eps,
                                     const double *shifts, glinalg_info *infos, cudaStream_t st)
{
    const long n = op->size;
    const Verb quiet;
    for (int q = 0; q < n_rhs; q++) {
        std::vector<double2 *> xs(n_shift);
        for (int j = 0; j < n_shift; j++) xs[j] = X + ((size_t)q * n_shift + j) * n;
        double *keep = infos[q].resSqmrhs;
        infos[q] = glinalg_info{};
        infos[q].resSqmrhs = keep;
        GL_TRY(cg_m_fp64(op, xs.data(), B + (size_t)q * n, n_shift, resid_freq_check, max_iter, eps,
                         shifts, false, quiet, &infos[q], st));
    }
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_cg_batch(const glinalg_operator *ops, int n_sys, double *const *phi,
                                           const double *const *phi0, int max_iter, double eps,
                                           const glinalg_solver_params *params, glinalg_info *infos)
{
    if (!ops || !phi || !phi0 || !infos || n_sys <= 0)
        return invalid_arg("!ops || !phi || !phi0 || !infos || n_sys <= 0");
    for (int q = 0; q < n_sys; q++)
        if (!ops[q] || !phi[q] || !phi0[q] ||
            !(ops[q]->kind == GLINALG_OP_STAGGERED_NORMAL || ops[q]->kind == GLINALG_OP_LAPLACE))
            return GLINALG_ERROR_INVALID_VALUE;
    GL_TRY(ensure_device());
    const bool dev = params && (params->flags & GLINALG_PTR_DEVICE);
    const int prec = params ? params->precision : GLINALG_PREC_DOUBLE;
    const double delta = params && params->delta > 0 ? params->delta : 0.0;  // 0: the per-precision default
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    std::vector<double2 *> xs(n_sys);
    std::vector<const double2 *> bs(n_sys);
    for (int q = 0; q < n_sys; q++) {
        const long n = ops[q]->size;
        xs[q] = (double2 *)phi[q];
        bs[q] = (const double2 *)phi0[q];
        if (!dev) {
            double2 *tx, *tb;
            GL_TRY(sc.alloc(&tx, n));
            GL_TRY(sc.alloc(&tb, n));
            GL_CUDA(cudaMemcpyAsync(tx, phi[q], sizeof(double2) * n, cudaMemcpyHostToDevice, st));
            GL_CUDA(cudaMemcpyAsync(tb, phi0[q], sizeof(double2) * n, cudaMemcpyHostToDevice, st));
            xs[q] = tx;
            bs[q] = tb;
        }
    }
    if (prec != GLINALG_PREC_DOUBLE) {
        // every system advanced by the same kernels (cg_batch.cu)
        std::vector<const glinalg_operator_s *> po(ops, ops + n_sys);
        GL_TRY(cg_batch_mixed(po.data(), n_sys, xs.data(), bs.data(), max_iter, eps, prec, delta, infos, st));
    } else {
        // FP64: the reference recurrence, one system after another
        const Verb quiet;
        for (int q = 0; q < n_sys; q++) {
            double *keep = infos[q].resSqmrhs;
            infos[q] = glinalg_info{};
            infos[q].resSqmrhs = keep;
            GL_TRY(cg_fp64(ops[q], xs[q], bs[q], max_iter, eps, quiet, &infos[q], st));
        }
    }
    if (!dev)
        for (int q = 0; q < n_sys; q++)
            GL_CUDA(cudaMemcpyAsync(phi[q], xs[q], sizeof(double2) * ops[q]->size, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}
