// capi_solvers.cu -- extern "C" solver entry points (include/glinalg.h): argument checks,
// host/device staging of phi and phi0, precision dispatch, then the device solvers.

#include <cmath>
#include <vector>

#include "solvers.h"

using namespace glinalg;

namespace {

struct SolveCall {
    cudaStream_t st;
    Scratch sc;
    Staged sg;
    bool dev = false;
    SolveCall() : st(lib_stream()), sc(st) {}
};

glinalg_status finish_call(SolveCall &c, double *phi, long n)
{
    GL_TRY(c.sg.finish(phi, n, c.dev, c.st));
    GL_CUDA(cudaStreamSynchronize(c.st));
    return GLINALG_SUCCESS;
}

glinalg_status prologue(glinalg_operator op, double *phi, const double *phi0, int size,
                        const glinalg_solver_params *params, glinalg_info *info, SolveCall &c)
{
    if (!info) return GLINALG_ERROR_INVALID_VALUE;
    GL_TRY(check_solver_args(op, phi, phi0, size, &c.dev, params));
    GL_TRY(c.sg.stage(c.sc, phi, phi0, op->size, c.dev, c.st));
    double *keep = info->resSqmrhs;
    int keep_n = info->n_rhs;
    *info = glinalg_info{};
    info->resSqmrhs = keep;
    info->n_rhs = keep_n;
    return GLINALG_SUCCESS;
}

int precision_of(const glinalg_solver_params *p) { return p ? p->precision : GLINALG_PREC_DOUBLE; }
double delta_of(const glinalg_solver_params *p) { return p && p->delta > 0 ? p->delta : 0.1; }

}  // namespace

extern "C" glinalg_status glinalg_cg(glinalg_operator op, double *phi, const double *phi0, int size,
                                     int max_iter, double eps, const glinalg_verbosity *verb,
                                     const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(ensure_device());
    SolveCall c;
    GL_TRY(prologue(op, phi, phi0, size, params, info, c));
    const Verb v = Verb::from(verb);
    const int prec = precision_of(params);
    if (prec == GLINALG_PREC_DOUBLE) GL_TRY(cg_fp64(op, c.sg.x, c.sg.b, max_iter, eps, v, info, c.st));
    else GL_TRY(cg_mixed(op, c.sg.x, c.sg.b, max_iter, eps, prec, delta_of(params), 0.0, v, info, c.st));
    return finish_call(c, phi, op->size);
}

static glinalg_status restart_entry(int which, glinalg_operator op, double *phi, const double *phi0,
                                    int size, int max_iter, double eps, int restart_freq,
                                    const glinalg_verbosity *verb,
                                    const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(ensure_device());
    if (restart_freq <= 0) {
        set_last_error("restart_freq must be positive");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if (precision_of(params) != GLINALG_PREC_DOUBLE) {
        set_last_error("restarted solvers run in FP64 only");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    SolveCall c;
    GL_TRY(prologue(op, phi, phi0, size, params, info, c));
    GL_TRY(restart_driver(which, op, c.sg.x, c.sg.b, max_iter, eps, restart_freq, Verb::from(verb), info, c.st));
    return finish_call(c, phi, op->size);
}

extern "C" glinalg_status glinalg_cg_restart(glinalg_operator op, double *phi, const double *phi0,
                                             int size, int max_iter, double eps, int restart_freq,
                                             const glinalg_verbosity *verb,
                                             const glinalg_solver_params *params, glinalg_info *info)
{
    return restart_entry(0, op, phi, phi0, size, max_iter, eps, restart_freq, verb, params, info);
}

extern "C" glinalg_status glinalg_bicgstab(glinalg_operator op, double *phi, const double *phi0,
                                           int size, int max_iter, double eps,
                                           const glinalg_verbosity *verb,
                                           const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(ensure_device());
    if (precision_of(params) != GLINALG_PREC_DOUBLE) {
        set_last_error("BiCGstab runs in FP64 only");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    SolveCall c;
    GL_TRY(prologue(op, phi, phi0, size, params, info, c));
    GL_TRY(bicgstab_fp64(op, c.sg.x, c.sg.b, max_iter, eps, Verb::from(verb), info, c.st));
    return finish_call(c, phi, op->size);
}

extern "C" glinalg_status glinalg_bicgstab_restart(glinalg_operator op, double *phi,
                                                   const double *phi0, int size, int max_iter,
                                                   double eps, int restart_freq,
                                                   const glinalg_verbosity *verb,
                                                   const glinalg_solver_params *params,
                                                   glinalg_info *info)
{
    return restart_entry(1, op, phi, phi0, size, max_iter, eps, restart_freq, verb, params, info);
}

extern "C" glinalg_status glinalg_gcr(glinalg_operator op, double *phi, const double *phi0, int size,
                                      int max_iter, double eps, const glinalg_verbosity *verb,
                                      const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(ensure_device());
    if (precision_of(params) != GLINALG_PREC_DOUBLE) {
        set_last_error("GCR runs in FP64 only");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    SolveCall c;
    GL_TRY(prologue(op, phi, phi0, size, params, info, c));
    GL_TRY(gcr_fp64(op, c.sg.x, c.sg.b, max_iter, eps, Verb::from(verb), info, c.st));
    return finish_call(c, phi, op->size);
}

extern "C" glinalg_status glinalg_gcr_restart(glinalg_operator op, double *phi, const double *phi0,
                                              int size, int max_iter, double eps, int restart_freq,
                                              const glinalg_verbosity *verb,
                                              const glinalg_solver_params *params,
                                              glinalg_info *info)
{
    return restart_entry(2, op, phi, phi0, size, max_iter, eps, restart_freq, verb, params, info);
}

extern "C" glinalg_status glinalg_cg_m(glinalg_operator op, double *const *phi, const double *phi0,
                                       int n_shift, int size, int resid_freq_check, int max_iter,
                                       double eps, const double *shifts, int worst_first,
                                       const glinalg_verbosity *verb,
                                       const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(ensure_device());
    if (!op || !phi || !phi0 || !shifts || !info || n_shift <= 0) return GLINALG_ERROR_INVALID_VALUE;
    if (resid_freq_check <= 0) {
        set_last_error("resid_freq_check must be positive");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if ((long)size != op->size) {
        set_last_error("size does not match the operator's field size");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    for (int j = 0; j < n_shift; j++)
        if (!phi[j]) return GLINALG_ERROR_INVALID_VALUE;
    if (precision_of(params) != GLINALG_PREC_DOUBLE) {
        set_last_error("CG-M runs its vectors in FP64 (the shift recurrences need it)");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    const bool dev = params && (params->flags & GLINALG_PTR_DEVICE);
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long n = op->size;
    std::vector<double2 *> X(n_shift);
    const double2 *b = (const double2 *)phi0;
    if (dev) {
        for (int j = 0; j < n_shift; j++) X[j] = (double2 *)phi[j];
    } else {
        for (int j = 0; j < n_shift; j++) GL_TRY(sc.alloc(&X[j], n));
        double2 *bb;
        GL_TRY(sc.alloc(&bb, n));
        GL_CUDA(cudaMemcpyAsync(bb, phi0, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        b = bb;
    }
    double *keep = info->resSqmrhs;
    *info = glinalg_info{};
    info->resSqmrhs = keep;
    GL_TRY(cg_m_fp64(op, X.data(), b, n_shift, resid_freq_check, max_iter, eps, shifts,
                     worst_first != 0, Verb::from(verb), info, st));
    if (!dev)
        for (int j = 0; j < n_shift; j++)
            GL_CUDA(cudaMemcpyAsync(phi[j], X[j], sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}
