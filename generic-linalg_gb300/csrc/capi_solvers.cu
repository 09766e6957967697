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
    if (!info) {
        set_last_error("null info");
        return GLINALG_ERROR_INVALID_VALUE;
    }
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
// The caller's reliable-update trigger, or 0: the mixed solvers then pick their per-precision
// default (0.01 for FP32 iterates, 0.1 for 16-bit ones).
double delta_of(const glinalg_solver_params *p) { return p && p->delta > 0 ? p->delta : 0.0; }
int wait_limit_of(const glinalg_solver_params *p) { return p ? p->wait_limit_us : 0; }

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
    else GL_TRY(cg_mixed(op, c.sg.x, c.sg.b, max_iter, eps, prec, delta_of(params), 0.0, v, info, c.st,
                         wait_limit_of(params)));
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
    if (!op || !phi || !phi0 || !shifts || !info || n_shift <= 0)
        return invalid_arg("!op || !phi || !phi0 || !shifts || !info || n_shift <= 0");
    if (resid_freq_check <= 0) {
        set_last_error("resid_freq_check must be positive");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if ((long)size != op->size) {
        set_last_error("size does not match the operator's field size");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    for (int j = 0; j < n_shift; j++)
        if (!phi[j]) return invalid_arg("!phi[j]");
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

// ---------------------------------------------------------------- sibling solvers

namespace {

glinalg_status fp64_only(const glinalg_solver_params *params, const char *what)
{
    if (precision_of(params) != GLINALG_PREC_DOUBLE) {
        set_last_error(std::string(what) + " runs in FP64 only");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return GLINALG_SUCCESS;
}

glinalg_status positive(int v, const char *what)
{
    if (v <= 0) {
        set_last_error(std::string(what) + " must be positive");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return GLINALG_SUCCESS;
}

// Runs one single-vector solve: argument checks, staging of phi / phi0, the solver, copy-back.
template <class F>
glinalg_status single_solve(glinalg_operator op, double *phi, const double *phi0, int size,
                            const glinalg_solver_params *params, glinalg_info *info, const char *what, F solve)
{
    GL_TRY(ensure_device());
    GL_TRY(fp64_only(params, what));
    SolveCall c;
    GL_TRY(prologue(op, phi, phi0, size, params, info, c));
    GL_TRY(solve(c));
    return finish_call(c, phi, op->size);
}

glinalg_status make_precond(const glinalg_precond *p, glinalg_operator op, Precond *out)
{
    *out = Precond{};
    if (!p) return GLINALG_SUCCESS;
    if (p->kind < GLINALG_PRECOND_IDENTITY || p->kind > GLINALG_PRECOND_MG) {
        set_last_error("unknown preconditioner kind");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if (p->kind == GLINALG_PRECOND_MG) {
        if (!p->mg) {
            set_last_error("the multigrid preconditioner needs a hierarchy (glinalg_mg_create)");
            return GLINALG_ERROR_INVALID_VALUE;
        }
        out->kind = GLINALG_PRECOND_MG;
        out->mg = p->mg;
        out->level = 0;
        return GLINALG_SUCCESS;
    }
    if (p->kind != GLINALG_PRECOND_IDENTITY && p->n_step < 0) {
        set_last_error("preconditioner n_step must not be negative");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if (p->op && p->op->size != op->size) {
        set_last_error("the preconditioner's operator has another field size");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    out->kind = p->kind;
    out->n_step = p->n_step;
    out->rel_res = p->rel_res;
    out->op = p->op;
    return GLINALG_SUCCESS;
}

// Multishift entry: staging of the n_shift solution vectors, then solver(X, b).
template <class F>
glinalg_status multishift_entry(glinalg_operator op, double *const *phi, const double *phi0, int n_shift,
                                int size, int resid_freq_check, const double *shifts,
                                const glinalg_solver_params *params, glinalg_info *info, const char *what,
                                F solve)
{
    GL_TRY(ensure_device());
    if (!op || !phi || !phi0 || !shifts || !info || n_shift <= 0)
        return invalid_arg("!op || !phi || !phi0 || !shifts || !info || n_shift <= 0");
    GL_TRY(positive(resid_freq_check, "resid_freq_check"));
    if ((long)size != op->size) {
        set_last_error("size does not match the operator's field size");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    for (int j = 0; j < n_shift; j++)
        if (!phi[j]) return invalid_arg("!phi[j]");
    GL_TRY(fp64_only(params, what));
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
    GL_TRY(solve(X.data(), b, st));
    if (!dev)
        for (int j = 0; j < n_shift; j++)
            GL_CUDA(cudaMemcpyAsync(phi[j], X[j], sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

}  // namespace

extern "C" glinalg_status glinalg_cr(glinalg_operator op, double *phi, const double *phi0, int size,
                                     int max_iter, double eps, const glinalg_verbosity *verb,
                                     const glinalg_solver_params *params, glinalg_info *info)
{
    return single_solve(op, phi, phi0, size, params, info, "CR", [&](SolveCall &c) {
        return cr_fp64(op, c.sg.x, c.sg.b, max_iter, eps, Verb::from(verb), info, c.st);
    });
}

extern "C" glinalg_status glinalg_cr_restart(glinalg_operator op, double *phi, const double *phi0, int size,
                                             int max_iter, double eps, int restart_freq,
                                             const glinalg_verbosity *verb,
                                             const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(positive(restart_freq, "restart_freq"));
    return single_solve(op, phi, phi0, size, params, info, "CR", [&](SolveCall &c) {
        return cr_restart_fp64(op, c.sg.x, c.sg.b, max_iter, eps, restart_freq, Verb::from(verb), info, c.st);
    });
}

extern "C" glinalg_status glinalg_minres(glinalg_operator op, double *phi, const double *phi0, int size,
                                         int max_iter, double eps, double omega,
                                         const glinalg_verbosity *verb, const glinalg_solver_params *params,
                                         glinalg_info *info)
{
    return single_solve(op, phi, phi0, size, params, info, "MinRes", [&](SolveCall &c) {
        return minres_fp64(op, c.sg.x, c.sg.b, max_iter, eps, omega, Verb::from(verb), info, c.st);
    });
}

extern "C" glinalg_status glinalg_bicgstab_l(glinalg_operator op, double *phi, const double *phi0, int size,
                                             int max_iter, double eps, int l, const glinalg_verbosity *verb,
                                             const glinalg_solver_params *params, glinalg_info *info)
{
    if (l < 1 || l > kMaxBicgstabL) {
        set_last_error("BiCGstab-l needs 1 <= l <= 16");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return single_solve(op, phi, phi0, size, params, info, "BiCGstab-l", [&](SolveCall &c) {
        return bicgstab_l_fp64(op, c.sg.x, c.sg.b, max_iter, eps, l, Verb::from(verb), info, c.st);
    });
}

extern "C" glinalg_status glinalg_bicgstab_l_restart(glinalg_operator op, double *phi, const double *phi0,
                                                     int size, int max_iter, double eps, int restart_freq, int l,
                                                     const glinalg_verbosity *verb,
                                                     const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(positive(restart_freq, "restart_freq"));
    if (l < 1 || l > kMaxBicgstabL) {
        set_last_error("BiCGstab-l needs 1 <= l <= 16");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return single_solve(op, phi, phi0, size, params, info, "BiCGstab-l", [&](SolveCall &c) {
        return bicgstab_l_restart_fp64(op, c.sg.x, c.sg.b, max_iter, eps, restart_freq, l, Verb::from(verb), info,
                                       c.st);
    });
}

extern "C" glinalg_status glinalg_cr_m(glinalg_operator op, double *const *phi, const double *phi0, int n_shift,
                                       int size, int resid_freq_check, int max_iter, double eps,
                                       const double *shifts, int worst_first, const glinalg_verbosity *verb,
                                       const glinalg_solver_params *params, glinalg_info *info)
{
    return multishift_entry(op, phi, phi0, n_shift, size, resid_freq_check, shifts, params, info, "CR-M",
                            [&](double2 *const *X, const double2 *b, cudaStream_t st) {
                                return cr_m_fp64(op, X, b, n_shift, resid_freq_check, max_iter, eps, shifts,
                                                 worst_first != 0, Verb::from(verb), info, st);
                            });
}

extern "C" glinalg_status glinalg_bicgstab_m(glinalg_operator op, double *const *phi, const double *phi0,
                                             int n_shift, int size, int resid_freq_check, int max_iter,
                                             double eps, const double *shifts, int worst_first,
                                             const glinalg_verbosity *verb, const glinalg_solver_params *params,
                                             glinalg_info *info)
{
    return multishift_entry(op, phi, phi0, n_shift, size, resid_freq_check, shifts, params, info, "BiCGstab-M",
                            [&](double2 *const *X, const double2 *b, cudaStream_t st) {
                                return bicgstab_m_fp64(op, X, b, n_shift, resid_freq_check, max_iter, eps, shifts,
                                                       worst_first != 0, Verb::from(verb), info, st);
                            });
}

static glinalg_status flex_entry(int mode, int restart_freq, glinalg_operator op, double *phi, const double *phi0,
                                 int size, int max_iter, double eps, const glinalg_precond *precond,
                                 const glinalg_verbosity *verb, const glinalg_solver_params *params,
                                 glinalg_info *info)
{
    if (!op) return invalid_arg("!op");
    Precond pc;
    GL_TRY(make_precond(precond, op, &pc));
    return single_solve(op, phi, phi0, size, params, info, mode == 0 ? "FPCG" : "VPGCR", [&](SolveCall &c) {
        const Verb v = Verb::from(verb);
        return restart_freq > 0
                   ? flex_restart_fp64(mode, op, c.sg.x, c.sg.b, max_iter, eps, restart_freq, pc, v, info, c.st)
                   : flex_fp64(mode, op, c.sg.x, c.sg.b, max_iter, eps, pc, v, info, c.st);
    });
}

extern "C" glinalg_status glinalg_cg_flex_precond(glinalg_operator op, double *phi, const double *phi0, int size,
                                                  int max_iter, double eps, const glinalg_precond *precond,
                                                  const glinalg_verbosity *verb,
                                                  const glinalg_solver_params *params, glinalg_info *info)
{
    return flex_entry(0, 0, op, phi, phi0, size, max_iter, eps, precond, verb, params, info);
}

extern "C" glinalg_status glinalg_cg_flex_precond_restart(glinalg_operator op, double *phi, const double *phi0,
                                                          int size, int max_iter, double eps, int restart_freq,
                                                          const glinalg_precond *precond,
                                                          const glinalg_verbosity *verb,
                                                          const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(positive(restart_freq, "restart_freq"));
    return flex_entry(0, restart_freq, op, phi, phi0, size, max_iter, eps, precond, verb, params, info);
}

extern "C" glinalg_status glinalg_gcr_var_precond(glinalg_operator op, double *phi, const double *phi0, int size,
                                                  int max_iter, double eps, const glinalg_precond *precond,
                                                  const glinalg_verbosity *verb,
                                                  const glinalg_solver_params *params, glinalg_info *info)
{
    return flex_entry(1, 0, op, phi, phi0, size, max_iter, eps, precond, verb, params, info);
}

extern "C" glinalg_status glinalg_gcr_var_precond_restart(glinalg_operator op, double *phi, const double *phi0,
                                                          int size, int max_iter, double eps, int restart_freq,
                                                          const glinalg_precond *precond,
                                                          const glinalg_verbosity *verb,
                                                          const glinalg_solver_params *params, glinalg_info *info)
{
    GL_TRY(positive(restart_freq, "restart_freq"));
    return flex_entry(1, restart_freq, op, phi, phi0, size, max_iter, eps, precond, verb, params, info);
}
