// mg_precond.cu -- the reference's multigrid preconditioner (mg_preconditioner,
// multigrid/aa_mg/mg_complex.cpp:514-824) over a hierarchy of device operators and null-vector
// levels, for the flexible solvers (glinalg_cg_flex_precond, glinalg_gcr_var_precond).
//
// One application at level l, for rhs r (the reference's order of steps):
//   z1 = pre-smoother(r) with n_pre[l] iterations from zero (tolerance 1e-20, so it runs them
//        all), r1 = r - A_l z1; without pre-smoothing z1 = 0, r1 = r;
//   with a coarse solver: r_c = R r1; on the coarsest level solve A_{l+1} e_c = r_c to
//        rel_res[l] with it; above it recurse (MLEVEL_SMOOTH, or MINRES) or run a flexible
//        solve of the coarse level preconditioned by the level below (MLEVEL_RECURSIVE: CG ->
//        restarted FPCG, GCR and CR -> restarted VPGCR); lhs = z1 + P e_c;
//   without one (a plain V cycle): recurse below the coarsest level, else lhs = z1;
//   z3 = post-smoother(r - A_l lhs) with n_post[l] iterations, lhs += z3.
// The MinRes smoother uses omega = 1, as the reference fixes it (mg_complex.cpp:560).  The
// reference's progress lines ("[L1 Presmooth]: ...") and its Dslash counters are not
// reproduced; the normal-equation variants (normal_eqn_mg, normal_eqn_smooth) and the
// BiCGstab / GMRES / SOR variants that have no device solver here are rejected at creation.

#include <vector>

#include "solvers.h"

struct glinalg_mg_level_s;

struct glinalg_mg_s {
    int n_refine = 0;
    std::vector<const glinalg_operator_s *> ops;     // n_refine + 1: A_0 (fine) .. A_n (coarsest)
    std::vector<const glinalg_mg_level_s *> levels;  // n_refine transfers
    glinalg_mg_params p{};
};

namespace glinalg {

glinalg_status mg_prolong(const glinalg_mg_level_s *l, double2 *fine, const double2 *coarse, cudaStream_t st);
glinalg_status mg_restrict(const glinalg_mg_level_s *l, double2 *coarse, const double2 *fine, cudaStream_t st);

namespace {

__global__ void k_axpby(double2 *__restrict__ out, const double2 *__restrict__ a, const double2 *__restrict__ b,
                        double sb, long n)
{
    // out = a + sb * b (sb = +1 or -1)
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double2 y = b[i];
        out[i] = sb > 0 ? cadd(a[i], y) : csub(a[i], y);
    }
}

int grid(long n)
{
    const long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

glinalg_status axpby(double2 *out, const double2 *a, const double2 *b, double sb, long n, cudaStream_t st)
{
    k_axpby<<<grid(n), 256, 0, st>>>(out, a, b, sb, n);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

// minv_unpreconditioned (generic_inverter.cpp:102-190) with tolerance 1e-20 and n iterations,
// from the zero guess in x
glinalg_status smooth(int type, const glinalg_operator_s *op, double2 *x, const double2 *b, int n, cudaStream_t st)
{
    const Verb none;
    glinalg_info in = {};
    const double tol = 1e-20;
    switch (type) {
    case GLINALG_MINV_CG: return cg_fp64(op, x, b, n, tol, none, &in, st);
    case GLINALG_MINV_CR: return cr_fp64(op, x, b, n, tol, none, &in, st);
    case GLINALG_MINV_GCR: return gcr_fp64(op, x, b, n, tol, none, &in, st);
    case GLINALG_MINV_BICGSTAB: return bicgstab_fp64(op, x, b, n, tol, none, &in, st);
    case GLINALG_MINV_BICGSTAB_L: return bicgstab_l_fp64(op, x, b, n, tol, n, none, &in, st);
    case GLINALG_MINV_MINRES: return minres_fp64(op, x, b, n, tol, 1.0, none, &in, st);
    default: set_last_error("unsupported multigrid smoother"); return GLINALG_ERROR_INVALID_VALUE;
    }
}

}  // namespace

glinalg_status mg_apply(const glinalg_mg_s *mg, int level, double2 *lhs, const double2 *rhs, const Verb &verb,
                        cudaStream_t st)
{
    const glinalg_mg_params &p = mg->p;
    const glinalg_operator_s *A = mg->ops[level];
    const long n = A->size;
    Scratch sc(st);
    double2 *z1, *r1, *tmp = nullptr;
    GL_TRY(sc.zeros(&z1, n));
    GL_TRY(sc.alloc(&r1, n));
    if (needs_tmp(A->kind)) GL_TRY(sc.alloc(&tmp, n));
    const bool smoothing = p.smoother != GLINALG_MINV_INVALID;
    if (p.n_pre_smooth[level] > 0 && smoothing) {
        GL_TRY(smooth(p.smoother, A, z1, rhs, p.n_pre_smooth[level], st));
        GL_TRY(launch_apply(A, r1, z1, tmp, nullptr, st));
        GL_TRY(axpby(r1, rhs, r1, -1.0, n, st));
    } else {
        GL_CUDA(cudaMemcpyAsync(r1, rhs, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    }
    const bool coarsest = level + 1 == mg->n_refine;
    const glinalg_mg_level_s *T = mg->levels[level];
    const long nc = mg->ops[level + 1]->size;
    if (p.coarse_solver != GLINALG_MG_NONE || !coarsest) {
        double2 *rc, *lc, *z2;
        GL_TRY(sc.alloc(&rc, nc));
        GL_TRY(sc.zeros(&lc, nc));
        GL_TRY(sc.alloc(&z2, n));
        GL_TRY(mg_restrict(T, rc, r1, st));
        const glinalg_operator_s *Ac = mg->ops[level + 1];
        glinalg_info in = {};
        const double rr = p.rel_res[level];
        if (p.coarse_solver != GLINALG_MG_NONE && coarsest) {
            switch (p.coarse_solver) {
            case GLINALG_MG_MINRES: GL_TRY(minres_fp64(Ac, lc, rc, p.n_max, rr, 1.0, verb, &in, st)); break;
            case GLINALG_MG_CG: GL_TRY(cg_fp64(Ac, lc, rc, p.n_max, rr, verb, &in, st)); break;
            case GLINALG_MG_GCR: GL_TRY(restart_driver(2, Ac, lc, rc, p.n_max, rr, p.n_restart, verb, &in, st)); break;
            case GLINALG_MG_BICGSTAB: GL_TRY(bicgstab_fp64(Ac, lc, rc, p.n_max, rr, verb, &in, st)); break;
            case GLINALG_MG_CR: GL_TRY(cr_restart_fp64(Ac, lc, rc, p.n_max, rr, p.n_restart, verb, &in, st)); break;
            case GLINALG_MG_BICGSTAB_L: GL_TRY(bicgstab_fp64(Ac, lc, rc, p.n_max, rr, verb, &in, st)); break;
            default: set_last_error("unsupported coarse solver"); return GLINALG_ERROR_INVALID_VALUE;
            }
        } else if (p.coarse_solver == GLINALG_MG_NONE || p.mlevel_type == GLINALG_MLEVEL_SMOOTH ||
                   p.coarse_solver == GLINALG_MG_MINRES) {
            GL_TRY(mg_apply(mg, level + 1, lc, rc, verb, st));
        } else {
            Precond below;
            below.kind = GLINALG_PRECOND_MG;
            below.mg = mg;
            below.level = level + 1;
            const int mode = p.coarse_solver == GLINALG_MG_CG ? 0 : 1;
            GL_TRY(flex_restart_fp64(mode, Ac, lc, rc, p.n_max, rr, p.n_restart, below, verb, &in, st));
        }
        GL_TRY(mg_prolong(T, z2, lc, st));
        GL_TRY(axpby(lhs, z1, z2, +1.0, n, st));
    } else {
        GL_CUDA(cudaMemcpyAsync(lhs, z1, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    }
    if (p.n_post_smooth[level] > 0 && smoothing) {
        double2 *r2, *z3;
        GL_TRY(sc.alloc(&r2, n));
        GL_TRY(sc.zeros(&z3, n));
        GL_TRY(launch_apply(A, r2, lhs, tmp, nullptr, st));
        GL_TRY(axpby(r2, rhs, r2, -1.0, n, st));
        GL_TRY(smooth(p.smoother, A, z3, r2, p.n_post_smooth[level], st));
        GL_TRY(axpby(lhs, lhs, z3, +1.0, n, st));
    }
    return GLINALG_SUCCESS;
}

}  // namespace glinalg

using namespace glinalg;

extern "C" glinalg_status glinalg_mg_create(int n_refine, const glinalg_operator *ops, const glinalg_mg_level *levels,
                                            const glinalg_mg_params *params, glinalg_mg *out)
{
    if (!out || !ops || !levels || !params)
        return invalid_arg("!out || !ops || !levels || !params");
    *out = nullptr;
    if (n_refine < 1 || n_refine > GLINALG_MG_MAX_LEVELS) {
        set_last_error("n_refine must be between 1 and GLINALG_MG_MAX_LEVELS");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    for (int l = 0; l <= n_refine; l++)
        if (!ops[l]) return invalid_arg("!ops[l]");
    for (int l = 0; l < n_refine; l++) {
        if (!levels[l]) return invalid_arg("!levels[l]");
        if (mg_level_fine_size(levels[l]) != ops[l]->size || mg_level_coarse_size(levels[l]) != ops[l + 1]->size) {
            set_last_error("the transfer levels do not match the operators' field sizes");
            return GLINALG_ERROR_INVALID_VALUE;
        }
    }
    const glinalg_mg_params &p = *params;
    if (p.normal_eqn_mg || p.normal_eqn_smooth) {
        set_last_error("normal-equation multigrid is not supported");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    const bool smoother_ok = p.smoother == GLINALG_MINV_INVALID || p.smoother == GLINALG_MINV_CG ||
                             p.smoother == GLINALG_MINV_CR || p.smoother == GLINALG_MINV_GCR ||
                             p.smoother == GLINALG_MINV_BICGSTAB || p.smoother == GLINALG_MINV_BICGSTAB_L ||
                             p.smoother == GLINALG_MINV_MINRES;
    if (!smoother_ok) {
        set_last_error("unsupported multigrid smoother (GMRES and SOR have no device solver here)");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if (p.coarse_solver < GLINALG_MG_NONE || p.coarse_solver > GLINALG_MG_BICGSTAB_L ||
        (n_refine > 1 && p.mlevel_type == GLINALG_MLEVEL_RECURSIVE &&
         (p.coarse_solver == GLINALG_MG_BICGSTAB || p.coarse_solver == GLINALG_MG_BICGSTAB_L))) {
        set_last_error("unsupported coarse solver for this hierarchy");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if ((p.coarse_solver == GLINALG_MG_GCR || p.coarse_solver == GLINALG_MG_CR ||
         (p.mlevel_type == GLINALG_MLEVEL_RECURSIVE && p.coarse_solver == GLINALG_MG_CG)) && p.n_restart <= 0) {
        set_last_error("n_restart must be positive for this coarse solver");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    auto *mg = new glinalg_mg_s();
    mg->n_refine = n_refine;
    mg->ops.assign(ops, ops + n_refine + 1);
    mg->levels.assign(levels, levels + n_refine);
    mg->p = p;
    *out = mg;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_destroy(glinalg_mg mg)
{
    delete mg;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_apply(glinalg_mg mg, double *lhs, const double *rhs, int flags)
{
    if (!mg || !lhs || !rhs) return invalid_arg("!mg || !lhs || !rhs");
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long n = mg->ops[0]->size;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    double2 *dl = (double2 *)lhs, *dr = (double2 *)rhs;
    if (!dev) {
        GL_TRY(sc.alloc(&dl, n));
        GL_TRY(sc.alloc(&dr, n));
        GL_CUDA(cudaMemcpyAsync(dr, rhs, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
    }
    GL_TRY(mg_apply(mg, 0, dl, dr, Verb(), st));
    if (!dev) GL_CUDA(cudaMemcpyAsync(lhs, dl, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}
