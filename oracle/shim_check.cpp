// shim_check.cpp -- test driver for generic-linalg_gb300/shim/glinalg_shim.cpp (test
// infrastructure, built by `make -C oracle shim` from the reference's unmodified sources).
//
// Links the reference's operators, stencils and solvers with the shim in place of the
// complex minv_vector_* overloads (the solver files that define them compiled under ref_*
// names), and calls through the reference's own interface.  One line per case on stdout, "case <name> <key>=<value> ...":
//   - every reference callback the library drives, through minv_vector_cg (complex);
//   - a callback the library does not drive, and a single-direction stencil apply;
//   - minv_vector_cg_m (complex), whose result must carry n_shift per-shift residuals;
//   - the other complex entry points (restarted CG, BiCGstab, GCR) and the sibling solvers
//     (CR, MinRes, BiCGstab-l, CR-M, BiCGstab-M, flexible CG, variably preconditioned GCR);
//   - preconditioner callbacks recognised by identity, and a foreign one refused;
//   - the real-valued overloads, which must run the reference's code.
// With a device the accelerated calls are compared with the reference's CG on the same input;
// without one they must fail with "glinalg: no CUDA device" (no CPU fallback).

#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <string>

#include "generic_bicgstab.h"
#include "generic_bicgstab_l.h"
#include "generic_bicgstab_m.h"
#include "generic_cg.h"
#include "generic_cg_flex_precond.h"
#include "generic_cg_m.h"
#include "generic_cr.h"
#include "generic_cr_m.h"
#include "generic_gcr.h"
#include "generic_gcr_var_precond.h"
#include "generic_minres.h"
#include "generic_precond.h"
#include "glinalg.h"
#include "mg_complex.h"
#include "operators.h"
#include "operators_stencil.h"
#include "u1_utils.h"

typedef void (*cmatvec)(complex<double> *, complex<double> *, void *);

// The reference's complex CG under its ref_* name (generic_cg.cpp:278).
inversion_info ref_minv_vector_cg(complex<double> *, complex<double> *, int, int, double, cmatvec, void *,
                                  inversion_verbose_struct *);

namespace {

const int L = 8, V = L * L;

void not_a_library_operator(complex<double> *lhs, complex<double> *rhs, void *)
{
    for (int i = 0; i < V; i++) lhs[i] = 2.0 * rhs[i];
}

void real_diagonal(double *lhs, double *rhs, void *)
{
    for (int i = 0; i < V; i++) lhs[i] = (1.0 + i % 7) * rhs[i];
}

void foreign_preconditioner(complex<double> *lhs, complex<double> *rhs, int size, void *, inversion_verbose_struct *)
{
    for (int i = 0; i < size; i++) lhs[i] = rhs[i];
}

// Largest error of x against the exact solution of the real diagonal system.
double max_err(const double *x, const complex<double> *b)
{
    double err = 0.0;
    for (int i = 0; i < V; i++) err = std::fmax(err, std::fabs(x[i] - b[i].real() / (1.0 + i % 7)));
    return err;
}

double rel_diff(const complex<double> *a, const complex<double> *b)
{
    double num = 0, den = 0;
    for (int i = 0; i < V; i++) {
        num += std::norm(a[i] - b[i]);
        den += std::norm(b[i]);
    }
    return std::sqrt(num / den);
}

void report(const char *name, const inversion_info &r, double diff = -1.0)
{
    std::printf("case %s success=%d iter=%d ops=%d diff=%.3e name=%s\n", name, r.success ? 1 : 0, r.iter,
                r.ops_count, diff, r.name.c_str());
}

}  // namespace

int main()
{
    const bool device = glinalg_device_count() > 0;
    std::printf("device %d\n", device ? 1 : 0);

    std::mt19937 gen(1337);
    complex<double> links[2 * V], b[V], x[V], xr[V];
    rand_gauge_u1(links, L, L, gen);
    std::normal_distribution<double> g(0.0, 1.0);
    for (int i = 0; i < V; i++) b[i] = complex<double>(g(gen), g(gen));

    staggered_u1_op stag = {links, 0.1, L, L, 1, 0.0};
    int dims[2] = {L, L};
    Lattice lat(2, dims, 1);
    stencil_2d sten(&lat, 1);
    get_square_staggered_u1_stencil(&sten, &stag);

    // Every callback the shim maps.  Hermitian ones are also solved by the reference's CG for
    // comparison when a device runs them.
    struct Cb {
        const char *name;
        cmatvec f;
        void *extra;
        bool hermitian;
    } cbs[] = {
        {"square_staggered_u1", square_staggered_u1, &stag, false},
        {"square_staggered_dagger_u1", square_staggered_dagger_u1, &stag, false},
        {"square_staggered_normal_u1", square_staggered_normal_u1, &stag, true},
        {"square_laplace_u1", square_laplace_u1, &stag, true},
        {"square_staggered_deo_u1", square_staggered_deo_u1, &stag, false},
        {"square_staggered_doe_u1", square_staggered_doe_u1, &stag, false},
        {"square_staggered_m2mdeodoe_u1", square_staggered_m2mdeodoe_u1, &stag, false},
        {"apply_stencil_2d", apply_stencil_2d, &sten, false},
        {"apply_stencil_2d_eo", apply_stencil_2d_eo, &sten, false},
        {"apply_stencil_2d_oe", apply_stencil_2d_oe, &sten, false},
        {"apply_square_staggered_m2mdeodoe_stencil", apply_square_staggered_m2mdeodoe_stencil, &sten, false},
        {"apply_stencil_2d_tb", apply_stencil_2d_tb, &sten, false},
        {"apply_stencil_2d_bt", apply_stencil_2d_bt, &sten, false},
        {"apply_square_staggered_m2mdtbdbt_stencil", apply_square_staggered_m2mdtbdbt_stencil, &sten, false},
        {"apply_square_staggered_normal_eo_stencil", apply_square_staggered_normal_eo_stencil, &sten, false},
        {"apply_square_staggered_normal_tb_stencil", apply_square_staggered_normal_tb_stencil, &sten, false},
        {"apply_square_staggered_dagger_eo_stencil", apply_square_staggered_dagger_eo_stencil, &sten, false},
        {"apply_square_staggered_dagger_tb_stencil", apply_square_staggered_dagger_tb_stencil, &sten, false},
    };
    for (const Cb &c : cbs) {
        for (int i = 0; i < V; i++) x[i] = 0.0;
        inversion_info r = minv_vector_cg(x, b, V, c.hermitian ? 1000 : 3, 1e-10, c.f, c.extra);
        double diff = -1.0;
        if (device && c.hermitian) {
            for (int i = 0; i < V; i++) xr[i] = 0.0;
            ref_minv_vector_cg(xr, b, V, 1000, 1e-10, c.f, c.extra, 0);
            diff = rel_diff(x, xr);
        }
        report(c.name, r, diff);
    }

    // A callback the library does not drive, and a single-direction stencil apply.
    report("unknown_callback", minv_vector_cg(x, b, V, 10, 1e-10, not_a_library_operator, &stag));
    stencil_2d one_dir(&lat, 1);
    get_square_staggered_u1_stencil(&one_dir, &stag);
    one_dir.sdir = DIR_XP1;
    report("single_direction_stencil", minv_vector_cg(x, b, V, 10, 1e-10, apply_stencil_2d, &one_dir));

    // Multishift CG: the result owns n_shift per-shift residuals, as the reference's does
    // (generic_cg_m.cpp:330), whether or not the solve ran.
    const int ns = 3;
    double shifts[ns] = {0.01, 0.1, 1.0};
    complex<double> xs[ns][V];
    complex<double> *phis[ns] = {xs[0], xs[1], xs[2]};
    inversion_info rm = minv_vector_cg_m(phis, b, ns, V, 1, 1000, 1e-10, shifts, square_staggered_normal_u1, &stag);
    report("cg_m", rm);
    std::printf("cg_m_resSqmrhs n_rhs=%d", rm.n_rhs);
    for (int n = 0; rm.resSqmrhs && n < ns; n++) std::printf(" %.6e", rm.resSqmrhs[n]);
    std::printf("\n");

    // The other complex entry points.
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("cg_restart", minv_vector_cg_restart(x, b, V, 1000, 1e-10, 16, square_staggered_normal_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("bicgstab", minv_vector_bicgstab(x, b, V, 1000, 1e-10, square_staggered_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("bicgstab_restart", minv_vector_bicgstab_restart(x, b, V, 1000, 1e-10, 16, square_staggered_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("gcr", minv_vector_gcr(x, b, V, 1000, 1e-10, square_staggered_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("gcr_restart", minv_vector_gcr_restart(x, b, V, 1000, 1e-10, 16, square_staggered_u1, &stag));

    // The sibling solvers.
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("cr", minv_vector_cr(x, b, V, 1000, 1e-10, square_staggered_normal_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("cr_restart", minv_vector_cr_restart(x, b, V, 1000, 1e-10, 16, square_staggered_normal_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("minres", minv_vector_minres(x, b, V, 1000, 1e-10, square_laplace_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("minres_omega", minv_vector_minres(x, b, V, 1000, 1e-10, 0.8, square_laplace_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("bicgstab_l", minv_vector_bicgstab_l(x, b, V, 1000, 1e-10, 2, square_staggered_u1, &stag));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("bicgstab_l_restart", minv_vector_bicgstab_l_restart(x, b, V, 1000, 1e-10, 16, 2, square_staggered_u1, &stag));
    inversion_info rcm = minv_vector_cr_m(phis, b, ns, V, 1, 1000, 1e-10, shifts, square_staggered_normal_u1, &stag);
    report("cr_m", rcm);
    std::printf("cr_m_resSqmrhs n_rhs=%d", rcm.n_rhs);
    for (int n = 0; rcm.resSqmrhs && n < ns; n++) std::printf(" %.6e", rcm.resSqmrhs[n]);
    std::printf("\n");
    report("bicgstab_m", minv_vector_bicgstab_m(phis, b, ns, V, 1, 1000, 1e-10, shifts, square_staggered_u1, &stag));

    // Preconditioned solvers: identity, MinRes and GCR preconditioners are recognised by
    // identity (their inner operator too); a foreign preconditioner is refused.
    minres_precond_struct_complex mr = {4, 0.1, square_staggered_normal_u1, &stag};
    gcr_precond_struct_complex gp = {4, 0.1, square_staggered_u1, &stag};
    minres_precond_struct_complex mr_foreign = {4, 0.1, not_a_library_operator, &stag};
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("cg_flex_identity", minv_vector_cg_flex_precond(x, b, V, 1000, 1e-10, square_staggered_normal_u1, &stag,
                                                           identity_preconditioner, 0));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("cg_flex_minres", minv_vector_cg_flex_precond(x, b, V, 1000, 1e-10, square_staggered_normal_u1, &stag,
                                                         minres_preconditioner, &mr));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("cg_flex_restart_minres",
           minv_vector_cg_flex_precond_restart(x, b, V, 1000, 1e-10, 12, square_staggered_normal_u1, &stag,
                                               minres_preconditioner, &mr));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("gcr_var_gcr", minv_vector_gcr_var_precond(x, b, V, 1000, 1e-10, square_staggered_u1, &stag,
                                                      gcr_preconditioner, &gp));
    for (int i = 0; i < V; i++) x[i] = 0.0;
    report("gcr_var_restart_gcr",
           minv_vector_gcr_var_precond_restart(x, b, V, 1000, 1e-10, 12, square_staggered_u1, &stag,
                                               gcr_preconditioner, &gp));
    report("precond_foreign_operator", minv_vector_gcr_var_precond(x, b, V, 10, 1e-10, square_staggered_u1, &stag,
                                                                   minres_preconditioner, &mr_foreign));
    report("precond_foreign_callback", minv_vector_gcr_var_precond(x, b, V, 10, 1e-10, square_staggered_u1, &stag,
                                                                   foreign_preconditioner, &mr));

    // Real-valued sibling overloads run the reference's code on the diagonal system.
    double rx2[V], rb2[V];
    for (int i = 0; i < V; i++) {
        rx2[i] = 0.0;
        rb2[i] = b[i].real();
    }
    inversion_info rcr = minv_vector_cr(rx2, rb2, V, 1000, 1e-12, real_diagonal, 0);
    report("real_cr", rcr, max_err(rx2, b));

    // The real-valued overload runs the reference's CG: the diagonal system is solved exactly.
    double rx[V], rb[V];
    for (int i = 0; i < V; i++) {
        rx[i] = 0.0;
        rb[i] = b[i].real();
    }
    inversion_info rr = minv_vector_cg(rx, rb, V, 1000, 1e-12, real_diagonal, 0);
    double err = 0.0;
    for (int i = 0; i < V; i++) err = std::fmax(err, std::fabs(rx[i] - rb[i] / (1.0 + i % 7)));
    report("real_cg", rr, err);
    return 0;
}
