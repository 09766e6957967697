// glinalg_shim.cpp -- routes the reference's complex minv_vector_* solvers to libglinalg_gb300.
//
// A reference program links this file in place of the solver files it replaces, which it
// compiles under ref_* names instead (-Dminv_vector_cg=ref_minv_vector_cg and so on) so that
// the real-valued overloads keep the reference's own code:
//   generic_cg.cpp, generic_cg_m.cpp, generic_bicgstab.cpp, generic_gcr.cpp (the hot path) and
//   generic_cr.cpp, generic_minres.cpp, generic_bicgstab_l.cpp, generic_cr_m.cpp,
//   generic_bicgstab_m.cpp, generic_cg_flex_precond.cpp, generic_gcr_var_precond.cpp.
// The overloads below have the reference's signatures (generic_cg.h:19,23; generic_cg_m.h:17;
// generic_bicgstab.h:20-21; generic_gcr.h:18,22; generic_cr.h:18,22; generic_minres.h:20-21;
// generic_bicgstab_l.h:20-21; generic_cr_m.h:28; generic_bicgstab_m.h:17;
// generic_cg_flex_precond.h:18,23; generic_gcr_var_precond.h:18,23).
//
// The operator is recognised by the callback's function-pointer identity; its extra_info
// (staggered_u1_op, operators.h:7-15, or stencil_2d, coarse_stencil.h:33-155) becomes a
// glinalg_op_desc.  Any other callback, and any device error, gives success = false and a name
// starting with "glinalg: " that says why (inverter_struct.h:14-89 has no error field).
// Nothing falls back to the CPU.
//
// Compile with -I<this library>/include plus the reference's include paths, and link with
// -lglinalg_gb300.

#include <complex>
#include <limits>
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

typedef void (*cmatvec)(complex<double> *, complex<double> *, void *);
typedef void (*rmatvec)(double *, double *, void *);
typedef void (*cprecond)(complex<double> *, complex<double> *, int, void *, inversion_verbose_struct *);
typedef void (*rprecond)(double *, double *, int, void *, inversion_verbose_struct *);

// The reference's solvers compiled from its unmodified sources under ref_* names; the
// real-valued overloads use them.
inversion_info ref_minv_vector_cg(double *, double *, int, int, double, rmatvec, void *, inversion_verbose_struct *);
inversion_info ref_minv_vector_cg_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                          inversion_verbose_struct *);
inversion_info ref_minv_vector_cg_m(double **, double *, int, int, int, int, double, double *, rmatvec, void *, bool,
                                    inversion_verbose_struct *);
inversion_info ref_minv_vector_bicgstab(double *, double *, int, int, double, rmatvec, void *,
                                        inversion_verbose_struct *);
inversion_info ref_minv_vector_bicgstab_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                                inversion_verbose_struct *);
inversion_info ref_minv_vector_gcr(double *, double *, int, int, double, rmatvec, void *, inversion_verbose_struct *);
inversion_info ref_minv_vector_gcr_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                           inversion_verbose_struct *);
inversion_info ref_minv_vector_cr(double *, double *, int, int, double, rmatvec, void *, inversion_verbose_struct *);
inversion_info ref_minv_vector_cr_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                          inversion_verbose_struct *);
inversion_info ref_minv_vector_minres(double *, double *, int, int, double, rmatvec, void *,
                                      inversion_verbose_struct *);
inversion_info ref_minv_vector_minres(double *, double *, int, int, double, double, rmatvec, void *,
                                      inversion_verbose_struct *);
inversion_info ref_minv_vector_bicgstab_l(double *, double *, int, int, double, int, rmatvec, void *,
                                          inversion_verbose_struct *);
inversion_info ref_minv_vector_bicgstab_l_restart(double *, double *, int, int, double, int, int, rmatvec, void *,
                                                  inversion_verbose_struct *);
inversion_info ref_minv_vector_cr_m(double **, double *, int, int, int, int, double, double *, rmatvec, void *, bool,
                                    inversion_verbose_struct *);
inversion_info ref_minv_vector_bicgstab_m(double **, double *, int, int, int, int, double, double *, rmatvec, void *,
                                          bool, inversion_verbose_struct *);
inversion_info ref_minv_vector_cg_flex_precond(double *, double *, int, int, double, rmatvec, void *, rprecond,
                                               void *, inversion_verbose_struct *);
inversion_info ref_minv_vector_cg_flex_precond_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                                       rprecond, void *, inversion_verbose_struct *);
inversion_info ref_minv_vector_gcr_var_precond(double *, double *, int, int, double, rmatvec, void *, rprecond,
                                               void *, inversion_verbose_struct *);
inversion_info ref_minv_vector_gcr_var_precond_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                                       rprecond, void *, inversion_verbose_struct *);

namespace {

// Operator kind of a reference callback, or -1 for a callback the library does not drive.
int kind_of(cmatvec f)
{
    if (f == square_staggered_u1) return GLINALG_OP_STAGGERED;
    if (f == square_staggered_dagger_u1) return GLINALG_OP_STAGGERED_DAGGER;
    if (f == square_staggered_normal_u1) return GLINALG_OP_STAGGERED_NORMAL;
    if (f == square_laplace_u1) return GLINALG_OP_LAPLACE;
    if (f == square_staggered_deo_u1) return GLINALG_OP_STAGGERED_DEO;
    if (f == square_staggered_doe_u1) return GLINALG_OP_STAGGERED_DOE;
    if (f == square_staggered_m2mdeodoe_u1) return GLINALG_OP_STAGGERED_M2MDEODOE;
    if (f == apply_stencil_2d) return GLINALG_OP_STENCIL;
    if (f == apply_stencil_2d_eo) return GLINALG_OP_STENCIL_EO;
    if (f == apply_stencil_2d_oe) return GLINALG_OP_STENCIL_OE;
    if (f == apply_square_staggered_m2mdeodoe_stencil) return GLINALG_OP_STENCIL_M2MDEODOE;
    if (f == apply_stencil_2d_tb) return GLINALG_OP_STENCIL_TB;
    if (f == apply_stencil_2d_bt) return GLINALG_OP_STENCIL_BT;
    if (f == apply_square_staggered_m2mdtbdbt_stencil) return GLINALG_OP_STENCIL_M2MDTBDBT;
    if (f == apply_square_staggered_normal_eo_stencil) return GLINALG_OP_STENCIL_NORMAL_EO;
    if (f == apply_square_staggered_normal_tb_stencil) return GLINALG_OP_STENCIL_NORMAL_TB;
    if (f == apply_square_staggered_dagger_eo_stencil) return GLINALG_OP_STENCIL_DAGGER_EO;
    if (f == apply_square_staggered_dagger_tb_stencil) return GLINALG_OP_STENCIL_DAGGER_TB;
    return -1;
}

bool is_function_kind(int kind)
{
    return kind <= GLINALG_OP_LAPLACE || (kind >= GLINALG_OP_STAGGERED_DEO && kind <= GLINALG_OP_STAGGERED_M2MDEODOE);
}

// The library operator behind (f, extra).  GLINALG_ERROR_UNSUPPORTED_OP for a callback the
// library does not drive (or a single-direction stencil apply), else glinalg_operator_create's
// status.
glinalg_status make_operator(cmatvec f, void *extra, glinalg_operator *op)
{
    *op = 0;
    const int kind = kind_of(f);
    if (kind < 0 || !extra) return GLINALG_ERROR_UNSUPPORTED_OP;
    glinalg_op_desc d = {};
    d.kind = kind;
    if (is_function_kind(kind)) {
        const staggered_u1_op *s = (const staggered_u1_op *)extra;
        d.lx = s->x_fine;
        d.ly = s->y_fine;
        d.nc = 1;
        d.mass = s->mass;
        d.links = (const double *)s->lattice;
    } else {
        stencil_2d *s = (stencil_2d *)extra;
        if (s->sdir != DIR_ALL) return GLINALG_ERROR_UNSUPPORTED_OP;
        d.lx = s->lat->get_lattice_dimension(0);
        d.ly = s->lat->get_lattice_dimension(1);
        d.nc = s->lat->get_nc();
        d.clover = (const double *)s->clover;
        d.hopping = (const double *)s->hopping;
        d.two_link = s->has_two ? (const double *)s->two_link : 0;
        d.shift[0] = s->shift.real();
        d.shift[1] = s->shift.imag();
        d.eo_shift[0] = s->eo_shift.real();
        d.eo_shift[1] = s->eo_shift.imag();
        d.dof_shift[0] = s->dof_shift.real();
        d.dof_shift[1] = s->dof_shift.imag();
    }
    return glinalg_operator_create(&d, op);
}

struct Verb {
    glinalg_verbosity v = {};
    glinalg_verbosity *ptr = 0;
    explicit Verb(const inversion_verbose_struct *r)
    {
        if (!r) return;
        v.verbosity = r->verbosity;
        v.verb_prefix = r->verb_prefix.c_str();
        v.precond_verbosity = r->precond_verbosity;
        v.precond_verb_prefix = r->precond_verb_prefix.c_str();
        ptr = &v;
    }
};

// Runs call(op, info) on the operator behind (f, extra) and fills r.  On any error r keeps
// success = false, its name says why, and every per-shift residual reads +infinity, so a
// caller's convergence check on resSqmrhs reports the failure.
template <class Call>
void run(cmatvec f, void *extra, inversion_info &r, Call call)
{
    glinalg_operator op;
    glinalg_info info = {};
    info.resSqmrhs = r.resSqmrhs;
    info.n_rhs = r.n_rhs > 0 ? r.n_rhs : 0;
    glinalg_status st = make_operator(f, extra, &op);
    if (st == GLINALG_SUCCESS) st = call(op, &info);
    if (op) glinalg_operator_destroy(op);
    if (st != GLINALG_SUCCESS) {
        r.name = std::string("glinalg: ") + glinalg_status_string(st);
        for (int i = 0; r.resSqmrhs && i < r.n_rhs; i++) r.resSqmrhs[i] = std::numeric_limits<double>::infinity();
        return;
    }
    r.resSq = info.resSq;
    r.iter = info.iter;
    r.success = info.success != 0;
    r.name = info.name;
    r.ops_count = info.ops_count;
}

// The library preconditioner behind a reference preconditioner callback (generic_precond.h),
// recognised by identity like the operators: identity_preconditioner, and
// minres_preconditioner / gcr_preconditioner with their {minres,gcr}_precond_struct_complex,
// whose inner operator must itself be one the library drives.  Any other callback
// (mg_preconditioner included: its hierarchy is built with glinalg_mg_create) is
// GLINALG_ERROR_UNSUPPORTED_OP.  *inner receives the operator the caller must destroy.
glinalg_status make_precond(cprecond pf, void *pinfo, glinalg_precond *p, glinalg_operator *inner)
{
    *p = glinalg_precond{};
    *inner = 0;
    if (pf == (cprecond)identity_preconditioner) {
        p->kind = GLINALG_PRECOND_IDENTITY;
        return GLINALG_SUCCESS;
    }
    if ((pf != (cprecond)minres_preconditioner && pf != (cprecond)gcr_preconditioner) || !pinfo)
        return GLINALG_ERROR_UNSUPPORTED_OP;
    // minres_precond_struct_complex and gcr_precond_struct_complex have the same fields
    const minres_precond_struct_complex *m = (const minres_precond_struct_complex *)pinfo;
    p->kind = pf == (cprecond)minres_preconditioner ? GLINALG_PRECOND_MINRES : GLINALG_PRECOND_GCR;
    p->n_step = m->n_step;
    p->rel_res = m->rel_res;
    const glinalg_status st = make_operator(m->matrix_vector, m->matrix_extra_data, inner);
    p->op = *inner;
    return st;
}

// run() for the flexibly / variably preconditioned solvers: the preconditioner is mapped
// first, and its inner operator lives for the call.
template <class Call>
void run_precond(cmatvec f, void *extra, cprecond pf, void *pinfo, inversion_info &r, Call call)
{
    glinalg_precond pc;
    glinalg_operator inner;
    const glinalg_status pst = make_precond(pf, pinfo, &pc, &inner);
    if (pst != GLINALG_SUCCESS) {
        if (inner) glinalg_operator_destroy(inner);
        r.name = std::string("glinalg: ") + glinalg_status_string(pst) + " (preconditioner)";
        return;
    }
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) { return call(op, &pc, info); });
    if (inner) glinalg_operator_destroy(inner);
}

}  // namespace

inversion_info minv_vector_cg(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                              cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_cg(op, (double *)phi, (const double *)phi0, size, max_iter, eps, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_cg_restart(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                      double eps, int restart_freq, cmatvec f, void *extra,
                                      inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_cg_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps, restart_freq,
                                  v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_bicgstab(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                    double eps, cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_bicgstab(op, (double *)phi, (const double *)phi0, size, max_iter, eps, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_bicgstab_restart(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                            double eps, int restart_freq, cmatvec f, void *extra,
                                            inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_bicgstab_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps,
                                        restart_freq, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_gcr(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                               cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_gcr(op, (double *)phi, (const double *)phi0, size, max_iter, eps, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_gcr_restart(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                       double eps, int restart_freq, cmatvec f, void *extra,
                                       inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_gcr_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps, restart_freq,
                                   v.ptr, 0, info);
    });
    return r;
}

// Like the reference (generic_cg_m.cpp:330), the result carries n_shift per-shift squared
// residuals |(A + shift_n) x_n - b|^2 in resSqmrhs, owned by the returned struct.
inversion_info minv_vector_cg_m(complex<double> **phi, complex<double> *phi0, int n_shift, int size,
                                int resid_freq_check, int max_iter, double eps, double *shifts, cmatvec f,
                                void *extra, bool worst_first, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r(n_shift);
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_cg_m(op, (double *const *)phi, (const double *)phi0, n_shift, size, resid_freq_check,
                            max_iter, eps, shifts, worst_first ? 1 : 0, v.ptr, 0, info);
    });
    return r;
}

// ---- sibling Krylov solvers

inversion_info minv_vector_cr(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                              cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_cr(op, (double *)phi, (const double *)phi0, size, max_iter, eps, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_cr_restart(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                      double eps, int restart_freq, cmatvec f, void *extra,
                                      inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_cr_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps, restart_freq,
                                  v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_minres(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                                  double omega, cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_minres(op, (double *)phi, (const double *)phi0, size, max_iter, eps, omega, v.ptr, 0, info);
    });
    return r;
}

// The short form is omega = 1 (generic_minres.cpp:234-237).
inversion_info minv_vector_minres(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                                  cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return minv_vector_minres(phi, phi0, size, max_iter, eps, 1.0, f, extra, verb);
}

inversion_info minv_vector_bicgstab_l(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                      double eps, int l, cmatvec f, void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_bicgstab_l(op, (double *)phi, (const double *)phi0, size, max_iter, eps, l, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_bicgstab_l_restart(complex<double> *phi, complex<double> *phi0, int size,
                                              int max_iter, double eps, int restart_freq, int l, cmatvec f,
                                              void *extra, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_bicgstab_l_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps,
                                          restart_freq, l, v.ptr, 0, info);
    });
    return r;
}

// As minv_vector_cg_m: the result owns n_shift per-shift residuals (generic_cr_m.cpp:342).
inversion_info minv_vector_cr_m(complex<double> **phi, complex<double> *phi0, int n_shift, int size,
                                int resid_freq_check, int max_iter, double eps, double *shifts, cmatvec f,
                                void *extra, bool worst_first, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r(n_shift);
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_cr_m(op, (double *const *)phi, (const double *)phi0, n_shift, size, resid_freq_check,
                            max_iter, eps, shifts, worst_first ? 1 : 0, v.ptr, 0, info);
    });
    return r;
}

// As minv_vector_cg_m (generic_bicgstab_m.cpp:424).
inversion_info minv_vector_bicgstab_m(complex<double> **phi, complex<double> *phi0, int n_shift, int size,
                                      int resid_freq_check, int max_iter, double eps, double *shifts, cmatvec f,
                                      void *extra, bool worst_first, inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r(n_shift);
    run(f, extra, r, [&](glinalg_operator op, glinalg_info *info) {
        return glinalg_bicgstab_m(op, (double *const *)phi, (const double *)phi0, n_shift, size, resid_freq_check,
                                  max_iter, eps, shifts, worst_first ? 1 : 0, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_cg_flex_precond(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                           double eps, cmatvec f, void *extra, cprecond pf, void *pinfo,
                                           inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run_precond(f, extra, pf, pinfo, r, [&](glinalg_operator op, const glinalg_precond *pc, glinalg_info *info) {
        return glinalg_cg_flex_precond(op, (double *)phi, (const double *)phi0, size, max_iter, eps, pc, v.ptr, 0,
                                       info);
    });
    return r;
}

inversion_info minv_vector_cg_flex_precond_restart(complex<double> *phi, complex<double> *phi0, int size,
                                                   int max_iter, double eps, int restart_freq, cmatvec f,
                                                   void *extra, cprecond pf, void *pinfo,
                                                   inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run_precond(f, extra, pf, pinfo, r, [&](glinalg_operator op, const glinalg_precond *pc, glinalg_info *info) {
        return glinalg_cg_flex_precond_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps,
                                               restart_freq, pc, v.ptr, 0, info);
    });
    return r;
}

inversion_info minv_vector_gcr_var_precond(complex<double> *phi, complex<double> *phi0, int size, int max_iter,
                                           double eps, cmatvec f, void *extra, cprecond pf, void *pinfo,
                                           inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run_precond(f, extra, pf, pinfo, r, [&](glinalg_operator op, const glinalg_precond *pc, glinalg_info *info) {
        return glinalg_gcr_var_precond(op, (double *)phi, (const double *)phi0, size, max_iter, eps, pc, v.ptr, 0,
                                       info);
    });
    return r;
}

inversion_info minv_vector_gcr_var_precond_restart(complex<double> *phi, complex<double> *phi0, int size,
                                                   int max_iter, double eps, int restart_freq, cmatvec f,
                                                   void *extra, cprecond pf, void *pinfo,
                                                   inversion_verbose_struct *verb)
{
    Verb v(verb);
    inversion_info r;
    run_precond(f, extra, pf, pinfo, r, [&](glinalg_operator op, const glinalg_precond *pc, glinalg_info *info) {
        return glinalg_gcr_var_precond_restart(op, (double *)phi, (const double *)phi0, size, max_iter, eps,
                                               restart_freq, pc, v.ptr, 0, info);
    });
    return r;
}

// Real-valued overloads: no real operator is on the accelerated path; the reference's code runs.
inversion_info minv_vector_cg(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f, void *extra,
                              inversion_verbose_struct *verb)
{
    return ref_minv_vector_cg(phi, phi0, size, max_iter, eps, f, extra, verb);
}

inversion_info minv_vector_cg_restart(double *phi, double *phi0, int size, int max_iter, double eps, int rf,
                                      rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_cg_restart(phi, phi0, size, max_iter, eps, rf, f, extra, verb);
}

inversion_info minv_vector_cg_m(double **phi, double *phi0, int n_shift, int size, int rfc, int max_iter, double eps,
                                double *shifts, rmatvec f, void *extra, bool wf, inversion_verbose_struct *verb)
{
    return ref_minv_vector_cg_m(phi, phi0, n_shift, size, rfc, max_iter, eps, shifts, f, extra, wf, verb);
}

inversion_info minv_vector_bicgstab(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f,
                                    void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_bicgstab(phi, phi0, size, max_iter, eps, f, extra, verb);
}

inversion_info minv_vector_bicgstab_restart(double *phi, double *phi0, int size, int max_iter, double eps, int rf,
                                            rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_bicgstab_restart(phi, phi0, size, max_iter, eps, rf, f, extra, verb);
}

inversion_info minv_vector_gcr(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f, void *extra,
                               inversion_verbose_struct *verb)
{
    return ref_minv_vector_gcr(phi, phi0, size, max_iter, eps, f, extra, verb);
}

inversion_info minv_vector_gcr_restart(double *phi, double *phi0, int size, int max_iter, double eps, int rf,
                                       rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_gcr_restart(phi, phi0, size, max_iter, eps, rf, f, extra, verb);
}

inversion_info minv_vector_cr(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f, void *extra,
                              inversion_verbose_struct *verb)
{
    return ref_minv_vector_cr(phi, phi0, size, max_iter, eps, f, extra, verb);
}

inversion_info minv_vector_cr_restart(double *phi, double *phi0, int size, int max_iter, double eps, int rf,
                                      rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_cr_restart(phi, phi0, size, max_iter, eps, rf, f, extra, verb);
}

inversion_info minv_vector_minres(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f,
                                  void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_minres(phi, phi0, size, max_iter, eps, f, extra, verb);
}

inversion_info minv_vector_minres(double *phi, double *phi0, int size, int max_iter, double eps, double omega,
                                  rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_minres(phi, phi0, size, max_iter, eps, omega, f, extra, verb);
}

inversion_info minv_vector_bicgstab_l(double *phi, double *phi0, int size, int max_iter, double eps, int l,
                                      rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_bicgstab_l(phi, phi0, size, max_iter, eps, l, f, extra, verb);
}

inversion_info minv_vector_bicgstab_l_restart(double *phi, double *phi0, int size, int max_iter, double eps, int rf,
                                              int l, rmatvec f, void *extra, inversion_verbose_struct *verb)
{
    return ref_minv_vector_bicgstab_l_restart(phi, phi0, size, max_iter, eps, rf, l, f, extra, verb);
}

inversion_info minv_vector_cr_m(double **phi, double *phi0, int n_shift, int size, int rfc, int max_iter, double eps,
                                double *shifts, rmatvec f, void *extra, bool wf, inversion_verbose_struct *verb)
{
    return ref_minv_vector_cr_m(phi, phi0, n_shift, size, rfc, max_iter, eps, shifts, f, extra, wf, verb);
}

inversion_info minv_vector_bicgstab_m(double **phi, double *phi0, int n_shift, int size, int rfc, int max_iter,
                                      double eps, double *shifts, rmatvec f, void *extra, bool wf,
                                      inversion_verbose_struct *verb)
{
    return ref_minv_vector_bicgstab_m(phi, phi0, n_shift, size, rfc, max_iter, eps, shifts, f, extra, wf, verb);
}

inversion_info minv_vector_cg_flex_precond(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f,
                                           void *extra, rprecond pf, void *pinfo, inversion_verbose_struct *verb)
{
    return ref_minv_vector_cg_flex_precond(phi, phi0, size, max_iter, eps, f, extra, pf, pinfo, verb);
}

inversion_info minv_vector_cg_flex_precond_restart(double *phi, double *phi0, int size, int max_iter, double eps,
                                                   int rf, rmatvec f, void *extra, rprecond pf, void *pinfo,
                                                   inversion_verbose_struct *verb)
{
    return ref_minv_vector_cg_flex_precond_restart(phi, phi0, size, max_iter, eps, rf, f, extra, pf, pinfo, verb);
}

inversion_info minv_vector_gcr_var_precond(double *phi, double *phi0, int size, int max_iter, double eps, rmatvec f,
                                           void *extra, rprecond pf, void *pinfo, inversion_verbose_struct *verb)
{
    return ref_minv_vector_gcr_var_precond(phi, phi0, size, max_iter, eps, f, extra, pf, pinfo, verb);
}

inversion_info minv_vector_gcr_var_precond_restart(double *phi, double *phi0, int size, int max_iter, double eps,
                                                   int rf, rmatvec f, void *extra, rprecond pf, void *pinfo,
                                                   inversion_verbose_struct *verb)
{
    return ref_minv_vector_gcr_var_precond_restart(phi, phi0, size, max_iter, eps, rf, f, extra, pf, pinfo, verb);
}
