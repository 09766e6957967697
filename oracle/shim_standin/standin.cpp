// standin.cpp -- definitions behind ref_standin.h (test infrastructure).  The operator and
// preconditioner callbacks exist so that the shim can recognise them by address; the library
// runs the operators, so their bodies are never reached here.  The real-valued solvers that
// the shim passes to the reference's own code (ref_minv_vector_*) are not built in this setting
// and report so.
#include "ref_standin.h"

typedef void (*rmatvec)(double *, double *, void *);
typedef void (*rprecond)(double *, double *, int, void *, inversion_verbose_struct *);

#define STANDIN_OP(name) \
    void name(complex<double> *, complex<double> *, void *) {}
STANDIN_OP(square_staggered_u1)
STANDIN_OP(square_staggered_dagger_u1)
STANDIN_OP(square_staggered_normal_u1)
STANDIN_OP(square_laplace_u1)
STANDIN_OP(square_staggered_deo_u1)
STANDIN_OP(square_staggered_doe_u1)
STANDIN_OP(square_staggered_m2mdeodoe_u1)
STANDIN_OP(apply_stencil_2d)
STANDIN_OP(apply_stencil_2d_eo)
STANDIN_OP(apply_stencil_2d_oe)
STANDIN_OP(apply_stencil_2d_tb)
STANDIN_OP(apply_stencil_2d_bt)
STANDIN_OP(apply_square_staggered_m2mdeodoe_stencil)
STANDIN_OP(apply_square_staggered_m2mdtbdbt_stencil)
STANDIN_OP(apply_square_staggered_normal_eo_stencil)
STANDIN_OP(apply_square_staggered_normal_tb_stencil)
STANDIN_OP(apply_square_staggered_dagger_eo_stencil)
STANDIN_OP(apply_square_staggered_dagger_tb_stencil)

void identity_preconditioner(complex<double> *, complex<double> *, int, void *, inversion_verbose_struct *) {}
void minres_preconditioner(complex<double> *, complex<double> *, int, void *, inversion_verbose_struct *) {}
void gcr_preconditioner(complex<double> *, complex<double> *, int, void *, inversion_verbose_struct *) {}

static inversion_info not_built()
{
    inversion_info r;
    r.name = "real-valued solver not built in this setting";
    return r;
}

inversion_info ref_minv_vector_cg(double *, double *, int, int, double, rmatvec, void *, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cg_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                          inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cg_m(double **, double *, int, int, int, int, double, double *, rmatvec, void *, bool,
                                    inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_bicgstab(double *, double *, int, int, double, rmatvec, void *,
                                        inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_bicgstab_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                                inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_gcr(double *, double *, int, int, double, rmatvec, void *, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_gcr_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                           inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cr(double *, double *, int, int, double, rmatvec, void *, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cr_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                          inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_minres(double *, double *, int, int, double, rmatvec, void *,
                                      inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_minres(double *, double *, int, int, double, double, rmatvec, void *,
                                      inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_bicgstab_l(double *, double *, int, int, double, int, rmatvec, void *,
                                          inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_bicgstab_l_restart(double *, double *, int, int, double, int, int, rmatvec, void *,
                                                  inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cr_m(double **, double *, int, int, int, int, double, double *, rmatvec, void *, bool,
                                    inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_bicgstab_m(double **, double *, int, int, int, int, double, double *, rmatvec, void *,
                                          bool, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cg_flex_precond(double *, double *, int, int, double, rmatvec, void *, rprecond,
                                               void *, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_cg_flex_precond_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                                       rprecond, void *, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_gcr_var_precond(double *, double *, int, int, double, rmatvec, void *, rprecond,
                                               void *, inversion_verbose_struct *)
{ return not_built(); }
inversion_info ref_minv_vector_gcr_var_precond_restart(double *, double *, int, int, double, int, rmatvec, void *,
                                                       rprecond, void *, inversion_verbose_struct *)
{ return not_built(); }
