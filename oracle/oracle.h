/*
 * oracle.h -- CPU oracle for the 2D U(1) lattice hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C99 restatement of generic-linalg's CPU algorithms for the operators
 * (staggered D, D^dagger, D^dagger D, gauge Laplacian, stencil_2d apply/eo/oe, the
 * staggered stencil builders, and the even/odd pieces D_eo, D_oe, m^2 - D_eo D_oe with the
 * prepare / reconstruct steps) and the Krylov solvers that call them (CG, restarted CG,
 * multishift CG, BiCGstab, restarted BiCGstab, GCR, restarted GCR) and their siblings (CR,
 * restarted CR, MinRes, multishift CR, BiCGstab-l, restarted BiCGstab-l, multishift BiCGstab,
 * flexibly preconditioned CG and variably preconditioned GCR, with their restarted forms).  Every function cites
 * the reference file:line it follows.  It exists so that tests, the smoke check and the
 * CPU-baseline leg of the benchmark have something to compare the CUDA path against.
 * The product (the CUDA library and its C-ABI) never links, loads or calls it.
 *
 * Parity pin: tests/golden/ holds outputs of the reference itself (compiled from its own
 * sources by oracle/Makefile into oracle/_ref/), and tests/test_oracle_golden.py checks
 * this oracle against them.
 *
 * Data layout (identical to the reference): a field is V = lx*ly complex<double> values,
 * site i = y*lx + x, stored as interleaved (re, im) doubles.  Links are U[2*i + mu],
 * mu = 0 for +x and mu = 1 for +y.  stencil_2d arrays use the reference's layout:
 * clover[c + nc*i], hopping[c + nc*i + dir*nc*V*nc], two_link[c + nc*i + dir*nc*V*nc]
 * with i = site*nc + row.
 */
#ifndef GLINALG_ORACLE_H
#define GLINALG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum orc_kind {
    ORC_STAGGERED = 0,        /* square_staggered_u1 */
    ORC_STAGGERED_DAGGER = 1, /* square_staggered_dagger_u1 */
    ORC_STAGGERED_NORMAL = 2, /* square_staggered_normal_u1 */
    ORC_LAPLACE = 3,          /* square_laplace_u1 */
    ORC_STENCIL = 4,          /* apply_stencil_2d (DIR_ALL) */
    ORC_STENCIL_EO = 5,       /* apply_stencil_2d_eo */
    ORC_STENCIL_OE = 6,       /* apply_stencil_2d_oe */
    ORC_STAGGERED_DEO = 7,    /* square_staggered_deo_u1 */
    ORC_STAGGERED_DOE = 8,    /* square_staggered_doe_u1 */
    ORC_STAGGERED_M2MDEODOE = 9, /* square_staggered_m2mdeodoe_u1 */
    ORC_STENCIL_M2MDEODOE = 10,  /* apply_square_staggered_m2mdeodoe_stencil */
    ORC_STENCIL_TB = 11,         /* apply_stencil_2d_tb */
    ORC_STENCIL_BT = 12,         /* apply_stencil_2d_bt */
    ORC_STENCIL_M2MDTBDBT = 13,  /* apply_square_staggered_m2mdtbdbt_stencil (mg_complex.cpp) */
    ORC_STENCIL_NORMAL_EO = 14,  /* apply_square_staggered_normal_eo_stencil */
    ORC_STENCIL_NORMAL_TB = 15,  /* apply_square_staggered_normal_tb_stencil */
    ORC_STENCIL_DAGGER_EO = 16,  /* apply_square_staggered_dagger_eo_stencil */
    ORC_STENCIL_DAGGER_TB = 17   /* apply_square_staggered_dagger_tb_stencil */
};

typedef struct {
    int kind;
    int lx, ly, nc;
    double mass;
    const double *links;      /* 2*lx*ly complex */
    const double *clover;     /* lx*ly*nc*nc complex */
    const double *hopping;    /* 4*lx*ly*nc*nc complex */
    const double *two_link;   /* 8*lx*ly*nc*nc complex or NULL */
    double shift[2], eo_shift[2], dof_shift[2];
} orc_op;

typedef struct {
    double resSq;
    int iter;
    int success;
    int ops_count;
    char name[64];
} orc_info;

/* Operators: lhs is overwritten, rhs is read. */
void orc_apply(const orc_op *op, double *lhs, const double *rhs);
long orc_op_size(const orc_op *op); /* number of complex entries of a field */

/* Even/odd preconditioning of the staggered operator, for op->kind ORC_STAGGERED_M2MDEODOE
 * (the function form: mass and links) or ORC_STENCIL_M2MDEODOE (the stencil form: shift and
 * hopping).  prepare: rhs_e = m rhs - D_eo rhs on even sites, 0 on odd sites.  reconstruct:
 * lhs_full = lhs_e on even sites, (rhs_o - D_oe lhs_e) / m on odd sites. */
void orc_eoprec_prepare(const orc_op *op, double *rhs_e, const double *rhs);
void orc_eoprec_reconstruct(const orc_op *op, double *lhs_full, const double *lhs_e, const double *rhs_o);

/* Top/bottom preconditioning of a coarse stencil (ORC_STENCIL_M2MDTBDBT). */
void orc_tbprec_prepare(const orc_op *op, double *rhs_t, const double *rhs);
void orc_tbprec_reconstruct(const orc_op *op, double *lhs_full, const double *lhs_t, const double *rhs_b);

/* One multigrid level (mg_operator_struct_complex at its current level): a fine lattice
 * lx x ly with nc_f dof per site blocked bx x by into (lx/bx) x (ly/by) coarse sites with nc_c
 * dof; null_vectors holds nc_c fields of lx*ly*nc_f complex, index (y*lx + x)*nc_f + dof. */
typedef struct {
    int lx, ly, nc_f, bx, by, nc_c;
    double *null_vectors;
} orc_mg_level;
void orc_mg_block_normalize(orc_mg_level *lv);
void orc_mg_block_orthonormalize(orc_mg_level *lv);
void orc_mg_prolong(const orc_mg_level *lv, double *fine, const double *coarse);
void orc_mg_restrict(const orc_mg_level *lv, double *coarse, const double *fine);
/* generate_coarse_from_fine_stencil: coarse clover (V_c*nc_c*nc_c) and hopping (4*that) of
 * P^dagger A P for a stencil-kind fine operator (its clover, 4 hops and shifts). */
void orc_mg_coarse_stencil(const orc_mg_level *lv, const orc_op *fine, int ignore_shifts, double *clover,
                           double *hopping);

/* Stencil builders (fill hopping[4*V], clover untouched, shift = mass). */
void orc_staggered_stencil(double *hopping, const double *links, int lx, int ly, int dagger);

/* BLAS-1 helpers (generic_vector.h). */
void orc_dot(const double *a, const double *b, long n, double out[2]);
double orc_norm2sq(const double *a, long n);
double orc_diffnorm2sq(const double *a, const double *b, long n);

/* Solvers.  hist (optional, may be NULL) receives the relative residual printed at each
 * iteration by the reference's DETAIL verbosity, hist_cap entries at most. */
void orc_cg(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
            double eps, orc_info *info, double *hist, int hist_cap);
void orc_cg_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                    double eps, int restart_freq, orc_info *info);
void orc_bicgstab(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                  double eps, orc_info *info, double *hist, int hist_cap);
void orc_bicgstab_restart(const orc_op *op, double *phi, const double *phi0, long size,
                          int max_iter, double eps, int restart_freq, orc_info *info);
void orc_gcr(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
             double eps, orc_info *info, double *hist, int hist_cap);
void orc_gcr_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                     double eps, int restart_freq, orc_info *info);
/* phi: n_shift solution vectors laid out back to back (n_shift*size complex). */
void orc_cg_m(const orc_op *op, double *phi, const double *phi0, int n_shift, long size,
              int resid_freq_check, int max_iter, double eps, const double *shifts,
              int worst_first, orc_info *info, double *resSqmrhs, double *hist, int hist_cap);

/* ---- sibling Krylov solvers ---- */
void orc_cr(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
            double eps, orc_info *info, double *hist, int hist_cap);
void orc_cr_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                    double eps, int restart_freq, orc_info *info);
void orc_minres(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                double eps, double omega, orc_info *info, double *hist, int hist_cap);
void orc_cr_m(const orc_op *op, double *phi, const double *phi0, int n_shift, long size,
              int resid_freq_check, int max_iter, double eps, const double *shifts,
              int worst_first, orc_info *info, double *resSqmrhs, double *hist, int hist_cap);
/* hist receives one entry per l-step cycle */
void orc_bicgstab_l(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                    double eps, int l, orc_info *info, double *hist, int hist_cap);
void orc_bicgstab_l_restart(const orc_op *op, double *phi, const double *phi0, long size,
                            int max_iter, double eps, int restart_freq, int l, orc_info *info);
void orc_bicgstab_m(const orc_op *op, double *phi, const double *phi0, int n_shift, long size,
                    int resid_freq_check, int max_iter, double eps, const double *shifts,
                    int worst_first, orc_info *info, double *resSqmrhs, double *hist, int hist_cap);

/* Preconditioners of the flexible solvers (generic_precond.h). */
enum orc_precond_kind { ORC_PRECOND_IDENTITY = 0, ORC_PRECOND_MINRES = 1, ORC_PRECOND_GCR = 2 };
typedef struct {
    int kind;
    int n_step;          /* iterations of the inner solve */
    double rel_res;      /* its relative-residual target */
    const orc_op *op;    /* its operator (matrix_vector of the precond struct) */
} orc_precond;
void orc_fpcg(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
              double eps, const orc_precond *pc, orc_info *info, double *hist, int hist_cap);
void orc_fpcg_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                      double eps, int restart_freq, const orc_precond *pc, orc_info *info);
void orc_vpgcr(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
               double eps, const orc_precond *pc, orc_info *info, double *hist, int hist_cap);
void orc_vpgcr_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                       double eps, int restart_freq, const orc_precond *pc, orc_info *info);

/* ---- gauge-field utilities (u1_utils.cpp) ---- */
void orc_plaquette_u1(const double *links, int lx, int ly, double out[2]);
double orc_topo_u1(const double *links, int lx, int ly);
void orc_gauge_trans_u1(double *links, const double *trans, int lx, int ly);
void orc_ape_smear_u1(double *smeared, const double *links, int lx, int ly, double alpha, int n_iter);

/* Adjoint force for S = phi^dagger (D^dagger D + sigma)^-1 phi with respect to the link
 * angles theta_mu(x) (U = exp(i theta)), given X = (D^dagger D + sigma)^-1 phi and Y = D X:
 * dS/dtheta_mu(x) = -2 Re( Y^dagger (dD/dtheta_mu(x)) X ).  out has 2*lx*ly reals. */
void orc_staggered_force(const double *links, double mass, int lx, int ly, const double *X,
                         const double *Y, double *out);

#ifdef __cplusplus
}
#endif
#endif
