/*
 * glinalg.h -- C-ABI of the GB300 (sm_103a) implementation of generic-linalg's hot path:
 * the 2D U(1) lattice operators (staggered D, D^dagger, D^dagger D, gauge Laplacian, the
 * generic stencil_2d operator) and the Krylov solvers that call them (CG, multishift CG,
 * BiCGstab, GCR and their restarted forms).
 *
 * Conventions shared with the reference (generic-linalg):
 *   - A complex field is an array of complex<double> stored as interleaved (re, im) doubles;
 *     site i = y*lx + x (x fastest), times nc colours for stencil operators
 *     (lattice/lattice.h:52-83).
 *   - Links: U[2*i + mu], mu = 0 for +x, mu = 1 for +y (operators.cpp:215-224).
 *   - stencil_2d coefficient arrays keep the reference's layout
 *     (stencil_2d/coarse_stencil.h:33-67): clover[c + nc*i], hopping[c + nc*i + d*nc*V*nc]
 *     for d in {+x,+y,-x,-y}, two_link[...] for {+2x,+x+y,+2y,-x+y,-2x,-x-y,-2y,+x-y}.
 *   - Solver arguments follow the reference's minv_vector_* signatures (phi = initial guess
 *     in / solution out, phi0 = source, size, max_iter, eps = relative tolerance), and the
 *     returned glinalg_info carries the fields of the reference's inversion_info.
 *
 * Every call is blocking: it returns after the device work it issued has finished.
 * Pointers are host pointers unless GLINALG_PTR_DEVICE is set in the relevant flags, in
 * which case they must be device pointers on the current CUDA device.  There is no CPU
 * fallback: without a usable CUDA device every compute entry point returns
 * GLINALG_ERROR_NO_DEVICE.
 */
#ifndef GLINALG_H
#define GLINALG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLINALG_ABI_VERSION 2

typedef enum glinalg_status {
    GLINALG_SUCCESS = 0,
    GLINALG_ERROR_INVALID_VALUE = 1,   /* bad argument (null pointer, size mismatch, ...) */
    GLINALG_ERROR_UNSUPPORTED_OP = 2,  /* operator kind the entry point cannot drive */
    GLINALG_ERROR_CUDA = 3,            /* a CUDA runtime call failed */
    GLINALG_ERROR_NO_DEVICE = 4,       /* no usable CUDA device */
    GLINALG_ERROR_OUT_OF_MEMORY = 5,
    GLINALG_ERROR_INTERNAL = 6
} glinalg_status;

/* Outcome of a solve, in glinalg_info.status (the call itself returns GLINALG_SUCCESS). */
typedef enum glinalg_solve_status {
    GLINALG_SOLVE_CONVERGED = 0,
    GLINALG_SOLVE_MAX_ITER = 1,   /* the reference's success == false */
    GLINALG_SOLVE_BREAKDOWN = 2,  /* a recurrence denominator was exactly zero */
    GLINALG_SOLVE_NONFINITE = 3,  /* NaN or Inf appeared in a residual norm */
    GLINALG_SOLVE_TIMEOUT = 4     /* a bounded device-side wait gave up (the call reports
                                     GLINALG_ERROR_INTERNAL; info is filled) */
} glinalg_solve_status;

/* Operator kinds.  Each names the reference callback it replaces. */
typedef enum glinalg_op_kind {
    GLINALG_OP_STAGGERED = 0,         /* square_staggered_u1          operators.cpp:184 */
    GLINALG_OP_STAGGERED_DAGGER = 1,  /* square_staggered_dagger_u1   operators.cpp:372 */
    GLINALG_OP_STAGGERED_NORMAL = 2,  /* square_staggered_normal_u1   operators.cpp:444 */
    GLINALG_OP_LAPLACE = 3,           /* square_laplace_u1            operators.cpp:73  */
    GLINALG_OP_STENCIL = 4,           /* apply_stencil_2d             coarse_stencil.cpp:12  */
    GLINALG_OP_STENCIL_EO = 5,        /* apply_stencil_2d_eo          coarse_stencil.cpp:395 */
    GLINALG_OP_STENCIL_OE = 6,        /* apply_stencil_2d_oe          coarse_stencil.cpp:560 */
    /* even/odd pieces of the staggered operator (staggered-kind descriptor: links, mass) */
    GLINALG_OP_STAGGERED_DEO = 7,     /* square_staggered_deo_u1      operators.cpp:455 */
    GLINALG_OP_STAGGERED_DOE = 8,     /* square_staggered_doe_u1      operators.cpp:499 */
    GLINALG_OP_STAGGERED_M2MDEODOE = 9, /* square_staggered_m2mdeodoe_u1 operators.cpp:566 */
    /* the stencil form of m^2 - D_eo D_oe (stencil descriptor, nc = 1, shift = mass) */
    GLINALG_OP_STENCIL_M2MDEODOE = 10, /* apply_square_staggered_m2mdeodoe_stencil operators_stencil.cpp:197 */
    /* top/bottom pieces of a coarse stencil (stencil descriptor, even nc) */
    GLINALG_OP_STENCIL_TB = 11,       /* apply_stencil_2d_tb          coarse_stencil.cpp:725  */
    GLINALG_OP_STENCIL_BT = 12,       /* apply_stencil_2d_bt          coarse_stencil.cpp:1120 */
    /* the multigrid code's stencil operators (m = the stencil's shift) */
    GLINALG_OP_STENCIL_M2MDTBDBT = 13, /* apply_square_staggered_m2mdtbdbt_stencil mg_complex.cpp:1228 */
    GLINALG_OP_STENCIL_NORMAL_EO = 14, /* apply_square_staggered_normal_eo_stencil mg_complex.cpp:1277 */
    GLINALG_OP_STENCIL_NORMAL_TB = 15, /* apply_square_staggered_normal_tb_stencil mg_complex.cpp:1305 */
    GLINALG_OP_STENCIL_DAGGER_EO = 16, /* apply_square_staggered_dagger_eo_stencil mg_complex.cpp:1335 */
    GLINALG_OP_STENCIL_DAGGER_TB = 17  /* apply_square_staggered_dagger_tb_stencil mg_complex.cpp:1355 */
} glinalg_op_kind;

/* Pointer-location flags. */
#define GLINALG_PTR_HOST 0
#define GLINALG_PTR_DEVICE 1

/* Operator description; replaces staggered_u1_op (operators.h:7-15) and stencil_2d
 * (coarse_stencil.h:33-67).  Arrays are read at glinalg_operator_create time and copied
 * to the device; the caller may free them afterwards. */
typedef struct glinalg_op_desc {
    int kind;               /* glinalg_op_kind */
    int lx, ly;             /* lattice extents (x_fine, y_fine) */
    int nc;                 /* colours per site for stencil kinds (1 otherwise) */
    double mass;            /* staggered_u1_op::mass (staggered and Laplace kinds) */
    const double *links;    /* 2*lx*ly complex; staggered and Laplace kinds */
    const double *clover;   /* lx*ly*nc*nc complex; stencil kinds */
    const double *hopping;  /* 4*lx*ly*nc*nc complex; stencil kinds */
    const double *two_link; /* 8*lx*ly*nc*nc complex or NULL (stencil_size 1) */
    double shift[2];        /* stencil_2d::shift     (re, im) */
    double eo_shift[2];     /* stencil_2d::eo_shift  (re, im) */
    double dof_shift[2];    /* stencil_2d::dof_shift (re, im) */
    int flags;              /* GLINALG_PTR_DEVICE if the arrays above are device pointers */
} glinalg_op_desc;

typedef struct glinalg_operator_s *glinalg_operator;

/* inversion_verbose_struct (verbosity.h:18-24); levels as inversion_verbose_level
 * (verbosity.h:9-16): -1 pass-through, 0 none, 1 summary, 2 restart detail, 3 detail.
 * Lines are printed to stdout in the reference's format after the solve completes. */
typedef struct glinalg_verbosity {
    int verbosity;
    const char *verb_prefix;
    int precond_verbosity;
    const char *precond_verb_prefix;
} glinalg_verbosity;

/* inversion_info (inverter_struct.h:14-43) plus device-side diagnostics. */
typedef struct glinalg_info {
    double resSq;        /* squared absolute true residual |b - A x|^2 (0 for CG-M, as in the reference) */
    int iter;            /* iterations */
    int success;         /* 1 if converged */
    int ops_count;       /* operator applications, counted as the reference counts them */
    char name[64];       /* "CG", "CG(n)", "CG-M", "BiCGStab", "GCR", ... */
    double *resSqmrhs;   /* caller-provided, n_rhs entries: per-shift |(A+s)x - b|^2 (CG-M) */
    int n_rhs;
    int status;          /* glinalg_solve_status */
    int reliable_updates;/* mixed precision: number of FP64 residual recomputations */
    double device_ms;    /* device time of the solve, CUDA events */
    double gbytes;       /* algorithmic bytes moved by the solve's kernels, in GB */
    double kernel_ms;    /* mixed CG: device time inside the persistent inner-loop kernel
                            (device clock, summed over its launches; 0 if it did not run);
                            mixed multishift: device time of the FP32 multishift phase (all
                            sources) */
    double kernel_gbytes;/* algorithmic bytes that kernel (phase, for this source) moved, in GB */
    int kernel_launches; /* its launches */
} glinalg_info;

/* Arithmetic of a solve. */
typedef enum glinalg_precision {
    GLINALG_PREC_DOUBLE = 0,  /* FP64 throughout, the reference's recurrence */
    GLINALG_PREC_SINGLE = 1,  /* FP32 inner iterations, FP64 reliable updates */
    GLINALG_PREC_HALF = 2,    /* FP16 field storage, FP32 links and arithmetic inner, FP64 reliable updates */
    GLINALG_PREC_BFLOAT = 3   /* BF16 field storage, FP32 links and arithmetic inner, FP64 reliable updates */
} glinalg_precision;

typedef struct glinalg_solver_params {
    int precision;     /* glinalg_precision; only CG on Hermitian kinds accepts != DOUBLE */
    double delta;      /* reliable-update trigger: recompute when |r| < delta * max|r| (0 -> 0.01
                          for SINGLE, 0.1 for HALF and BFLOAT) */
    int flags;         /* GLINALG_PTR_DEVICE: phi / phi0 are device pointers */
    int wait_limit_us; /* bound on each wait of the mixed CG's persistent kernels for other
                          blocks (grid barriers, border and partial-sum polls), in microseconds:
                          0 = the default (2 s); < 0 = give up at the first check that finds the
                          data missing (a diagnostic).  A wait that runs out ends the kernel
                          cleanly: the call returns GLINALG_ERROR_INTERNAL with info->status
                          GLINALG_SOLVE_TIMEOUT, and the device stays usable.  No counterpart
                          in the reference (its solvers never wait on a device). */
} glinalg_solver_params;

/* ---- library ---- */
int glinalg_abi_version(void);
const char *glinalg_status_string(glinalg_status s);
/* Text of the last error raised on the calling host thread ("" if none). */
const char *glinalg_last_error(void);
/* Number of CUDA devices the library can use (0 if none). */
int glinalg_device_count(void);
/* Issue the library's work on `stream` (a cudaStream_t of the current device) instead of
 * its own non-blocking stream; use = 0 goes back to the library's stream.  Calls still
 * return only after their work has finished. */
glinalg_status glinalg_set_stream(void *stream, int use);

/* The library takes the work vectors of its calls from a stream-ordered memory pool per device
 * that keeps what calls free, so that repeated calls do not map device memory again.  This
 * returns the pools' unused memory to the device; later calls allocate it again. */
glinalg_status glinalg_release_memory(void);

/* ---- operators ---- */
glinalg_status glinalg_operator_create(const glinalg_op_desc *desc, glinalg_operator *out);
glinalg_status glinalg_operator_destroy(glinalg_operator op);
/* The reference's tests shift the operator by editing staggered_u1_op::mass between solves
 * (tests/multishift/multishift.cpp:446); this is the same edit. */
glinalg_status glinalg_operator_set_mass(glinalg_operator op, double mass);
/* Copies a stencil-kind operator's clover (lx*ly*nc*nc complex) and hopping (4 times that)
 * out of the device, in the stencil_2d layout (either pointer may be NULL). */
glinalg_status glinalg_operator_stencil_get(glinalg_operator op, double *clover, double *hopping, int flags);
/* Number of complex entries of a field (lx*ly, times nc for stencil kinds). */
long glinalg_operator_size(glinalg_operator op);
/* lhs = A rhs, the operator callback of the reference (lhs overwritten, rhs untouched). */
glinalg_status glinalg_operator_apply(glinalg_operator op, double *lhs, const double *rhs,
                                      int flags);

/* Even/odd preconditioning of M x = b (M = m + D_stag).  op: GLINALG_OP_STAGGERED_M2MDEODOE
 * (replacing square_staggered_eoprec_prepare / _reconstruct, operators.cpp:543 / :592) or
 * GLINALG_OP_STENCIL_M2MDEODOE (apply_square_staggered_eoprec_prepare_stencil / _reconstruct_
 * stencil, operators_stencil.cpp:181 / :220).  prepare: rhs_e = m rhs - D_eo rhs on even sites,
 * 0 on odd sites.  reconstruct: lhs_full = lhs_e on even sites, (rhs_o - D_oe lhs_e) / m on
 * odd sites (m: the mass, or Re(shift) for the stencil form).  Fields have op's size;
 * GLINALG_PTR_DEVICE in flags marks device pointers. */
glinalg_status glinalg_eoprec_prepare(glinalg_operator op, double *rhs_e, const double *rhs, int flags);
/* The same two steps for the top/bottom colour halves of a coarse stencil, op of kind
 * GLINALG_OP_STENCIL_M2MDTBDBT (apply_square_staggered_tbprec_prepare_stencil /
 * _reconstruct_stencil, mg_complex.cpp:1211 / :1252): rhs_t = m rhs - D_tb rhs on the top
 * colours, 0 on the bottom ones; lhs_full = lhs_t on the top colours, (rhs_b - D_bt lhs_t) /
 * Re(m) on the bottom ones. */
glinalg_status glinalg_tbprec_prepare(glinalg_operator op, double *rhs_t, const double *rhs, int flags);
glinalg_status glinalg_tbprec_reconstruct(glinalg_operator op, double *lhs_full, const double *lhs_t,
                                          const double *rhs_b, int flags);
glinalg_status glinalg_eoprec_reconstruct(glinalg_operator op, double *lhs_full, const double *lhs_e,
                                          const double *rhs_o, int flags);

/* get_square_staggered_u1_stencil / get_square_staggered_dagger_u1_stencil
 * (operators_stencil.cpp:14-63, :120-169): fills hopping_out (4*lx*ly complex) with the
 * staggered hopping coefficients and shift_out (1 complex) with the mass. */
glinalg_status glinalg_staggered_stencil(const double *links, int lx, int ly, double mass,
                                         int dagger, double *hopping_out, double *shift_out,
                                         int flags);

/* ---- BLAS-1 on fields (generic_vector.h) ---- */
glinalg_status glinalg_dot(const double *a, const double *b, long n, double out[2], int flags);
glinalg_status glinalg_norm2sq(const double *a, long n, double *out, int flags);

/* ---- solvers (the reference's minv_vector_* calling convention) ---- */
/* minv_vector_cg                generic_cg.cpp:278 */
glinalg_status glinalg_cg(glinalg_operator op, double *phi, const double *phi0, int size,
                          int max_iter, double eps, const glinalg_verbosity *verb,
                          const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_cg_restart        generic_cg.cpp:387 */
glinalg_status glinalg_cg_restart(glinalg_operator op, double *phi, const double *phi0, int size,
                                  int max_iter, double eps, int restart_freq,
                                  const glinalg_verbosity *verb,
                                  const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_bicgstab          generic_bicgstab.cpp:205 */
glinalg_status glinalg_bicgstab(glinalg_operator op, double *phi, const double *phi0, int size,
                                int max_iter, double eps, const glinalg_verbosity *verb,
                                const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_bicgstab_restart  generic_bicgstab.cpp:345 */
glinalg_status glinalg_bicgstab_restart(glinalg_operator op, double *phi, const double *phi0,
                                        int size, int max_iter, double eps, int restart_freq,
                                        const glinalg_verbosity *verb,
                                        const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_gcr               generic_gcr.cpp:202 */
glinalg_status glinalg_gcr(glinalg_operator op, double *phi, const double *phi0, int size,
                           int max_iter, double eps, const glinalg_verbosity *verb,
                           const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_gcr_restart       generic_gcr.cpp:337 */
glinalg_status glinalg_gcr_restart(glinalg_operator op, double *phi, const double *phi0, int size,
                                   int max_iter, double eps, int restart_freq,
                                   const glinalg_verbosity *verb,
                                   const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_cg_m              generic_cg_m.cpp:312.  phi: n_shift pointers to solution
 * vectors (zeroed, then written); shifts must be sorted ascending as in the reference and
 * are left unchanged on return; info->resSqmrhs (n_shift entries) receives the explicit
 * squared residual of every shifted system. */
glinalg_status glinalg_cg_m(glinalg_operator op, double *const *phi, const double *phi0,
                            int n_shift, int size, int resid_freq_check, int max_iter,
                            double eps, const double *shifts, int worst_first,
                            const glinalg_verbosity *verb, const glinalg_solver_params *params,
                            glinalg_info *info);

/* ---- sibling solvers: the reference's other Krylov methods on the same operators (FP64) ---- */

/* minv_vector_cr                 generic_cr.cpp:198 (A Hermitian).  As in the reference,
 * info->success is 1 whenever max_iter > 0 (generic_cr.cpp:288 compares k with max_iter, a
 * value the loop never reaches); info->status says whether the tolerance was met. */
glinalg_status glinalg_cr(glinalg_operator op, double *phi, const double *phi0, int size,
                          int max_iter, double eps, const glinalg_verbosity *verb,
                          const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_cr_restart         generic_cr.cpp:326 */
glinalg_status glinalg_cr_restart(glinalg_operator op, double *phi, const double *phi0, int size,
                                  int max_iter, double eps, int restart_freq,
                                  const glinalg_verbosity *verb,
                                  const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_minres (with omega) generic_minres.cpp:130: minimal residual, x += omega alpha r */
glinalg_status glinalg_minres(glinalg_operator op, double *phi, const double *phi0, int size,
                              int max_iter, double eps, double omega,
                              const glinalg_verbosity *verb, const glinalg_solver_params *params,
                              glinalg_info *info);
/* minv_vector_bicgstab_l         generic_bicgstab_l.cpp:317 (1 <= l <= 16) */
glinalg_status glinalg_bicgstab_l(glinalg_operator op, double *phi, const double *phi0, int size,
                                  int max_iter, double eps, int l, const glinalg_verbosity *verb,
                                  const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_bicgstab_l_restart generic_bicgstab_l.cpp:564 */
glinalg_status glinalg_bicgstab_l_restart(glinalg_operator op, double *phi, const double *phi0,
                                          int size, int max_iter, double eps, int restart_freq, int l,
                                          const glinalg_verbosity *verb,
                                          const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_cr_m               generic_cr_m.cpp:323 and
 * minv_vector_bicgstab_m         generic_bicgstab_m.cpp:402: arguments as glinalg_cg_m.  The
 * multishift summary line reads "CG-M" for every method, as the reference prints it. */
glinalg_status glinalg_cr_m(glinalg_operator op, double *const *phi, const double *phi0,
                            int n_shift, int size, int resid_freq_check, int max_iter,
                            double eps, const double *shifts, int worst_first,
                            const glinalg_verbosity *verb, const glinalg_solver_params *params,
                            glinalg_info *info);
glinalg_status glinalg_bicgstab_m(glinalg_operator op, double *const *phi, const double *phi0,
                                  int n_shift, int size, int resid_freq_check, int max_iter,
                                  double eps, const double *shifts, int worst_first,
                                  const glinalg_verbosity *verb,
                                  const glinalg_solver_params *params, glinalg_info *info);

/* Preconditioners of the flexible solvers (generic_precond.h): the reference passes a
 * callback plus a struct; here the kind selects the callback and the fields are the struct's. */
typedef enum glinalg_precond_kind {
    GLINALG_PRECOND_IDENTITY = 0, /* identity_preconditioner  generic_precond.cpp:34 */
    GLINALG_PRECOND_MINRES = 1,   /* minres_preconditioner    generic_precond.cpp:53 */
    GLINALG_PRECOND_GCR = 2,      /* gcr_preconditioner       generic_precond.cpp:70 */
    GLINALG_PRECOND_MG = 3        /* mg_preconditioner        mg_complex.cpp:514 (field mg) */
} glinalg_precond_kind;
typedef struct glinalg_mg_s *glinalg_mg;
typedef struct glinalg_precond {
    int kind;             /* glinalg_precond_kind */
    int n_step;           /* {minres,gcr}_precond_struct_complex::n_step */
    double rel_res;       /* ::rel_res */
    glinalg_operator op;  /* ::matrix_vector / matrix_extra_data; NULL: the solve's operator */
    glinalg_mg mg;        /* GLINALG_PRECOND_MG: the hierarchy (glinalg_mg_create) */
} glinalg_precond;

/* minv_vector_cg_flex_precond    generic_cg_flex_precond.cpp:223 (NULL precond: identity) */
glinalg_status glinalg_cg_flex_precond(glinalg_operator op, double *phi, const double *phi0,
                                       int size, int max_iter, double eps,
                                       const glinalg_precond *precond,
                                       const glinalg_verbosity *verb,
                                       const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_cg_flex_precond_restart generic_cg_flex_precond.cpp:367 */
glinalg_status glinalg_cg_flex_precond_restart(glinalg_operator op, double *phi, const double *phi0,
                                               int size, int max_iter, double eps, int restart_freq,
                                               const glinalg_precond *precond,
                                               const glinalg_verbosity *verb,
                                               const glinalg_solver_params *params,
                                               glinalg_info *info);
/* minv_vector_gcr_var_precond    generic_gcr_var_precond.cpp:220 */
glinalg_status glinalg_gcr_var_precond(glinalg_operator op, double *phi, const double *phi0,
                                       int size, int max_iter, double eps,
                                       const glinalg_precond *precond,
                                       const glinalg_verbosity *verb,
                                       const glinalg_solver_params *params, glinalg_info *info);
/* minv_vector_gcr_var_precond_restart generic_gcr_var_precond.cpp:369 */
glinalg_status glinalg_gcr_var_precond_restart(glinalg_operator op, double *phi, const double *phi0,
                                               int size, int max_iter, double eps, int restart_freq,
                                               const glinalg_precond *precond,
                                               const glinalg_verbosity *verb,
                                               const glinalg_solver_params *params,
                                               glinalg_info *info);

/* ---- U(1) gauge fields (u1_utils.h); links are 2*lx*ly complex, U[2*i + mu] ---- */

/* read_gauge_u1 / write_gauge_u1 (u1_utils.cpp:17 / :44): the reference's text format, one
 * phase per line, x outermost, then y, then mu (fixed notation, 20 decimals on write).  Host
 * arrays; read fails with GLINALG_ERROR_INVALID_VALUE if the file holds fewer phases. */
glinalg_status glinalg_read_gauge_u1(double *links, int lx, int ly, const char *path);
glinalg_status glinalg_write_gauge_u1(const double *links, int lx, int ly, const char *path);
/* unit_gauge_u1 (u1_utils.cpp:69) */
glinalg_status glinalg_unit_gauge_u1(double *links, int lx, int ly, int flags);
/* get_plaquette_u1 (u1_utils.cpp:190): the average plaquette, out = (re, im) */
glinalg_status glinalg_plaquette_u1(const double *links, int lx, int ly, double out[2], int flags);
/* get_topo_u1 (u1_utils.cpp:210): sum of plaquette phases over 2 pi */
glinalg_status glinalg_topo_u1(const double *links, int lx, int ly, double *out, int flags);
/* apply_gauge_trans_u1 (u1_utils.cpp:128): U_mu(x) = g(x) U_mu(x) g(x+mu)^*, in place;
 * trans: lx*ly complex */
glinalg_status glinalg_apply_gauge_trans_u1(double *links, const double *trans, int lx, int ly, int flags);
/* apply_ape_smear_u1 (u1_utils.cpp:145): n_iter APE sweeps with weight alpha, each projected
 * back onto U(1); smeared and links may not overlap */
glinalg_status glinalg_apply_ape_smear_u1(double *smeared, const double *links, int lx, int ly,
                                          double alpha, int n_iter, int flags);

/* ---- multigrid transfer and coarse operators (multigrid/aa_mg/mg_complex.cpp) ---- */

/* One level of mg_operator_struct_complex (mg_complex.h): a fine lattice lx x ly with
 * nc_fine dof per site, blocked bx x by onto (lx/bx) x (ly/by) coarse sites with nc_coarse
 * dof.  null_vectors: nc_coarse fields of lx*ly*nc_fine complex (null_vectors[level][c][f],
 * f = (y*lx + x)*nc_fine + dof), copied to the device. */
typedef struct glinalg_mg_level_s *glinalg_mg_level;
glinalg_status glinalg_mg_level_create(int lx, int ly, int nc_fine, int bx, int by, int nc_coarse,
                                       const double *null_vectors, int flags, glinalg_mg_level *out);
glinalg_status glinalg_mg_level_destroy(glinalg_mg_level lv);
glinalg_status glinalg_mg_get_null_vectors(glinalg_mg_level lv, double *out, int flags);
/* block_normalize / block_orthonormalize (mg_complex.cpp:191 / :259), in place */
glinalg_status glinalg_mg_block_normalize(glinalg_mg_level lv);
glinalg_status glinalg_mg_block_orthonormalize(glinalg_mg_level lv);
/* prolong (mg_complex.cpp:372): fine = P coarse; restrict (:421): coarse = P^dagger fine */
glinalg_status glinalg_mg_prolong(glinalg_mg_level lv, double *fine, const double *coarse, int flags);
glinalg_status glinalg_mg_restrict(glinalg_mg_level lv, double *coarse, const double *fine, int flags);
/* generate_coarse_from_fine_stencil (mg_complex.cpp:827): a new GLINALG_OP_STENCIL operator on
 * the coarse lattice holding P^dagger A P of the fine stencil operator `fine` (clover, the
 * four hops and, unless ignore_shifts, its shift / eo_shift / dof_shift; two-link terms do not
 * enter, as in the reference).  The coarse operator's own shifts are zero. */
glinalg_status glinalg_mg_coarse_stencil(glinalg_mg_level lv, glinalg_operator fine, int ignore_shifts,
                                         glinalg_operator *coarse_out);

/* The multigrid preconditioner mg_preconditioner (mg_complex.cpp:514) over a hierarchy of
 * n_refine levels: ops[0] the fine operator, ops[l+1] the operator of the coarse lattice of
 * levels[l] (for instance from glinalg_mg_coarse_stencil), levels[l] the transfer from
 * ops[l] to ops[l+1].  params mirrors mg_precond_struct_complex (mg_complex.h). */
#define GLINALG_MG_MAX_LEVELS 8
/* minv_inverter (generic_inverters.h:70-81): the smoother */
#define GLINALG_MINV_INVALID -1
#define GLINALG_MINV_CG 0
#define GLINALG_MINV_CR 1
#define GLINALG_MINV_GCR 2
#define GLINALG_MINV_BICGSTAB 3
#define GLINALG_MINV_BICGSTAB_L 4
#define GLINALG_MINV_MINRES 7
/* inner_solver (mg.h:5-14): the coarse solver */
#define GLINALG_MG_NONE 0
#define GLINALG_MG_MINRES 1
#define GLINALG_MG_CG 2
#define GLINALG_MG_GCR 3
#define GLINALG_MG_BICGSTAB 4
#define GLINALG_MG_CR 5
#define GLINALG_MG_BICGSTAB_L 6
/* mg_multilevel_type (mg_complex.h) */
#define GLINALG_MLEVEL_SMOOTH 0
#define GLINALG_MLEVEL_RECURSIVE 1
typedef struct glinalg_mg_params {
    int smoother;                              /* in_smooth_type (GLINALG_MINV_*) */
    double omega_smooth;                       /* kept for the interface; the MinRes smoother uses 1 */
    int n_pre_smooth[GLINALG_MG_MAX_LEVELS];   /* per level */
    int n_post_smooth[GLINALG_MG_MAX_LEVELS];
    int normal_eqn_mg, normal_eqn_smooth;      /* must be 0: normal-equation variants not supported */
    int mlevel_type;                           /* GLINALG_MLEVEL_* */
    int coarse_solver;                         /* in_solve_type (GLINALG_MG_*) */
    int n_max, n_restart;
    double rel_res[GLINALG_MG_MAX_LEVELS];
} glinalg_mg_params;
glinalg_status glinalg_mg_create(int n_refine, const glinalg_operator *ops, const glinalg_mg_level *levels,
                                 const glinalg_mg_params *params, glinalg_mg *out);
glinalg_status glinalg_mg_destroy(glinalg_mg mg);
/* One application lhs = M^-1 rhs on the finest level (fields of ops[0]'s size). */
glinalg_status glinalg_mg_apply(glinalg_mg mg, double *lhs, const double *rhs, int flags);

/* ---- batched solves (no reference counterpart: the reference solves systems one at a
 * time in a loop; these run many independent systems in one device launch sequence) ---- */

/* Multishift CG for n_rhs independent sources of one operator, all shifts and sources
 * iterated together.  phi: n_rhs*n_shift*size complex (rhs-major, then shift), phi0:
 * n_rhs*size complex.  infos: n_rhs entries (each with resSqmrhs of n_shift entries or NULL).
 * Same recurrence per source as glinalg_cg_m. */
glinalg_status glinalg_cg_m_multi(glinalg_operator op, double *phi, const double *phi0,
                                  int n_rhs, int n_shift, int size, int resid_freq_check,
                                  int max_iter, double eps, const double *shifts,
                                  const glinalg_solver_params *params, glinalg_info *infos);

/* CG on n_sys independent Hermitian systems (staggered-normal or Laplace kinds, any sizes)
 * advanced together with per-system convergence masks.  phi[s] / phi0[s] have
 * glinalg_operator_size(ops[s]) complex entries. */
glinalg_status glinalg_cg_batch(const glinalg_operator *ops, int n_sys, double *const *phi,
                                const double *const *phi0, int max_iter, double eps,
                                const glinalg_solver_params *params, glinalg_info *infos);

/* ---- adjoint force (no reference counterpart) ----
 * For S(theta) = phi^dagger (D^dagger D + sigma)^-1 phi with U_mu(x) = exp(i theta_mu(x)):
 * given X = (D^dagger D + sigma)^-1 phi and Y = D X, writes
 * dS/dtheta_mu(x) = -2 Re(Y^dagger dD/dtheta_mu(x) X) to grad[2*i + mu] (2*lx*ly reals).
 * op must be a staggered kind (its links and mass define D). */
glinalg_status glinalg_staggered_force(glinalg_operator op, const double *X, const double *Y,
                                       double *grad, int flags);
/* Forward solve plus force: X = (D^dagger D + sigma)^-1 phi by CG to relative residual eps
 * (params->precision selects the arithmetic), Y = D X, grad as above, *action = Re(phi^dagger X).
 * X_out may be NULL. */
glinalg_status glinalg_staggered_action_grad(glinalg_operator op, const double *phi, double sigma,
                                             double eps, int max_iter, double *action,
                                             double *grad, double *X_out,
                                             const glinalg_solver_params *params,
                                             glinalg_info *info);

/* ---- allocation-free operator ----
 * No counterpart in the reference.  For callers that must not allocate device memory while
 * they run (an application that has reserved HBM for its own pools, a code path under another
 * framework's allocator or memory budget, a latency-critical loop that cannot afford
 * cudaMalloc / cudaFree): lhs = D^dagger D rhs, the staggered normal operator of
 * square_staggered_normal_u1, on caller-provided DEVICE buffers (links: 2*lx*ly complex,
 * lhs / rhs: lx*ly complex), enqueued on `stream` (a cudaStream_t, NULL for the legacy default
 * stream); the call returns without waiting, and lhs is complete once that stream has reached
 * the work (synchronise the stream before reading it on the host).  The intermediate D rhs lives in a fixed array inside
 * the library (GLINALG_NOALLOC_MAX_SITES complex values, 4 MiB, held on every GPU that loads
 * the library until exit); lattices with more sites are rejected with
 * GLINALG_ERROR_INVALID_VALUE.  The first call on a device looks up that array's address;
 * make it before any stream capture.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller. */
#define GLINALG_NOALLOC_MAX_SITES (1L << 18)
glinalg_status glinalg_staggered_normal_apply_noalloc(const double *links, double mass, int lx,
                                                      int ly, double *lhs, const double *rhs,
                                                      void *stream);

/* ---- measurement ----
 * Times the two inner-iteration kernels of the mixed-precision CG (A: direction update +
 * D p + norm; B: D^dagger t + solution/residual update + norm) on op's lattice, each launched
 * n_launch times on its own between CUDA events, on resident buffers.  ms[0], ms[1]: mean
 * duration of one launch of A and B; bytes[0], bytes[1]: algorithmic bytes one launch moves.
 * op must be GLINALG_OP_STAGGERED_NORMAL; precision SINGLE, HALF or BFLOAT. */
glinalg_status glinalg_profile_mixed_kernels(glinalg_operator op, int precision, int n_launch,
                                             double ms[2], double bytes[2]);
/* Times the persistent inner-loop kernel the autotuner picked for op's lattice and precision
 * (a mixed-precision solve must have run on it): n_launch launches of exactly n_iter inner CG
 * iterations each, bracketed by CUDA events on the library stream.  ms: mean milliseconds per
 * launch; bytes: algorithmic bytes per launch; cand: the kernel (as glinalg_tuned_persist).
 * Staggered normal operator only. */
glinalg_status glinalg_profile_persist_kernel(glinalg_operator op, int precision, int n_launch, int n_iter,
                                              double *ms, double *bytes, int *cand);
/* Measured shared-memory bandwidth of the current device: 2 blocks of 1024 threads per SM
 * stream conflict-free 128-bit loads from shared memory (5 timed launches, CUDA events on the
 * library stream).  gbs: bytes loaded per second / 1e9; ms (may be NULL): one launch.  No
 * counterpart in the reference: the denominator of the on-chip roofline of the resident CG. */
glinalg_status glinalg_probe_smem_bandwidth(double *gbs, double *ms);
/* Tile shape the autotuner picked for op's lattice and precision (an index into the
 * library's candidate list: 0 = 32x16, 1 = 32x32, 2 = 32x32 (4 rows of 8), 3 = 32x32
 * (16 rows of 2) sites per block), or -1 if no mixed solve has run on this lattice yet. */
int glinalg_tuned_tile(glinalg_operator op, int precision);
/* Persistent inner-loop kernel the autotuner picked for op's lattice and precision: 0-3 the
 * register-tiled kernel (16 warps x 4 rows, 16 x 8, 32 x 2, 16 x 2), 4-5 the bulk-copy kernel
 * (256 x 4 and 512 x 2 tiles), 6-8 the rectangle-resident kernel (FP32 only: 16 warps with
 * x_lo in registers, 32 warps, 16 warps with x_lo in memory); -1 if none serves the lattice or
 * no mixed solve has run on it yet. */
int glinalg_tuned_persist(glinalg_operator op, int precision);

/* ---- inputs the way the reference's tests make them (host side) ----
 * A generator is one std::mt19937 stream (as `std::mt19937 generator(seed)` in the tests);
 * successive calls continue the stream. */
typedef struct glinalg_rng_s *glinalg_rng;
glinalg_status glinalg_rng_create(uint32_t seed, glinalg_rng *out);
glinalg_status glinalg_rng_destroy(glinalg_rng rng);
/* rand_gauge_u1 (u1_utils.cpp:79-87): U = exp(i theta), theta uniform in (-pi, pi). */
glinalg_status glinalg_rng_gauge_u1(glinalg_rng rng, double *links, int lx, int ly);
/* gauss_gauge_u1 (u1_utils.cpp:92-112): theta normal with variance 1/beta. */
glinalg_status glinalg_rng_gauss_gauge_u1(glinalg_rng rng, double *links, int lx, int ly,
                                          double beta);
/* rand_trans_u1 (u1_utils.cpp:116): a random gauge transform, lx*ly complex */
glinalg_status glinalg_rng_trans_u1(glinalg_rng rng, double *trans, int lx, int ly);
/* gaussian<complex> (generic_vector.h:48-60): re and im independent N(0,1). */
glinalg_status glinalg_rng_gaussian(glinalg_rng rng, double *v, long n_complex);

#ifdef __cplusplus
}
#endif
#endif /* GLINALG_H */
