// solvers.h -- internal solver entry points on device pointers (x in/out, b in).
#pragma once

#include "solver_util.h"

namespace glinalg {

// sigma: diagonal shift added to the operator (the reference's CG has none; used by the force)
glinalg_status cg_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                       double eps, const Verb &verb, glinalg_info *info, cudaStream_t st,
                       double sigma = 0.0);
glinalg_status bicgstab_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b,
                             int max_iter, double eps, const Verb &verb, glinalg_info *info,
                             cudaStream_t st);
glinalg_status gcr_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                        double eps, const Verb &verb, glinalg_info *info, cudaStream_t st);
glinalg_status cg_m_fp64(const glinalg_operator_s *op, double2 *const *X, const double2 *b,
                         int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                         bool worst_first, const Verb &verb, glinalg_info *info, cudaStream_t st);
// Multishift CG of n_rhs sources advanced together (cgm_batch.cu); X: n_rhs * n_shift fields
// (source-major), B: n_rhs fields.  Staggered-normal and Laplace kinds, n_shift <= 32.
bool cg_m_batch_supported(const glinalg_operator_s *op, int n_shift);
glinalg_status cg_m_batch(const glinalg_operator_s *op, double2 *X, const double2 *B, int n_rhs,
                          int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                          glinalg_info *infos, cudaStream_t st);
// The same in mixed precision (cgm_mixed.cu): an FP32 multishift over every source (FP64
// scalar recurrences), then every shifted system refined by the mixed CG to eps, FP64-true.
// Staggered-normal kind, n_shift <= 32.  phase1_iters / phase2_iters (may be null): per source,
// the multishift iterations and the refinement iterations summed over its shifts.
bool cg_m_batch_mixed_supported(const glinalg_operator_s *op, int n_shift);
glinalg_status cg_m_batch_mixed(const glinalg_operator_s *op, double2 *X, const double2 *B, int n_rhs,
                                int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                                glinalg_info *infos, cudaStream_t st, int *phase1_iters = nullptr,
                                int *phase2_iters = nullptr);
// Mixed-precision CG (FP64 reliable updates) on nsys independent systems of any sizes,
// staggered-normal or Laplace kinds, advanced together (cg_batch.cu).  X[q], B[q]: device fields.
glinalg_status cg_batch_mixed(const glinalg_operator_s *const *ops, int nsys, double2 *const *X,
                              const double2 *const *B, int max_iter, double eps, int precision, double delta,
                              glinalg_info *infos, cudaStream_t st);
// which: 0 CG, 1 BiCGstab, 2 GCR
glinalg_status restart_driver(int which, const glinalg_operator_s *op, double2 *x,
                              const double2 *b, int max_iter, double eps, int restart_freq,
                              const Verb &verb, glinalg_info *info, cudaStream_t st);

// ---- sibling solvers (solvers_more.cu) ----
// A preconditioner of the flexible solvers: kind GLINALG_PRECOND_*, n_step inner iterations
// to rel_res on op (null: the solve's own operator).
struct Precond {
    int kind = GLINALG_PRECOND_IDENTITY;
    int n_step = 0;
    double rel_res = 0.0;
    const glinalg_operator_s *op = nullptr;
    const glinalg_mg_s *mg = nullptr;  // GLINALG_PRECOND_MG
    int level = 0;                     // the level the multigrid preconditioner starts on
};
// One application of the multigrid preconditioner at `level` (mg_precond.cu).
glinalg_status mg_apply(const glinalg_mg_s *mg, int level, double2 *lhs, const double2 *rhs, const Verb &verb,
                        cudaStream_t st);
long mg_level_fine_size(const glinalg_mg_level_s *l);
long mg_level_coarse_size(const glinalg_mg_level_s *l);
glinalg_status cr_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                       double eps, const Verb &verb, glinalg_info *info, cudaStream_t st);
glinalg_status cr_restart_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                               double eps, int restart_freq, const Verb &verb, glinalg_info *info,
                               cudaStream_t st);
glinalg_status minres_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                           double eps, double omega, const Verb &verb, glinalg_info *info, cudaStream_t st);
glinalg_status cr_m_fp64(const glinalg_operator_s *op, double2 *const *X, const double2 *b, int n_shift,
                         int rfc, int max_iter, double eps, const double *shifts, bool worst_first,
                         const Verb &verb, glinalg_info *info, cudaStream_t st);
glinalg_status bicgstab_m_fp64(const glinalg_operator_s *op, double2 *const *X, const double2 *b,
                               int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                               bool worst_first, const Verb &verb, glinalg_info *info, cudaStream_t st);
constexpr int kMaxBicgstabL = 16;
glinalg_status bicgstab_l_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                               double eps, int l, const Verb &verb, glinalg_info *info, cudaStream_t st);
glinalg_status bicgstab_l_restart_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b,
                                       int max_iter, double eps, int restart_freq, int l, const Verb &verb,
                                       glinalg_info *info, cudaStream_t st);
// mode 0: flexibly preconditioned CG; mode 1: variably preconditioned GCR
glinalg_status flex_fp64(int mode, const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                         double eps, const Precond &pc, const Verb &verb, glinalg_info *info, cudaStream_t st);
glinalg_status flex_restart_fp64(int mode, const glinalg_operator_s *op, double2 *x, const double2 *b,
                                 int max_iter, double eps, int restart_freq, const Precond &pc,
                                 const Verb &verb, glinalg_info *info, cudaStream_t st);

// The FP64 CG on the staggered normal operator as one persistent cooperative kernel
// (cg64_fused.cu): whether it serves op (lx a multiple of 32, no shift; GLINALG_FP64_FUSED=0
// turns it off), and the solve.
bool cg64_fused_applies(const glinalg_operator_s *op, double sigma);
glinalg_status cg64_fused(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter, double eps,
                          const Verb &verb, glinalg_info *info, cudaStream_t st, int wait_limit_us = 0);

// FP64 staggered passes with the 1/2 and eta(x) folded into a hopping table H (2 complex per
// site, built by launch_make_hop64 from op's links): out = D in (sign +1) or D^dagger in
// (sign -1), nothing written while *done is set.  Staggered kinds with lx a multiple of 32.
glinalg_status launch_make_hop64(double2 *H, const glinalg_operator_s *op, cudaStream_t st);
glinalg_status launch_stag64(double2 *out, const double2 *in, const double2 *H, const glinalg_operator_s *op,
                             double sign, const int *done, cudaStream_t st);

// Mixed-precision CG with FP64 reliable updates (cg_mixed.cu).  sigma: diagonal shift added to
// the operator (0 for the plain system).  wait_limit_us: glinalg_solver_params::wait_limit_us.
glinalg_status cg_mixed(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                        double eps, int precision, double delta, double sigma, const Verb &verb,
                        glinalg_info *info, cudaStream_t st, int wait_limit_us = 0);

}  // namespace glinalg
