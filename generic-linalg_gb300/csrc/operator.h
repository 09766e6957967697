// operator.h -- the device-resident operator object behind glinalg_operator and the
// launchers of its kernels.
#pragma once

#include "common.cuh"

struct glinalg_operator_s {
    int kind = 0;
    int lx = 0, ly = 0, nc = 1;
    double mass = 0.0;
    long vol = 0;   // lx*ly sites
    long size = 0;  // complex entries of a field (vol * nc)
    int device = 0;

    // FP64 device copies of the reference's data.
    double2 *U = nullptr;         // links, U[2*i+mu]
    double2 *clover = nullptr;    // stencil kinds
    double2 *hopping = nullptr;
    double2 *two_link = nullptr;
    double2 shift{0, 0}, eo_shift{0, 0}, dof_shift{0, 0};

    ~glinalg_operator_s();
};

namespace glinalg {

bool is_staggered(int kind);
bool is_stencil(int kind);     // kinds described by a stencil_2d (clover, hopping, shifts)
bool is_hermitian(int kind);   // D^dagger D, the gauge Laplacian, m^2 - D_eo D_oe
bool needs_tmp(int kind);      // two-pass kinds: launch_apply needs a scratch field

// lhs = A rhs on `stream` (device pointers).  tmp: a scratch field of op->size entries for
// the normal operator (may be null for other kinds).  done: optional device flag; when it
// points at a non-zero value the kernels return without writing (used inside solver loops).
glinalg_status launch_apply(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs,
                            double2 *tmp, const int *done, cudaStream_t stream);

// lhs = (A + sigma) rhs, optionally skipped when *done is set.
glinalg_status launch_apply_sigma(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs,
                                  double2 *tmp, double sigma, const int *done, cudaStream_t stream);
// lhs = (A + sigma) rhs.
glinalg_status launch_apply_shifted(const glinalg_operator_s *op, double2 *lhs,
                                    const double2 *rhs, double2 *tmp, double sigma,
                                    cudaStream_t stream);

// apply_stencil_2d (parity 0), _eo (1), _oe (2), _tb (3) or _bt (4) of a stencil-described
// operator.  With comb_r, out = (comb_s2 comb_r - out) - (the stencil applied to in).
glinalg_status launch_stencil_parity(const glinalg_operator_s *op, double2 *out, const double2 *in, int parity,
                                     const int *done, cudaStream_t stream, const double2 *comb_r = nullptr,
                                     double2 comb_s2 = double2{0.0, 0.0});

// Even/odd preconditioning (eoprec.cu): D_eo, D_oe and m^2 - D_eo D_oe applied; the prepare and
// reconstruct steps; the even part of a field; x = x_e on even sites.
glinalg_status launch_eo_apply(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs, double2 *tmp,
                               const int *done, cudaStream_t stream);
glinalg_status launch_eo_prepare(const glinalg_operator_s *op, double2 *rhs_e, const double2 *rhs,
                                 cudaStream_t stream);
glinalg_status launch_eo_reconstruct(const glinalg_operator_s *op, double2 *full, const double2 *lhs_e,
                                     const double2 *rhs_o, cudaStream_t stream);
glinalg_status launch_even_part(const glinalg_operator_s *op, double2 *out, const double2 *in,
                                cudaStream_t stream);
glinalg_status launch_even_into(const glinalg_operator_s *op, double2 *x, const double2 *xe,
                                cudaStream_t stream);

// The coarse-level stencil operators of the multigrid code (coarse_ops.cu): m^2 - D_tb D_bt,
// the normal_eo / normal_tb and dagger_eo / dagger_tb forms; tmp: one scratch field.
glinalg_status launch_coarse_piece(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs, double2 *tmp,
                                   const int *done, cudaStream_t stream);
glinalg_status launch_tb_prepare(const glinalg_operator_s *op, double2 *rhs_t, const double2 *rhs,
                                 cudaStream_t stream);
glinalg_status launch_tb_reconstruct(const glinalg_operator_s *op, double2 *full, const double2 *lhs_t,
                                     const double2 *rhs_b, cudaStream_t stream);

// Staggered-only pieces (used by the force and by the fused solver kernels).
glinalg_status launch_staggered(const glinalg_operator_s *op, double2 *out, const double2 *in,
                                double sign, const int *done, cudaStream_t stream);

// The library's stream on the current device and its device-side scratch allocator.
cudaStream_t lib_stream();
// Stream-ordered allocation from the library's memory pool of the current device (freed with
// cudaFreeAsync; the pool keeps freed memory for the next call).
cudaError_t lib_malloc_async(void **p, size_t bytes, cudaStream_t st);
void set_user_stream(cudaStream_t s, bool use);
// A private stream of the current device used only to capture CUDA graphs.
cudaStream_t capture_stream();
glinalg_status ensure_device();

// Bytes an application of the operator moves (algorithmic), for info->gbytes.
double apply_bytes(const glinalg_operator_s *op);

}  // namespace glinalg
