// coarse_ops.cu -- the stencil operators of the multigrid code on a coarse level
// (multigrid/aa_mg/mg_complex.cpp:1211-1375), built from the top/bottom stencil passes
// (apply_stencil_2d_tb / _bt, coarse_stencil.cpp:725 / :1120).  The colours of a coarse site
// split into a top half (colour < nc/2) and a bottom half; for a staggered fine operator
// they play the role the even and odd sites play on the fine lattice.  m is the stencil's
// complex shift, squared as the reference's std::complex product.
#include "operator.h"

namespace glinalg {

namespace {

// top / bottom colour of element i (site-major, colour fastest)
__device__ __forceinline__ bool is_top(long i, int nc) { return (int)(i % nc) < nc / 2; }

// mode 0: top elements out = coef b - out (bottom ones are left as the tb pass made them, zero);
// mode 1: bottom elements out = inv (b - out), top elements out = a
__global__ void k_tb_combine(double2 *__restrict__ out, const double2 *__restrict__ a,
                             const double2 *__restrict__ b, double2 coef, double inv, long n, int nc, int mode,
                             const int *__restrict__ done)
{
    if (done && *done) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const bool top = is_top(i, nc);
        if (mode == 0) {
            if (top) out[i] = csub(cmul(coef, b[i]), out[i]);
        } else {
            out[i] = top ? a[i] : cscale(inv, csub(b[i], out[i]));
        }
    }
}

// lattice_epsilon (eo = 1: -1 on odd sites) or lattice_sigma3 (eo = 0: -1 on the bottom colours
// when nc is even), lattice/lattice_functions.h:11-55; in place allowed
__global__ void k_sign(double2 *__restrict__ out, const double2 *__restrict__ in, int lx, int nc, long n, int eo,
                       const int *__restrict__ done)
{
    if (done && *done) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        bool plus;
        if (eo) {
            const long site = i / nc;
            const int y = (int)(site / lx), x = (int)(site - (long)y * lx);
            plus = ((x + y) & 1) == 0;
        } else {
            plus = (nc & 1) || is_top(i, nc);
        }
        const double2 v = in[i];
        out[i] = plus ? v : cneg(v);
    }
}

int grid(long n)
{
    const long b = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

double2 shift_sq(double2 s) { return cmk(s.x * s.x - s.y * s.y, s.x * s.y + s.y * s.x); }

}  // namespace

glinalg_status launch_coarse_piece(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs, double2 *tmp,
                                   const int *done, cudaStream_t st)
{
    if (!tmp) return GLINALG_ERROR_INTERNAL;
    const long n = op->size;
    const int g = grid(n);
    switch (op->kind) {
    case GLINALG_OP_STENCIL_M2MDTBDBT:  // mg_complex.cpp:1228-1249
        GL_TRY(launch_stencil_parity(op, tmp, rhs, 4, done, st));
        GL_TRY(launch_stencil_parity(op, lhs, tmp, 3, done, st));
        k_tb_combine<<<g, 256, 0, st>>>(lhs, nullptr, rhs, shift_sq(op->shift), 0.0, n, op->nc, 0, done);
        break;
    case GLINALG_OP_STENCIL_NORMAL_EO:  // mg_complex.cpp:1277-1302
    case GLINALG_OP_STENCIL_NORMAL_TB: {  // :1305-1330
        const int a = op->kind == GLINALG_OP_STENCIL_NORMAL_EO ? 1 : 3;
        const int b = op->kind == GLINALG_OP_STENCIL_NORMAL_EO ? 2 : 4;
        // lhs = b(a(rhs)); then lhs = (m^2 rhs - lhs) - a(b(rhs))
        GL_TRY(launch_stencil_parity(op, tmp, rhs, a, done, st));
        GL_TRY(launch_stencil_parity(op, lhs, tmp, b, done, st));
        GL_TRY(launch_stencil_parity(op, tmp, rhs, b, done, st));
        GL_TRY(launch_stencil_parity(op, lhs, tmp, a, done, st, rhs, shift_sq(op->shift)));
        break;
    }
    case GLINALG_OP_STENCIL_DAGGER_EO:  // mg_complex.cpp:1335-1352
    case GLINALG_OP_STENCIL_DAGGER_TB: {  // :1355-1372
        const int eo = op->kind == GLINALG_OP_STENCIL_DAGGER_EO;
        k_sign<<<g, 256, 0, st>>>(tmp, rhs, op->lx, op->nc, n, eo, done);
        GL_TRY(launch_stencil_parity(op, lhs, tmp, 0, done, st));
        k_sign<<<g, 256, 0, st>>>(lhs, lhs, op->lx, op->nc, n, eo, done);
        break;
    }
    default: return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

// apply_square_staggered_tbprec_prepare_stencil (mg_complex.cpp:1211-1225)
glinalg_status launch_tb_prepare(const glinalg_operator_s *op, double2 *rhs_t, const double2 *rhs, cudaStream_t st)
{
    GL_TRY(launch_stencil_parity(op, rhs_t, rhs, 3, nullptr, st));
    k_tb_combine<<<grid(op->size), 256, 0, st>>>(rhs_t, nullptr, rhs, op->shift, 0.0, op->size, op->nc, 0, nullptr);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

// apply_square_staggered_tbprec_reconstruct_stencil (mg_complex.cpp:1252-1274)
glinalg_status launch_tb_reconstruct(const glinalg_operator_s *op, double2 *full, const double2 *lhs_t,
                                     const double2 *rhs_b, cudaStream_t st)
{
    GL_TRY(launch_stencil_parity(op, full, lhs_t, 4, nullptr, st));
    k_tb_combine<<<grid(op->size), 256, 0, st>>>(full, lhs_t, rhs_b, cmk(0.0, 0.0), 1.0 / op->shift.x, op->size,
                                                 op->nc, 1, nullptr);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

}  // namespace glinalg
