// eoprec.cu -- even/odd preconditioning of the staggered operator M = m + D_stag: the pieces
// D_eo and D_oe, the even-site operator m^2 - D_eo D_oe (function and stencil forms), and the
// prepare / reconstruct steps of an even/odd solve of M x = b.
//
// On an even-only field, D^dagger D = m^2 - D_eo D_oe - D_oe D_eo reduces to m^2 - D_eo D_oe, so
// CG on the even system converges like CG on one parity block of D^dagger D, on the same field
// layout (site i = y*lx + x; odd sites carry zeros).  Site parity: even when x + y is even
// (lattice/lattice.h:128-139).  The per-site arithmetic follows the reference's order, so
// results agree with it to rounding (FMA contraction) only.
#include "operator.h"
#include "sites.cuh"
#include "solver_util.h"

namespace glinalg {

namespace {

__device__ __forceinline__ bool site_even(long i, int lx)
{
    const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
    return ((x + y) & 1) == 0;
}

// square_staggered_deo_u1 (odd = 0) / square_staggered_doe_u1 (odd = 1), operators.cpp:455-541:
// the hopping part of square_staggered_u1 at the sites of one parity, zero at the others.
__global__ void k_stag_parity(double2 *__restrict__ out, const double2 *__restrict__ in,
                              const double2 *__restrict__ U, int lx, int ly, int odd,
                              const int *__restrict__ done)
{
    if (done && *done) return;
    const long vol = (long)lx * ly;
    auto ld = [in](long j) { return in[j]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x)
        out[i] = (site_even(i, lx) == (odd == 0)) ? stag_hop_site(ld, U, lx, ly, +1.0, i) : cmk(0.0, 0.0);
}

// The second half of square_staggered_m2mdeodoe_u1 (operators.cpp:578-586): on even sites
// out = m*m in - D_eo tmp (tmp = D_oe in), zero on odd sites.
__global__ void k_m2m_even(double2 *__restrict__ out, const double2 *__restrict__ in,
                           const double2 *__restrict__ tmp, const double2 *__restrict__ U, double m2, int lx,
                           int ly, const int *__restrict__ done)
{
    if (done && *done) return;
    const long vol = (long)lx * ly;
    auto ld = [tmp](long j) { return tmp[j]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x)
        out[i] = site_even(i, lx) ? csub(cscale(m2, in[i]), stag_hop_site(ld, U, lx, ly, +1.0, i)) : cmk(0.0, 0.0);
}

// square_staggered_eoprec_prepare (operators.cpp:543-563): on even sites
// rhs_e = m rhs - D_eo rhs, zero on odd sites.
__global__ void k_eo_prepare(double2 *__restrict__ rhs_e, const double2 *__restrict__ rhs,
                             const double2 *__restrict__ U, double mass, int lx, int ly)
{
    const long vol = (long)lx * ly;
    auto ld = [rhs](long j) { return rhs[j]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x)
        rhs_e[i] = site_even(i, lx) ? csub(cscale(mass, rhs[i]), stag_hop_site(ld, U, lx, ly, +1.0, i)) : cmk(0.0, 0.0);
}

// square_staggered_eoprec_reconstruct (operators.cpp:592-620): on odd sites
// full = inv_mass (rhs_o - D_oe lhs_e), on even sites full = lhs_e.
__global__ void k_eo_reconstruct(double2 *__restrict__ full, const double2 *__restrict__ lhs_e,
                                 const double2 *__restrict__ rhs_o, const double2 *__restrict__ U,
                                 double inv_mass, int lx, int ly)
{
    const long vol = (long)lx * ly;
    auto ld = [lhs_e](long j) { return lhs_e[j]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x)
        full[i] = site_even(i, lx) ? lhs_e[i]
                                   : cscale(inv_mass, csub(rhs_o[i], stag_hop_site(ld, U, lx, ly, +1.0, i)));
}

// The pointwise steps of the stencil forms (operators_stencil.cpp:179-236), after an
// apply_stencil_2d_eo / _oe pass left its result in out:
//   mode 0 (prepare, m2mdeodoe): even sites out = coef b - out (odd sites are already zero);
//   mode 1 (reconstruct): odd sites out = inv (b - out), even sites out = a.
__global__ void k_eo_combine(double2 *__restrict__ out, const double2 *__restrict__ a,
                             const double2 *__restrict__ b, double2 coef, double inv, int lx, int ly, int mode,
                             const int *__restrict__ done)
{
    if (done && *done) return;
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x) {
        const bool even = site_even(i, lx);
        if (mode == 0) {
            if (even) out[i] = csub(cmul(coef, b[i]), out[i]);
        } else {
            out[i] = even ? a[i] : cscale(inv, csub(b[i], out[i]));
        }
    }
}

// Copies the even sites of `in` and zeroes the odd ones.
__global__ void k_even_part(double2 *__restrict__ out, const double2 *__restrict__ in, int lx, int ly)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x)
        out[i] = site_even(i, lx) ? in[i] : cmk(0.0, 0.0);
}

// x = x_e on even sites; odd sites keep x.
__global__ void k_even_into(double2 *__restrict__ x, const double2 *__restrict__ xe, int lx, int ly)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x)
        if (site_even(i, lx)) x[i] = xe[i];
}

int eo_grid(long n)
{
    const long b = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// shift * shift as the reference forms it (std::complex product, operators_stencil.cpp:211)
double2 shift_squared(double2 s) { return cmk(s.x * s.x - s.y * s.y, s.x * s.y + s.y * s.x); }

}  // namespace

glinalg_status launch_eo_apply(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs, double2 *tmp,
                               const int *done, cudaStream_t st)
{
    const int g = eo_grid(op->vol);
    switch (op->kind) {
    case GLINALG_OP_STAGGERED_DEO:
    case GLINALG_OP_STAGGERED_DOE:
        k_stag_parity<<<g, 256, 0, st>>>(lhs, rhs, op->U, op->lx, op->ly,
                                         op->kind == GLINALG_OP_STAGGERED_DOE ? 1 : 0, done);
        break;
    case GLINALG_OP_STAGGERED_M2MDEODOE:
        if (!tmp) return GLINALG_ERROR_INTERNAL;
        k_stag_parity<<<g, 256, 0, st>>>(tmp, rhs, op->U, op->lx, op->ly, 1, done);
        k_m2m_even<<<g, 256, 0, st>>>(lhs, rhs, tmp, op->U, op->mass * op->mass, op->lx, op->ly, done);
        break;
    case GLINALG_OP_STENCIL_M2MDEODOE:
        if (!tmp) return GLINALG_ERROR_INTERNAL;
        GL_TRY(launch_stencil_parity(op, tmp, rhs, 2, done, st));
        GL_TRY(launch_stencil_parity(op, lhs, tmp, 1, done, st));
        k_eo_combine<<<g, 256, 0, st>>>(lhs, nullptr, rhs, shift_squared(op->shift), 0.0, op->lx, op->ly, 0, done);
        break;
    default: return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_eo_prepare(const glinalg_operator_s *op, double2 *rhs_e, const double2 *rhs, cudaStream_t st)
{
    const int g = eo_grid(op->vol);
    if (op->kind == GLINALG_OP_STAGGERED_M2MDEODOE) {
        k_eo_prepare<<<g, 256, 0, st>>>(rhs_e, rhs, op->U, op->mass, op->lx, op->ly);
    } else if (op->kind == GLINALG_OP_STENCIL_M2MDEODOE) {
        GL_TRY(launch_stencil_parity(op, rhs_e, rhs, 1, nullptr, st));
        k_eo_combine<<<g, 256, 0, st>>>(rhs_e, nullptr, rhs, op->shift, 0.0, op->lx, op->ly, 0, nullptr);
    } else {
        set_last_error("even/odd preconditioning needs an m^2 - D_eo D_oe operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_eo_reconstruct(const glinalg_operator_s *op, double2 *full, const double2 *lhs_e,
                                     const double2 *rhs_o, cudaStream_t st)
{
    const int g = eo_grid(op->vol);
    if (op->kind == GLINALG_OP_STAGGERED_M2MDEODOE) {
        k_eo_reconstruct<<<g, 256, 0, st>>>(full, lhs_e, rhs_o, op->U, 1.0 / op->mass, op->lx, op->ly);
    } else if (op->kind == GLINALG_OP_STENCIL_M2MDEODOE) {
        GL_TRY(launch_stencil_parity(op, full, lhs_e, 2, nullptr, st));
        k_eo_combine<<<g, 256, 0, st>>>(full, lhs_e, rhs_o, cmk(0.0, 0.0), 1.0 / op->shift.x, op->lx, op->ly, 1,
                                        nullptr);
    } else {
        set_last_error("even/odd preconditioning needs an m^2 - D_eo D_oe operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_even_part(const glinalg_operator_s *op, double2 *out, const double2 *in, cudaStream_t st)
{
    k_even_part<<<eo_grid(op->vol), 256, 0, st>>>(out, in, op->lx, op->ly);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_even_into(const glinalg_operator_s *op, double2 *x, const double2 *xe, cudaStream_t st)
{
    k_even_into<<<eo_grid(op->vol), 256, 0, st>>>(x, xe, op->lx, op->ly);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

}  // namespace glinalg

using namespace glinalg;

// The C-ABI steps: fields staged to the device when they are host pointers.
static glinalg_status eo_step(glinalg_operator op, double *out, const double *a, const double *b, int flags,
                              bool reconstruct)
{
    if (!op || !out || !a || (reconstruct && !b))
        return invalid_arg("!op || !out || !a || (reconstruct && !b)");
    const bool tb = op->kind == GLINALG_OP_STENCIL_M2MDTBDBT;
    if (op->kind != GLINALG_OP_STAGGERED_M2MDEODOE && op->kind != GLINALG_OP_STENCIL_M2MDEODOE && !tb) {
        set_last_error("even/odd preconditioning needs an m^2 - D_eo D_oe operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    const bool dev = flags & GLINALG_PTR_DEVICE;
    const long n = op->size;
    const size_t bytes = sizeof(double2) * (size_t)n;
    Scratch sc(st);
    double2 *d_out = (double2 *)out, *d_a = (double2 *)a, *d_b = (double2 *)b;
    if (!dev) {
        GL_TRY(sc.alloc(&d_out, n));
        GL_TRY(sc.alloc(&d_a, n));
        GL_CUDA(cudaMemcpyAsync(d_a, a, bytes, cudaMemcpyHostToDevice, st));
        if (reconstruct) {
            GL_TRY(sc.alloc(&d_b, n));
            GL_CUDA(cudaMemcpyAsync(d_b, b, bytes, cudaMemcpyHostToDevice, st));
        }
    }
    if (tb) {
        if (reconstruct) GL_TRY(launch_tb_reconstruct(op, d_out, d_a, d_b, st));
        else GL_TRY(launch_tb_prepare(op, d_out, d_a, st));
    } else {
        if (reconstruct) GL_TRY(launch_eo_reconstruct(op, d_out, d_a, d_b, st));
        else GL_TRY(launch_eo_prepare(op, d_out, d_a, st));
    }
    if (!dev) GL_CUDA(cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_eoprec_prepare(glinalg_operator op, double *rhs_e, const double *rhs, int flags)
{
    return eo_step(op, rhs_e, rhs, nullptr, flags, false);
}

extern "C" glinalg_status glinalg_eoprec_reconstruct(glinalg_operator op, double *lhs_full, const double *lhs_e,
                                                     const double *rhs_o, int flags)
{
    return eo_step(op, lhs_full, lhs_e, rhs_o, flags, true);
}

extern "C" glinalg_status glinalg_tbprec_prepare(glinalg_operator op, double *rhs_t, const double *rhs, int flags)
{
    if (op && op->kind != GLINALG_OP_STENCIL_M2MDTBDBT) {
        set_last_error("top/bottom preconditioning needs an m^2 - D_tb D_bt stencil operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    return eo_step(op, rhs_t, rhs, nullptr, flags, false);
}

extern "C" glinalg_status glinalg_tbprec_reconstruct(glinalg_operator op, double *lhs_full, const double *lhs_t,
                                                     const double *rhs_b, int flags)
{
    if (op && op->kind != GLINALG_OP_STENCIL_M2MDTBDBT) {
        set_last_error("top/bottom preconditioning needs an m^2 - D_tb D_bt stencil operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    return eo_step(op, lhs_full, lhs_t, rhs_b, flags, true);
}
