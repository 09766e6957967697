// force.cu -- adjoint force for S(theta) = phi^dagger (D^dagger D + sigma)^-1 phi with respect
// to the U(1) link angles (U_mu(x) = exp(i theta_mu(x))).  No counterpart in the reference,
// which has no derivatives; the operator conventions are those of square_staggered_u1
// (operators.cpp:184-239).
//
// With X = (D^dagger D + sigma)^-1 phi and Y = D X,
//   dS/dtheta = -X^dagger (dD^dagger D + D^dagger dD) X = -2 Re(Y^dagger dD X).
// U_x(s) enters D in row s as -1/2 U psi(s+x) and in row s+x as +1/2 U^* psi(s); U_y(s) the
// same with eta(s) = (-1)^x.  With dU/dtheta = i U:
//   dS/dtheta_x(s) = -Im( Y(s)^* U X(s+x) + Y(s+x)^* U^* X(s) )
//   dS/dtheta_y(s) = -eta(s) Im( Y(s)^* U X(s+y) + Y(s+y)^* U^* X(s) )
// One thread per site writes both link derivatives of that site: it reads X, Y at the site
// and its +x, +y neighbours and its two links (FP64: 16*(2+4) + 32 = 128 B read, 16 B written).

#include <cmath>
#include <vector>

#include "solvers.h"

namespace glinalg {

__global__ void k_staggered_force(double *__restrict__ grad, const double2 *__restrict__ U,
                                  const double2 *__restrict__ X, const double2 *__restrict__ Y,
                                  int lx, int ly)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x) {
        const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
        const long ixp = (long)y * lx + (x + 1 == lx ? 0 : x + 1);
        const long iyp = (long)(y + 1 == ly ? 0 : y + 1) * lx + x;
        const double eta = (x & 1) ? -1.0 : 1.0;
        const double2 xi = X[i], yi = Y[i];
        const double2 ux = U[2 * i], uy = U[2 * i + 1];
        // Im(conj(a) * u * b) + Im(conj(c) * conj(u) * d)
        const double2 fx = cadd(cmul(cconj(yi), cmul(ux, X[ixp])), cmul(cconj(Y[ixp]), cmul(cconj(ux), xi)));
        const double2 fy = cadd(cmul(cconj(yi), cmul(uy, X[iyp])), cmul(cconj(Y[iyp]), cmul(cconj(uy), xi)));
        grad[2 * i] = -fx.y;
        grad[2 * i + 1] = -eta * fy.y;
    }
}

glinalg_status launch_force(const glinalg_operator_s *op, double *grad, const double2 *X,
                            const double2 *Y, cudaStream_t st)
{
    long g = (op->vol + 255) / 256, cap = (long)sm_count() * 16;
    k_staggered_force<<<(int)(g < 1 ? 1 : (g > cap ? cap : g)), 256, 0, st>>>(grad, op->U, X, Y, op->lx, op->ly);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

}  // namespace glinalg

using namespace glinalg;

extern "C" glinalg_status glinalg_staggered_force(glinalg_operator op, const double *X,
                                                  const double *Y, double *grad, int flags)
{
    if (!op || !X || !Y || !grad) return invalid_arg("!op || !X || !Y || !grad");
    if (!is_staggered(op->kind)) {
        set_last_error("the force needs a staggered operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long n = op->vol;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    const double2 *dX = (const double2 *)X, *dY = (const double2 *)Y;
    double *dg = grad;
    if (!dev) {
        double2 *tx, *ty;
        GL_TRY(sc.alloc(&tx, n));
        GL_TRY(sc.alloc(&ty, n));
        GL_TRY(sc.alloc(&dg, 2 * n));
        GL_CUDA(cudaMemcpyAsync(tx, X, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(ty, Y, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        dX = tx;
        dY = ty;
    }
    GL_TRY(launch_force(op, dg, dX, dY, st));
    if (!dev) GL_CUDA(cudaMemcpyAsync(grad, dg, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_staggered_action_grad(glinalg_operator op, const double *phi,
                                                        double sigma, double eps, int max_iter,
                                                        double *action, double *grad, double *X_out,
                                                        const glinalg_solver_params *params,
                                                        glinalg_info *info)
{
    if (!op || !phi || !grad || !info) return invalid_arg("!op || !phi || !grad || !info");
    if (op->kind != GLINALG_OP_STAGGERED_NORMAL) {
        set_last_error("action_grad needs the staggered normal operator (D^dagger D)");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long n = op->vol;
    const bool dev = params && (params->flags & GLINALG_PTR_DEVICE);
    const int prec = params ? params->precision : GLINALG_PREC_DOUBLE;
    const double delta = params && params->delta > 0 ? params->delta : 0.0;  // 0: the per-precision default
    const double2 *dphi = (const double2 *)phi;
    double2 *X, *Y;
    double *dg = grad;
    if (!dev) {
        double2 *t;
        GL_TRY(sc.alloc(&t, n));
        GL_CUDA(cudaMemcpyAsync(t, phi, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        dphi = t;
        GL_TRY(sc.alloc(&dg, 2 * n));
    }
    if (dev && X_out) X = (double2 *)X_out;
    else GL_TRY(sc.alloc(&X, n));
    GL_TRY(sc.alloc(&Y, n));
    GL_CUDA(cudaMemsetAsync(X, 0, sizeof(double2) * n, st));
    double *keep = info->resSqmrhs;
    *info = glinalg_info{};
    info->resSqmrhs = keep;
    const Verb quiet;
    if (prec == GLINALG_PREC_DOUBLE) GL_TRY(cg_fp64(op, X, dphi, max_iter, eps, quiet, info, st, sigma));
    else GL_TRY(cg_mixed(op, X, dphi, max_iter, eps, prec, delta, sigma, quiet, info, st));
    GL_TRY(launch_staggered(op, Y, X, +1.0, nullptr, st));
    GL_TRY(launch_force(op, dg, X, Y, st));
    // action = Re <phi, X>
    double *partials;
    unsigned *cnt;
    double2 *res;
    GL_TRY(sc.alloc(&partials, 2 * (size_t)reduction_blocks(n)));
    GL_TRY(sc.zeros(&cnt, 1));
    GL_TRY(sc.alloc(&res, 1));
    GL_TRY(launch_dot(dphi, X, n, partials, cnt, res, st));
    double2 hres;
    GL_CUDA(cudaMemcpyAsync(&hres, res, sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (!dev) {
        GL_CUDA(cudaMemcpyAsync(grad, dg, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
        if (X_out) GL_CUDA(cudaMemcpyAsync(X_out, X, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    }
    GL_CUDA(cudaStreamSynchronize(st));
    if (action) *action = hres.x;
    return GLINALG_SUCCESS;
}
