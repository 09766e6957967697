// gauge.cu -- U(1) gauge-field utilities of u1_utils.cpp: the text file format
// (read_gauge_u1 / write_gauge_u1, :17-65), the unit field (:69-75), random gauge transforms
// (rand_trans_u1 / apply_gauge_trans_u1, :116-142), APE smearing (:145-187), the average
// plaquette (:190-207) and the topological charge (:210-226).
//
// Links use the operators' layout U[2*i + mu], site i = y*lx + x.  The file format, as the
// reference writes it, lists the phase arg(U) of every link with x outermost, then y, then mu,
// one number per line in fixed notation with 20 decimals.  File work runs on the host; the
// per-link arithmetic runs on the device, one thread per site.

#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "operator.h"
#include "solver_util.h"

namespace glinalg {

namespace {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ double2 polar1(double th)
{
    double s, c;
    sincos(th, &s, &c);
    return make_double2(c, s);
}

// sum over sites of w = U_x(x) U_y(x+x) U_x(x+y)^* U_y(x)^* (both components) and of arg(w),
// each product formed left to right as in get_plaquette_u1 / get_topo_u1
__global__ void __launch_bounds__(kRedThreads)
k_plaquette(const double2 *__restrict__ U, int lx, int ly, double *partials, unsigned *counter, double *out3)
{
    const long vol = (long)lx * ly;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < vol; i += (long)gridDim.x * kRedThreads) {
        const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
        const int xp = x + 1 == lx ? 0 : x + 1, yp = y + 1 == ly ? 0 : y + 1;
        const double2 w = cmul(cmul(cmul(U[2 * i], U[2 * ((long)y * lx + xp) + 1]), cconj(U[2 * ((long)yp * lx + x)])),
                               cconj(U[2 * i + 1]));
        v[0] += w.x;
        v[1] += w.y;
        v[2] += atan2(w.y, w.x);
    }
    if (grid_sum<3, kRedThreads>(v, partials, counter) && threadIdx.x == 0) {
        out3[0] = v[0];
        out3[1] = v[1];
        out3[2] = v[2];
    }
}

// U_mu(x) = g(x) U_mu(x) g(x + mu)^* (apply_gauge_trans_u1)
__global__ void k_gauge_trans(double2 *__restrict__ U, const double2 *__restrict__ g, int lx, int ly)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x) {
        const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
        const int xp = x + 1 == lx ? 0 : x + 1, yp = y + 1 == ly ? 0 : y + 1;
        const double2 gi = g[i];
        U[2 * i] = cmul(cmul(gi, U[2 * i]), cconj(g[(long)y * lx + xp]));
        U[2 * i + 1] = cmul(cmul(gi, U[2 * i + 1]), cconj(g[(long)yp * lx + x]));
    }
}

// One APE sweep: S = T + alpha (staple) + alpha (staple) per link with the reference's
// products (apply_ape_smear_u1, :161-171), then out = polar(1, arg(S)) (:175-178).
__global__ void k_ape_sweep(double2 *__restrict__ out, const double2 *__restrict__ T, int lx, int ly, double alpha)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x) {
        const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
        const int xp = x + 1 == lx ? 0 : x + 1, yp = y + 1 == ly ? 0 : y + 1;
        const int xm = x == 0 ? lx - 1 : x - 1, ym = y == 0 ? ly - 1 : y - 1;
        auto L = [&](int xx, int yy, int mu) { return T[2 * ((long)yy * lx + xx) + mu]; };
        double2 v = L(x, y, 0);
        v = cadd(v, cmul(cmul(cscale(alpha, L(x, y, 1)), L(x, yp, 0)), cconj(L(xp, y, 1))));
        v = cadd(v, cmul(cmul(cscale(alpha, cconj(L(x, ym, 1))), L(x, ym, 0)), L(xp, ym, 1)));
        out[2 * i] = polar1(atan2(v.y, v.x));
        v = L(x, y, 1);
        v = cadd(v, cmul(cmul(cscale(alpha, cconj(L(xm, y, 0))), L(xm, y, 1)), L(xm, yp, 0)));
        v = cadd(v, cmul(cmul(cscale(alpha, L(x, y, 0)), L(xp, y, 1)), cconj(L(x, yp, 0))));
        out[2 * i + 1] = polar1(atan2(v.y, v.x));
    }
}

__global__ void k_fill_one(double2 *__restrict__ U, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        U[i] = make_double2(1.0, 0.0);
}

int grid_for(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

glinalg_status check_lattice(const void *p, int lx, int ly)
{
    if (!p || lx <= 0 || ly <= 0) {
        set_last_error("null field or non-positive lattice extent");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return GLINALG_SUCCESS;
}

// Device copy of a field given by the caller (host pointers are staged, device pointers used).
glinalg_status stage_in(Scratch &sc, const double *src, long n_complex, bool dev, double2 **out, cudaStream_t st)
{
    if (dev) {
        *out = (double2 *)src;
        return GLINALG_SUCCESS;
    }
    GL_TRY(sc.alloc(out, n_complex));
    GL_CUDA(cudaMemcpyAsync(*out, src, sizeof(double2) * n_complex, cudaMemcpyHostToDevice, st));
    return GLINALG_SUCCESS;
}

glinalg_status plaq_sums(const double *links, int lx, int ly, int flags, double sums[3])
{
    GL_TRY(check_lattice(links, lx, ly));
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long vol = (long)lx * ly;
    double2 *U;
    GL_TRY(stage_in(sc, links, 2 * vol, flags & GLINALG_PTR_DEVICE, &U, st));
    double *partials, *out;
    unsigned *cnt;
    GL_TRY(sc.alloc(&partials, 3 * (size_t)reduction_blocks(vol)));
    GL_TRY(sc.zeros(&cnt, 1));
    GL_TRY(sc.alloc(&out, 3));
    k_plaquette<<<reduction_blocks(vol), kRedThreads, 0, st>>>(U, lx, ly, partials, cnt, out);
    GL_CUDA(cudaGetLastError());
    GL_CUDA(cudaMemcpyAsync(sums, out, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

}  // namespace

}  // namespace glinalg

using namespace glinalg;

extern "C" glinalg_status glinalg_read_gauge_u1(double *links, int lx, int ly, const char *path)
{
    GL_TRY(check_lattice(links, lx, ly));
    if (!path) return invalid_arg("!path");
    std::ifstream in(path);
    if (!in) {
        set_last_error(std::string("cannot open ") + path);
        return GLINALG_ERROR_INVALID_VALUE;
    }
    std::complex<double> *U = reinterpret_cast<std::complex<double> *>(links);
    for (int x = 0; x < lx; x++)
        for (int y = 0; y < ly; y++)
            for (int mu = 0; mu < 2; mu++) {
                double ph;
                if (!(in >> ph)) {
                    set_last_error(std::string(path) + ": fewer than 2*lx*ly phases");
                    return GLINALG_ERROR_INVALID_VALUE;
                }
                U[(long)y * 2 * lx + x * 2 + mu] = std::polar(1.0, ph);
            }
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_write_gauge_u1(const double *links, int lx, int ly, const char *path)
{
    GL_TRY(check_lattice(links, lx, ly));
    if (!path) return invalid_arg("!path");
    FILE *f = std::fopen(path, "w");
    if (!f) {
        set_last_error(std::string("cannot write ") + path);
        return GLINALG_ERROR_INVALID_VALUE;
    }
    const std::complex<double> *U = reinterpret_cast<const std::complex<double> *>(links);
    for (int x = 0; x < lx; x++)
        for (int y = 0; y < ly; y++)
            for (int mu = 0; mu < 2; mu++) std::fprintf(f, "%.20f\n", std::arg(U[(long)y * 2 * lx + x * 2 + mu]));
    if (std::fclose(f) != 0) {
        set_last_error(std::string("error writing ") + path);
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_unit_gauge_u1(double *links, int lx, int ly, int flags)
{
    GL_TRY(check_lattice(links, lx, ly));
    const long n = 2L * lx * ly;
    if (!(flags & GLINALG_PTR_DEVICE)) {
        for (long i = 0; i < n; i++) {
            links[2 * i] = 1.0;
            links[2 * i + 1] = 0.0;
        }
        return GLINALG_SUCCESS;
    }
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    k_fill_one<<<grid_for(n), 256, 0, st>>>((double2 *)links, n);
    GL_CUDA(cudaGetLastError());
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_plaquette_u1(const double *links, int lx, int ly, double out[2], int flags)
{
    if (!out) return invalid_arg("!out");
    double s[3];
    GL_TRY(plaq_sums(links, lx, ly, flags, s));
    const double v = (double)((long)lx * ly);
    out[0] = s[0] / v;
    out[1] = s[1] / v;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_topo_u1(const double *links, int lx, int ly, double *out, int flags)
{
    if (!out) return invalid_arg("!out");
    double s[3];
    GL_TRY(plaq_sums(links, lx, ly, flags, s));
    *out = 0.5 * s[2] / kPi;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_apply_gauge_trans_u1(double *links, const double *trans, int lx, int ly, int flags)
{
    GL_TRY(check_lattice(links, lx, ly));
    if (!trans) return invalid_arg("!trans");
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long vol = (long)lx * ly;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    double2 *U, *g;
    GL_TRY(stage_in(sc, links, 2 * vol, dev, &U, st));
    GL_TRY(stage_in(sc, trans, vol, dev, &g, st));
    k_gauge_trans<<<grid_for(vol), 256, 0, st>>>(U, g, lx, ly);
    GL_CUDA(cudaGetLastError());
    if (!dev) GL_CUDA(cudaMemcpyAsync(links, U, sizeof(double2) * 2 * vol, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_apply_ape_smear_u1(double *smeared, const double *links, int lx, int ly,
                                                     double alpha, int n_iter, int flags)
{
    GL_TRY(check_lattice(links, lx, ly));
    if (!smeared || n_iter < 0) return invalid_arg("!smeared || n_iter < 0");
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long vol = (long)lx * ly;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    double2 *a, *b;
    GL_TRY(sc.alloc(&a, 2 * vol));
    GL_TRY(sc.alloc(&b, 2 * vol));
    GL_CUDA(cudaMemcpyAsync(a, links, sizeof(double2) * 2 * vol,
                            dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    for (int it = 0; it < n_iter; it++) {
        k_ape_sweep<<<grid_for(vol), 256, 0, st>>>(b, a, lx, ly, alpha);
        std::swap(a, b);
    }
    GL_CUDA(cudaGetLastError());
    GL_CUDA(cudaMemcpyAsync(smeared, a, sizeof(double2) * 2 * vol,
                            dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}
