// sites.cuh -- the FP64 U(1) operators at one site, shared by the single-field kernels and
// the batched solvers so that both compute every site with the same arithmetic.
// `in(j)` returns the input field at site j (a plain load, or a value formed on the fly).
#pragma once

#include "common.cuh"

namespace glinalg {

__device__ __forceinline__ int wrap_p(int v, int n) { return v + 1 == n ? 0 : v + 1; }
__device__ __forceinline__ int wrap_m(int v, int n) { return v == 0 ? n - 1 : v - 1; }

// The hopping part of square_staggered_u1 (sign = +1) / square_staggered_dagger_u1
// (sign = -1) at site i (operators.cpp:207-231, :395-426), which is also
// square_staggered_deo_u1 / _doe_u1 at a site of their parity (operators.cpp:455-541):
// -1/2 sum_mu eta_mu(x) [U_mu(x) psi(x+mu) - U_mu(x-mu)^* psi(x-mu)], eta_x = 1,
// eta_y = (-1)^x, accumulated in the reference's order +x, -x, +y, -y, then halved.
template <class In>
__device__ __forceinline__ double2 stag_hop_site(In in, const double2 *__restrict__ U, int lx, int ly,
                                                 double sign, long i)
{
    const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
    const int xp = wrap_p(x, lx), xm = wrap_m(x, lx), yp = wrap_p(y, ly), ym = wrap_m(y, ly);
    const double eta = (x & 1) ? -1.0 : 1.0;
    const long row = (long)y * lx;
    double2 acc = cmk(0.0, 0.0), t;
    t = cmul(U[2 * i], in(row + xp));
    acc = sign > 0 ? csub(acc, t) : cadd(acc, t);
    t = cmul(cconj(U[2 * (row + xm)]), in(row + xm));
    acc = sign > 0 ? cadd(acc, t) : csub(acc, t);
    t = cmul(cscale(eta, U[2 * i + 1]), in((long)yp * lx + x));
    acc = sign > 0 ? csub(acc, t) : cadd(acc, t);
    t = cmul(cscale(eta, cconj(U[2 * ((long)ym * lx + x) + 1])), in((long)ym * lx + x));
    acc = sign > 0 ? cadd(acc, t) : csub(acc, t);
    return cscale(0.5, acc);
}

// square_staggered_u1 (sign = +1) / square_staggered_dagger_u1 (sign = -1) at site i
// (operators.cpp:184-239, :372-441): the hopping part plus m psi(x); the dagger flips the
// hopping sign and keeps the mass.
template <class In>
__device__ __forceinline__ double2 stag_site(In in, const double2 *__restrict__ U, double mass,
                                             int lx, int ly, double sign, long i)
{
    return cadd(stag_hop_site(in, U, lx, ly, sign, i), cscale(mass, in(i)));
}

// square_laplace_u1 at site i (operators.cpp:73-120): (4 + mass) psi(x)
// - sum_mu [U_mu(x) psi(x+mu) + U_mu(x-mu)^* psi(x-mu)].
template <class In>
__device__ __forceinline__ double2 lap_site(In in, const double2 *__restrict__ U, double mass,
                                            int lx, int ly, long i)
{
    const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
    const int xp = wrap_p(x, lx), xm = wrap_m(x, lx), yp = wrap_p(y, ly), ym = wrap_m(y, ly);
    const long row = (long)y * lx;
    double2 acc = cmk(0.0, 0.0);
    acc = csub(acc, cmul(U[2 * i], in(row + xp)));
    acc = csub(acc, cmul(cconj(U[2 * (row + xm)]), in(row + xm)));
    acc = csub(acc, cmul(U[2 * i + 1], in((long)yp * lx + x)));
    acc = csub(acc, cmul(cconj(U[2 * ((long)ym * lx + x) + 1]), in((long)ym * lx + x)));
    return cadd(acc, cscale(4.0 + mass, in(i)));
}

}  // namespace glinalg
