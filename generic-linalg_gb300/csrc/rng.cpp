// rng.cpp -- host-side input generators with the reference tests' streams: one
// std::mt19937 per generator, U(1) links from std::uniform_real_distribution(-pi, pi)
// (rand_gauge_u1, u1_utils.cpp:79-87) or std::normal_distribution(0, 1/sqrt(beta))
// (gauss_gauge_u1, u1_utils.cpp:92-112), Gaussian fields from std::normal_distribution(0,1)
// drawn re then im (gaussian<complex>, generic_vector.h:48-60).  Using the same standard
// library distributions as the reference's tests gives the same numbers from the same seed.

#include <cmath>
#include <complex>
#include <random>

#include "glinalg.h"

struct glinalg_rng_s {
    std::mt19937 gen;
    explicit glinalg_rng_s(uint32_t seed) : gen(seed) {}
};

namespace {
const double kPi = 3.14159265358979323846;
}

extern "C" glinalg_status glinalg_rng_create(uint32_t seed, glinalg_rng *out)
{
    if (!out) return GLINALG_ERROR_INVALID_VALUE;
    *out = new glinalg_rng_s(seed);
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_rng_destroy(glinalg_rng rng)
{
    delete rng;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_rng_gauge_u1(glinalg_rng rng, double *links, int lx, int ly)
{
    if (!rng || !links || lx <= 0 || ly <= 0) return GLINALG_ERROR_INVALID_VALUE;
    std::uniform_real_distribution<> dist(-kPi, kPi);
    std::complex<double> *U = reinterpret_cast<std::complex<double> *>(links);
    for (long i = 0; i < 2L * lx * ly; i++) U[i] = std::polar(1.0, dist(rng->gen));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_rng_gauss_gauge_u1(glinalg_rng rng, double *links, int lx, int ly,
                                                     double beta)
{
    if (!rng || !links || lx <= 0 || ly <= 0) return GLINALG_ERROR_INVALID_VALUE;
    if (beta < 0) beta = -beta;
    if (beta == 0) return glinalg_rng_gauge_u1(rng, links, lx, ly);
    std::normal_distribution<> dist(0.0, 1.0 / std::sqrt(beta));
    std::complex<double> *U = reinterpret_cast<std::complex<double> *>(links);
    for (long i = 0; i < 2L * lx * ly; i++) U[i] = std::polar(1.0, dist(rng->gen));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_rng_gaussian(glinalg_rng rng, double *v, long n_complex)
{
    if (!rng || !v || n_complex < 0) return GLINALG_ERROR_INVALID_VALUE;
    std::normal_distribution<> dist(0.0, 1.0);
    // The reference writes complex<T>(dist(g), dist(g)) (generic_vector.h:58); the order in
    // which the two arguments are evaluated is unspecified in C++, and GCC evaluates them
    // right to left, so the imaginary part is drawn first.  Drawing in that order here
    // reproduces the fields of the reference's tests as built by GCC.
    for (long i = 0; i < n_complex; i++) {
        const double im = dist(rng->gen);
        const double re = dist(rng->gen);
        v[2 * i] = re;
        v[2 * i + 1] = im;
    }
    return GLINALG_SUCCESS;
}

// rand_trans_u1 (u1_utils.cpp:116-126): lx*ly phases uniform in (-pi, pi).
extern "C" glinalg_status glinalg_rng_trans_u1(glinalg_rng rng, double *trans, int lx, int ly)
{
    if (!rng || !trans || lx <= 0 || ly <= 0) return GLINALG_ERROR_INVALID_VALUE;
    std::uniform_real_distribution<> dist(-kPi, kPi);
    std::complex<double> *g = reinterpret_cast<std::complex<double> *>(trans);
    for (long i = 0; i < (long)lx * ly; i++) g[i] = std::polar(1.0, dist(rng->gen));
    return GLINALG_SUCCESS;
}
