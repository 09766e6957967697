/*
 * inputs.cpp -- the reference tests' input generators, restated for the CPU oracle (TEST
 * INFRASTRUCTURE ONLY: tests, the smoke check and the CPU legs of the benchmark use it; the
 * product never links it).
 *
 * The reference draws every input from one std::mt19937 per program:
 *   - rand_gauge_u1 (u1_utils/u1_utils.cpp:79-87): for each of the 2*lx*ly links in memory
 *     order, U = polar(1, theta) with theta from uniform_real_distribution<>(-pi, pi);
 *   - gauss_gauge_u1 (u1_utils.cpp:92-112): the same with theta from
 *     normal_distribution<>(0, 1/sqrt(beta)) (beta = 0 falls back to rand_gauge_u1);
 *   - rand_trans_u1 (u1_utils.cpp:116-126): lx*ly phases from uniform(-pi, pi);
 *   - gaussian<complex<double>> (generic_vector.h:48-60): complex(dist(g), dist(g)) with
 *     normal_distribution<>(0, 1).  The two arguments' evaluation order is unspecified in
 *     C++; GCC evaluates them right to left, so the imaginary part is drawn first.
 * The distributions are the standard library's (libstdc++), as in the reference, so the same
 * seed gives the same numbers bit for bit.
 */
#include <cmath>
#include <complex>
#include <random>

namespace {
const double kPi = 3.14159265358979323846;
}

struct orc_rng_s {
    std::mt19937 gen;
    explicit orc_rng_s(unsigned seed) : gen(seed) {}
};

extern "C" {

orc_rng_s *orc_rng_create(unsigned seed) { return new orc_rng_s(seed); }

void orc_rng_destroy(orc_rng_s *g) { delete g; }

void orc_rng_gauge_u1(orc_rng_s *g, double *links, int lx, int ly)
{
    std::uniform_real_distribution<> dist(-kPi, kPi);
    std::complex<double> *U = reinterpret_cast<std::complex<double> *>(links);
    const long n = 2L * lx * ly;
    for (long i = 0; i < n; i++) U[i] = std::polar(1.0, dist(g->gen));
}

void orc_rng_gauss_gauge_u1(orc_rng_s *g, double *links, int lx, int ly, double beta)
{
    if (beta < 0) beta = -beta;
    if (beta == 0) {
        orc_rng_gauge_u1(g, links, lx, ly);
        return;
    }
    std::normal_distribution<> dist(0.0, 1.0 / std::sqrt(beta));
    std::complex<double> *U = reinterpret_cast<std::complex<double> *>(links);
    const long n = 2L * lx * ly;
    for (long i = 0; i < n; i++) U[i] = std::polar(1.0, dist(g->gen));
}

void orc_rng_trans_u1(orc_rng_s *g, double *trans, int lx, int ly)
{
    std::uniform_real_distribution<> dist(-kPi, kPi);
    std::complex<double> *t = reinterpret_cast<std::complex<double> *>(trans);
    const long n = (long)lx * ly;
    for (long i = 0; i < n; i++) t[i] = std::polar(1.0, dist(g->gen));
}

void orc_rng_gaussian(orc_rng_s *g, double *v, long n_complex)
{
    std::normal_distribution<> dist(0.0, 1.0);
    for (long i = 0; i < n_complex; i++) {
        const double im = dist(g->gen);
        const double re = dist(g->gen);
        v[2 * i] = re;
        v[2 * i + 1] = im;
    }
}

}  // extern "C"
