// solver_util.cu -- shared solver plumbing (see solver_util.h), the generic BLAS-1 kernels
// (generic_vector.h:87-169) and the library-level C-ABI entry points.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <mutex>

#include "solver_util.h"

namespace glinalg {

static thread_local std::string t_last_error;
void set_last_error(const std::string &msg) { t_last_error = msg; }

bool use_graphs()
{
    static const bool on = [] {
        const char *e = std::getenv("GLINALG_SOLVER_GRAPHS");
        return !(e && e[0] == '0');
    }();
    return on;
}

__global__ void k_loop_guard(const int *done, cudaGraphConditionalHandle h)
{
    if (threadIdx.x == 0 && blockIdx.x == 0 && *done) cudaGraphSetConditional(h, 0);
}

glinalg_status Staged::stage(Scratch &sc, double *phi, const double *phi0, long n, bool dev,
                             cudaStream_t st)
{
    if (dev) {
        x = (double2 *)phi;
        b = (const double2 *)phi0;
        return GLINALG_SUCCESS;
    }
    double2 *bb = nullptr;
    GL_TRY(sc.alloc(&x, n));
    GL_TRY(sc.alloc(&bb, n));
    GL_CUDA(cudaMemcpyAsync(x, phi, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(bb, phi0, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
    b = bb;
    return GLINALG_SUCCESS;
}

glinalg_status Staged::finish(double *phi, long n, bool dev, cudaStream_t st)
{
    if (!dev) GL_CUDA(cudaMemcpyAsync(phi, x, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    return GLINALG_SUCCESS;
}

EventTimer::EventTimer()
{
    cudaEventCreate(&a);
    cudaEventCreate(&b);
}
EventTimer::~EventTimer()
{
    cudaEventDestroy(a);
    cudaEventDestroy(b);
}
double EventTimer::ms()
{
    float m = 0.f;
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&m, a, b);
    return (double)m;
}

// ---------------------------------------------------------------- BLAS-1 kernels

__global__ void __launch_bounds__(kRedThreads)
k_norm2(const double2 *__restrict__ a, long n, double *partials, unsigned *counter, double *out)
{
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads)
        v[0] += cabs2(a[i]);
    if (grid_sum<1, kRedThreads>(v, partials, counter) && threadIdx.x == 0) *out = v[0];
}

// <a, b> = sum conj(a_i) b_i (generic_vector.h:102-114)
__global__ void __launch_bounds__(kRedThreads)
k_dot(const double2 *__restrict__ a, const double2 *__restrict__ b, long n, double *partials,
      unsigned *counter, double2 *out)
{
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        double2 d = cmul(cconj(a[i]), b[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, counter) && threadIdx.x == 0) *out = cmk(v[0], v[1]);
}

__global__ void __launch_bounds__(kRedThreads)
k_diffnorm2(const double2 *__restrict__ a, const double2 *__restrict__ b, long n,
            double *partials, unsigned *counter, double *out)
{
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads)
        v[0] += cabs2(csub(a[i], b[i]));
    if (grid_sum<1, kRedThreads>(v, partials, counter) && threadIdx.x == 0) *out = v[0];
}

__global__ void k_sub(double2 *__restrict__ out, const double2 *__restrict__ a,
                      const double2 *__restrict__ b, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = csub(a[i], b[i]);
}

glinalg_status launch_norm2(const double2 *a, long n, double *partials, unsigned *counter,
                            double *out, cudaStream_t st)
{
    k_norm2<<<reduction_blocks(n), kRedThreads, 0, st>>>(a, n, partials, counter, out);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}
glinalg_status launch_dot(const double2 *a, const double2 *b, long n, double *partials,
                          unsigned *counter, double2 *out, cudaStream_t st)
{
    k_dot<<<reduction_blocks(n), kRedThreads, 0, st>>>(a, b, n, partials, counter, out);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}
glinalg_status launch_diffnorm2(const double2 *a, const double2 *b, long n, double *partials,
                                unsigned *counter, double *out, cudaStream_t st)
{
    k_diffnorm2<<<reduction_blocks(n), kRedThreads, 0, st>>>(a, b, n, partials, counter, out);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}
glinalg_status launch_sub(double2 *out, const double2 *a, const double2 *b, long n, cudaStream_t st)
{
    long g = (n + 255) / 256;
    if (g > (long)sm_count() * 16) g = (long)sm_count() * 16;
    k_sub<<<(int)(g < 1 ? 1 : g), 256, 0, st>>>(out, a, b, n);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

// ---------------------------------------------------------------- verbosity

Verb Verb::from(const glinalg_verbosity *v)
{
    Verb r;
    if (!v) return r;
    r.present = true;
    r.level = v->verbosity;
    r.prefix = v->verb_prefix ? v->verb_prefix : "";
    r.precond_level = v->precond_verbosity;
    r.precond_prefix = v->precond_verb_prefix ? v->precond_verb_prefix : "";
    return r;
}

Verb Verb::restart_inner() const
{
    Verb r;
    r.present = true;  // the reference always passes a struct to the inner solve
    if (present) {
        r.level = (level == 2 || level == 1) ? 0 : level;
        r.prefix = prefix;
        r.precond_level = precond_level;
        r.precond_prefix = precond_prefix;
    }
    return r;
}

Verb Verb::precond_inner() const
{
    Verb r;
    r.present = true;  // the reference always passes a struct to the preconditioner
    if (present) {
        r.level = precond_level == -1 ? level : precond_level;
        r.prefix = precond_prefix;
    }
    return r;
}

void Verb::resid(const std::string &alg, int iter, int ops, double relres) const
{
    if (present && level == 3)
        std::cout << prefix << alg << " Iter " << iter << " Ops " << ops << " RelRes " << relres << "\n" << std::flush;
}
void Verb::summary(const std::string &alg, bool success, int iter, int ops, double relres) const
{
    if (present && (level == 1 || level == 2 || level == 3))
        std::cout << prefix << alg << " Success " << (success ? "Y" : "N") << " Iter " << iter
                  << " Ops " << ops << " RelRes " << relres << "\n" << std::flush;
}
void Verb::summary_multi(bool success, int iter, int ops, const double *relres, int n) const
{
    if (present && (level == 1 || level == 2 || level == 3)) {
        std::cout << prefix << "CG-M " << " Success " << (success ? "Y" : "N") << " Iter " << iter
                  << " Ops " << ops << " RelRes ";
        for (int i = 0; i < n; i++) std::cout << relres[i] << " ";
        std::cout << "\n" << std::flush;
    }
}
void Verb::restart(const std::string &alg, int iter, int ops, double relres) const
{
    if (present && (level == 2 || level == 3))
        std::cout << prefix << alg << " Iter " << iter << " Ops " << ops << " RelRes " << relres << "\n" << std::flush;
}

void fill_name(glinalg_info *info, const std::string &name)
{
    std::strncpy(info->name, name.c_str(), sizeof(info->name) - 1);
    info->name[sizeof(info->name) - 1] = 0;
}

glinalg_status check_solver_args(glinalg_operator op, const void *phi, const void *phi0,
                                 int size, bool *dev, const glinalg_solver_params *params)
{
    if (!op || !phi || !phi0) {
        set_last_error("null operator, phi or phi0");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if ((long)size != op->size) {
        set_last_error("size does not match the operator's field size");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    *dev = params && (params->flags & GLINALG_PTR_DEVICE);
    return GLINALG_SUCCESS;
}

}  // namespace glinalg

using namespace glinalg;

// ---------------------------------------------------------------- library C-ABI

extern "C" int glinalg_abi_version(void) { return GLINALG_ABI_VERSION; }

extern "C" const char *glinalg_status_string(glinalg_status s)
{
    switch (s) {
    case GLINALG_SUCCESS: return "success";
    case GLINALG_ERROR_INVALID_VALUE: return "invalid value";
    case GLINALG_ERROR_UNSUPPORTED_OP: return "unsupported operator";
    case GLINALG_ERROR_CUDA: return "CUDA error";
    case GLINALG_ERROR_NO_DEVICE: return "no CUDA device";
    case GLINALG_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case GLINALG_ERROR_INTERNAL: return "internal error";
    }
    return "unknown status";
}

extern "C" const char *glinalg_last_error(void) { return t_last_error.c_str(); }

extern "C" int glinalg_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// BLAS-1 entry points: one reduction on the device, result copied to the host.
static glinalg_status reduce_entry(int which, const double *a, const double *b, long n,
                                   double *out, int flags)
{
    if (!a || !out || n < 0 || (which == 1 && !b))
        return invalid_arg("!a || !out || n < 0 || (which == 1 && !b)");
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const bool dev = flags & GLINALG_PTR_DEVICE;
    const double2 *da = (const double2 *)a, *db = (const double2 *)b;
    if (!dev) {
        double2 *ta = nullptr, *tb = nullptr;
        GL_TRY(sc.alloc(&ta, n));
        GL_CUDA(cudaMemcpyAsync(ta, a, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        da = ta;
        if (which == 1) {
            GL_TRY(sc.alloc(&tb, n));
            GL_CUDA(cudaMemcpyAsync(tb, b, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
            db = tb;
        }
    }
    double *partials = nullptr;
    unsigned *counter = nullptr;
    double2 *res = nullptr;
    GL_TRY(sc.alloc(&partials, 2 * (size_t)reduction_blocks(n)));
    GL_TRY(sc.zeros(&counter, 1));
    GL_TRY(sc.zeros(&res, 1));
    if (which == 0) GL_TRY(launch_norm2(da, n, partials, counter, (double *)res, st));
    else GL_TRY(launch_dot(da, db, n, partials, counter, res, st));
    double2 h;
    GL_CUDA(cudaMemcpyAsync(&h, res, sizeof(double2), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    out[0] = h.x;
    if (which == 1) out[1] = h.y;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_dot(const double *a, const double *b, long n, double out[2],
                                      int flags)
{
    return reduce_entry(1, a, b, n, out, flags);
}

extern "C" glinalg_status glinalg_norm2sq(const double *a, long n, double *out, int flags)
{
    return reduce_entry(0, a, nullptr, n, out, flags);
}
