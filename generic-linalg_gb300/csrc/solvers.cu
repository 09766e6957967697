// solvers.cu -- FP64 Krylov solvers with the reference's recurrences, on the device:
//   CG        generic_cg.cpp:278-382        (+ restarted :387-427)
//   BiCGstab  generic_bicgstab.cpp:205-341  (+ restarted :345-385)
//   GCR       generic_gcr.cpp:202-333       (+ restarted :337-378)
//   CG-M      generic_cg_m.cpp:312-600
//
// Every scalar of the recurrences (alpha, beta, rho, omega, zeta, ...) lives in a device
// struct and is computed by the last block of the reduction that produces it, so an
// iteration never waits for the host.  CG, BiCGstab and CG-M run their iteration body as a
// CUDA graph with a conditional WHILE node; the body's last kernel ends the loop once the
// stopping test (the reference's, term for term) has fired.  GCR, whose work per iteration
// grows with the iteration count, is driven from the host one iteration at a time.

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "solver_util.h"
#include "solvers.h"

namespace glinalg {

// ================================================================= CG

struct CgDev {
    double2 alpha;
    double beta;
    double rsq, rsq_new, bsq;
    double eps;
    int k, max_iter, done, status, iters, napply;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
};

__device__ __forceinline__ void finish_dev(int *done, int *status, int st)
{
    *status = st;
    *done = 1;
}

__global__ void __launch_bounds__(kRedThreads)
k_cg_alpha(const double2 *__restrict__ p, const double2 *__restrict__ Ap, long n, CgDev *s,
           double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        double2 d = cmul(cconj(p[i]), Ap[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        if (v[0] == 0.0 && v[1] == 0.0) {
            s->iters = s->k + 1;
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->alpha = cdiv(cmk(s->rsq, 0.0), cmk(v[0], v[1]));
    }
}

__global__ void __launch_bounds__(kRedThreads)
k_cg_update(double2 *__restrict__ x, double2 *__restrict__ r, const double2 *__restrict__ p,
            const double2 *__restrict__ Ap, long n, CgDev *s, double *partials)
{
    if (s->done) return;
    const double2 a = s->alpha;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        x[i] = cadd(x[i], cmul(a, p[i]));
        double2 ri = csub(r[i], cmul(a, Ap[i]));
        r[i] = ri;
        v[0] += cabs2(ri);
    }
    if (grid_sum<1, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0) {
        const double rn = v[0];
        const int k = s->k;
        const double bsqrt = sqrt(s->bsq);
        s->rsq_new = rn;
        if (k < s->hist_cap) s->hist[k] = sqrt(rn) / bsqrt;
        const bool last = (k == s->max_iter - 1);
        if (!isfinite(rn)) {
            s->iters = k + 1;
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        } else if (sqrt(rn) < s->eps * bsqrt || last) {
            s->iters = k + 1;
            finish_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
        } else {
            s->beta = rn / s->rsq;
            s->rsq = rn;
            s->k = k + 1;
            s->napply++;
        }
    }
}

__global__ void k_cg_xpay(double2 *__restrict__ p, const double2 *__restrict__ r, long n,
                          const CgDev *s)
{
    if (s->done) return;
    const double b = s->beta;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        p[i] = cadd(r[i], cscale(b, p[i]));
}

static int vec_grid(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

glinalg_status cg_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                       double eps, const Verb &verb, glinalg_info *info, cudaStream_t st,
                       double sigma)
{
    if (cg64_fused_applies(op, sigma)) return cg64_fused(op, x, b, max_iter, eps, verb, info, st);
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *p, *Ap, *tmp = nullptr;
    double *partials, *hist;
    CgDev *s;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&p, n));
    GL_TRY(sc.alloc(&Ap, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 2 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&s, 1));
    CgDev h = {};
    h.eps = eps;
    h.max_iter = max_iter;
    h.hist = hist;
    h.hist_cap = hist_cap;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    // setup (generic_cg.cpp:303-321): |b|, r = b - A x, p = r, Ap = A p, rsq = |r|^2
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[2], &s->bsq, st));
    GL_TRY(launch_apply_sigma(op, p, x, tmp, sigma, nullptr, st));
    GL_TRY(launch_sub(r, b, p, n, st));
    GL_CUDA(cudaMemcpyAsync(p, r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply_sigma(op, Ap, p, tmp, sigma, nullptr, st));
    GL_TRY(launch_norm2(r, n, partials, &s->cnt[2], &s->rsq, st));

    if (max_iter > 0) {
        const int vg = vec_grid(n);
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            k_cg_alpha<<<nb, kRedThreads, 0, cs>>>(p, Ap, n, s, partials);
            k_cg_update<<<nb, kRedThreads, 0, cs>>>(x, r, p, Ap, n, s, partials);
            k_cg_xpay<<<vg, 256, 0, cs>>>(p, r, n, s);
            GL_TRY(launch_apply_sigma(op, Ap, p, tmp, sigma, &s->done, cs));
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    // true residual (generic_cg.cpp:366-367)
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply_sigma(op, Ap, x, tmp, sigma, nullptr, st));
    GL_TRY(launch_diffnorm2(Ap, b, n, partials, &s->cnt[2], truersq, st));
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    std::vector<double> hh(hist_cap);
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));

    int iters, applies;
    bool success;
    if (max_iter > 0) {
        iters = h.iters;
        applies = h.napply;
        success = h.status == GLINALG_SOLVE_CONVERGED;
    } else {  // the loop never runs: k stays 0 (generic_cg.cpp:356-364)
        iters = 1;
        applies = 0;
        success = !(0 == max_iter - 1);
        h.status = success ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER;
    }
    const double bsqrt = std::sqrt(h.bsq);
    for (int k = 0; k < std::min(iters, hist_cap); k++) verb.resid("CG", k + 1, 2 + k, hh[k]);
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = 3 + applies;
    info->status = h.status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)(iters) * (176.0 * n + apply_bytes(op)) + 3 * apply_bytes(op)) * 1e-9;
    fill_name(info, "CG");
    verb.summary("CG", info->success != 0, iters, info->ops_count, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= BiCGstab

struct BiDev {
    double2 rho, alpha, omega, beta;
    double rsq, bsq, eps;
    int k, max_iter, done, status, iters, napply;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
};

__global__ void __launch_bounds__(kRedThreads)
k_bi_alpha(const double2 *__restrict__ r0, const double2 *__restrict__ Ap, long n, BiDev *s,
           double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        double2 d = cmul(cconj(r0[i]), Ap[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        if (v[0] == 0.0 && v[1] == 0.0) {
            s->iters = s->k + 1;
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->alpha = cdiv(s->rho, cmk(v[0], v[1]));
    }
}

// s = r - alpha Ap
__global__ void k_bi_s(double2 *__restrict__ sv, const double2 *__restrict__ r,
                       const double2 *__restrict__ Ap, long n, const BiDev *s)
{
    if (s->done) return;
    const double2 a = s->alpha;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        sv[i] = csub(r[i], cmul(a, Ap[i]));
}

// omega = <As, s> / <As, As>
__global__ void __launch_bounds__(kRedThreads)
k_bi_omega(const double2 *__restrict__ As, const double2 *__restrict__ sv, long n, BiDev *s,
           double *partials)
{
    if (s->done) return;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        double2 a = As[i];
        double2 d = cmul(cconj(a), sv[i]);
        v[0] += d.x;
        v[1] += d.y;
        v[2] += cabs2(a);
    }
    if (grid_sum<3, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0) {
        if (v[2] == 0.0) {
            s->iters = s->k + 1;
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->omega = cdiv(cmk(v[0], v[1]), cmk(v[2], 0.0));
    }
}

// x = x + alpha p + omega s; r = s - omega As; |r|^2 and <r0, r>
__global__ void __launch_bounds__(kRedThreads)
k_bi_update(double2 *__restrict__ x, double2 *__restrict__ r, const double2 *__restrict__ p,
            const double2 *__restrict__ sv, const double2 *__restrict__ As,
            const double2 *__restrict__ r0, long n, BiDev *s, double *partials)
{
    if (s->done) return;
    const double2 a = s->alpha, w = s->omega;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 si = sv[i];
        x[i] = cadd(cadd(x[i], cmul(a, p[i])), cmul(w, si));
        const double2 ri = csub(si, cmul(w, As[i]));
        r[i] = ri;
        v[0] += cabs2(ri);
        const double2 d = cmul(cconj(r0[i]), ri);
        v[1] += d.x;
        v[2] += d.y;
    }
    if (grid_sum<3, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0) {
        const double rn = v[0];
        const int k = s->k;
        const double bsqrt = sqrt(s->bsq);
        s->rsq = rn;
        if (k < s->hist_cap) s->hist[k] = sqrt(rn) / bsqrt;
        const bool last = (k == s->max_iter - 1);
        if (!isfinite(rn)) {
            s->iters = k + 1;
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        } else if (sqrt(rn) < s->eps * bsqrt || last) {
            s->iters = k + 1;
            finish_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
        } else {
            const double2 rho_new = cmk(v[1], v[2]);
            // beta = rhoNew/rho * (alpha/omega)   (generic_bicgstab.cpp:296)
            s->beta = cmul(cdiv(rho_new, s->rho), cdiv(s->alpha, s->omega));
            s->rho = rho_new;
            s->k = k + 1;
            s->napply++;
        }
    }
}

// p = r + beta (p - omega Ap)
__global__ void k_bi_p(double2 *__restrict__ p, const double2 *__restrict__ r,
                       const double2 *__restrict__ Ap, long n, const BiDev *s)
{
    if (s->done) return;
    const double2 bt = s->beta, w = s->omega;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        p[i] = cadd(r[i], cmul(bt, csub(p[i], cmul(w, Ap[i]))));
}

__global__ void k_store_dot(const double2 *res, BiDev *s) { s->rho = *res; }

glinalg_status bicgstab_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b,
                             int max_iter, double eps, const Verb &verb, glinalg_info *info,
                             cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *r0, *p, *Ap, *sv, *As, *tmp = nullptr, *dres;
    double *partials, *hist;
    BiDev *s;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&r0, n));
    GL_TRY(sc.alloc(&p, n));
    GL_TRY(sc.alloc(&Ap, n));
    GL_TRY(sc.alloc(&sv, n));
    GL_TRY(sc.alloc(&As, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 3 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&s, 1));
    GL_TRY(sc.alloc(&dres, 1));
    BiDev h = {};
    h.eps = eps;
    h.max_iter = max_iter;
    h.hist = hist;
    h.hist_cap = hist_cap;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    // setup (generic_bicgstab.cpp:238-255)
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[3], &s->bsq, st));
    GL_TRY(launch_apply(op, Ap, x, tmp, nullptr, st));
    GL_TRY(launch_sub(r, b, Ap, n, st));
    GL_CUDA(cudaMemcpyAsync(r0, r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_CUDA(cudaMemcpyAsync(p, r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_dot(r0, r, n, partials, &s->cnt[3], dres, st));
    k_store_dot<<<1, 1, 0, st>>>(dres, s);
    GL_TRY(launch_apply(op, Ap, p, tmp, nullptr, st));

    if (max_iter > 0) {
        const int vg = vec_grid(n);
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            k_bi_alpha<<<nb, kRedThreads, 0, cs>>>(r0, Ap, n, s, partials);
            k_bi_s<<<vg, 256, 0, cs>>>(sv, r, Ap, n, s);
            GL_TRY(launch_apply(op, As, sv, tmp, &s->done, cs));
            k_bi_omega<<<nb, kRedThreads, 0, cs>>>(As, sv, n, s, partials);
            k_bi_update<<<nb, kRedThreads, 0, cs>>>(x, r, p, sv, As, r0, n, s, partials);
            k_bi_p<<<vg, 256, 0, cs>>>(p, r, Ap, n, s);
            GL_TRY(launch_apply(op, Ap, p, tmp, &s->done, cs));
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply(op, Ap, x, tmp, nullptr, st));
    GL_TRY(launch_diffnorm2(Ap, b, n, partials, &s->cnt[3], truersq, st));
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    std::vector<double> hh(hist_cap);
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));

    int iters, ops;
    bool success;
    if (max_iter > 0) {
        iters = h.iters;
        // setup 2, As every iteration, Ap every iteration that did not stop, final check 1
        ops = 2 + iters + h.napply + 1;
        success = h.status == GLINALG_SOLVE_CONVERGED;
    } else {
        iters = 1;
        ops = 3;
        success = !(0 == max_iter - 1);
        h.status = success ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER;
    }
    const double bsqrt = std::sqrt(h.bsq);
    for (int k = 0; k < std::min(iters, hist_cap); k++) verb.resid("BiCGStab", k + 1, 3 + 2 * k, hh[k]);
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = ops;
    info->status = h.status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)iters * (2 * apply_bytes(op) + 400.0 * n) + 3 * apply_bytes(op)) * 1e-9;
    fill_name(info, "BiCGStab");
    verb.summary("BiCGStab", info->success != 0, iters, ops, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= GCR

struct GcrDev {
    double2 alpha;
    double rsq, bsq, eps;
    int k, max_iter, done, status;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
};

// alpha = <Ap, r> / |Ap|^2 ; stores |Ap|^2 (generic_gcr.cpp:256)
__global__ void __launch_bounds__(kRedThreads)
k_gcr_alpha(const double2 *__restrict__ Ap, const double2 *__restrict__ r, long n, GcrDev *s,
            double *apnorm_slot, double *partials)
{
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 a = Ap[i];
        const double2 d = cmul(cconj(a), r[i]);
        v[0] += d.x;
        v[1] += d.y;
        v[2] += cabs2(a);
    }
    if (grid_sum<3, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        *apnorm_slot = v[2];
        if (v[2] == 0.0) {
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->alpha = cmk(v[0] / v[2], v[1] / v[2]);
    }
}

__global__ void __launch_bounds__(kRedThreads)
k_gcr_update(double2 *__restrict__ x, double2 *__restrict__ r, const double2 *__restrict__ p,
             const double2 *__restrict__ Ap, long n, GcrDev *s, double *partials)
{
    if (s->done) return;
    const double2 a = s->alpha;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        x[i] = cadd(x[i], cmul(a, p[i]));
        const double2 ri = csub(r[i], cmul(a, Ap[i]));
        r[i] = ri;
        v[0] += cabs2(ri);
    }
    if (grid_sum<1, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0) {
        const double rn = v[0];
        const int k = s->k;
        const double bsqrt = sqrt(s->bsq);
        s->rsq = rn;
        if (k < s->hist_cap) s->hist[k] = sqrt(rn) / bsqrt;
        const bool last = (k == s->max_iter - 1);
        if (!isfinite(rn)) finish_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        else if (sqrt(rn) < s->eps * bsqrt || last)
            finish_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
        else s->k = k + 1;
    }
}

// beta_i = -<Ap_i, Ar> / |Ap_i|^2 for i in [i0, i0 + cnt), cnt <= 8 (generic_gcr.cpp:286)
constexpr int kGcrDots = 8;
__global__ void __launch_bounds__(kRedThreads)
k_gcr_betas(double2 *const *__restrict__ Aps, const double2 *__restrict__ Ar, long n, int i0,
            int cnt, const double *__restrict__ apnorm, double2 *betas, double *partials,
            unsigned *counter)
{
    double v[2 * kGcrDots];
#pragma unroll
    for (int j = 0; j < 2 * kGcrDots; j++) v[j] = 0.0;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 ar = Ar[i];
#pragma unroll
        for (int j = 0; j < kGcrDots; j++) {
            if (j < cnt) {
                const double2 d = cmul(cconj(Aps[i0 + j][i]), ar);
                v[2 * j] += d.x;
                v[2 * j + 1] += d.y;
            }
        }
    }
    if (grid_sum<2 * kGcrDots, kRedThreads>(v, partials, counter) && threadIdx.x == 0) {
        for (int j = 0; j < cnt; j++) {
            const double nn = apnorm[i0 + j];
            betas[i0 + j] = cmk(-v[2 * j] / nn, -v[2 * j + 1] / nn);
        }
    }
}

// p = r + sum_i beta_i p_i ; Ap = Ar + sum_i beta_i Ap_i  (in order i = 0..k)
__global__ void k_gcr_combine(double2 *__restrict__ p, double2 *__restrict__ Ap,
                              const double2 *__restrict__ r, const double2 *__restrict__ Ar,
                              double2 *const *__restrict__ ps, double2 *const *__restrict__ Aps,
                              const double2 *__restrict__ betas, int m, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double2 pv = r[i], av = Ar[i];
        for (int j = 0; j < m; j++) {
            const double2 bj = betas[j];
            pv = cadd(pv, cmul(bj, ps[j][i]));
            av = cadd(av, cmul(bj, Aps[j][i]));
        }
        p[i] = pv;
        Ap[i] = av;
    }
}

glinalg_status gcr_fp64(const glinalg_operator_s *op, double2 *phi, const double2 *b, int max_iter,
                        double eps, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *x, *r, *Ar, *tmp = nullptr, *betas;
    double *partials, *hist, *apnorm;
    double2 **d_ps, **d_Aps;
    GcrDev *s;
    const int cap = (max_iter > 0 ? max_iter : 1) + 1;
    const int hist_cap = verb.level == 3 ? cap : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&x, n));
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&Ar, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 2 * kGcrDots * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&apnorm, cap));
    GL_TRY(sc.alloc(&betas, cap));
    GL_TRY(sc.alloc(&d_ps, cap));
    GL_TRY(sc.alloc(&d_Aps, cap));
    GL_TRY(sc.alloc(&s, 1));
    GcrDev h = {};
    h.eps = eps;
    h.max_iter = max_iter;
    h.hist = hist;
    h.hist_cap = hist_cap;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));
    std::vector<double2 *> ps, Aps;  // host mirror of the stored directions
    std::vector<double2 *> hp(cap), hAp(cap);
    auto new_vec = [&](double2 **v) { return sc.alloc(v, n); };
    double2 *p, *Ap;
    GL_TRY(new_vec(&p));
    GL_TRY(new_vec(&Ap));

    EventTimer tm;
    tm.start(st);
    GL_CUDA(cudaMemcpyAsync(x, phi, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[2], &s->bsq, st));
    GL_TRY(launch_apply(op, p, x, tmp, nullptr, st));
    GL_TRY(launch_sub(r, b, p, n, st));
    GL_CUDA(cudaMemcpyAsync(p, r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply(op, Ap, p, tmp, nullptr, st));
    int ops = 2, k = 0, status = GLINALG_SOLVE_CONVERGED;
    const int vg = vec_grid(n);
    for (k = 0; k < max_iter; k++) {
        hp[k] = p;
        hAp[k] = Ap;
        GL_CUDA(cudaMemcpyAsync(d_ps + k, &hp[k], sizeof(double2 *), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(d_Aps + k, &hAp[k], sizeof(double2 *), cudaMemcpyHostToDevice, st));
        k_gcr_alpha<<<nb, kRedThreads, 0, st>>>(Ap, r, n, s, apnorm + k, partials);
        k_gcr_update<<<nb, kRedThreads, 0, st>>>(x, r, p, Ap, n, s, partials);
        GL_CUDA(cudaGetLastError());
        int done_status[2];
        GL_CUDA(cudaMemcpyAsync(done_status, &s->done, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
        GL_CUDA(cudaStreamSynchronize(st));
        if (done_status[0]) {
            status = done_status[1];
            break;
        }
        GL_TRY(launch_apply(op, Ar, r, tmp, nullptr, st));
        ops++;
        for (int i0 = 0; i0 <= k; i0 += kGcrDots) {
            const int cnt = std::min(kGcrDots, k + 1 - i0);
            k_gcr_betas<<<nb, kRedThreads, 0, st>>>(d_Aps, Ar, n, i0, cnt, apnorm, betas, partials, &s->cnt[3]);
        }
        GL_TRY(new_vec(&p));
        GL_TRY(new_vec(&Ap));
        k_gcr_combine<<<vg, 256, 0, st>>>(p, Ap, r, Ar, d_ps, d_Aps, betas, k + 1, n);
        GL_CUDA(cudaGetLastError());
    }
    int iters;
    bool success;
    if (max_iter > 0) {
        iters = k + 1;
        success = status == GLINALG_SOLVE_CONVERGED;
    } else {
        iters = 1;
        success = !(0 == max_iter - 1);
        status = success ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER;
    }
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply(op, Ar, x, tmp, nullptr, st));
    ops++;
    GL_TRY(launch_diffnorm2(Ar, b, n, partials, &s->cnt[2], truersq, st));
    GL_CUDA(cudaMemcpyAsync(phi, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    std::vector<double> hh(hist_cap);
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    const double bsqrt = std::sqrt(h.bsq);
    for (int j = 0; j < std::min(iters, hist_cap); j++) verb.resid("GCR", j + 1, 2 + j, hh[j]);
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = ops;
    info->status = status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)iters * (apply_bytes(op) + 192.0 * n) +
                    (double)iters * (iters + 1) * 0.5 * 48.0 * n + 3 * apply_bytes(op)) * 1e-9;
    fill_name(info, "GCR");
    verb.summary("GCR", info->success != 0, iters, ops, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= CG-M

struct CgmDev {
    double2 alpha, beta, beta_prev;
    double rsq, rsq_new, bsq, eps;
    int k, max_iter, done, status, iters, napply;
    int n_rem, n_rem_before, rfc, worst_first, n_shift;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
    // per slot (the reference's permuted position), n_shift entries each
    double2 *zeta, *zeta_prev, *beta_s, *alpha_s;
    double *shifts;
    int *map;  // slot -> original shift index
};

// beta = -rsq / <p, Ap>, then zeta and beta_s of every live shift (generic_cg_m.cpp:396-412)
__global__ void __launch_bounds__(kRedThreads)
k_cgm_beta(const double2 *__restrict__ p, const double2 *__restrict__ Ap, long n, CgmDev *s,
           double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(p[i]), Ap[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        if (v[0] == 0.0 && v[1] == 0.0) {
            s->iters = s->k + 1;
            s->n_rem_before = 0;
            finish_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        const double2 beta_prev = s->beta;
        const double2 beta = cdiv(cmk(-s->rsq, 0.0), cmk(v[0], v[1]));
        const double2 alpha = s->alpha;
        s->beta_prev = beta_prev;
        s->beta = beta;
        for (int j = 0; j < s->n_rem; j++) {
            const double2 z = s->zeta[j], zp = s->zeta_prev[j];
            const double sh = s->shifts[j];
            const double2 num = cmul(cmul(z, zp), beta_prev);
            const double2 one_m = cmk(1.0 - sh * beta.x, -(sh * beta.y));
            const double2 den = cadd(cmul(cmul(beta, alpha), csub(zp, z)), cmul(cmul(zp, beta_prev), one_m));
            const double2 zn = cdiv(num, den);
            s->zeta[j] = zn;
            s->zeta_prev[j] = z;
            s->beta_s[j] = cdiv(cmul(beta, zn), z);
        }
        s->n_rem_before = s->n_rem;
    }
}

// r = r + beta Ap; |r|^2; convergence bookkeeping (generic_cg_m.cpp:423-513, scalars only)
__global__ void __launch_bounds__(kRedThreads)
k_cgm_r(double2 *__restrict__ r, const double2 *__restrict__ Ap, long n, CgmDev *s,
        double *partials)
{
    if (s->done) return;
    const double2 bt = s->beta;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 ri = cadd(r[i], cmul(bt, Ap[i]));
        r[i] = ri;
        v[0] += cabs2(ri);
    }
    if (!(grid_sum<1, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0)) return;
    const double rn = v[0];
    const int k = s->k;
    const double bsqrt = sqrt(s->bsq), srn = sqrt(rn);
    s->rsq_new = rn;
    if (k < s->hist_cap) s->hist[k] = srn / bsqrt;
    if (k % s->rfc == 0) {
        for (int j = 0; j < s->n_rem; j++) {
            if (cabsd(s->zeta[j]) * srn < s->eps * bsqrt) {
                s->n_rem--;
                const int e = s->n_rem;
                if (e != j) {
                    int ti = s->map[e]; s->map[e] = s->map[j]; s->map[j] = ti;
                    double2 tc;
                    tc = s->alpha_s[e]; s->alpha_s[e] = s->alpha_s[j]; s->alpha_s[j] = tc;
                    tc = s->beta_s[e]; s->beta_s[e] = s->beta_s[j]; s->beta_s[j] = tc;
                    tc = s->zeta[e]; s->zeta[e] = s->zeta[j]; s->zeta[j] = tc;
                    tc = s->zeta_prev[e]; s->zeta_prev[e] = s->zeta_prev[j]; s->zeta_prev[j] = tc;
                    double td = s->shifts[e]; s->shifts[e] = s->shifts[j]; s->shifts[j] = td;
                    j--;
                }
            }
        }
    }
    const bool last = (k == s->max_iter - 1);
    if (!isfinite(rn)) {
        s->iters = k + 1;
        finish_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        return;
    }
    if ((s->worst_first && cabsd(s->zeta[0]) * srn < s->eps * bsqrt) || s->n_rem == 0 || last) {
        s->iters = k + 1;
        finish_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
        return;
    }
    const double2 alpha = cmk(rn / s->rsq, 0.0);
    s->alpha = alpha;
    s->rsq = rn;
    for (int j = 0; j < s->n_rem; j++)
        s->alpha_s[j] = cdiv(cmul(cmul(alpha, s->zeta[j]), s->beta_s[j]), cmul(s->zeta_prev[j], s->beta));
    s->k = k + 1;
    s->napply++;
}

// x_s -= beta_s p_s for the shifts live before this iteration's check; then (unless the
// solve stopped) p_s = zeta_s r + alpha_s p_s for the shifts still live and p = r + alpha p.
__global__ void k_cgm_vec(double2 *const *__restrict__ X, double2 *const *__restrict__ P,
                          double2 *__restrict__ p, const double2 *__restrict__ r, long n,
                          const CgmDev *s)
{
    const int nb = s->n_rem_before;
    const int na = s->done ? 0 : s->n_rem;
    const bool upd_p = !s->done;
    const double2 alpha = s->alpha;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double2 ri = r[i];
        for (int j = 0; j < nb; j++) {
            const int o = s->map[j];
            double2 *xs = X[o];
            double2 *ps = P[o];
            const double2 pv = ps[i];
            xs[i] = csub(xs[i], cmul(s->beta_s[j], pv));
            if (j < na) ps[i] = cadd(cmul(s->zeta[j], ri), cmul(s->alpha_s[j], pv));
        }
        if (upd_p) p[i] = cadd(ri, cmul(alpha, p[i]));
    }
}

__global__ void k_cgm_init(double2 *const *X, double2 *const *P, const double2 *b, int ns, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double2 bi = b[i];
        for (int j = 0; j < ns; j++) {
            X[j][i] = cmk(0.0, 0.0);
            P[j][i] = bi;
        }
    }
}

glinalg_status cg_m_fp64(const glinalg_operator_s *op, double2 *const *X_host, const double2 *b,
                         int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                         bool worst_first, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *p, *Ap, *tmp = nullptr;
    double *partials, *hist;
    CgmDev *s;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&p, n));
    GL_TRY(sc.alloc(&Ap, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 2 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&s, 1));
    double2 *zeta, *zeta_prev, *beta_s, *alpha_s;
    double *d_shifts;
    int *map;
    double2 **dX, **dP;
    GL_TRY(sc.alloc(&zeta, n_shift));
    GL_TRY(sc.alloc(&zeta_prev, n_shift));
    GL_TRY(sc.alloc(&beta_s, n_shift));
    GL_TRY(sc.alloc(&alpha_s, n_shift));
    GL_TRY(sc.alloc(&d_shifts, n_shift));
    GL_TRY(sc.alloc(&map, n_shift));
    GL_TRY(sc.alloc(&dX, n_shift));
    GL_TRY(sc.alloc(&dP, n_shift));
    std::vector<double2 *> hP(n_shift);
    for (int j = 0; j < n_shift; j++) GL_TRY(sc.alloc(&hP[j], n));
    std::vector<double2> ones(n_shift, cmk(1.0, 0.0)), zeros(n_shift, cmk(0.0, 0.0));
    std::vector<int> hmap(n_shift);
    for (int j = 0; j < n_shift; j++) hmap[j] = j;
    GL_CUDA(cudaMemcpyAsync(zeta, ones.data(), sizeof(double2) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(zeta_prev, ones.data(), sizeof(double2) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(beta_s, ones.data(), sizeof(double2) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(alpha_s, zeros.data(), sizeof(double2) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(d_shifts, shifts, sizeof(double) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(map, hmap.data(), sizeof(int) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(dX, X_host, sizeof(double2 *) * n_shift, cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(dP, hP.data(), sizeof(double2 *) * n_shift, cudaMemcpyHostToDevice, st));
    CgmDev h = {};
    h.beta = cmk(1.0, 0.0);
    h.alpha = cmk(0.0, 0.0);
    h.eps = eps;
    h.max_iter = max_iter;
    h.n_rem = n_shift;
    h.n_shift = n_shift;
    h.rfc = rfc;
    h.worst_first = worst_first ? 1 : 0;
    h.hist = hist;
    h.hist_cap = hist_cap;
    h.zeta = zeta;
    h.zeta_prev = zeta_prev;
    h.beta_s = beta_s;
    h.alpha_s = alpha_s;
    h.shifts = d_shifts;
    h.map = map;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    const int vg = vec_grid(n);
    // setup (generic_cg_m.cpp:372-391): x_s = 0, p_s = b, p = r = b, Ap = A p
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[2], &s->bsq, st));
    k_cgm_init<<<vg, 256, 0, st>>>(dX, dP, b, n_shift, n);
    GL_CUDA(cudaMemcpyAsync(p, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_CUDA(cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply(op, Ap, p, tmp, nullptr, st));
    GL_TRY(launch_norm2(r, n, partials, &s->cnt[2], &s->rsq, st));
    if (max_iter > 0) {
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            k_cgm_beta<<<nb, kRedThreads, 0, cs>>>(p, Ap, n, s, partials);
            k_cgm_r<<<nb, kRedThreads, 0, cs>>>(r, Ap, n, s, partials);
            k_cgm_vec<<<vg, 256, 0, cs>>>(dX, dP, p, r, n, s);
            GL_TRY(launch_apply(op, Ap, p, tmp, &s->done, cs));
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    // explicit residuals of the shifted systems in the caller's order (:561-572)
    double *res;
    GL_TRY(sc.alloc(&res, n_shift));
    for (int j = 0; j < n_shift; j++) {
        GL_TRY(launch_apply_shifted(op, Ap, X_host[j], tmp, shifts[j], st));
        GL_TRY(launch_diffnorm2(Ap, b, n, partials, &s->cnt[2], res + j, st));
    }
    tm.stop(st);
    std::vector<double> hres(n_shift), hh(hist_cap);
    GL_CUDA(cudaMemcpyAsync(hres.data(), res, sizeof(double) * n_shift, cudaMemcpyDeviceToHost, st));
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    double bsq = 0;
    GL_CUDA(cudaMemcpyAsync(&bsq, &s->bsq, sizeof(double), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    int iters, applies;
    bool success;
    if (max_iter > 0) {
        iters = h.iters;
        applies = h.napply;
        success = h.status == GLINALG_SOLVE_CONVERGED;
    } else {
        iters = 1;
        applies = 0;
        success = !(0 == max_iter - 1);
        h.status = success ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER;
    }
    const double bsqrt = std::sqrt(bsq);
    for (int k = 0; k < std::min(iters, hist_cap); k++) verb.resid("CG-M", k + 1, 1 + k, hh[k]);
    std::vector<double> relres(n_shift);
    for (int j = 0; j < n_shift; j++) {
        relres[j] = std::sqrt(hres[j]) / bsqrt;
        if (info->resSqmrhs) info->resSqmrhs[j] = hres[j];
    }
    info->n_rhs = n_shift;
    info->resSq = 0.0;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = 1 + applies + n_shift;
    info->status = h.status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)iters * (apply_bytes(op) + 112.0 * n + 64.0 * n * n_shift) +
                    (n_shift + 1) * apply_bytes(op)) * 1e-9;
    fill_name(info, "CG-M");
    verb.summary_multi(info->success != 0, iters, info->ops_count, relres.data(), n_shift);
    return GLINALG_SUCCESS;
}

// ================================================================= restarts

// generic_cg.cpp:387-427 (and the BiCGstab / GCR twins): repeat the inner solve with
// max_iter = restart_freq until converged or the iteration budget is spent.
glinalg_status restart_driver(int which, const glinalg_operator_s *op, double2 *x,
                              const double2 *b, int max_iter, double eps, int restart_freq,
                              const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    static const char *names[3] = {"CG", "BiCGStab", "GCR"};
    const std::string nm = std::string(names[which]) + "(" + std::to_string(restart_freq) + ")";
    Verb inner = verb.restart_inner();
    glinalg_info in = {};
    int iter = 0, ops = 0;
    double ms = 0, gb = 0, bsqrt = 0;
    {
        Scratch sc(st);
        double *partials, *bsq;
        unsigned *cnt;
        GL_TRY(sc.alloc(&partials, (size_t)reduction_blocks(op->size)));
        GL_TRY(sc.zeros(&cnt, 1));
        GL_TRY(sc.alloc(&bsq, 1));
        GL_TRY(launch_norm2(b, op->size, partials, cnt, bsq, st));
        double hb = 0;
        GL_CUDA(cudaMemcpyAsync(&hb, bsq, sizeof(double), cudaMemcpyDeviceToHost, st));
        GL_CUDA(cudaStreamSynchronize(st));
        bsqrt = std::sqrt(hb);
    }
    do {
        in = {};
        if (which == 0) GL_TRY(cg_fp64(op, x, b, restart_freq, eps, inner, &in, st));
        else if (which == 1) GL_TRY(bicgstab_fp64(op, x, b, restart_freq, eps, inner, &in, st));
        else GL_TRY(gcr_fp64(op, x, b, restart_freq, eps, inner, &in, st));
        iter += in.iter;
        ops += in.ops_count;
        ms += in.device_ms;
        gb += in.gbytes;
        verb.restart(nm, iter, ops, std::sqrt(in.resSq) / bsqrt);
    } while (iter < max_iter && in.success == 0 && std::sqrt(in.resSq) / bsqrt > eps);
    double *keep = info->resSqmrhs;
    *info = in;
    info->resSqmrhs = keep;
    info->iter = iter;
    info->ops_count = ops;
    info->device_ms = ms;
    info->gbytes = gb;
    verb.summary(nm, in.success != 0, iter, ops, std::sqrt(in.resSq) / bsqrt);
    fill_name(info, nm);
    const bool ok = !(std::sqrt(in.resSq) / bsqrt > eps);
    info->success = ok ? 1 : 0;
    if (ok) info->status = GLINALG_SOLVE_CONVERGED;
    else if (info->status == GLINALG_SOLVE_CONVERGED) info->status = GLINALG_SOLVE_MAX_ITER;
    return GLINALG_SUCCESS;
}

}  // namespace glinalg
