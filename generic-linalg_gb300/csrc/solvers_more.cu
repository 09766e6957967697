// solvers_more.cu -- the reference's sibling Krylov solvers on the device, FP64, with the
// reference's recurrences, stopping rules and operator counts:
//   CR          generic_cr.cpp:198-323            (+ restarted :326-366)
//   MinRes (MR) generic_minres.cpp:130-231
//   CR-M        generic_cr_m.cpp:323-622
//   BiCGstab-l  generic_bicgstab_l.cpp:317-561    (+ restarted :564-604)
//   BiCGstab-M  generic_bicgstab_m.cpp:402-774
//   FPCG        generic_cg_flex_precond.cpp:223-364 (+ restarted :367-415)
//   VPGCR       generic_gcr_var_precond.cpp:220-366 (+ restarted :369-411)
// and the preconditioners of generic_precond.cpp:34-77 (identity, MinRes, GCR).
//
// As in solvers.cu, every scalar of a recurrence lives in a device struct and is computed by
// the last block of the reduction that produces it.  CR, MinRes, CR-M, BiCGstab-l and
// BiCGstab-M run their iteration as a CUDA graph with a conditional WHILE node.  FPCG and
// VPGCR keep every search direction, so their work grows with the iteration count, and they
// call a preconditioner between iterations: they are driven from the host one iteration at a
// time, like GCR.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <sstream>
#include <string>
#include <vector>

#include "solvers.h"

namespace glinalg {

namespace {

__device__ __forceinline__ void stop_dev(int *done, int *status, int st)
{
    *status = st;
    *done = 1;
}

int vgrid(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

#define GRID_LOOP(i, n) \
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < (n); i += (long)gridDim.x * blockDim.x)

// reads |b|^2 into *bsq on the host (one synchronisation, before a solve starts)
glinalg_status host_bnorm(const double2 *b, long n, double *out, cudaStream_t st)
{
    Scratch sc(st);
    double *partials, *bsq;
    unsigned *cnt;
    GL_TRY(sc.alloc(&partials, (size_t)reduction_blocks(n)));
    GL_TRY(sc.zeros(&cnt, 1));
    GL_TRY(sc.alloc(&bsq, 1));
    GL_TRY(launch_norm2(b, n, partials, cnt, bsq, st));
    GL_CUDA(cudaMemcpyAsync(out, bsq, sizeof(double), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

}  // namespace

// ================================================================= CR

struct CrDev {
    double2 alpha, beta;
    double Apsq, bsq, eps;
    int k, max_iter, done, status, iters, napply;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
};

// |Ap|^2 and <Ap, r>, then alpha = <Ap, r> / |Ap|^2 (generic_cr.cpp:250, :262)
__global__ void __launch_bounds__(kRedThreads)
k_cr_alpha(const double2 *__restrict__ Ap, const double2 *__restrict__ r, long n, CrDev *s, double *partials)
{
    if (s->done) return;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 a = Ap[i];
        const double2 d = cmul(cconj(a), r[i]);
        v[0] += cabs2(a);
        v[1] += d.x;
        v[2] += d.y;
    }
    if (grid_sum<3, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        s->Apsq = v[0];
        if (v[0] == 0.0) {
            s->iters = s->k + 1;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->alpha = cmk(v[1] / v[0], v[2] / v[0]);
    }
}

// x += alpha p, r -= alpha Ap, |r|^2 and the stopping test (generic_cr.cpp:265-281)
__global__ void __launch_bounds__(kRedThreads)
k_cr_update(double2 *__restrict__ x, double2 *__restrict__ r, const double2 *__restrict__ p,
            const double2 *__restrict__ Ap, long n, CrDev *s, double *partials)
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
        if (k < s->hist_cap) s->hist[k] = sqrt(rn) / bsqrt;
        const bool last = (k == s->max_iter - 1);
        if (!isfinite(rn)) {
            s->iters = k + 1;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        } else if (sqrt(rn) < s->eps * bsqrt || last) {
            s->iters = k + 1;
            stop_dev(&s->done, &s->status, sqrt(rn) < s->eps * bsqrt ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER);
        } else {
            s->k = k + 1;
            s->napply++;
        }
    }
}

// beta = -<Ap, Ar> / |Ap|^2 (generic_cr.cpp:290)
__global__ void __launch_bounds__(kRedThreads)
k_cr_beta(const double2 *__restrict__ Ap, const double2 *__restrict__ Ar, long n, CrDev *s, double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(Ap[i]), Ar[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0)
        s->beta = cmk(-v[0] / s->Apsq, -v[1] / s->Apsq);
}

// p = r + beta p, Ap = Ar + beta Ap (generic_cr.cpp:294-298)
__global__ void k_cr_dir(double2 *__restrict__ p, double2 *__restrict__ Ap, const double2 *__restrict__ r,
                         const double2 *__restrict__ Ar, long n, const CrDev *s)
{
    if (s->done) return;
    const double2 bt = s->beta;
    GRID_LOOP(i, n)
    {
        p[i] = cadd(r[i], cmul(bt, p[i]));
        Ap[i] = cadd(Ar[i], cmul(bt, Ap[i]));
    }
}

glinalg_status cr_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                       double eps, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *p, *Ap, *Ar, *tmp = nullptr;
    double *partials, *hist;
    CrDev *s;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&p, n));
    GL_TRY(sc.alloc(&Ap, n));
    GL_TRY(sc.alloc(&Ar, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 3 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&s, 1));
    CrDev h = {};
    h.eps = eps;
    h.max_iter = max_iter;
    h.hist = hist;
    h.hist_cap = hist_cap;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    // setup (generic_cr.cpp:228-245): r = b - A x, p = r, Ap = A p
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[3], &s->bsq, st));
    GL_TRY(launch_apply(op, p, x, tmp, nullptr, st));
    GL_TRY(launch_sub(r, b, p, n, st));
    GL_CUDA(cudaMemcpyAsync(p, r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply(op, Ap, p, tmp, nullptr, st));
    if (max_iter > 0) {
        const int vg = vgrid(n);
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            k_cr_alpha<<<nb, kRedThreads, 0, cs>>>(Ap, r, n, s, partials);
            k_cr_update<<<nb, kRedThreads, 0, cs>>>(x, r, p, Ap, n, s, partials);
            GL_TRY(launch_apply(op, Ar, r, tmp, &s->done, cs));
            k_cr_beta<<<nb, kRedThreads, 0, cs>>>(Ap, Ar, n, s, partials);
            k_cr_dir<<<vg, 256, 0, cs>>>(p, Ap, r, Ar, n, s);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply(op, p, x, tmp, nullptr, st));
    GL_TRY(launch_diffnorm2(p, b, n, partials, &s->cnt[3], truersq, st));
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
        // generic_cr.cpp:288 tests k == max_iter, which the loop (it breaks at max_iter - 1)
        // never reaches: the reference's complex CR reports success whenever max_iter > 0.
        // status still tells whether the tolerance was met.
        success = h.status == GLINALG_SOLVE_CONVERGED || h.status == GLINALG_SOLVE_MAX_ITER;
    } else {
        iters = 1;
        applies = 0;
        success = false;
        h.status = GLINALG_SOLVE_MAX_ITER;
    }
    const double bsqrt = std::sqrt(h.bsq);
    for (int k = 0; k < std::min(iters, hist_cap); k++) verb.resid("CR", k + 1, 2 + k, hh[k]);
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = 3 + applies;
    info->status = h.status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)iters * (224.0 * n + apply_bytes(op)) + 3 * apply_bytes(op)) * 1e-9;
    fill_name(info, "CR");
    verb.summary("CR", info->success != 0, iters, info->ops_count, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= MinRes

struct MrDev {
    double2 alpha;
    double omega, bsq, eps;
    int k, max_iter, done, status, iters;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
};

// alpha = omega <Ar, r> / |Ar|^2 (generic_minres.cpp:174-179), with p = A r
__global__ void __launch_bounds__(kRedThreads)
k_mr_alpha(const double2 *__restrict__ p, const double2 *__restrict__ r, long n, MrDev *s, double *partials)
{
    if (s->done) return;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 a = p[i];
        const double2 d = cmul(cconj(a), r[i]);
        v[0] += cabs2(a);
        v[1] += d.x;
        v[2] += d.y;
    }
    if (grid_sum<3, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        if (v[0] == 0.0) {
            s->iters = s->k;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->alpha = cmk((v[1] / v[0]) * s->omega, (v[2] / v[0]) * s->omega);
    }
}

// x += alpha r, r -= alpha p, |r|^2; the loop ends on the tolerance or after max_iter
// iterations (generic_minres.cpp:182-196)
__global__ void __launch_bounds__(kRedThreads)
k_mr_update(double2 *__restrict__ x, double2 *__restrict__ r, const double2 *__restrict__ p, long n, MrDev *s,
            double *partials)
{
    if (s->done) return;
    const double2 a = s->alpha;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 ri = r[i];
        x[i] = cadd(x[i], cmul(a, ri));
        const double2 rn = csub(ri, cmul(a, p[i]));
        r[i] = rn;
        v[0] += cabs2(rn);
    }
    if (grid_sum<1, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0) {
        const double rn = v[0];
        const int k = s->k;
        const double bsqrt = sqrt(s->bsq);
        if (k < s->hist_cap) s->hist[k] = sqrt(rn) / bsqrt;
        if (!isfinite(rn)) {
            s->iters = k + 1;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        } else if (sqrt(rn) < s->eps * bsqrt) {
            s->iters = k;  // the reference breaks before k++ (generic_minres.cpp:193-196)
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_CONVERGED);
        } else if (k + 1 == s->max_iter) {
            s->iters = k + 1;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_MAX_ITER);
        } else {
            s->k = k + 1;
        }
    }
}

glinalg_status minres_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                           double eps, double omega, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *p, *tmp = nullptr;
    double *partials, *hist;
    MrDev *s;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&p, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 3 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&s, 1));
    MrDev h = {};
    h.eps = eps;
    h.omega = omega;
    h.max_iter = max_iter;
    h.hist = hist;
    h.hist_cap = hist_cap;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    // setup (generic_minres.cpp:155-163): r = b - A x
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[3], &s->bsq, st));
    GL_TRY(launch_apply(op, p, x, tmp, nullptr, st));
    GL_TRY(launch_sub(r, b, p, n, st));
    if (max_iter > 0) {
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            GL_TRY(launch_apply(op, p, r, tmp, &s->done, cs));
            k_mr_alpha<<<nb, kRedThreads, 0, cs>>>(p, r, n, s, partials);
            k_mr_update<<<nb, kRedThreads, 0, cs>>>(x, r, p, n, s, partials);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply(op, p, x, tmp, nullptr, st));
    GL_TRY(launch_diffnorm2(p, b, n, partials, &s->cnt[3], truersq, st));
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    std::vector<double> hh(hist_cap);
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));

    int iters, ran;
    if (max_iter > 0) {
        iters = h.iters;
        // iterations that ran: the converged one is not counted in iters (k before k++)
        ran = h.status == GLINALG_SOLVE_CONVERGED ? iters + 1 : iters;
    } else {
        iters = 0;
        ran = 0;
        h.status = GLINALG_SOLVE_MAX_ITER;
    }
    const bool success = iters != max_iter && h.status == GLINALG_SOLVE_CONVERGED;
    std::ostringstream nm;
    nm << "MR_" << omega;
    const double bsqrt = std::sqrt(h.bsq);
    for (int k = 0; k < std::min(ran, hist_cap); k++) verb.resid(nm.str(), k + 1, 2 + k, hh[k]);
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = 2 + ran;
    info->status = h.status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)ran * (112.0 * n + apply_bytes(op)) + 2 * apply_bytes(op)) * 1e-9;
    fill_name(info, "Minimum Residual (MinRes)");
    verb.summary(nm.str(), success, iters, info->ops_count, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= multishift: shared state

// Device state of a multishift solve (CR-M and BiCGstab-M).  The per-shift arrays are indexed
// by slot, the reference's permuted position: a shift that converges is swapped behind the
// live ones (generic_cr_m.cpp:445-496), and map[slot] is its original index.
struct MsDev {
    double2 alpha, beta, beta_prev, psi, delta, delta_prev, chi;
    double Apsq, rsq, bsq, eps;
    int k, max_iter, done, status, iters, napply;
    int n_rem, n_rem_before, rfc, worst_first, n_shift;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
    double2 *zeta, *zeta_prev, *beta_s, *alpha_s;
    double2 *chi_s, *rho_s, *rho_s_prev;  // BiCGstab-M
    double2 *c_x, *c_s1, *c_s2, *c_s3, *c_s4;  // BiCGstab-M: per-slot coefficients of the vector updates
    double *shifts;
    int *map;
};

// Swaps slot j with slot e (the last live one) in every per-shift array.
__device__ void ms_swap(MsDev *s, int j, int e, bool bicg)
{
    int ti = s->map[e]; s->map[e] = s->map[j]; s->map[j] = ti;
    double2 tc;
#define SW(a) tc = s->a[e]; s->a[e] = s->a[j]; s->a[j] = tc
    SW(alpha_s); SW(beta_s); SW(zeta); SW(zeta_prev);
    if (bicg) { SW(chi_s); SW(rho_s); SW(rho_s_prev); }
#undef SW
    double td = s->shifts[e]; s->shifts[e] = s->shifts[j]; s->shifts[j] = td;
}

// zeta_{k+1}, zeta_k and beta_s of every live shift (generic_cr_m.cpp:408-419, the CG-M
// recurrence of Jegerlehner, hep-lat/9612014)
__device__ void ms_zeta(MsDev *s, double2 beta, double2 beta_prev, double2 alpha)
{
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
}

__global__ void k_ms_init(double2 *const *X, double2 *const *P, const double2 *b, int ns, long n)
{
    GRID_LOOP(i, n)
    {
        const double2 bi = b[i];
        for (int j = 0; j < ns; j++) {
            X[j][i] = cmk(0.0, 0.0);
            P[j][i] = bi;
        }
    }
}

// ================================================================= CR-M

// beta = -<Ap, r> / |Ap|^2, then zeta and beta_s (generic_cr_m.cpp:404-419)
__global__ void __launch_bounds__(kRedThreads)
k_crm_beta(const double2 *__restrict__ Ap, const double2 *__restrict__ r, long n, MsDev *s, double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(Ap[i]), r[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        if (s->Apsq == 0.0) {
            s->iters = s->k + 1;
            s->n_rem_before = 0;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        const double2 beta_prev = s->beta;
        const double2 beta = cmk(-v[0] / s->Apsq, -v[1] / s->Apsq);
        s->beta_prev = beta_prev;
        s->beta = beta;
        ms_zeta(s, beta, beta_prev, s->alpha);
        s->n_rem_before = s->n_rem;
    }
}

// r = r + beta Ap, |r|^2, shift retirement and the stopping test (generic_cr_m.cpp:422-504)
__global__ void __launch_bounds__(kRedThreads)
k_crm_r(double2 *__restrict__ r, const double2 *__restrict__ Ap, long n, MsDev *s, double *partials)
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
    s->rsq = rn;
    if (k < s->hist_cap) s->hist[k] = srn / bsqrt;
    if (k % s->rfc == 0) {
        for (int j = 0; j < s->n_rem; j++) {
            if (cabsd(s->zeta[j]) * srn < s->eps * bsqrt) {
                s->n_rem--;
                if (s->n_rem != j) {
                    ms_swap(s, j, s->n_rem, false);
                    j--;
                }
            }
        }
    }
    const bool last = (k == s->max_iter - 1);
    if (!isfinite(rn)) {
        s->iters = k + 1;
        stop_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
    } else if ((s->worst_first && cabsd(s->zeta[0]) * srn < s->eps * bsqrt) || s->n_rem == 0 || last) {
        s->iters = k + 1;
        stop_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
    }
}

// alpha = -<Ap, Ar> / |Ap|^2 and alpha_s of the live shifts (generic_cr_m.cpp:511-518)
__global__ void __launch_bounds__(kRedThreads)
k_crm_alpha(const double2 *__restrict__ Ap, const double2 *__restrict__ Ar, long n, MsDev *s, double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(Ap[i]), Ar[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0) {
        const double2 alpha = cmk(-v[0] / s->Apsq, -v[1] / s->Apsq);
        s->alpha = alpha;
        for (int j = 0; j < s->n_rem; j++)
            s->alpha_s[j] = cdiv(cmul(cmul(alpha, s->zeta[j]), s->beta_s[j]), cmul(s->zeta_prev[j], s->beta));
        s->k = s->k + 1;
        s->napply++;
    }
}

// x_s -= beta_s p_s for the shifts live before this iteration's check; then, unless the solve
// stopped, p_s = zeta_s r + alpha_s p_s for the live shifts, p = r + alpha p,
// Ap = Ar + alpha Ap and |Ap|^2 (generic_cr_m.cpp:413-418, :516-534)
__global__ void __launch_bounds__(kRedThreads)
k_crm_vec(double2 *const *__restrict__ X, double2 *const *__restrict__ P, double2 *__restrict__ p,
          double2 *__restrict__ Ap, const double2 *__restrict__ r, const double2 *__restrict__ Ar, long n,
          MsDev *s, double *partials)
{
    const int nb = s->n_rem_before;
    const bool live = !s->done;
    const int na = live ? s->n_rem : 0;
    const double2 alpha = s->alpha;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 ri = r[i];
        for (int j = 0; j < nb; j++) {
            const int o = s->map[j];
            double2 *xs = X[o];
            double2 *ps = P[o];
            const double2 pv = ps[i];
            xs[i] = csub(xs[i], cmul(s->beta_s[j], pv));
            if (j < na) ps[i] = cadd(cmul(s->zeta[j], ri), cmul(s->alpha_s[j], pv));
        }
        if (live) {
            p[i] = cadd(ri, cmul(alpha, p[i]));
            const double2 a = cadd(Ar[i], cmul(alpha, Ap[i]));
            Ap[i] = a;
            v[0] += cabs2(a);
        }
    }
    if (!live) return;
    if (grid_sum<1, kRedThreads>(v, partials, &s->cnt[3]) && threadIdx.x == 0) s->Apsq = v[0];
}

// Allocates and fills the per-shift arrays of a multishift solve and the device state.
struct MsSetup {
    double2 **dX = nullptr, **dP = nullptr;
    std::vector<double2 *> hP;
    MsDev h = {};
    MsDev *s = nullptr;
    glinalg_status make(Scratch &sc, double2 *const *X_host, long n, int n_shift, int rfc, int max_iter,
                        double eps, const double *shifts, bool worst_first, int hist_cap, double *hist,
                        bool bicg, cudaStream_t st)
    {
        double2 *zeta, *zeta_prev, *beta_s, *alpha_s;
        double *d_shifts;
        int *map;
        GL_TRY(sc.alloc(&zeta, n_shift));
        GL_TRY(sc.alloc(&zeta_prev, n_shift));
        GL_TRY(sc.alloc(&beta_s, n_shift));
        GL_TRY(sc.alloc(&alpha_s, n_shift));
        GL_TRY(sc.alloc(&d_shifts, n_shift));
        GL_TRY(sc.alloc(&map, n_shift));
        GL_TRY(sc.alloc(&dX, n_shift));
        GL_TRY(sc.alloc(&dP, n_shift));
        hP.resize(n_shift);
        for (int j = 0; j < n_shift; j++) GL_TRY(sc.alloc(&hP[j], n));
        std::vector<double2> ones(n_shift, cmk(1.0, 0.0)), zeros(n_shift, cmk(0.0, 0.0));
        std::vector<int> hmap(n_shift);
        for (int j = 0; j < n_shift; j++) hmap[j] = j;
        const size_t zb = sizeof(double2) * n_shift;
        GL_CUDA(cudaMemcpyAsync(zeta, ones.data(), zb, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(zeta_prev, ones.data(), zb, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(beta_s, ones.data(), zb, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(alpha_s, zeros.data(), zb, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(d_shifts, shifts, sizeof(double) * n_shift, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(map, hmap.data(), sizeof(int) * n_shift, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(dX, X_host, sizeof(double2 *) * n_shift, cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(dP, hP.data(), sizeof(double2 *) * n_shift, cudaMemcpyHostToDevice, st));
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
        if (bicg) {
            double2 **arr[8] = {&h.chi_s, &h.rho_s, &h.rho_s_prev, &h.c_x, &h.c_s1, &h.c_s2, &h.c_s3, &h.c_s4};
            for (double2 **a : arr) GL_TRY(sc.alloc(a, n_shift));
            GL_CUDA(cudaMemcpyAsync(h.chi_s, zeros.data(), zb, cudaMemcpyHostToDevice, st));
            GL_CUDA(cudaMemcpyAsync(h.rho_s, ones.data(), zb, cudaMemcpyHostToDevice, st));
            GL_CUDA(cudaMemcpyAsync(h.rho_s_prev, ones.data(), zb, cudaMemcpyHostToDevice, st));
        }
        GL_TRY(sc.alloc(&s, 1));
        GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));
        return GLINALG_SUCCESS;
    }
};

// The end of a multishift solve: explicit residuals |(A + sigma_j) x_j - b|^2 in the caller's
// order (generic_cr_m.cpp:581-593), the info fields and the summary line.
static glinalg_status ms_finish(const glinalg_operator_s *op, double2 *const *X_host, const double2 *b,
                                int n_shift, const double *shifts, int max_iter, MsDev *s, double *hist,
                                int hist_cap, double2 *work, double2 *tmp, double *partials, Scratch &sc,
                                EventTimer &tm, const Verb &verb, const char *name, int ops_base,
                                int ops_step, double gbytes_per_iter, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    MsDev h;
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double *res;
    GL_TRY(sc.alloc(&res, n_shift));
    for (int j = 0; j < n_shift; j++) {
        GL_TRY(launch_apply_shifted(op, work, X_host[j], tmp, shifts[j], st));
        GL_TRY(launch_diffnorm2(work, b, n, partials, &s->cnt[3], res + j, st));
    }
    tm.stop(st);
    std::vector<double> hres(n_shift), hh(hist_cap);
    GL_CUDA(cudaMemcpyAsync(hres.data(), res, sizeof(double) * n_shift, cudaMemcpyDeviceToHost, st));
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
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
    const double bsqrt = std::sqrt(h.bsq);
    for (int k = 0; k < std::min(iters, hist_cap); k++) verb.resid(name, k + 1, ops_base + ops_step * k, hh[k]);
    std::vector<double> relres(n_shift);
    for (int j = 0; j < n_shift; j++) {
        relres[j] = std::sqrt(hres[j]) / bsqrt;
        if (info->resSqmrhs) info->resSqmrhs[j] = hres[j];
    }
    info->n_rhs = n_shift;
    info->resSq = 0.0;  // the reference leaves it at 0 (generic_cr_m.cpp:618)
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = 1 + applies + n_shift;
    info->status = h.status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)iters * gbytes_per_iter + (n_shift + 1) * apply_bytes(op)) * 1e-9;
    fill_name(info, name);
    verb.summary_multi(info->success != 0, iters, info->ops_count, relres.data(), n_shift);
    return GLINALG_SUCCESS;
}

glinalg_status cr_m_fp64(const glinalg_operator_s *op, double2 *const *X_host, const double2 *b, int n_shift,
                         int rfc, int max_iter, double eps, const double *shifts, bool worst_first,
                         const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *p, *Ap, *Ar, *tmp = nullptr;
    double *partials, *hist;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.alloc(&p, n));
    GL_TRY(sc.alloc(&Ap, n));
    GL_TRY(sc.alloc(&Ar, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 2 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    MsSetup m;
    GL_TRY(m.make(sc, X_host, n, n_shift, rfc, max_iter, eps, shifts, worst_first, hist_cap, hist, false, st));
    MsDev *s = m.s;

    EventTimer tm;
    tm.start(st);
    // setup (generic_cr_m.cpp:383-401): x_s = 0, p_s = p = r = b, Ap = A p, |Ap|^2
    const int vg = vgrid(n);
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[3], &s->bsq, st));
    k_ms_init<<<vg, 256, 0, st>>>(m.dX, m.dP, b, n_shift, n);
    GL_CUDA(cudaMemcpyAsync(p, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_CUDA(cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply(op, Ap, p, tmp, nullptr, st));
    GL_TRY(launch_norm2(Ap, n, partials, &s->cnt[3], &s->Apsq, st));
    if (max_iter > 0) {
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            k_crm_beta<<<nb, kRedThreads, 0, cs>>>(Ap, r, n, s, partials);
            k_crm_r<<<nb, kRedThreads, 0, cs>>>(r, Ap, n, s, partials);
            GL_TRY(launch_apply(op, Ar, r, tmp, &s->done, cs));
            k_crm_alpha<<<nb, kRedThreads, 0, cs>>>(Ap, Ar, n, s, partials);
            k_crm_vec<<<nb, kRedThreads, 0, cs>>>(m.dX, m.dP, p, Ap, r, Ar, n, s, partials);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    return ms_finish(op, X_host, b, n_shift, shifts, max_iter, s, hist, hist_cap, Ap, tmp, partials, sc, tm,
                     verb, "CR-M", 1, 1, apply_bytes(op) + 176.0 * n + 64.0 * n * n_shift, info, st);
}

// ================================================================= BiCGstab-M

// The shadow vector of the reference is conj(b) (generic_bicgstab_m.cpp:491-492), so
// <wdag, v> = sum_i conj(wdag_i) v_i = sum_i b_i v_i; wdag is kept as a field.

__global__ void k_conj(double2 *__restrict__ out, const double2 *__restrict__ in, long n)
{
    GRID_LOOP(i, n) out[i] = cconj(in[i]);
}

// delta = <wdag, r>, psi = <wdag, As> / delta (generic_bicgstab_m.cpp:493-496)
__global__ void __launch_bounds__(kRedThreads)
k_bm_setup(const double2 *__restrict__ wdag, const double2 *__restrict__ r, const double2 *__restrict__ As,
           long n, MsDev *s, double *partials)
{
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 wc = cconj(wdag[i]);
        const double2 d1 = cmul(wc, r[i]), d2 = cmul(wc, As[i]);
        v[0] += d1.x;
        v[1] += d1.y;
        v[2] += d2.x;
        v[3] += d2.y;
    }
    if (grid_sum<4, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        const double2 delta = cmk(v[0], v[1]);
        s->delta = s->delta_prev = delta;
        s->psi = cdiv(cmk(v[2], v[3]), delta);
    }
}

// beta = -1 / psi, w = r + beta As (generic_bicgstab_m.cpp:502-511)
__global__ void k_bm_w(double2 *__restrict__ w, const double2 *__restrict__ r, const double2 *__restrict__ As,
                       long n, MsDev *s)
{
    if (s->done) return;
    const double2 beta = cdiv(cmk(-1.0, 0.0), s->psi);
    GRID_LOOP(i, n) w[i] = cadd(r[i], cmul(beta, As[i]));
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s->beta_prev = s->beta;
        s->beta = beta;
    }
}

// chi = <Aw, w> / |Aw|^2, then the per-shift zeta, beta_s, chi_s and rho_s
// (generic_bicgstab_m.cpp:517-549)
__global__ void __launch_bounds__(kRedThreads)
k_bm_chi(const double2 *__restrict__ Aw, const double2 *__restrict__ w, long n, MsDev *s, double *partials)
{
    if (s->done) return;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 a = Aw[i];
        const double2 d = cmul(cconj(a), w[i]);
        v[0] += d.x;
        v[1] += d.y;
        v[2] += cabs2(a);
    }
    if (grid_sum<3, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0) {
        const double2 chi = cmk(v[0] / v[2], v[1] / v[2]);
        s->chi = chi;
        s->napply++;  // Aw = A w
        ms_zeta(s, s->beta, s->beta_prev, s->alpha);
        for (int j = 0; j < s->n_rem; j++) {
            const double sh = s->shifts[j];
            const double2 den = cmk(1.0 + chi.x * sh, chi.y * sh);
            s->chi_s[j] = cdiv(chi, den);
            const double2 rho = s->rho_s[j];
            s->rho_s[j] = cdiv(rho, den);
            s->rho_s_prev[j] = rho;
            s->c_x[j] = cmul(cmul(s->chi_s[j], rho), s->zeta[j]);
        }
        s->n_rem_before = s->n_rem;
    }
}

// r_prev = r, r = w - chi Aw, x_s = x_s - beta_s s_s + chi_s rho_s_prev zeta_s w; |r|^2 and
// <wdag, r>; then shift retirement, the stopping test, and the next alpha, alpha_s and the
// coefficients of the s_s update (generic_bicgstab_m.cpp:523-622)
__global__ void __launch_bounds__(kRedThreads)
k_bm_r(double2 *__restrict__ r, double2 *__restrict__ r_prev, const double2 *__restrict__ w,
       const double2 *__restrict__ Aw, const double2 *__restrict__ wdag, double2 *const *__restrict__ X,
       double2 *const *__restrict__ S, long n, MsDev *s, double *partials)
{
    if (s->done) return;
    const double2 chi = s->chi;
    const int nb = s->n_rem_before;
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 wi = w[i];
        r_prev[i] = r[i];
        const double2 rn = csub(wi, cmul(chi, Aw[i]));
        r[i] = rn;
        for (int j = 0; j < nb; j++) {
            const int o = s->map[j];
            double2 *xs = X[o];
            xs[i] = cadd(csub(xs[i], cmul(s->beta_s[j], S[o][i])), cmul(s->c_x[j], wi));
        }
        const double2 d = cmul(cconj(wdag[i]), rn);
        v[0] += cabs2(rn);
        v[1] += d.x;
        v[2] += d.y;
    }
    if (!(grid_sum<3, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0)) return;
    const double rn = v[0];
    const int k = s->k;
    const double bsqrt = sqrt(s->bsq), srn = sqrt(rn);
    s->rsq = rn;
    if (k < s->hist_cap) s->hist[k] = srn / bsqrt;
    if (k % s->rfc == 0) {
        for (int j = 0; j < s->n_rem; j++) {
            if (cabsd(cmul(s->zeta[j], s->rho_s[j])) * srn < s->eps * bsqrt) {
                s->n_rem--;
                if (s->n_rem != j) {
                    ms_swap(s, j, s->n_rem, true);
                    j--;
                }
            }
        }
    }
    const bool last = (k == s->max_iter - 1);
    if (rn != rn) {
        s->iters = k + 1;
        stop_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        return;
    }
    if ((s->worst_first && cabsd(cmul(s->zeta[0], s->rho_s[0])) * srn < s->eps * bsqrt) || s->n_rem == 0 || last) {
        s->iters = k + 1;
        stop_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
        return;
    }
    s->delta_prev = s->delta;
    s->delta = cmk(v[1], v[2]);
    const double2 alpha = cdiv(cmul(cneg(s->beta), s->delta), cmul(s->delta_prev, chi));
    s->alpha = alpha;
    for (int j = 0; j < s->n_rem; j++) {
        s->alpha_s[j] = cdiv(cmul(cmul(alpha, s->zeta[j]), s->beta_s[j]), cmul(s->zeta_prev[j], s->beta));
        s->c_s1[j] = cmul(s->zeta[j], s->rho_s[j]);
        s->c_s2[j] = cdiv(s->chi_s[j], s->beta_s[j]);
        s->c_s3[j] = cmul(s->zeta[j], s->rho_s_prev[j]);
        s->c_s4[j] = cmul(s->zeta_prev[j], s->rho_s_prev[j]);
    }
}

// s = r + alpha (s - chi As); s_s = zeta rho r + alpha_s (s_s - chi_s / beta_s (zeta rho_prev w
// - zeta_prev rho_prev r_prev)), or s_s = s for a zero shift (generic_bicgstab_m.cpp:624-650)
__global__ void k_bm_s(double2 *__restrict__ sv, const double2 *__restrict__ r, const double2 *__restrict__ As,
                       const double2 *__restrict__ w, const double2 *__restrict__ r_prev,
                       double2 *const *__restrict__ S, long n, const MsDev *s)
{
    if (s->done) return;
    const double2 alpha = s->alpha, chi = s->chi;
    const int na = s->n_rem;
    GRID_LOOP(i, n)
    {
        const double2 ri = r[i];
        const double2 snew = cadd(ri, cmul(alpha, csub(sv[i], cmul(chi, As[i]))));
        sv[i] = snew;
        const double2 wi = w[i], rp = r_prev[i];
        for (int j = 0; j < na; j++) {
            double2 *ss = S[s->map[j]];
            if (fabs(s->shifts[j]) != 0.0) {
                const double2 inner = csub(cmul(s->c_s3[j], wi), cmul(s->c_s4[j], rp));
                ss[i] = cadd(cmul(s->c_s1[j], ri), cmul(s->alpha_s[j], csub(ss[i], cmul(s->c_s2[j], inner))));
            } else {
                ss[i] = snew;
            }
        }
    }
}

// psi = <wdag, As> / delta; psi == 0 is a breakdown (generic_bicgstab_m.cpp:656-663)
__global__ void __launch_bounds__(kRedThreads)
k_bm_psi(const double2 *__restrict__ wdag, const double2 *__restrict__ As, long n, MsDev *s, double *partials)
{
    if (s->done) return;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(wdag[i]), As[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[3]) && threadIdx.x == 0) {
        s->napply++;  // As = A s
        const double2 psi = cdiv(cmk(v[0], v[1]), s->delta);
        s->psi = psi;
        if (cabsd(psi) == 0.0) {
            s->iters = s->k + 1;
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->k = s->k + 1;
    }
}

glinalg_status bicgstab_m_fp64(const glinalg_operator_s *op, double2 *const *X_host, const double2 *b,
                               int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                               bool worst_first, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r, *r_prev, *sv, *As, *w, *Aw, *wdag, *tmp = nullptr;
    double *partials, *hist;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nb = reduction_blocks(n);
    double2 **vs[7] = {&r, &r_prev, &sv, &As, &w, &Aw, &wdag};
    for (double2 **v : vs) GL_TRY(sc.alloc(v, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 4 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    MsSetup m;
    GL_TRY(m.make(sc, X_host, n, n_shift, rfc, max_iter, eps, shifts, worst_first, hist_cap, hist, true, st));
    MsDev *s = m.s;

    EventTimer tm;
    tm.start(st);
    // setup (generic_bicgstab_m.cpp:474-496): x_s = 0, s_s = s = r = r_prev = b, As = A s,
    // wdag = conj(r), delta, psi
    const int vg = vgrid(n);
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[3], &s->bsq, st));
    k_ms_init<<<vg, 256, 0, st>>>(m.dX, m.dP, b, n_shift, n);
    GL_CUDA(cudaMemcpyAsync(sv, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_CUDA(cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_CUDA(cudaMemcpyAsync(r_prev, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply(op, As, sv, tmp, nullptr, st));
    k_conj<<<vg, 256, 0, st>>>(wdag, r, n);
    k_bm_setup<<<nb, kRedThreads, 0, st>>>(wdag, r, As, n, s, partials);
    GL_CUDA(cudaGetLastError());
    if (max_iter > 0) {
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            k_bm_w<<<vg, 256, 0, cs>>>(w, r, As, n, s);
            GL_TRY(launch_apply(op, Aw, w, tmp, &s->done, cs));
            k_bm_chi<<<nb, kRedThreads, 0, cs>>>(Aw, w, n, s, partials);
            k_bm_r<<<nb, kRedThreads, 0, cs>>>(r, r_prev, w, Aw, wdag, m.dX, m.dP, n, s, partials);
            k_bm_s<<<vg, 256, 0, cs>>>(sv, r, As, w, r_prev, m.dP, n, s);
            GL_TRY(launch_apply(op, As, sv, tmp, &s->done, cs));
            k_bm_psi<<<nb, kRedThreads, 0, cs>>>(wdag, As, n, s, partials);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    return ms_finish(op, X_host, b, n_shift, shifts, max_iter, s, hist, hist_cap, Aw, tmp, partials, sc, tm,
                     verb, "BICGSTAB-M", 2, 2, 2 * apply_bytes(op) + 288.0 * n + 96.0 * n * n_shift, info, st);
}

// ================================================================= BiCGstab-l

constexpr int kMaxL = kMaxBicgstabL;

struct BlDev {
    double2 rho0, rho1, alpha, omega, beta;
    double bsq, eps;
    int k, max_iter, l, done, status, iters, success;
    unsigned cnt[4];
    double *hist;
    int hist_cap;
    double sigma[kMaxL + 1];
    double2 gamma[kMaxL + 1], gp[kMaxL + 1], gpp[kMaxL + 1];
    double2 tau[(kMaxL + 1) * (kMaxL + 1)];
};

// rho1 = <r0, r_j>, beta = alpha rho1 / rho0, rho0 = rho1; the cycle's first step first sets
// rho0 = -omega rho0 (generic_bicgstab_l.cpp:391-400)
__global__ void __launch_bounds__(kRedThreads)
k_bl_rho(const double2 *__restrict__ r0, double2 *const *__restrict__ R, int j, long n, BlDev *s, double *partials)
{
    if (s->done) return;
    const double2 *rj = R[j];
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(r0[i]), rj[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        if (j == 0) s->rho0 = cmul(s->rho0, cneg(s->omega));
        const double2 rho1 = cmk(v[0], v[1]);
        s->rho1 = rho1;
        s->beta = cdiv(cmul(s->alpha, rho1), s->rho0);
        s->rho0 = rho1;
    }
}

// u_i = r_i - beta u_i for i = 0..j (generic_bicgstab_l.cpp:402-409)
__global__ void k_bl_u(double2 *const *__restrict__ R, double2 *const *__restrict__ U, int j, long n,
                       const BlDev *s)
{
    if (s->done) return;
    const double2 beta = s->beta;
    GRID_LOOP(h, n)
    {
        for (int i = 0; i <= j; i++) U[i][h] = csub(R[i][h], cmul(beta, U[i][h]));
    }
}

// alpha = rho0 / <r0, u_{j+1}> (generic_bicgstab_l.cpp:415)
__global__ void __launch_bounds__(kRedThreads)
k_bl_alpha(const double2 *__restrict__ r0, double2 *const *__restrict__ U, int j, long n, BlDev *s,
           double *partials)
{
    if (s->done) return;
    const double2 *u = U[j + 1];
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 d = cmul(cconj(r0[i]), u[i]);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[1]) && threadIdx.x == 0)
        s->alpha = cdiv(s->rho0, cmk(v[0], v[1]));
}

// r_i = r_i - alpha u_{i+1} for i = 0..j, x = x + alpha u_0 (generic_bicgstab_l.cpp:417-432)
__global__ void k_bl_r(double2 *const *__restrict__ R, double2 *const *__restrict__ U, double2 *__restrict__ x,
                       int j, long n, const BlDev *s)
{
    if (s->done) return;
    const double2 alpha = s->alpha;
    GRID_LOOP(h, n)
    {
        for (int i = 0; i <= j; i++) R[i][h] = csub(R[i][h], cmul(alpha, U[i + 1][h]));
        x[h] = cadd(x[h], cmul(alpha, U[0][h]));
    }
}

// One step of the modified Gram-Schmidt of the MR part (generic_bicgstab_l.cpp:438-456): with
// iu > 0, first r_j -= tau[iu][j] r_iu; then either tau[id][j] = <r_id, r_j> / sigma[id]
// (id > 0) or sigma[j] = |r_j|^2 and gamma'_j = <r_j, r_0> / sigma[j] (id == 0).  After the
// last step (j == l, id == 0) the last block also forms gamma, omega and gamma''
// (generic_bicgstab_l.cpp:459-479).
__global__ void __launch_bounds__(kRedThreads)
k_bl_gs(double2 *const *__restrict__ R, int j, int iu, int id, long n, BlDev *s, double *partials)
{
    if (s->done) return;
    const int L1 = s->l + 1;
    double2 *rj = R[j];
    const double2 *ru = iu > 0 ? R[iu] : nullptr;
    const double2 *rd = id > 0 ? R[id] : R[0];
    const double2 t = iu > 0 ? s->tau[iu * L1 + j] : cmk(0.0, 0.0);
    double v[3] = {0.0, 0.0, 0.0};
    for (long h = blockIdx.x * (long)kRedThreads + threadIdx.x; h < n; h += (long)gridDim.x * kRedThreads) {
        double2 x = rj[h];
        if (iu > 0) {
            x = csub(x, cmul(t, ru[h]));
            rj[h] = x;
        }
        if (id > 0) {
            const double2 d = cmul(cconj(rd[h]), x);
            v[0] += d.x;
            v[1] += d.y;
        } else {
            const double2 d = cmul(cconj(x), rd[h]);
            v[0] += d.x;
            v[1] += d.y;
            v[2] += cabs2(x);
        }
    }
    if (!(grid_sum<3, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0)) return;
    if (id > 0) {
        const double sg = s->sigma[id];
        s->tau[id * L1 + j] = cmk(v[0] / sg, v[1] / sg);
        return;
    }
    s->sigma[j] = v[2];
    s->gp[j] = cmk(v[0] / v[2], v[1] / v[2]);
    const int l = s->l;
    if (j < l) return;
    s->gamma[l] = s->gp[l];
    s->omega = s->gamma[l];
    for (int jj = l - 1; jj > 0; jj--) {
        double2 g = s->gp[jj];
        for (int i = jj + 1; i <= l; i++) g = csub(g, cmul(s->tau[jj * L1 + i], s->gamma[i]));
        s->gamma[jj] = g;
    }
    for (int jj = 1; jj < l; jj++) {
        double2 g = s->gamma[jj + 1];
        for (int i = jj + 1; i < l; i++) g = cadd(g, cmul(s->tau[jj * L1 + i], s->gamma[i + 1]));
        s->gpp[jj] = g;
    }
}

// x += gamma_1 r_0, u_0 -= gamma_l u_l, r_0 -= gamma'_l r_l, then for j = 1..l-1: u_0 -= gamma_j
// u_j, x += gamma''_j r_j, r_0 -= gamma'_j r_j; sigma_0 = |r_0|^2 and the stopping test
// (generic_bicgstab_l.cpp:482-510)
__global__ void __launch_bounds__(kRedThreads)
k_bl_final(double2 *const *__restrict__ R, double2 *const *__restrict__ U, double2 *__restrict__ x, long n,
           BlDev *s, double *partials)
{
    if (s->done) return;
    const int l = s->l;
    double v[1] = {0.0};
    for (long h = blockIdx.x * (long)kRedThreads + threadIdx.x; h < n; h += (long)gridDim.x * kRedThreads) {
        double2 xv = x[h], u0 = U[0][h], r0 = R[0][h];
        xv = cadd(xv, cmul(s->gamma[1], r0));
        u0 = csub(u0, cmul(s->gamma[l], U[l][h]));
        r0 = csub(r0, cmul(s->gp[l], R[l][h]));
        for (int j = 1; j < l; j++) {
            const double2 rj = R[j][h];
            u0 = csub(u0, cmul(s->gamma[j], U[j][h]));
            xv = cadd(xv, cmul(s->gpp[j], rj));
            r0 = csub(r0, cmul(s->gp[j], rj));
        }
        x[h] = xv;
        U[0][h] = u0;
        R[0][h] = r0;
        v[0] += cabs2(r0);
    }
    if (!(grid_sum<1, kRedThreads>(v, partials, &s->cnt[3]) && threadIdx.x == 0)) return;
    const double sg = v[0];
    const int k = s->k;
    const double bsqrt = sqrt(s->bsq);
    s->sigma[0] = sg;
    const int cyc = k / l;
    if (cyc < s->hist_cap) s->hist[cyc] = sqrt(sg) / bsqrt;
    if (!isfinite(sg)) {
        s->iters = k + 1;
        s->success = 0;
        stop_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
    } else if (sqrt(sg) < s->eps * bsqrt) {
        // success is judged against max_iter - 1 (generic_bicgstab_l.cpp:515)
        s->iters = k + 1;
        s->success = k >= s->max_iter - 1 ? 0 : 1;
        stop_dev(&s->done, &s->status, GLINALG_SOLVE_CONVERGED);
    } else if (k + l >= s->max_iter) {
        s->iters = k + l + 1;
        s->success = 0;
        stop_dev(&s->done, &s->status, GLINALG_SOLVE_MAX_ITER);
    } else {
        s->k = k + l;
    }
}

glinalg_status bicgstab_l_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                               double eps, int l, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    Scratch sc(st);
    double2 *r0, *tmp = nullptr, **dR, **dU;
    double *partials, *hist;
    BlDev *s;
    const int ncyc = max_iter > 0 ? (max_iter + l - 1) / l : 1;
    const int hist_cap = verb.level == 3 ? ncyc : 0;
    const int nb = reduction_blocks(n);
    std::vector<double2 *> hR(l + 1), hU(l + 1);
    GL_TRY(sc.alloc(&r0, n));
    for (int i = 0; i <= l; i++) {
        GL_TRY(sc.zeros(&hR[i], n));
        GL_TRY(sc.zeros(&hU[i], n));
    }
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&dR, l + 1));
    GL_TRY(sc.alloc(&dU, l + 1));
    GL_TRY(sc.alloc(&partials, 3 * (size_t)nb));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&s, 1));
    GL_CUDA(cudaMemcpyAsync(dR, hR.data(), sizeof(double2 *) * (l + 1), cudaMemcpyHostToDevice, st));
    GL_CUDA(cudaMemcpyAsync(dU, hU.data(), sizeof(double2 *) * (l + 1), cudaMemcpyHostToDevice, st));
    BlDev h = {};
    h.rho0 = cmk(1.0, 0.0);
    h.alpha = cmk(0.0, 0.0);
    h.omega = cmk(1.0, 0.0);
    h.eps = eps;
    h.max_iter = max_iter;
    h.l = l;
    h.hist = hist;
    h.hist_cap = hist_cap;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    // setup (generic_bicgstab_l.cpp:374-384): r_0 = b - A x, sigma_0, r0 (shadow) = r_0, u_0 = 0
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[3], &s->bsq, st));
    GL_TRY(launch_apply(op, hU[0], x, tmp, nullptr, st));
    GL_TRY(launch_sub(hR[0], b, hU[0], n, st));
    GL_CUDA(cudaMemcpyAsync(r0, hR[0], sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_CUDA(cudaMemsetAsync(hU[0], 0, sizeof(double2) * n, st));
    if (max_iter > 0) {
        const int vg = vgrid(n);
        GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
            for (int j = 0; j < l; j++) {
                k_bl_rho<<<nb, kRedThreads, 0, cs>>>(r0, dR, j, n, s, partials);
                k_bl_u<<<vg, 256, 0, cs>>>(dR, dU, j, n, s);
                GL_TRY(launch_apply(op, hU[j + 1], hU[j], tmp, &s->done, cs));
                k_bl_alpha<<<nb, kRedThreads, 0, cs>>>(r0, dU, j, n, s, partials);
                k_bl_r<<<vg, 256, 0, cs>>>(dR, dU, x, j, n, s);
                GL_TRY(launch_apply(op, hR[j + 1], hR[j], tmp, &s->done, cs));
            }
            for (int j = 1; j <= l; j++) {
                if (j == 1) {
                    k_bl_gs<<<nb, kRedThreads, 0, cs>>>(dR, 1, 0, 0, n, s, partials);
                } else {
                    k_bl_gs<<<nb, kRedThreads, 0, cs>>>(dR, j, 0, 1, n, s, partials);
                    for (int i = 1; i < j; i++)
                        k_bl_gs<<<nb, kRedThreads, 0, cs>>>(dR, j, i, i + 1 < j ? i + 1 : 0, n, s, partials);
                }
            }
            k_bl_final<<<nb, kRedThreads, 0, cs>>>(dR, dU, x, n, s, partials);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply(op, hU[0], x, tmp, nullptr, st));
    GL_TRY(launch_diffnorm2(hU[0], b, n, partials, &s->cnt[3], truersq, st));
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    std::vector<double> hh(hist_cap);
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));

    int iters, cycles;
    bool success;
    if (max_iter > 0) {
        iters = h.iters;
        success = h.success != 0;
        cycles = (iters - 1 + (h.status == GLINALG_SOLVE_CONVERGED || h.status == GLINALG_SOLVE_NONFINITE ? l : 0)) / l;
    } else {
        iters = 1;
        success = false;
        cycles = 0;
        h.status = GLINALG_SOLVE_MAX_ITER;
    }
    const std::string nm = "BiCGStab-" + std::to_string(l);
    const double bsqrt = std::sqrt(h.bsq);
    for (int c = 0; c < std::min(cycles, hist_cap); c++) verb.resid(nm, (c + 1) * l, 1 + 2 * l * (c + 1), hh[c]);
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = 2 + 2 * l * cycles;
    info->status = h.status;
    info->device_ms = tm.ms();
    // per cycle: 2l applications, the BiCG updates (~3 (j+1) fields per step), MR (~l^2 / 2 passes)
    info->gbytes = ((double)cycles * (2.0 * l * apply_bytes(op) + 16.0 * n * (4.0 * l * l + 10.0 * l)) +
                    2 * apply_bytes(op)) * 1e-9;
    fill_name(info, nm);
    verb.summary(nm, success, iters, info->ops_count, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= preconditioners

// identity_preconditioner copies (generic_precond.cpp:34-42); minres_preconditioner runs
// n_step MinRes iterations (omega 1) and gcr_preconditioner n_step GCR iterations, both to
// rel_res and from the guess in z (the callers zero it; generic_precond.cpp:53-77).  Their
// own operator counts do not enter the outer solve's ops_count, as in the reference.
glinalg_status precond_apply(const Precond &pc, const glinalg_operator_s *op, double2 *z, const double2 *r,
                             const Verb &vprec, cudaStream_t st)
{
    const glinalg_operator_s *pop = pc.op ? pc.op : op;
    glinalg_info tmp = {};
    switch (pc.kind) {
    case GLINALG_PRECOND_MINRES: return minres_fp64(pop, z, r, pc.n_step, pc.rel_res, 1.0, vprec, &tmp, st);
    case GLINALG_PRECOND_GCR: return gcr_fp64(pop, z, r, pc.n_step, pc.rel_res, vprec, &tmp, st);
    case GLINALG_PRECOND_MG: return mg_apply(pc.mg, pc.level, z, r, vprec, st);
    default:
        GL_CUDA(cudaMemcpyAsync(z, r, sizeof(double2) * op->size, cudaMemcpyDeviceToDevice, st));
        return GLINALG_SUCCESS;
    }
}

// ================================================================= FPCG / VPGCR

struct FxDev {
    double2 alpha;
    double rsq, bsq, eps;
    int k, max_iter, done, status;
    unsigned cnt[4];
};

// FPCG (mode 0): alpha = <p, r> / <p, Ap>, keeping <p, Ap> (generic_cg_flex_precond.cpp:286);
// VPGCR (mode 1): alpha = <Ap, r> / |Ap|^2, keeping |Ap|^2 (generic_gcr_var_precond.cpp:284).
// den[k] keeps the denominator for the later A-orthogonalisations against this direction.
__global__ void __launch_bounds__(kRedThreads)
k_fx_alpha(const double2 *__restrict__ p, const double2 *__restrict__ Ap, const double2 *__restrict__ r, long n,
           int mode, FxDev *s, double2 *den, double *partials)
{
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 a = Ap[i], ri = r[i];
        if (mode == 0) {
            const double2 pc = cconj(p[i]);
            const double2 d1 = cmul(pc, ri), d2 = cmul(pc, a);
            v[0] += d1.x;
            v[1] += d1.y;
            v[2] += d2.x;
            v[3] += d2.y;
        } else {
            const double2 d1 = cmul(cconj(a), ri);
            v[0] += d1.x;
            v[1] += d1.y;
            v[2] += cabs2(a);
        }
    }
    if (grid_sum<4, kRedThreads>(v, partials, &s->cnt[0]) && threadIdx.x == 0) {
        const double2 d = cmk(v[2], v[3]);
        den[s->k] = d;
        if (v[2] == 0.0 && v[3] == 0.0) {
            stop_dev(&s->done, &s->status, GLINALG_SOLVE_BREAKDOWN);
            return;
        }
        s->alpha = mode == 0 ? cdiv(cmk(v[0], v[1]), d) : cmk(v[0] / v[2], v[1] / v[2]);
    }
}

// x += alpha p, r -= alpha Ap, |r|^2 and the stopping test (generic_cg_flex_precond.cpp:290-301)
__global__ void __launch_bounds__(kRedThreads)
k_fx_update(double2 *__restrict__ x, double2 *__restrict__ r, const double2 *__restrict__ p,
            const double2 *__restrict__ Ap, long n, FxDev *s, double *partials)
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
        const bool last = (k == s->max_iter - 1);
        if (!isfinite(rn)) stop_dev(&s->done, &s->status, GLINALG_SOLVE_NONFINITE);
        else if (sqrt(rn) < s->eps * bsqrt || last)
            stop_dev(&s->done, &s->status, last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED);
        else s->k = k + 1;
    }
}

// beta_i = -<Ap_i, y> / den[i] for i in [i0, i0 + cnt), cnt <= 8; y = z (FPCG,
// generic_cg_flex_precond.cpp:319) or A z (VPGCR, generic_gcr_var_precond.cpp:317)
constexpr int kFxDots = 8;
__global__ void __launch_bounds__(kRedThreads)
k_fx_betas(double2 *const *__restrict__ Aps, const double2 *__restrict__ y, long n, int i0, int cnt,
           const double2 *__restrict__ den, int mode, double2 *betas, double *partials, unsigned *counter)
{
    double v[2 * kFxDots];
#pragma unroll
    for (int j = 0; j < 2 * kFxDots; j++) v[j] = 0.0;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 yi = y[i];
#pragma unroll
        for (int j = 0; j < kFxDots; j++) {
            if (j < cnt) {
                const double2 d = cmul(cconj(Aps[i0 + j][i]), yi);
                v[2 * j] += d.x;
                v[2 * j + 1] += d.y;
            }
        }
    }
    if (grid_sum<2 * kFxDots, kRedThreads>(v, partials, counter) && threadIdx.x == 0) {
        for (int j = 0; j < cnt; j++) {
            const double2 d = cmk(-v[2 * j], -v[2 * j + 1]);
            const double2 dn = den[i0 + j];
            betas[i0 + j] = mode == 0 ? cdiv(d, dn) : cmk(d.x / dn.x, d.y / dn.x);
        }
    }
}

// p = z + sum_i beta_i p_i, Ap = Az + sum_i beta_i Ap_i, in order i = 0..m-1
__global__ void k_fx_combine(double2 *__restrict__ p, double2 *__restrict__ Ap, const double2 *__restrict__ z,
                             const double2 *__restrict__ Az, double2 *const *__restrict__ ps,
                             double2 *const *__restrict__ Aps, const double2 *__restrict__ betas, int m, long n)
{
    GRID_LOOP(i, n)
    {
        double2 pv = z[i], av = Az[i];
        for (int j = 0; j < m; j++) {
            const double2 bj = betas[j];
            pv = cadd(pv, cmul(bj, ps[j][i]));
            av = cadd(av, cmul(bj, Aps[j][i]));
        }
        p[i] = pv;
        Ap[i] = av;
    }
}

// mode 0: flexibly preconditioned CG, updating phi in place (generic_cg_flex_precond.cpp:223-364);
// mode 1: variably preconditioned GCR (generic_gcr_var_precond.cpp:220-366).  Driven from the
// host one iteration at a time; the DETAIL lines are printed as the iterations complete, so
// the preconditioner's own lines interleave with them as in the reference.
glinalg_status flex_fp64(int mode, const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                         double eps, const Precond &pc, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    const long n = op->size;
    const char *alg = mode == 0 ? "FPCG" : "VPGCR";
    Scratch sc(st);
    double2 *r, *z, *Az, *tmp = nullptr, *betas, *den;
    double *partials;
    double2 **d_ps, **d_Aps;
    FxDev *s;
    const int cap = (max_iter > 0 ? max_iter : 1) + 1;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.zeros(&z, n));
    GL_TRY(sc.alloc(&Az, n));
    if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partials, 2 * kFxDots * (size_t)nb));
    GL_TRY(sc.alloc(&den, cap));
    GL_TRY(sc.alloc(&betas, cap));
    GL_TRY(sc.alloc(&d_ps, cap));
    GL_TRY(sc.alloc(&d_Aps, cap));
    GL_TRY(sc.alloc(&s, 1));
    FxDev h = {};
    h.eps = eps;
    h.max_iter = max_iter;
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));
    std::vector<double2 *> hp(cap), hAp(cap);
    double2 *p, *Ap;
    GL_TRY(sc.alloc(&p, n));
    GL_TRY(sc.alloc(&Ap, n));
    const Verb vprec = verb.precond_inner();
    double bsq = 0.0;

    EventTimer tm;
    tm.start(st);
    // setup: r = b - A x, z = M^-1 r, p = z, Ap = A p
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[2], &s->bsq, st));
    GL_CUDA(cudaMemcpyAsync(&bsq, &s->bsq, sizeof(double), cudaMemcpyDeviceToHost, st));
    GL_TRY(launch_apply(op, p, x, tmp, nullptr, st));
    GL_TRY(launch_sub(r, b, p, n, st));
    GL_TRY(precond_apply(pc, op, z, r, vprec, st));
    GL_CUDA(cudaMemcpyAsync(p, z, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    GL_TRY(launch_apply(op, Ap, p, tmp, nullptr, st));
    GL_CUDA(cudaStreamSynchronize(st));
    const double bsqrt = std::sqrt(bsq);
    int ops = 2, k = 0, status = GLINALG_SOLVE_CONVERGED, stored = 0;
    const int vg = vgrid(n);
    for (k = 0; k < max_iter; k++) {
        hp[k] = p;
        hAp[k] = Ap;
        stored++;
        GL_CUDA(cudaMemcpyAsync(d_ps + k, &hp[k], sizeof(double2 *), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(d_Aps + k, &hAp[k], sizeof(double2 *), cudaMemcpyHostToDevice, st));
        k_fx_alpha<<<nb, kRedThreads, 0, st>>>(p, Ap, r, n, mode, s, den, partials);
        k_fx_update<<<nb, kRedThreads, 0, st>>>(x, r, p, Ap, n, s, partials);
        GL_CUDA(cudaGetLastError());
        FxDev hs;
        GL_CUDA(cudaMemcpyAsync(&hs, s, sizeof(hs), cudaMemcpyDeviceToHost, st));
        GL_CUDA(cudaStreamSynchronize(st));
        if (hs.status != GLINALG_SOLVE_BREAKDOWN) verb.resid(alg, k + 1, ops, std::sqrt(hs.rsq) / bsqrt);
        if (hs.done) {
            status = hs.status;
            break;
        }
        GL_CUDA(cudaMemsetAsync(z, 0, sizeof(double2) * n, st));
        GL_TRY(precond_apply(pc, op, z, r, vprec, st));
        GL_TRY(launch_apply(op, Az, z, tmp, nullptr, st));
        ops++;
        const double2 *y = mode == 0 ? z : Az;
        for (int i0 = 0; i0 <= k; i0 += kFxDots) {
            const int cnt = std::min(kFxDots, k + 1 - i0);
            k_fx_betas<<<nb, kRedThreads, 0, st>>>(d_Aps, y, n, i0, cnt, den, mode, betas, partials, &s->cnt[3]);
        }
        GL_TRY(sc.alloc(&p, n));
        GL_TRY(sc.alloc(&Ap, n));
        k_fx_combine<<<vg, 256, 0, st>>>(p, Ap, z, Az, d_ps, d_Aps, betas, k + 1, n);
        GL_CUDA(cudaGetLastError());
    }
    int iters;
    bool success;
    if (max_iter > 0) {
        // FPCG reports k + 1; VPGCR the number of stored directions (generic_gcr_var_precond.cpp:350-362),
        // the same once the loop has run
        iters = k + 1;
        success = status == GLINALG_SOLVE_CONVERGED;
    } else {
        iters = mode == 0 ? 1 : 0;
        success = !(0 == max_iter - 1);
        status = success ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER;
    }
    (void)stored;
    double *truersq;
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(launch_apply(op, Az, x, tmp, nullptr, st));
    ops++;
    GL_TRY(launch_diffnorm2(Az, b, n, partials, &s->cnt[2], truersq, st));
    tm.stop(st);
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    info->resSq = tr;
    info->iter = iters;
    info->success = success ? 1 : 0;
    info->ops_count = ops;
    info->status = status;
    info->device_ms = tm.ms();
    info->gbytes = ((double)iters * (apply_bytes(op) + 208.0 * n) + (double)iters * (iters + 1) * 0.5 * 48.0 * n +
                    3 * apply_bytes(op)) * 1e-9;
    fill_name(info, mode == 0 ? "Flexibly Preconditioned CG" : "Variably Preconditioned GCR");
    verb.summary(alg, info->success != 0, iters, ops, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

// ================================================================= restarts

// The restart loop of generic_cr.cpp:326-366 and its twins: run the inner solve with
// max_iter = restart_freq until it succeeds, the iteration budget is spent or the true
// residual meets the tolerance.  Two reference variations: the flexible CG
// (generic_cg_flex_precond.cpp:396-404) recomputes the true residual once more at the end
// (one more operator application), and it and the variably preconditioned GCR print the last
// inner solve's operator count in their summary line (summary_inner_ops).
template <class F>
static glinalg_status restart_loop(const std::string &nm, const glinalg_operator_s *op, double2 *x,
                                   const double2 *b, int max_iter, double eps, const Verb &verb,
                                   bool final_apply, bool summary_inner_ops, glinalg_info *info, cudaStream_t st,
                                   F inner_solve)
{
    const Verb inner = verb.restart_inner();
    glinalg_info in = {};
    int iter = 0, ops = 0;
    double ms = 0, gb = 0, bsq = 0;
    GL_TRY(host_bnorm(b, op->size, &bsq, st));
    const double bsqrt = std::sqrt(bsq);
    do {
        in = {};
        GL_TRY(inner_solve(inner, &in));
        iter += in.iter;
        ops += in.ops_count;
        ms += in.device_ms;
        gb += in.gbytes;
        verb.restart(nm, iter, ops, std::sqrt(in.resSq) / bsqrt);
    } while (iter < max_iter && in.success == 0 && std::sqrt(in.resSq) / bsqrt > eps);
    const int inner_ops = in.ops_count;
    if (final_apply) {
        Scratch sc(st);
        double2 *ax, *tmp = nullptr;
        double *partials, *tr;
        unsigned *cnt;
        GL_TRY(sc.alloc(&ax, op->size));
        if (needs_tmp(op->kind)) GL_TRY(sc.alloc(&tmp, op->size));
        GL_TRY(sc.alloc(&partials, (size_t)reduction_blocks(op->size)));
        GL_TRY(sc.zeros(&cnt, 1));
        GL_TRY(sc.alloc(&tr, 1));
        GL_TRY(launch_apply(op, ax, x, tmp, nullptr, st));
        GL_TRY(launch_diffnorm2(ax, b, op->size, partials, cnt, tr, st));
        GL_CUDA(cudaMemcpyAsync(&in.resSq, tr, sizeof(double), cudaMemcpyDeviceToHost, st));
        GL_CUDA(cudaStreamSynchronize(st));
        ops++;
    }
    double *keep = info->resSqmrhs;
    *info = in;
    info->resSqmrhs = keep;
    info->iter = iter;
    info->ops_count = ops;
    info->device_ms = ms;
    info->gbytes = gb;
    verb.summary(nm, in.success != 0, iter, summary_inner_ops ? inner_ops : ops, std::sqrt(in.resSq) / bsqrt);
    fill_name(info, nm);
    const bool ok = !(std::sqrt(in.resSq) / bsqrt > eps);
    info->success = ok ? 1 : 0;
    if (ok) info->status = GLINALG_SOLVE_CONVERGED;
    else if (info->status == GLINALG_SOLVE_CONVERGED) info->status = GLINALG_SOLVE_MAX_ITER;
    return GLINALG_SUCCESS;
}

glinalg_status cr_restart_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                               double eps, int restart_freq, const Verb &verb, glinalg_info *info, cudaStream_t st)
{
    return restart_loop("CR(" + std::to_string(restart_freq) + ")", op, x, b, max_iter, eps, verb, false, false,
                        info, st, [&](const Verb &v, glinalg_info *in) {
                            return cr_fp64(op, x, b, restart_freq, eps, v, in, st);
                        });
}

glinalg_status bicgstab_l_restart_fp64(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                                       double eps, int restart_freq, int l, const Verb &verb, glinalg_info *info,
                                       cudaStream_t st)
{
    const std::string nm = "BiCGStab-" + std::to_string(l) + "(" + std::to_string(restart_freq) + ")";
    return restart_loop(nm, op, x, b, max_iter, eps, verb, false, false, info, st,
                        [&](const Verb &v, glinalg_info *in) {
                            return bicgstab_l_fp64(op, x, b, restart_freq, eps, l, v, in, st);
                        });
}

glinalg_status flex_restart_fp64(int mode, const glinalg_operator_s *op, double2 *x, const double2 *b,
                                 int max_iter, double eps, int restart_freq, const Precond &pc, const Verb &verb,
                                 glinalg_info *info, cudaStream_t st)
{
    const std::string nm = std::string(mode == 0 ? "Flexibly Preconditioned Restarted CG("
                                                 : "Variably Preconditioned Restarted GCR(") +
                           std::to_string(restart_freq) + ")";
    return restart_loop(nm, op, x, b, max_iter, eps, verb, mode == 0, true, info, st,
                        [&](const Verb &v, glinalg_info *in) {
                            return flex_fp64(mode, op, x, b, restart_freq, eps, pc, v, in, st);
                        });
}

}  // namespace glinalg
