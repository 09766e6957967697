// cgm_batch.cu -- multishift CG for many sources of one operator, every source and every
// shift advanced by the same kernels (glinalg_cg_m_multi).  The reference solves one source
// per minv_vector_cg_m call (tests/multishift/multishift.cpp:446-489); here all sources run
// in one CUDA graph.
//
// Per source, the recurrence is the one of generic_cg_m.cpp:312-600 (worst_first off):
// beta = -|r|^2 / <p, Ap>; zeta_s and beta_s of every live shift (:396-412); r += beta Ap;
// every resid_freq_check iterations, shifts with |zeta_s| |r| < eps |b| retire to the end of
// the live range (:466-513); alpha = |r_new|^2 / |r|^2, alpha_s (:505-511); x_s -= beta_s p_s;
// p_s = zeta_s r + alpha_s p_s; p = r + alpha p; Ap = A p.  Sources stop independently.
//
// The graph is one conditional WHILE loop whose body is, for all sources at once
// (grid.y = source):
//   C  r += beta Ap and |r|^2; in the source's last block: convergence checks, alpha, alpha_s
//   A  x_s -= beta_s p_s, p_s = zeta_s r + alpha_s p_s, p' = r + alpha p, then t = D p'
//      (staggered normal operator) or Ap = L p' and <p', Ap> (gauge Laplacian)
//   B  Ap = D^dagger t and <p', Ap>; in the source's last block: beta, zeta_s, beta_s
//   tail: sources that stopped in this pass are marked finished; all finished ends the loop.
// p' alternates between two buffers so that A can form it at a site's neighbours while
// other blocks write it.  Every reduction runs over the same blocks and elements, in the same
// order, as the single-source solver's, and every site uses the same arithmetic (sites.cuh),
// so each source follows the single-source solve up to the rounding of multiply-adds that the
// compiler contracts differently (iteration counts agree).

#include <vector>

#include "sites.cuh"
#include "solvers.h"

namespace glinalg {
namespace {

constexpr int kMaxBatchShifts = 32;

int vec_grid(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

struct MsSrc {  // scalar state of one source
    double2 alpha, beta;
    double rsq, bsq;
    int k, done, status, iters, napply, n_rem, n_rem_before, pad;
    unsigned cnt[2];
};

struct MsArgs {
    MsSrc *src;
    double2 *zeta, *zeta_prev, *beta_s, *alpha_s;  // [q * ns + slot]
    double *shifts;                                 // [q * ns + slot], permuted with the slots
    int *map;                                       // [q * ns + slot] -> caller's shift index
    double2 *X, *P;                                 // [(q * ns + j) * n], j = caller's index
    double2 *r, *p0, *p1, *t, *Ap;                  // [q * n]
    const double2 *b;                               // [q * n]
    const double2 *U;
    double *partials;                               // [q * 2 * gridDim.x]
    double *res;                                    // [q * ns]: final explicit residuals
    int *all_done;
    double mass, eps;
    int lx, ly, ns, nrhs, rfc, max_iter, normal;    // normal: D^dagger D, else Laplace
    long n;
};

__device__ __forceinline__ double *row_partials(const MsArgs &a, int q)
{
    return a.partials + (size_t)q * 2 * gridDim.x;
}

// Same scalar updates as the single-source k_cgm_beta (given <p, Ap>).
__device__ void ms_beta_scalars(const MsArgs &a, MsSrc *s, int q, double re, double im)
{
    if (re == 0.0 && im == 0.0) {
        s->iters = s->k + 1;
        s->n_rem_before = 0;
        s->status = GLINALG_SOLVE_BREAKDOWN;
        s->done = 1;
        return;
    }
    const double2 beta_prev = s->beta;
    const double2 beta = cdiv(cmk(-s->rsq, 0.0), cmk(re, im));
    const double2 alpha = s->alpha;
    s->beta = beta;
    double2 *zeta = a.zeta + q * a.ns, *zeta_prev = a.zeta_prev + q * a.ns;
    double2 *beta_s = a.beta_s + q * a.ns;
    const double *sh = a.shifts + q * a.ns;
    for (int j = 0; j < s->n_rem; j++) {
        const double2 z = zeta[j], zp = zeta_prev[j];
        const double2 num = cmul(cmul(z, zp), beta_prev);
        const double2 one_m = cmk(1.0 - sh[j] * beta.x, -(sh[j] * beta.y));
        const double2 den = cadd(cmul(cmul(beta, alpha), csub(zp, z)), cmul(cmul(zp, beta_prev), one_m));
        const double2 zn = cdiv(num, den);
        zeta[j] = zn;
        zeta_prev[j] = z;
        beta_s[j] = cdiv(cmul(beta, zn), z);
    }
    s->n_rem_before = s->n_rem;
}

// C: r += beta Ap, |r|^2, then the source's bookkeeping (single-source k_cgm_r).
__global__ void __launch_bounds__(kRedThreads) k_ms_C(MsArgs a)
{
    const int q = blockIdx.y;
    MsSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    double2 *r = a.r + q * n;
    const double2 *Ap = a.Ap + q * n;
    const double2 bt = s->beta;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 ri = cadd(r[i], cmul(bt, Ap[i]));
        r[i] = ri;
        v[0] += cabs2(ri);
    }
    if (!(grid_sum_row<1, kRedThreads>(v, row_partials(a, q), &s->cnt[1]) && threadIdx.x == 0)) return;
    const double rn = v[0];
    const int k = s->k;
    const double bsqrt = sqrt(s->bsq), srn = sqrt(rn);
    const int o = q * a.ns;
    if (k % a.rfc == 0) {
        for (int j = 0; j < s->n_rem; j++) {
            if (cabsd(a.zeta[o + j]) * srn < a.eps * bsqrt) {
                s->n_rem--;
                const int e = s->n_rem;
                if (e != j) {
                    int ti = a.map[o + e]; a.map[o + e] = a.map[o + j]; a.map[o + j] = ti;
                    double2 tc;
                    tc = a.alpha_s[o + e]; a.alpha_s[o + e] = a.alpha_s[o + j]; a.alpha_s[o + j] = tc;
                    tc = a.beta_s[o + e]; a.beta_s[o + e] = a.beta_s[o + j]; a.beta_s[o + j] = tc;
                    tc = a.zeta[o + e]; a.zeta[o + e] = a.zeta[o + j]; a.zeta[o + j] = tc;
                    tc = a.zeta_prev[o + e]; a.zeta_prev[o + e] = a.zeta_prev[o + j]; a.zeta_prev[o + j] = tc;
                    double td = a.shifts[o + e]; a.shifts[o + e] = a.shifts[o + j]; a.shifts[o + j] = td;
                    j--;
                }
            }
        }
    }
    const bool last = (k == a.max_iter - 1);
    if (!isfinite(rn)) {
        s->iters = k + 1;
        s->status = GLINALG_SOLVE_NONFINITE;
        s->done = 1;
        return;
    }
    if (s->n_rem == 0 || last) {
        s->iters = k + 1;
        s->status = last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED;
        s->done = 1;
        return;
    }
    const double2 alpha = cmk(rn / s->rsq, 0.0);
    s->alpha = alpha;
    s->rsq = rn;
    for (int j = 0; j < s->n_rem; j++)
        a.alpha_s[o + j] = cdiv(cmul(cmul(alpha, a.zeta[o + j]), a.beta_s[o + j]), cmul(a.zeta_prev[o + j], s->beta));
    s->k = k + 1;
    s->napply++;
}

// A: shift updates and p' = r + alpha p at every site of the source, then the first operator
// pass on p'.  setup = 1: p' = p0 as stored (the source), no shift updates.
__global__ void __launch_bounds__(kRedThreads) k_ms_A(MsArgs a, int setup)
{
    const int q = blockIdx.y;
    MsSrc *s = a.src + q;
    const int done = s->done;
    if (done == 2) return;
    __shared__ double2 sb[kMaxBatchShifts], sz[kMaxBatchShifts], sa[kMaxBatchShifts];
    __shared__ long soff[kMaxBatchShifts];
    const int nb = setup ? 0 : s->n_rem_before;
    const int na = done ? 0 : s->n_rem;
    const long n = a.n;
    for (int j = threadIdx.x; j < nb; j += kRedThreads) {
        const int o = q * a.ns + j;
        sb[j] = a.beta_s[o];
        sz[j] = a.zeta[o];
        sa[j] = a.alpha_s[o];
        soff[j] = ((long)q * a.ns + a.map[o]) * n;
    }
    __syncthreads();
    const int k = s->k;
    const double2 alpha = s->alpha;
    const double2 *r = a.r + q * n;
    const double2 *pold = ((k & 1) ? a.p0 : a.p1) + q * n;
    double2 *pnew = ((k & 1) ? a.p1 : a.p0) + q * n;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        if (nb) {
            const double2 ri = r[i];
            for (int j = 0; j < nb; j++) {
                double2 *xs = a.X + soff[j];
                double2 *ps = a.P + soff[j];
                const double2 pv = ps[i];
                xs[i] = csub(xs[i], cmul(sb[j], pv));
                if (j < na) ps[i] = cadd(cmul(sz[j], ri), cmul(sa[j], pv));
            }
        }
        if (done) continue;  // the source stopped: final solution update only
        if (!setup) pnew[i] = cadd(r[i], cmul(alpha, pold[i]));
        if (a.normal) {
            if (setup) {
                auto ld = [pnew](long j) { return pnew[j]; };
                a.t[q * n + i] = stag_site(ld, a.U, a.mass, a.lx, a.ly, +1.0, i);
            } else {
                auto ld = [r, pold, alpha](long j) { return cadd(r[j], cmul(alpha, pold[j])); };
                a.t[q * n + i] = stag_site(ld, a.U, a.mass, a.lx, a.ly, +1.0, i);
            }
        } else {
            double2 api, pi;
            if (setup) {
                auto ld = [pnew](long j) { return pnew[j]; };
                api = lap_site(ld, a.U, a.mass, a.lx, a.ly, i);
                pi = pnew[i];
            } else {
                auto ld = [r, pold, alpha](long j) { return cadd(r[j], cmul(alpha, pold[j])); };
                api = lap_site(ld, a.U, a.mass, a.lx, a.ly, i);
                pi = ld(i);
            }
            a.Ap[q * n + i] = api;
            const double2 d = cmul(cconj(pi), api);
            v[0] += d.x;
            v[1] += d.y;
        }
    }
    if (a.normal || done) return;
    if (grid_sum_row<2, kRedThreads>(v, row_partials(a, q), &s->cnt[0]) && threadIdx.x == 0)
        ms_beta_scalars(a, s, q, v[0], v[1]);
}

// B (staggered normal operator): Ap = D^dagger t, <p', Ap>, beta and the shift scalars.
__global__ void __launch_bounds__(kRedThreads) k_ms_B(MsArgs a)
{
    const int q = blockIdx.y;
    MsSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    const double2 *pc = ((s->k & 1) ? a.p1 : a.p0) + q * n;
    const double2 *t = a.t + q * n;
    auto ld = [t](long j) { return t[j]; };
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 api = stag_site(ld, a.U, a.mass, a.lx, a.ly, -1.0, i);
        a.Ap[q * n + i] = api;
        const double2 d = cmul(cconj(pc[i]), api);
        v[0] += d.x;
        v[1] += d.y;
    }
    if (grid_sum_row<2, kRedThreads>(v, row_partials(a, q), &s->cnt[0]) && threadIdx.x == 0)
        ms_beta_scalars(a, s, q, v[0], v[1]);
}

__global__ void k_ms_tail(MsArgs a)
{
    if (threadIdx.x != 0) return;
    int fin = 0;
    for (int q = 0; q < a.nrhs; q++) {
        MsSrc *s = a.src + q;
        if (s->done == 1) s->done = 2;
        fin += s->done == 2;
    }
    if (fin == a.nrhs) *a.all_done = 1;
}

// |b|^2 and |r|^2 (= |b|^2 bit for bit, same reduction) of every source
__global__ void __launch_bounds__(kRedThreads) k_ms_norms(MsArgs a)
{
    const int q = blockIdx.y;
    MsSrc *s = a.src + q;
    const long n = a.n;
    const double2 *b = a.b + q * n;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads)
        v[0] += cabs2(b[i]);
    if (grid_sum_row<1, kRedThreads>(v, row_partials(a, q), &s->cnt[1]) && threadIdx.x == 0) {
        s->bsq = v[0];
        s->rsq = v[0];
    }
}

// x_s = 0, p_s = b, r = p = b (generic_cg_m.cpp:372-391)
__global__ void k_ms_init(MsArgs a)
{
    const int q = blockIdx.y;
    const long n = a.n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double2 bi = a.b[q * n + i];
        for (int j = 0; j < a.ns; j++) {
            a.X[((long)q * a.ns + j) * n + i] = cmk(0.0, 0.0);
            a.P[((long)q * a.ns + j) * n + i] = bi;
        }
        a.r[q * n + i] = bi;
        a.p0[q * n + i] = bi;
    }
}

// Explicit residual |(A + sigma_j) x_j - b|^2 of shift j (caller's order) for every source:
// pass 1 t = D x_j (staggered normal only), pass 2 the rest and the reduction.
__global__ void k_ms_res1(MsArgs a, int j)
{
    const int q = blockIdx.y;
    const long n = a.n;
    const double2 *x = a.X + ((long)q * a.ns + j) * n;
    auto ld = [x](long m) { return x[m]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        a.t[q * n + i] = stag_site(ld, a.U, a.mass, a.lx, a.ly, +1.0, i);
}

__global__ void __launch_bounds__(kRedThreads) k_ms_res2(MsArgs a, int j, double sigma)
{
    const int q = blockIdx.y;
    MsSrc *s = a.src + q;
    const long n = a.n;
    const double2 *x = a.X + ((long)q * a.ns + j) * n;
    const double2 *b = a.b + q * n;
    const double2 *t = a.t + q * n;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        double2 o;
        if (a.normal) {
            auto ld = [t](long m) { return t[m]; };
            o = stag_site(ld, a.U, a.mass, a.lx, a.ly, -1.0, i);
        } else {
            auto ld = [x](long m) { return x[m]; };
            o = lap_site(ld, a.U, a.mass, a.lx, a.ly, i);
        }
        if (sigma != 0.0) o = cadd(o, cscale(sigma, x[i]));
        v[0] += cabs2(csub(o, b[i]));
    }
    if (grid_sum_row<1, kRedThreads>(v, row_partials(a, q), &s->cnt[1]) && threadIdx.x == 0)
        a.res[q * a.ns + j] = v[0];
}

}  // namespace

bool cg_m_batch_supported(const glinalg_operator_s *op, int n_shift)
{
    return (op->kind == GLINALG_OP_STAGGERED_NORMAL || op->kind == GLINALG_OP_LAPLACE) &&
           n_shift <= kMaxBatchShifts;
}

// X: n_rhs * n_shift * n device values (source-major, then shift); B: n_rhs * n.
glinalg_status cg_m_batch(const glinalg_operator_s *op, double2 *X, const double2 *B, int n_rhs,
                          int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                          glinalg_info *infos, cudaStream_t st)
{
    const long n = op->size;
    const int ns = n_shift;
    Scratch sc(st);
    MsArgs a = {};
    const int nb = reduction_blocks(n);
    GL_TRY(sc.zeros(&a.src, n_rhs));
    GL_TRY(sc.alloc(&a.zeta, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.zeta_prev, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.beta_s, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.alpha_s, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.shifts, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.map, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.P, (size_t)n_rhs * ns * n));
    GL_TRY(sc.alloc(&a.r, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.p0, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.p1, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.Ap, (size_t)n_rhs * n));
    if (op->kind == GLINALG_OP_STAGGERED_NORMAL) GL_TRY(sc.alloc(&a.t, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.partials, (size_t)n_rhs * 2 * nb));
    GL_TRY(sc.alloc(&a.res, (size_t)n_rhs * ns));
    GL_TRY(sc.zeros(&a.all_done, 1));
    {
        std::vector<double2> ones((size_t)n_rhs * ns, cmk(1.0, 0.0)), zeros((size_t)n_rhs * ns, cmk(0.0, 0.0));
        std::vector<double> hs((size_t)n_rhs * ns);
        std::vector<int> hm((size_t)n_rhs * ns);
        for (int q = 0; q < n_rhs; q++)
            for (int j = 0; j < ns; j++) {
                hs[(size_t)q * ns + j] = shifts[j];
                hm[(size_t)q * ns + j] = j;
            }
        GL_CUDA(cudaMemcpyAsync(a.zeta, ones.data(), sizeof(double2) * ones.size(), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(a.zeta_prev, ones.data(), sizeof(double2) * ones.size(), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(a.beta_s, ones.data(), sizeof(double2) * ones.size(), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(a.alpha_s, zeros.data(), sizeof(double2) * zeros.size(), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(a.shifts, hs.data(), sizeof(double) * hs.size(), cudaMemcpyHostToDevice, st));
        GL_CUDA(cudaMemcpyAsync(a.map, hm.data(), sizeof(int) * hm.size(), cudaMemcpyHostToDevice, st));
        std::vector<MsSrc> hsrc(n_rhs);
        for (auto &s : hsrc) {
            s = MsSrc{};
            s.beta = cmk(1.0, 0.0);
            s.alpha = cmk(0.0, 0.0);
            s.n_rem = ns;
        }
        GL_CUDA(cudaMemcpyAsync(a.src, hsrc.data(), sizeof(MsSrc) * n_rhs, cudaMemcpyHostToDevice, st));
    }
    a.X = X;
    a.b = B;
    a.U = op->U;
    a.mass = op->mass;
    a.eps = eps;
    a.lx = op->lx;
    a.ly = op->ly;
    a.ns = ns;
    a.nrhs = n_rhs;
    a.rfc = rfc;
    a.max_iter = max_iter;
    a.normal = op->kind == GLINALG_OP_STAGGERED_NORMAL;
    a.n = n;

    EventTimer tm;
    tm.start(st);
    const dim3 rg(nb, n_rhs), vg(vec_grid(n), n_rhs);
    k_ms_init<<<vg, 256, 0, st>>>(a);
    k_ms_norms<<<rg, kRedThreads, 0, st>>>(a);
    GL_CUDA(cudaGetLastError());
    if (max_iter > 0) {
        // setup: Ap = A b and the first beta
        k_ms_A<<<rg, kRedThreads, 0, st>>>(a, 1);
        if (a.normal) k_ms_B<<<rg, kRedThreads, 0, st>>>(a);
        k_ms_tail<<<1, 32, 0, st>>>(a);
        GL_CUDA(cudaGetLastError());
        GL_TRY(run_loop(st, a.all_done, [&](cudaStream_t cs) -> glinalg_status {
            k_ms_C<<<rg, kRedThreads, 0, cs>>>(a);
            k_ms_A<<<rg, kRedThreads, 0, cs>>>(a, 0);
            if (a.normal) k_ms_B<<<rg, kRedThreads, 0, cs>>>(a);
            k_ms_tail<<<1, 32, 0, cs>>>(a);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    // explicit residuals of every shifted system (generic_cg_m.cpp:561-572)
    for (int j = 0; j < ns; j++) {
        if (a.normal) k_ms_res1<<<vg, 256, 0, st>>>(a, j);
        k_ms_res2<<<rg, kRedThreads, 0, st>>>(a, j, shifts[j]);
    }
    GL_CUDA(cudaGetLastError());
    tm.stop(st);
    std::vector<MsSrc> hsrc(n_rhs);
    std::vector<double> hres((size_t)n_rhs * ns);
    GL_CUDA(cudaMemcpyAsync(hsrc.data(), a.src, sizeof(MsSrc) * n_rhs, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaMemcpyAsync(hres.data(), a.res, sizeof(double) * hres.size(), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    const double ms = tm.ms();
    for (int q = 0; q < n_rhs; q++) {
        const MsSrc &h = hsrc[q];
        glinalg_info *info = &infos[q];
        double *keep = info->resSqmrhs;
        *info = glinalg_info{};
        info->resSqmrhs = keep;
        int iters, applies, status = h.status;
        if (max_iter > 0) {
            iters = h.iters;
            applies = h.napply;
        } else {
            iters = 1;
            applies = 0;
            status = !(0 == max_iter - 1) ? GLINALG_SOLVE_CONVERGED : GLINALG_SOLVE_MAX_ITER;
        }
        if (keep)
            for (int j = 0; j < ns; j++) keep[j] = hres[(size_t)q * ns + j];
        info->n_rhs = ns;
        info->resSq = 0.0;
        info->iter = iters;
        info->success = status == GLINALG_SOLVE_CONVERGED ? 1 : 0;
        info->ops_count = 1 + applies + ns;
        info->status = status;
        info->device_ms = ms;
        info->gbytes = ((double)iters * (apply_bytes(op) + 112.0 * n + 64.0 * n * ns) + (ns + 1) * apply_bytes(op)) * 1e-9;
        fill_name(info, "CG-M");
    }
    return GLINALG_SUCCESS;
}

}  // namespace glinalg
