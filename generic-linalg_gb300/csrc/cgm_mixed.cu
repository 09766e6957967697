// cgm_mixed.cu -- multishift CG for many sources of the staggered normal operator in mixed
// precision (glinalg_cg_m_multi with precision GLINALG_PREC_SINGLE).
//
// Phase 1: the multishift recurrence of generic_cg_m.cpp:312-600 for every source at once,
// with the vectors (r, p, A p, every shift's p_s and x_s) and the operator in FP32 and the
// scalar recurrences (beta, alpha, zeta_s, beta_s, alpha_s: complex, as in the reference) in
// FP64.  FP32 shifted solutions stop improving once their true residuals reach about 1e-7 of
// |b|: the base residual is updated with an FP32 operator, and every rounding of that update
// is missing from the shifted solutions, which the recurrence never recomputes.  So phase 1
// stops each shift at max(eps, kPhase1Tol).
// Phase 2: every (source, shift) system is refined from its phase-1 solution by the mixed CG
// with FP64 reliable updates (cg_batch_mixed: all systems advanced together) to the FP64-true
// relative residual eps.  D^dagger D + sigma with mass m is exactly D^dagger D with mass
// sqrt(m^2 + sigma) (D = m + D_hop with D_hop anti-Hermitian, so D^dagger D = m^2 +
// D_hop^dagger D_hop), so each shifted system is a staggered normal system of its own mass.
//
// Phase-1 kernels, for all sources at once (grid.y = source), mirroring cgm_batch.cu:
//   C  r += beta Ap and |r|^2; in the source's last block: retire converged shifts, alpha,
//      alpha_s
//   A  x_s -= beta_s p_s, p_s = zeta_s r + alpha_s p_s, p' = r + alpha p, then t = D p'
//   B  Ap = D^dagger t and <p', Ap>; in the source's last block: beta, zeta_s, beta_s
//   tail: sources that stopped in this pass are marked finished; all finished ends the loop.
// Sums: FP32 per thread, FP64 across threads and blocks.  The operator uses a FP32 hopping
// table with the 1/2 and eta(x) folded in (exact: powers of two and signs).

#include <cmath>
#include <vector>

#include "solvers.h"
#include "stag_tiles.cuh"

namespace glinalg {
namespace {

constexpr int kMaxMixShifts = 32;
// Phase-1 target: the FP32 shifted solutions' true residuals level off near 1e-7 |b|.
constexpr double kPhase1Tol = 1e-6;

int mvec_grid(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

struct MxSrc {  // scalar state of one source (FP64)
    double2 alpha, beta;
    double rsq, bsq;
    int k, done, status, iters, napply, n_rem, n_rem_before, shift_updates;
    unsigned cnt[2];
};

struct MxArgs {
    MxSrc *src;
    double2 *zeta, *zeta_prev, *beta_s, *alpha_s;  // [q * ns + slot]
    double *shifts;                                 // [q * ns + slot], permuted with the slots
    int *map;                                       // [q * ns + slot] -> caller's shift index
    float2 *Xs, *Ps;                                // [(q * ns + j) * n], j = caller's index
    float2 *r, *p0, *p1, *t, *Ap;                   // [q * n]
    const double2 *b;                               // [q * n]
    const float2 *H;                                // [2 i]: 1/2 U_x(i), 1/2 eta(x) U_y(i)
    double *partials;                               // [q * 2 * gridDim.x]
    int *all_done;
    float mass;
    double eps;
    int lx, ly, ns, nrhs, rfc, max_iter;
    long n;
};

__device__ __forceinline__ float2 f2(double2 v) { return make_float2((float)v.x, (float)v.y); }

__device__ __forceinline__ double *mrow_partials(const MxArgs &a, int q)
{
    return a.partials + (size_t)q * 2 * gridDim.x;
}

// hs = H_x f(x+1) - H_x(x-1)^* f(x-1) + H_y f(y+1) - H_y(y-1)^* f(y-1): D f = m f - hs,
// D^dagger f = m f + hs.
template <class In>
__device__ __forceinline__ float2 hop32(In in, const float2 *__restrict__ H, int lx, int ly, long i)
{
    const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
    const int xp = x + 1 == lx ? 0 : x + 1, xm = x == 0 ? lx - 1 : x - 1;
    const int yp = y + 1 == ly ? 0 : y + 1, ym = y == 0 ? ly - 1 : y - 1;
    const long row = (long)y * lx;
    float2 acc = fmul(H[2 * i], in(row + xp));
    acc = fsub(acc, fmulc(H[2 * (row + xm)], in(row + xm)));
    acc = fadd(acc, fmul(H[2 * i + 1], in((long)yp * lx + x)));
    acc = fsub(acc, fmulc(H[2 * ((long)ym * lx + x) + 1], in((long)ym * lx + x)));
    return acc;
}

__global__ void k_mx_hop(float2 *__restrict__ H, const double2 *__restrict__ U, int lx, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % lx);
        const double ey = (x & 1) ? -0.5 : 0.5;
        const double2 ux = U[2 * i], uy = U[2 * i + 1];
        H[2 * i] = make_float2((float)(0.5 * ux.x), (float)(0.5 * ux.y));
        H[2 * i + 1] = make_float2((float)(ey * uy.x), (float)(ey * uy.y));
    }
}

// beta, zeta_s, beta_s from <p, Ap> (generic_cg_m.cpp:396-412), in FP64.
__device__ void mx_beta_scalars(const MxArgs &a, MxSrc *s, int q, double re, double im)
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
    s->shift_updates += s->n_rem;
}

// C: r += beta Ap, |r|^2, then the source's bookkeeping (generic_cg_m.cpp:424-513).
__global__ void __launch_bounds__(kRedThreads) k_mx_C(MxArgs a)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    float2 *r = a.r + q * n;
    const float2 *Ap = a.Ap + q * n;
    const float2 bt = f2(s->beta);
    float vf = 0.f;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const float2 ri = fadd(r[i], fmul(bt, Ap[i]));
        r[i] = ri;
        vf += fn2(ri);
    }
    double v[1] = {(double)vf};
    if (!(grid_sum_row<1, kRedThreads>(v, mrow_partials(a, q), &s->cnt[1]) && threadIdx.x == 0)) return;
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

// A: shift updates and p' = r + alpha p at every site of the source, then t = D p'.
// setup = 1: p' = p0 as stored (the source), no shift updates.
__global__ void __launch_bounds__(kRedThreads) k_mx_A(MxArgs a, int setup)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    const int done = s->done;
    if (done == 2) return;
    __shared__ float2 sb[kMaxMixShifts], sz[kMaxMixShifts], sa[kMaxMixShifts];
    __shared__ long soff[kMaxMixShifts];
    const int nb = setup ? 0 : s->n_rem_before;
    const int na = done ? 0 : s->n_rem;
    const long n = a.n;
    for (int j = threadIdx.x; j < nb; j += kRedThreads) {
        const int o = q * a.ns + j;
        sb[j] = f2(a.beta_s[o]);
        sz[j] = f2(a.zeta[o]);
        sa[j] = f2(a.alpha_s[o]);
        soff[j] = ((long)q * a.ns + a.map[o]) * n;
    }
    __syncthreads();
    const int k = s->k;
    const float2 alpha = f2(s->alpha);
    const float2 *r = a.r + q * n;
    const float2 *pold = ((k & 1) ? a.p0 : a.p1) + q * n;
    float2 *pnew = ((k & 1) ? a.p1 : a.p0) + q * n;
    const float mass = a.mass;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        if (nb) {
            const float2 ri = r[i];
            for (int j = 0; j < nb; j++) {
                float2 *xs = a.Xs + soff[j];
                float2 *ps = a.Ps + soff[j];
                const float2 pv = ps[i];
                xs[i] = fsub(xs[i], fmul(sb[j], pv));
                if (j < na) ps[i] = fadd(fmul(sz[j], ri), fmul(sa[j], pv));
            }
        }
        if (done) continue;  // the source stopped: final solution update only
        float2 pc;
        float2 hs;
        if (setup) {
            auto ld = [pnew](long j) { return pnew[j]; };
            pc = pnew[i];
            hs = hop32(ld, a.H, a.lx, a.ly, i);
        } else {
            auto ld = [r, pold, alpha](long j) { return fadd(r[j], fmul(alpha, pold[j])); };
            pc = ld(i);
            pnew[i] = pc;
            hs = hop32(ld, a.H, a.lx, a.ly, i);
        }
        a.t[q * n + i] = fsub(fscale(mass, pc), hs);
    }
}

// B: Ap = D^dagger t, <p', Ap>, then beta and the shift scalars.
__global__ void __launch_bounds__(kRedThreads) k_mx_B(MxArgs a)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    const float2 *pc = ((s->k & 1) ? a.p1 : a.p0) + q * n;
    const float2 *t = a.t + q * n;
    auto ld = [t](long j) { return t[j]; };
    const float mass = a.mass;
    float vr = 0.f, vi = 0.f;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const float2 api = fadd(fscale(mass, t[i]), hop32(ld, a.H, a.lx, a.ly, i));
        a.Ap[q * n + i] = api;
        const float2 d = fmulc(pc[i], api);
        vr += d.x;
        vi += d.y;
    }
    double v[2] = {(double)vr, (double)vi};
    if (grid_sum_row<2, kRedThreads>(v, mrow_partials(a, q), &s->cnt[0]) && threadIdx.x == 0)
        mx_beta_scalars(a, s, q, v[0], v[1]);
}

__global__ void k_mx_tail(MxArgs a)
{
    if (threadIdx.x != 0) return;
    int fin = 0;
    for (int q = 0; q < a.nrhs; q++) {
        MxSrc *s = a.src + q;
        if (s->done == 1) s->done = 2;
        fin += s->done == 2;
    }
    if (fin == a.nrhs) *a.all_done = 1;
}

// |b|^2 of every source (FP64)
__global__ void __launch_bounds__(kRedThreads) k_mx_norms(MxArgs a)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    const long n = a.n;
    const double2 *b = a.b + q * n;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads)
        v[0] += cabs2(b[i]);
    if (grid_sum_row<1, kRedThreads>(v, mrow_partials(a, q), &s->cnt[1]) && threadIdx.x == 0) {
        s->bsq = v[0];
        s->rsq = v[0];
    }
}

// x_s = 0, p_s = b, r = p = b (generic_cg_m.cpp:372-391), in FP32
__global__ void k_mx_init(MxArgs a)
{
    const int q = blockIdx.y;
    const long n = a.n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 bi = f2(a.b[q * n + i]);
        for (int j = 0; j < a.ns; j++) {
            a.Xs[((long)q * a.ns + j) * n + i] = make_float2(0.f, 0.f);
            a.Ps[((long)q * a.ns + j) * n + i] = bi;
        }
        a.r[q * n + i] = bi;
        a.p0[q * n + i] = bi;
    }
}

// X (FP64, the caller's) = Xs (FP32), for every source and shift
__global__ void k_mx_widen(double2 *__restrict__ X, const float2 *__restrict__ Xs, long total)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const float2 v = Xs[i];
        X[i] = make_double2((double)v.x, (double)v.y);
    }
}

}  // namespace

bool cg_m_batch_mixed_supported(const glinalg_operator_s *op, int n_shift)
{
    return op->kind == GLINALG_OP_STAGGERED_NORMAL && n_shift <= kMaxMixShifts;
}

glinalg_status cg_m_batch_mixed(const glinalg_operator_s *op, double2 *X, const double2 *B, int n_rhs,
                                int n_shift, int rfc, int max_iter, double eps, const double *shifts,
                                glinalg_info *infos, cudaStream_t st, int *phase1_iters, int *phase2_iters)
{
    const long n = op->size;
    const int ns = n_shift;
    Scratch sc(st);
    MxArgs a = {};
    const int nb = reduction_blocks(n);
    GL_TRY(sc.zeros(&a.src, n_rhs));
    GL_TRY(sc.alloc(&a.zeta, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.zeta_prev, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.beta_s, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.alpha_s, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.shifts, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.map, (size_t)n_rhs * ns));
    GL_TRY(sc.alloc(&a.Xs, (size_t)n_rhs * ns * n));
    GL_TRY(sc.alloc(&a.Ps, (size_t)n_rhs * ns * n));
    GL_TRY(sc.alloc(&a.r, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.p0, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.p1, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.Ap, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.t, (size_t)n_rhs * n));
    float2 *H;
    GL_TRY(sc.alloc(&H, 2 * (size_t)n));
    a.H = H;
    GL_TRY(sc.alloc(&a.partials, (size_t)n_rhs * 2 * nb));
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
        std::vector<MxSrc> hsrc(n_rhs);
        for (auto &s : hsrc) {
            s = MxSrc{};
            s.beta = cmk(1.0, 0.0);
            s.alpha = cmk(0.0, 0.0);
            s.n_rem = ns;
        }
        GL_CUDA(cudaMemcpyAsync(a.src, hsrc.data(), sizeof(MxSrc) * n_rhs, cudaMemcpyHostToDevice, st));
    }
    a.b = B;
    a.mass = (float)op->mass;
    a.eps = std::max(eps, kPhase1Tol);
    a.lx = op->lx;
    a.ly = op->ly;
    a.ns = ns;
    a.nrhs = n_rhs;
    a.rfc = rfc;
    a.max_iter = max_iter;
    a.n = n;

    EventTimer tm;
    tm.start(st);
    const dim3 rg(nb, n_rhs), vg(mvec_grid(n), n_rhs);
    k_mx_hop<<<mvec_grid(n), 256, 0, st>>>(H, op->U, op->lx, n);
    k_mx_init<<<vg, 256, 0, st>>>(a);
    k_mx_norms<<<rg, kRedThreads, 0, st>>>(a);
    GL_CUDA(cudaGetLastError());
    if (max_iter > 0) {
        // setup: Ap = A b and the first beta
        k_mx_A<<<rg, kRedThreads, 0, st>>>(a, 1);
        k_mx_B<<<rg, kRedThreads, 0, st>>>(a);
        k_mx_tail<<<1, 32, 0, st>>>(a);
        GL_CUDA(cudaGetLastError());
        GL_TRY(run_loop(st, a.all_done, [&](cudaStream_t cs) -> glinalg_status {
            k_mx_C<<<rg, kRedThreads, 0, cs>>>(a);
            k_mx_A<<<rg, kRedThreads, 0, cs>>>(a, 0);
            k_mx_B<<<rg, kRedThreads, 0, cs>>>(a);
            k_mx_tail<<<1, 32, 0, cs>>>(a);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
    const long total = (long)n_rhs * ns * n;
    k_mx_widen<<<mvec_grid(total), 256, 0, st>>>(X, a.Xs, total);
    GL_CUDA(cudaGetLastError());
    EventTimer t1;  // the FP32 multishift phase ends here
    t1.start(st);
    std::vector<MxSrc> hsrc(n_rhs);
    GL_CUDA(cudaMemcpyAsync(hsrc.data(), a.src, sizeof(MxSrc) * n_rhs, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));

    // ---- phase 2: every (source, shift) system from its phase-1 solution to eps, FP64-true
    const int nsys = n_rhs * ns;
    std::vector<glinalg_operator_s> views(nsys);
    std::vector<const glinalg_operator_s *> ops(nsys);
    std::vector<double2 *> xs(nsys);
    std::vector<const double2 *> bs(nsys);
    std::vector<glinalg_info> inf2(nsys);
    for (int q = 0; q < n_rhs; q++)
        for (int j = 0; j < ns; j++) {
            const int y = q * ns + j;
            glinalg_operator_s &v = views[y];
            v.kind = GLINALG_OP_STAGGERED_NORMAL;
            v.lx = op->lx;
            v.ly = op->ly;
            v.mass = std::sqrt(op->mass * op->mass + shifts[j]);
            v.vol = op->vol;
            v.size = op->size;
            v.device = op->device;
            v.U = op->U;  // shared, not owned: cleared below before the views go away
            ops[y] = &v;
            xs[y] = X + (size_t)y * n;
            bs[y] = B + (size_t)q * n;
            inf2[y] = glinalg_info{};
        }
    glinalg_status s2 = cg_batch_mixed(ops.data(), nsys, xs.data(), bs.data(), max_iter, eps, GLINALG_PREC_SINGLE,
                                       0.0, inf2.data(), st);
    for (auto &v : views) v.U = nullptr;
    GL_TRY(s2);
    tm.stop(st);
    t1.stop(st);
    GL_CUDA(cudaStreamSynchronize(st));
    const double ms = tm.ms(), ms2 = t1.ms();
    for (int q = 0; q < n_rhs; q++) {
        const MxSrc &h = hsrc[q];
        glinalg_info *info = &infos[q];
        double *keep = info->resSqmrhs;
        *info = glinalg_info{};
        info->resSqmrhs = keep;
        int status = max_iter > 0 ? h.status : GLINALG_SOLVE_MAX_ITER;
        int refine = 0, rel = 0, ok = 1;
        double gb = 0.0;
        for (int j = 0; j < ns; j++) {
            const glinalg_info &g = inf2[(size_t)q * ns + j];
            refine += g.iter;
            rel += g.reliable_updates;
            gb += g.gbytes;
            if (!g.success) {
                ok = 0;
                if (status == GLINALG_SOLVE_CONVERGED) status = g.status;
            }
            if (keep) keep[j] = g.resSq;
        }
        if (status == GLINALG_SOLVE_MAX_ITER && ok && max_iter > 0) status = GLINALG_SOLVE_CONVERGED;
        if (phase1_iters) phase1_iters[q] = max_iter > 0 ? h.iters : 0;
        if (phase2_iters) phase2_iters[q] = refine;
        info->n_rhs = ns;
        info->resSq = 0.0;
        info->iter = max_iter > 0 ? h.iters : 1;
        info->success = (ok && status == GLINALG_SOLVE_CONVERGED) ? 1 : 0;
        info->ops_count = 1 + h.napply + refine + rel;
        info->status = status;
        info->reliable_updates = rel;
        info->device_ms = ms;
        // phase 1 per iteration: C r, Ap in, r out (3 words); A r, p in, p', t out, 2 links (6);
        // B t in, Ap out, p' in, 2 links (5); per live shift and iteration x_s, p_s in and out
        // (4); FP32 words
        const double gb1 = ((double)h.iters * 14.0 + 4.0 * h.shift_updates) * 8.0 * n * 1e-9;
        info->gbytes = gb1 + gb;
        // the FP32 multishift phase of the whole batch (every source), and its bytes for this source
        info->kernel_ms = ms - ms2;
        info->kernel_gbytes = gb1;
        fill_name(info, "CG-M-FP32");
    }
    return GLINALG_SUCCESS;
}

}  // namespace glinalg
