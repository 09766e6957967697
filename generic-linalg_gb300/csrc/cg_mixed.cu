// cg_mixed.cu -- CG on a Hermitian operator (staggered D^dagger D or the gauge Laplacian, plus
// an optional diagonal shift sigma) with reduced-precision inner iterations and FP64
// reliable updates.
//
// Algorithm: conjugate gradients with reliable updates (Sleijpen & van der Vorst 1996; the
// mixed-precision form of Clark et al., arXiv:0911.3191).  The inner loop runs the CG
// recurrence in FP32 arithmetic.  Storage per variant (direction vectors p, t / links /
// accumulators r, x_lo): SINGLE FP32 / FP32 / FP32; HALF FP16 / FP16 / FP32; BFLOAT
// BF16 / FP32 / FP32 (BF16 links, 8-bit mantissa, make the inner operator too inexact for
// kappa ~ 1e4 systems: defect correction needs |A_sloppy - A| kappa < 1).
// Whenever the iterated residual has dropped by `delta` since the last update (or claims
// convergence), the FP64 solution is advanced by the low-precision correction and the
// residual is recomputed in FP64 from the FP64 operator, r = b - A x; the search direction is
// re-orthogonalised against the new residual and the recurrence continues.  The solve stops
// only on an FP64-true relative residual below eps.
//
// Reduced-precision vectors are stored scaled: r_true ~= scale * r_lo with scale chosen at
// every reliable update so that entries of r_lo are O(1), which keeps FP16 in range.
//
// Per inner iteration (staggered normal operator), two kernels (stag_tiles.cuh tiling):
//   A: p' = r + beta p (read p from one buffer, write p' to the other), t = D p',
//      |t|^2 (+ sigma |p'|^2) -> alpha = rsq / <p', A p'>
//   B: Ap = D^dagger t (+ sigma p'), x_lo += alpha p', r -= alpha Ap, |r|^2 -> beta or update
// For the Laplacian, A stores Ap and B reads it.  The tile shape of the staggered kernels is
// picked per lattice by timing the candidates on first use (autotune below).
//
// The whole solve is one CUDA graph: an outer WHILE node (until FP64 convergence) whose body
// holds an inner WHILE node (inner iterations until a reliable update is due) followed by the
// reliable-update kernels.  The last block of each inner kernel's reduction ends the inner
// loop itself when an update is due or the solve has stopped.

#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cuda/atomic>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "mixed_state.cuh"
#include "stag_bulk.cuh"
#include "stag_resident.cuh"
#include "stag_resident_eo.cuh"
#include "stag_resident_s.cuh"

namespace glinalg {

// ---------------------------------------------------------------- staggered inner kernels

// A: p' = r + beta p_old ; t = D p' ; |t|^2 + sigma |p'|^2
template <class S, class R, class LK, int BY, int NY, bool XS>
__global__ void __launch_bounds__(32 * BY)
k_stA(const R *__restrict__ r, const S *__restrict__ p_old, S *__restrict__ p_new,
      S *__restrict__ t, const LK *__restrict__ H, float mass, float sigma, int lx, int ly,
      MxDev *s, double *partials, cudaGraphConditionalHandle cond, int use_cond)
{
    if (s->done || s->reliable) return;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int ybase = blockIdx.y * (BY * NY) + threadIdx.y * NY;
    float acc[1] = {tile_A<S, R, LK, NY, XS, false>(r, p_old, p_new, t, H, (float)s->beta, mass, sigma, lx, ly,
                                                     threadIdx.x, x, x < lx, ybase)};
    double out[1];
    if (grid_sum_f<1, 32 * BY>(acc, partials, &s->cnt[0], out) && threadIdx.x == 0 && threadIdx.y == 0)
        mx_after_A(s, out[0], cond, use_cond);
}

// B: Ap = D^dagger t + sigma p' ; x_lo += alpha p' ; r -= alpha Ap ; |r|^2
template <class S, class R, class LK, int BY, int NY, bool XS>
__global__ void __launch_bounds__(32 * BY)
k_stB(const S *__restrict__ t, const S *__restrict__ p, R *__restrict__ r,
      float2 *__restrict__ xlo, const LK *__restrict__ H, float mass, float sigma, int lx, int ly,
      int dir_parity, MxDev *s, double *partials, cudaGraphConditionalHandle cond, int use_cond)
{
    if (s->done || s->reliable) return;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int ybase = blockIdx.y * (BY * NY) + threadIdx.y * NY;
    float acc[1] = {tile_B<S, R, LK, NY, XS, false>(t, p, r, xlo, H, (float)s->alpha, mass, sigma, lx, ly,
                                                     threadIdx.x, x, x < lx, ybase)};
    double out[1];
    if (grid_sum_f<1, 32 * BY>(acc, partials, &s->cnt[1], out) && threadIdx.x == 0 && threadIdx.y == 0)
        mx_after_B(s, out[0], dir_parity, cond, use_cond);
}

// ---------------------------------------------------------------- Laplacian inner kernels

constexpr int kLBX = 32, kLBY = 8, kLNT = kLBX * kLBY;

// Inner iterations per pass of the inner WHILE body (even).  Every body pass is one device-side
// graph launch; more iterations per pass amortise its latency, and the kernels of the
// iterations after the stopping one return at once.
constexpr int kInnerUnroll = 8;

// Keeps the GPU busy for about `ns` nanoseconds (bounded: reads %globaltimer), so that work
// queued behind it starts without host launch latency in between; used by the timing hook.
__global__ void k_busy_wait(long long ns)
{
    long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (int i = 0; i < (1 << 22); i++) {
        long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 >= ns) break;
    }
}

// A: p' = r + beta p_old, Ap = (4 + m + sigma) p' - sum_mu [U p'(+mu) + U^* p'(-mu)]
template <class S, class R, class LK>
__global__ void __launch_bounds__(kLNT)
k_lapA(const R *__restrict__ r, const S *__restrict__ p_old, S *__restrict__ p_new,
       S *__restrict__ Ap, const LK *__restrict__ G, float diag, int lx, int ly, MxDev *s,
       double *partials, cudaGraphConditionalHandle cond, int use_cond)
{
    if (s->done || s->reliable) return;
    const float beta = (float)s->beta;
    const int x = blockIdx.x * kLBX + threadIdx.x, y = blockIdx.y * kLBY + threadIdx.y;
    float acc[1] = {0.f};
    if (x < lx && y < ly) {
        const int xp = x + 1 == lx ? 0 : x + 1, xm = x == 0 ? lx - 1 : x - 1;
        const int yp = y + 1 == ly ? 0 : y + 1, ym = y == 0 ? ly - 1 : y - 1;
        const long i = (long)y * lx + x;
        auto P = [&](long j) { return fadd(Fmt<R>::ld(r, j), fscale(beta, Fmt<S>::ld(p_old, j))); };
        const float2 pc = P(i);
        float2 hs = fmul(Fmt<LK>::ld(G, 2 * i), P((long)y * lx + xp));
        hs = fadd(hs, fmulc(Fmt<LK>::ld(G, 2 * ((long)y * lx + xm)), P((long)y * lx + xm)));
        hs = fadd(hs, fmul(Fmt<LK>::ld(G, 2 * i + 1), P((long)yp * lx + x)));
        hs = fadd(hs, fmulc(Fmt<LK>::ld(G, 2 * ((long)ym * lx + x) + 1), P((long)ym * lx + x)));
        const float2 av = fsub(fscale(diag, pc), hs);
        Fmt<S>::st(p_new, i, pc);
        Fmt<S>::st(Ap, i, av);
        const float2 pq = Fmt<S>::round(pc), aq = Fmt<S>::round(av);
        acc[0] = pq.x * aq.x + pq.y * aq.y;  // Re <p, Ap>
    }
    double out[1];
    if (grid_sum_f<1, kLNT>(acc, partials, &s->cnt[0], out) && threadIdx.x == 0 && threadIdx.y == 0)
        mx_after_A(s, out[0], cond, use_cond);
}

// B: x_lo += alpha p', r -= alpha Ap
template <class S, class R>
__global__ void __launch_bounds__(kLNT)
k_lapB(const S *__restrict__ Ap, const S *__restrict__ p, R *__restrict__ r,
       float2 *__restrict__ xlo, int lx, int ly, int dir_parity, MxDev *s, double *partials,
       cudaGraphConditionalHandle cond, int use_cond)
{
    if (s->done || s->reliable) return;
    const float alpha = (float)s->alpha;
    const int x = blockIdx.x * kLBX + threadIdx.x, y = blockIdx.y * kLBY + threadIdx.y;
    float acc[1] = {0.f};
    if (x < lx && y < ly) {
        const long i = (long)y * lx + x;
        const float2 pc = Fmt<S>::ld(p, i);
        xlo[i] = fadd(xlo[i], fscale(alpha, pc));
        const float2 rn = Fmt<R>::round(fsub(Fmt<R>::ld(r, i), fscale(alpha, Fmt<S>::ld(Ap, i))));
        Fmt<R>::st(r, i, rn);
        acc[0] = fn2(rn);
    }
    double out[1];
    if (grid_sum_f<1, kLNT>(acc, partials, &s->cnt[1], out) && threadIdx.x == 0 && threadIdx.y == 0)
        mx_after_B(s, out[0], dir_parity, cond, use_cond);
}

// ---------------------------------------------------------------- reliable update kernels

// R1: x_hi += scale * x_lo ; x_lo = 0
__global__ void k_mx_R1(double2 *__restrict__ x, float2 *__restrict__ xlo, long n, const MxDev *s)
{
    if (s->done) return;
    const double sc = s->scale;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 d = xlo[i];
        const double2 xv = x[i];
        x[i] = cmk(xv.x + sc * (double)d.x, xv.y + sc * (double)d.y);
        xlo[i] = make_float2(0.f, 0.f);
    }
}

// After the FP64 true residual |r_hi|^2 = rt of n sites: stop (converged, non-finite, an exactly
// zero residual, the iteration cap) or rescale for the next inner cycle.  One thread.
static __device__ void mx_true_residual(MxDev *s, double rt, long n)
{
    s->rsq_old_true = s->rsq * s->scale * s->scale;  // |r|^2 at the start of the last iteration
    s->rsq_true = rt;
    s->n_reliable++;
    const double bsqrt = sqrt(s->bsq);
    if (!isfinite(rt)) {
        s->status = GLINALG_SOLVE_NONFINITE;
        s->done = 1;
        return;
    }
    if (sqrt(rt) < s->eps * bsqrt) {
        s->status = GLINALG_SOLVE_CONVERGED;
        s->done = 1;
        return;
    }
    if (rt == 0.0) {
        // an exactly zero residual (a zero source with a zero guess): x is exact, and the
        // rescale below would divide by zero; the FP64 CG stops the same way (<p, Ap> = 0)
        s->status = GLINALG_SOLVE_BREAKDOWN;
        s->done = 1;
        return;
    }
    if (s->k >= s->max_iter) {
        s->status = GLINALG_SOLVE_MAX_ITER;
        s->done = 1;
        return;
    }
    const double new_scale = sqrt(rt / (double)n);
    // p keeps its meaning under the new scale: p_lo_new = p_lo_old * (old/new)
    s->pscale = s->scale / new_scale;
    s->scale = new_scale;
    s->rmax = sqrt(rt);
}

// R2: r_hi = b - (Ax + sigma x) ; |r_hi|^2 -> scale, convergence
__global__ void __launch_bounds__(kRedThreads)
k_mx_R2(double2 *__restrict__ rhi, const double2 *__restrict__ b, const double2 *__restrict__ Ax,
        const double2 *__restrict__ x, long n, MxDev *s, double *partials)
{
    if (s->done) return;
    const double sg = s->sigma;
    double v[1] = {0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 ax = cadd(Ax[i], cscale(sg, x[i]));
        const double2 ri = csub(b[i], ax);
        rhi[i] = ri;
        v[0] += cabs2(ri);
    }
    if (grid_sum<1, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0) mx_true_residual(s, v[0], n);
}

// R3: r_lo = r_hi / scale ; p_lo *= f ; reduce <r_lo, p_lo> (real part) and |r_lo|^2.
// p_lo is the buffer holding the current direction (p0 or p1 by s->parity).
template <class S, class R>
__global__ void __launch_bounds__(kRedThreads)
k_mx_R3(R *__restrict__ rlo, S *p0, S *p1, const double2 *__restrict__ rhi, long n, MxDev *s,
        double *partials)
{
    if (s->done) return;
    S *plo = s->parity ? p1 : p0;
    const double inv = 1.0 / s->scale;
    const float f = (float)s->pscale;
    double v[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const double2 rh = rhi[i];
        Fmt<R>::st(rlo, i, make_float2((float)(rh.x * inv), (float)(rh.y * inv)));
        const float2 pq = fscale(f, Fmt<S>::ld(plo, i));
        Fmt<S>::st(plo, i, pq);
        const float2 rq = Fmt<R>::ld(rlo, i), pr = Fmt<S>::ld(plo, i);
        v[0] += (double)(rq.x * pr.x + rq.y * pr.y);
        v[1] += (double)fn2(rq);
    }
    if (grid_sum<2, kRedThreads>(v, partials, &s->cnt[3]) && threadIdx.x == 0) {
        const double rr = v[1];
        s->rp = rr > 0.0 ? v[0] / rr : 0.0;
        // beta = |r_true|^2 / |r_old|^2 (both in true units), expressed in the new scale
        const double sc2 = s->scale * s->scale;
        s->beta = s->rsq_old_true > 0.0 ? (rr * sc2) / s->rsq_old_true : 0.0;
        s->rsq = rr;
    }
}

// R4: p0 = p_lo - rp * r_lo (restore r orthogonal to p); the direction is in p0 afterwards
// (the tail kernel resets s->parity).
template <class S, class R>
__global__ void k_mx_R4(S *p0, const S *p1, const R *__restrict__ rlo, long n, const MxDev *s)
{
    if (s->done) return;
    const S *plo = s->parity ? p1 : p0;
    const float rp = (float)s->rp;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        Fmt<S>::st(p0, i, fsub(Fmt<S>::ld(plo, i), fscale(rp, Fmt<R>::ld(rlo, i))));
}

__global__ void k_mx_outer_tail(MxDev *s, cudaGraphConditionalHandle outer, int use_cond)
{
    if (threadIdx.x != 0) return;
    s->outer++;
    if (s->outer > s->max_iter + 2 && !s->done) {
        s->status = GLINALG_SOLVE_MAX_ITER;
        s->done = 1;
    }
    if (s->done) {
        if (use_cond) cudaGraphSetConditional(outer, 0);
        return;
    }
    s->reliable = 0;
    s->parity = 0;
}

__global__ void k_mx_arm_inner(const MxDev *s, cudaGraphConditionalHandle inner)
{
    if (threadIdx.x == 0) cudaGraphSetConditional(inner, s->done ? 0u : 1u);
}

// ---------------------------------------------------------------- link preparation

template <class L>
__global__ void k_make_hop(L *__restrict__ H, const double2 *__restrict__ U, int lx, int ly)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % lx);
        const double eta = (x & 1) ? -1.0 : 1.0;
        H[2 * i] = Fmt<L>::from(cscale(-0.5, U[2 * i]));
        H[2 * i + 1] = Fmt<L>::from(cscale(-0.5 * eta, U[2 * i + 1]));
    }
}
template <class L>
__global__ void k_copy_links(L *__restrict__ G, const double2 *__restrict__ U, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        G[i] = Fmt<L>::from(U[i]);
}

static int vgrid(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

// ---------------------------------------------------------------- persistent inner loop
//
// One cooperative launch runs inner iterations until a reliable update is due: one block of
// 32 x 32 threads per SM, each warp walking a static list of 32 x NY tiles (the tile code of
// k_stA / k_stB), two grid-wide barriers per iteration (after the |t|^2 and after the |r|^2
// partial sums), and every block summing the per-block partials in the same order, so all
// blocks hold bitwise-identical scalars without a broadcast.  Fields written by other blocks
// during the launch are read with ld.global.cg (L2), never through the non-coherent L1.

template <class S, class R, class LK, int BY, int NY>
__global__ void __launch_bounds__(32 * BY, 1)
k_persist(const LK *__restrict__ H, R *r, S *p0, S *p1, S *t, float2 *xlo, float mass, float sigma,
          int lx, int ly, MxDev *s, GridSync *gs, double *partA, double *partB)
{
    __shared__ double sm[33];
    __shared__ int skip;
    // one read of the solve state per block, so that a block never splits here: block 0 of a
    // launch whose waits ran out may set s->done while other blocks are still starting
    if (threadIdx.x == 0 && threadIdx.y == 0) skip = s->done || s->reliable;
    __syncthreads();
    if (skip) return;
    const long long t_start = gtimer();
    const unsigned nb = gridDim.x;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int ntx = lx / 32, ntiles = ntx * ((ly + NY - 1) / NY);
    const int gw = blockIdx.x * BY + warp, nw = nb * BY;
    double rsq = s->rsq, beta = s->beta, rmax = s->rmax, rn = 0.0;
    const double scale = s->scale, delta = s->delta, eps = s->eps, bsqrt = sqrt(s->bsq);
    int k = s->k;
    const int max_iter = s->max_iter;
    int j = 0, status = -1;
    bool reliable = false;
    const long long lim = peer_wait_ns(s);
    for (;;) {
        const S *pold = (j & 1) ? p1 : p0;
        S *pnew = (j & 1) ? p0 : p1;
        const float fb = (float)beta;
        // ---- A: p' = r + beta p_old ; t = D p' ; |t|^2 + sigma |p'|^2
        float acc = 0.f;
        for (int tile = gw; tile < ntiles; tile += nw)
            acc += tile_A<S, R, LK, NY, true, true>(r, pold, pnew, t, H, fb, mass, sigma, lx, ly, lane,
                                                    (tile % ntx) * 32 + lane, true, (tile / ntx) * NY);
        block_partial(acc, partA, sm);
        if (!grid_sync(gs, nb, lim)) { status = GLINALG_SOLVE_TIMEOUT; break; }
        const double pAp = grid_total(partA, nb, sm);
        if (!(pAp > 0.0) || !isfinite(pAp)) {
            status = pAp == 0.0 ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
            break;
        }
        const float alpha = (float)(rsq / pAp);
        // ---- B: Ap = D^dagger t + sigma p' ; x_lo += alpha p' ; r -= alpha Ap ; |r|^2
        acc = 0.f;
        for (int tile = gw; tile < ntiles; tile += nw)
            acc += tile_B<S, R, LK, NY, true, true>(t, pnew, r, xlo, H, alpha, mass, sigma, lx, ly, lane,
                                                    (tile % ntx) * 32 + lane, true, (tile / ntx) * NY);
        block_partial(acc, partB, sm);
        if (!grid_sync(gs, nb, lim)) { status = GLINALG_SOLVE_TIMEOUT; break; }
        rn = grid_total(partB, nb, sm);
        j++;
        k++;
        if (!isfinite(rn)) { status = GLINALG_SOLVE_NONFINITE; break; }
        const double rho = sqrt(rn) * scale;
        if (rho > rmax) rmax = rho;
        if (rho < delta * rmax || rho < eps * bsqrt || k >= max_iter) {
            reliable = true;
            break;
        }
        beta = rn / rsq;
        rsq = rn;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
        s->k = k;
        s->rmax = rmax;
        s->rsq = rsq;
        s->beta = beta;
        s->rsq_new = rn;
        s->parity = j & 1;
        if (status >= 0) {
            s->status = status;
            s->done = 1;
        }
        if (reliable) s->reliable = 1;
        s->inner_ns += gtimer() - t_start;
        s->inner_iters += j;
        s->inner_launches += 1;
    }
}

template <class S, class R, class LK>
struct PersistKernel {
    using F = void (*)(const LK *, R *, S *, S *, S *, float2 *, float, float, int, int, MxDev *, GridSync *,
                       double *, double *);
    // the rectangle-resident kernel synchronises through phase words and takes its rectangle
    // grid as two more arguments
    using FR = void (*)(const LK *, R *, S *, float2 *, float, float, int, int, MxDev *, res::PhaseFlags *,
                        unsigned long long *, int, int);
    F f = nullptr;
    FR fr = nullptr;
    res::Plan plan;
    int by = 0, ny = 0;
    int grid = 0;
    int smem = 0;  // dynamic shared memory per block
    bool ok() const { return f || fr; }
};

// Persistent-kernel shapes (warps per block, rows per thread); one block per SM.  Candidates
// 4 and 5 are the bulk-copy kernel (stag_bulk.cuh: 16 warps, tiles staged through shared
// memory); candidates 6-8 are the rectangle-resident kernel (stag_resident.cuh, FP32 only):
// 16 warps with x_lo in registers, 32 warps, 16 warps with x_lo in global memory; candidates
// 9 and 10 its single-reduction form (k_resident1) with 16 and 32 warps; candidates 11 and 12
// the two-reduction form with x_lo in tensor memory, 16 and 32 warps; candidates 13 and 14 the
// same with the links in tensor memory too.  Candidate 15 is the rectangle-resident kernel of
// the 16-bit variants (stag_resident_s.cuh: t = D p' formed from the stored p' each iteration).
constexpr int kNumPersist = 16;
constexpr int kResident16Cand = 15;
static const int kPersistBY[kNumPersist] = {16, 16, 32, 16, bulk::kBY, bulk::kBY, res::kWX * 4, res::kWX * 8,
                                            res::kWX * 4, res::kWX * 4, res::kWX * 8, res::kWX * 4, res::kWX * 8,
                                            res::kWX * 4, res::kWX * 8, res::kWX * ress::kWY};
static const int kPersistNY[kNumPersist] = {4, 8, 2, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
constexpr int kResidentCand = 6;  // 6 .. 14
static bool is_resident(int c) { return c >= kResidentCand && c <= kResidentCand + 8; }
static int resident_wy(int c)
{
    return c == kResidentCand + 1 || c == kResidentCand + 4 || c == kResidentCand + 6 || c == kResidentCand + 8 ? 8 : 4;
}
// where x_lo (and the links) live (kXGlobal, kXReg, kXTmem, kXTmemL)
static int resident_xmode(int c)
{
    if (c == kResidentCand) return kXReg;
    if (c >= kResidentCand + 7) return kXTmemL;
    return c >= kResidentCand + 5 ? kXTmem : kXGlobal;
}
static bool resident_single(int c) { return c == kResidentCand + 3 || c == kResidentCand + 4; }

// The rectangle grid of the resident kernel on this device (its static shared memory, the
// reduction scratch, comes out of the same per-block budget: 512 bytes are kept for it).
static res::Plan resident_plan(int lx, int ly, int wy)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return res::Plan{};
    }
    return res::plan(lx, ly, sm_count(), (size_t)std::max(0, optin - 512), wy);
}

// The rectangle grid of the 16-bit resident kernel (S: the storage of p' and t, LK: the links).
static res::Plan resident16_plan(int lx, int ly, size_t s_bytes, size_t lk_bytes)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return res::Plan{};
    }
    return ress::plan(lx, ly, sm_count(), (size_t)std::max(0, optin - 512), s_bytes, lk_bytes);
}

// storage bytes of the variant's p' / t (FP32: 8; FP16, BF16: 4) and links (FP32 in every
// variant: 8)
static size_t variant_s_bytes(int variant) { return variant == 1 ? 8 : 4; }
static size_t variant_lk_bytes(int) { return 8; }

static bool persist_applies(int lx, int ly);

// Whether persistent candidate c serves an lx x ly lattice in variant `variant` (the FP32
// resident kernels serve the FP32 variant, candidate 15 the 16-bit ones).
static bool persist_cand_applies(int c, int lx, int ly, int variant)
{
    if (is_resident(c)) return variant == 1 && resident_plan(lx, ly, resident_wy(c)).ok;
    if (c == kResident16Cand)
        return (variant == 2 || variant == 3) &&
               resident16_plan(lx, ly, variant_s_bytes(variant), variant_lk_bytes(variant)).ok;
    if (!persist_applies(lx, ly)) return false;
    if (c == 4) return bulk_applies<bulk::Geom256x4>(lx, ly, sm_count());
    if (c == 5) return bulk_applies<bulk::Geom512x2>(lx, ly, sm_count());
    return c >= 0 && c < kNumPersist;
}

// Whether any persistent candidate serves the lattice.
static bool any_persist_applies(int lx, int ly, int variant)
{
    for (int c = 0; c < kNumPersist; c++)
        if (persist_cand_applies(c, lx, ly, variant)) return true;
    return false;
}

template <class S, class R, class LK>
static void resident_kernel(PersistKernel<S, R, LK> &pk, int lx, int ly, int wy, int xmode, bool single)
{
    if constexpr (std::is_same<S, float2>::value && std::is_same<R, float2>::value &&
                  std::is_same<LK, float2>::value) {
        pk.plan = resident_plan(lx, ly, wy);
        if (!pk.plan.ok || pk.plan.gx * pk.plan.gy > (single ? res::kMaxBlocks1 : res::kMaxBlocks)) return;
        if (single) {
            if (wy == 4) {
                switch (pk.plan.ny) {
                case 4: pk.fr = k_resident1<4, 4>; break;
                case 8: pk.fr = k_resident1<8, 4>; break;
                default: pk.fr = k_resident1<14, 4>; break;
                }
            } else {
                switch (pk.plan.ny) {
                case 2: pk.fr = k_resident1<2, 8>; break;
                case 4: pk.fr = k_resident1<4, 8>; break;
                default: pk.fr = k_resident1<7, 8>; break;
                }
            }
        } else if (wy == 4 && xmode == kXReg) {
            switch (pk.plan.ny) {
            case 4: pk.fr = k_resident<4, 4, kXReg>; break;
            case 8: pk.fr = k_resident<8, 4, kXReg>; break;
            default: pk.fr = k_resident<14, 4, kXReg>; break;
            }
        } else if (wy == 4 && xmode == kXTmem) {
            switch (pk.plan.ny) {
            case 4: pk.fr = k_resident<4, 4, kXTmem>; break;
            case 8: pk.fr = k_resident<8, 4, kXTmem>; break;
            default: pk.fr = k_resident<14, 4, kXTmem>; break;
            }
        } else if (wy == 4 && xmode == kXTmemL) {
            switch (pk.plan.ny) {
            case 4: pk.fr = k_resident<4, 4, kXTmemL>; break;
            case 8: pk.fr = k_resident<8, 4, kXTmemL>; break;
            default: pk.fr = k_resident<14, 4, kXTmemL>; break;
            }
        } else if (xmode == kXTmemL) {
            switch (pk.plan.ny) {
            case 2: pk.fr = k_resident<2, 8, kXTmemL>; break;
            case 4: pk.fr = k_resident<4, 8, kXTmemL>; break;
            default: pk.fr = k_resident<7, 8, kXTmemL>; break;
            }
        } else if (wy == 4) {
            switch (pk.plan.ny) {
            case 4: pk.fr = k_resident<4, 4, kXGlobal>; break;
            case 8: pk.fr = k_resident<8, 4, kXGlobal>; break;
            default: pk.fr = k_resident<14, 4, kXGlobal>; break;
            }
        } else if (xmode == kXTmem) {
            switch (pk.plan.ny) {
            case 2: pk.fr = k_resident<2, 8, kXTmem>; break;
            case 4: pk.fr = k_resident<4, 8, kXTmem>; break;
            default: pk.fr = k_resident<7, 8, kXTmem>; break;
            }
        } else {
            switch (pk.plan.ny) {
            case 2: pk.fr = k_resident<2, 8, kXGlobal>; break;
            case 4: pk.fr = k_resident<4, 8, kXGlobal>; break;
            default: pk.fr = k_resident<7, 8, kXGlobal>; break;
            }
        }
        pk.smem = (int)pk.plan.smem;
        pk.grid = pk.plan.gx * pk.plan.gy;
    }
}

template <class S, class R, class LK>
static PersistKernel<S, R, LK> persist_cand(int c, int lx, int ly)
{
    PersistKernel<S, R, LK> pk;
    if (c < 0 || c >= kNumPersist) return pk;
    pk.by = kPersistBY[c];
    pk.ny = kPersistNY[c];
    if (is_resident(c) || c == kResident16Cand) {
        if (c == kResident16Cand) {
            pk.plan = resident16_plan(lx, ly, sizeof(S), sizeof(LK));
            if (!pk.plan.ok) return pk;
            pk.smem = (int)pk.plan.smem;
            pk.grid = pk.plan.gx * pk.plan.gy;
            if constexpr (std::is_same<R, float2>::value) {
                switch (pk.plan.ny) {
                case 4: pk.fr = k_resident_s<4, S, LK>; break;
                case 8: pk.fr = k_resident_s<8, S, LK>; break;
                default: pk.fr = k_resident_s<14, S, LK>; break;
                }
            }
        } else {
            resident_kernel<S, R, LK>(pk, lx, ly, resident_wy(c), resident_xmode(c), resident_single(c));
        }
        if (!pk.fr) return pk;
        const void *fp = reinterpret_cast<const void *>(pk.fr);
        int per_sm = 0;
        if (cudaFuncSetAttribute(fp, cudaFuncAttributeMaxDynamicSharedMemorySize, pk.smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp, 32 * pk.by, pk.smem) != cudaSuccess ||
            per_sm < 1 || pk.grid > sm_count() * per_sm) {
            cudaGetLastError();
            pk.fr = nullptr;
        }
        return pk;
    }
    switch (c) {
    case 0: pk.f = k_persist<S, R, LK, 16, 4>; break;
    case 1: pk.f = k_persist<S, R, LK, 16, 8>; break;
    case 2: pk.f = k_persist<S, R, LK, 32, 2>; break;
    case 4: pk.f = k_persist_bulk<S, R, LK, bulk::Geom256x4>; break;
    case 5: pk.f = k_persist_bulk<S, R, LK, bulk::Geom512x2>; break;
    default: pk.f = k_persist<S, R, LK, 16, 2>; break;
    }
    if (c >= 4) {
        pk.smem = c == 4 ? bulk::Layout<S, R, LK, bulk::Geom256x4>::SMEM : bulk::Layout<S, R, LK, bulk::Geom512x2>::SMEM;
        if (cudaFuncSetAttribute(pk.f, cudaFuncAttributeMaxDynamicSharedMemorySize, pk.smem) != cudaSuccess) {
            cudaGetLastError();
            pk.f = nullptr;
            return pk;
        }
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pk.f, 32 * pk.by, pk.smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        pk.f = nullptr;
        return pk;
    }
    pk.grid = sm_count();
    return pk;
}

// The persistent path serves lattices with lx a multiple of 32 and enough tiles to give
// every warp of the grid work.
static bool persist_applies(int lx, int ly)
{
    return lx % 32 == 0 && (long)(lx / 32) * ((ly + 7) / 8) >= (long)sm_count() * 16;
}

// GLINALG_PERSIST=0 disables the persistent inner loop (the per-kernel graph path runs).
static bool persist_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("GLINALG_PERSIST");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Cooperative launch of the persistent kernel (capturable into a graph).
template <class S, class R, class LK>
static cudaError_t launch_persist(const PersistKernel<S, R, LK> &pk, cudaStream_t st, const LK *H, R *r, S *p0,
                                  S *p1, S *t, float2 *xlo, float mass, float sigma, int lx, int ly, MxDev *s,
                                  GridSync *gs, double *partA, double *partB, res::PhaseFlags *pf,
                                  unsigned long long *mbox)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(pk.grid);
    cfg.blockDim = dim3(32, pk.by);
    cfg.dynamicSmemBytes = pk.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (pk.fr)
        return cudaLaunchKernelEx(&cfg, pk.fr, H, r, p0, xlo, mass, sigma, lx, ly, s, pf, mbox, pk.plan.ty,
                                  pk.plan.gx);
    return cudaLaunchKernelEx(&cfg, pk.f, H, r, p0, p1, t, xlo, mass, sigma, lx, ly, s, gs, partA, partB);
}

// ---------------------------------------------------------------- tile shapes and autotuning

template <class S, class R, class LK>
struct StagKernels {
    using FA = void (*)(const R *, const S *, S *, S *, const LK *, float, float, int, int, MxDev *,
                        double *, cudaGraphConditionalHandle, int);
    using FB = void (*)(const S *, const S *, R *, float2 *, const LK *, float, float, int, int, int,
                        MxDev *, double *, cudaGraphConditionalHandle, int);
    FA A;
    FB B;
    int by, ny;
    dim3 block() const { return dim3(32, by); }
    dim3 grid(int lx, int ly) const { return dim3((lx + 31) / 32, (ly + by * ny - 1) / (by * ny)); }
};

// Tile-shape candidates (BY thread rows, NY sites per thread along y).
constexpr int kNumTiles = 4;
static const int kTileBY[kNumTiles] = {8, 8, 4, 16};
static const int kTileNY[kNumTiles] = {2, 4, 8, 2};

template <class S, class R, class LK, int BY, int NY>
static StagKernels<S, R, LK> make_kernels(bool xs)
{
    StagKernels<S, R, LK> k;
    k.A = xs ? k_stA<S, R, LK, BY, NY, true> : k_stA<S, R, LK, BY, NY, false>;
    k.B = xs ? k_stB<S, R, LK, BY, NY, true> : k_stB<S, R, LK, BY, NY, false>;
    k.by = BY;
    k.ny = NY;
    return k;
}

template <class S, class R, class LK>
static StagKernels<S, R, LK> kernels_for(int cand, bool xs)
{
    switch (cand) {
    case 0: return make_kernels<S, R, LK, 8, 2>(xs);
    case 1: return make_kernels<S, R, LK, 8, 4>(xs);
    case 2: return make_kernels<S, R, LK, 4, 8>(xs);
    default: return make_kernels<S, R, LK, 16, 2>(xs);
    }
}

static long max_tile_blocks(int lx, int ly)
{
    long m = 0;
    for (int c = 0; c < kNumTiles; c++) {
        long b = (long)((lx + 31) / 32) * ((ly + kTileBY[c] * kTileNY[c] - 1) / (kTileBY[c] * kTileNY[c]));
        m = std::max(m, b);
    }
    return m;
}

static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, int> g_tuned;  // (device, lx, ly, variant) -> candidate

// Times every tile candidate on the solve's own buffers (A then B, 8 launches each after one
// warm-up) and returns the fastest; cached per device, lattice and variant.
template <class S, class R, class LK>
static int autotune(const glinalg_operator_s *op, int variant, R *r, S *p0, S *p1, S *t, float2 *xlo,
                    const LK *L, MxDev *s, double *partials, cudaStream_t st)
{
    const int lx = op->lx, ly = op->ly;
    const auto key = std::make_tuple(op->device, lx, ly, variant);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) return it->second;
    }
    // GLINALG_TILE=<candidate> fixes the shape: timing picks can differ between processes, and
    // a different tile changes the order of the reductions (results differ at rounding level)
    if (const char *e = std::getenv("GLINALG_TILE")) {
        const int c = std::atoi(e);
        if (c >= 0 && c < kNumTiles) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned[key] = c;
            return c;
        }
    }
    const bool xs = lx % 32 == 0;
    // a state under which the kernels neither stop nor trigger an update: rsq = 0 gives
    // alpha = 0 (updates add zero but run in full); delta = eps = 0 never trigger
    MxDev h = {};
    h.beta = 0.5;
    h.scale = 1.0;
    h.rmax = 1e300;
    h.max_iter = 0x7fffffff;
    std::vector<double2> ones(op->size, cmk(1.0, 0.0));
    double2 *d1 = nullptr;
    if (lib_malloc_async((void **)&d1, sizeof(double2) * op->size, st) != cudaSuccess) return 1;
    cudaMemcpyAsync(d1, ones.data(), sizeof(double2) * op->size, cudaMemcpyHostToDevice, st);
    k_copy_links<R><<<vgrid(op->size), 256, 0, st>>>(r, d1, op->size);
    cudaFreeAsync(d1, st);
    int best = 1;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int c = 0; c < kNumTiles; c++) {
        auto k = kernels_for<S, R, LK>(c, xs);
        float tot = 0.f;
        for (int it = 0; it < 9; it++) {
            cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st);
            k_busy_wait<<<1, 1, 0, st>>>(30000);  // keep launch latency out of the events
            cudaEventRecord(e0, st);
            k.A<<<k.grid(lx, ly), k.block(), 0, st>>>(r, p0, p1, t, L, (float)op->mass, 0.f, lx, ly, s, partials, 0, 0);
            k.B<<<k.grid(lx, ly), k.block(), 0, st>>>(t, p1, r, xlo, L, (float)op->mass, 0.f, lx, ly, 1, s, partials, 0, 0);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (it > 0) tot += ms;
        }
        if (cudaGetLastError() == cudaSuccess && tot < best_ms) {
            best_ms = tot;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
    return best;
}

static std::map<std::tuple<int, int, int, int>, int> g_ptuned;  // persistent shape per lattice

// The tuned persistent candidate, or -1 when none serves the lattice.
static int persist_tuned(int lx, int ly, int variant)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_ptuned.find(std::make_tuple(dev, lx, ly, variant));
    return it == g_ptuned.end() ? -1 : it->second;
}

// Times every persistent shape on 16 CG iterations of A x = 1 (from r = 1, p = 0) and keeps
// the fastest for this device, lattice and variant.
template <class S, class R, class LK>
static void autotune_persist(const glinalg_operator_s *op, int variant, R *r, S *p0, S *p1, S *t, float2 *xlo,
                             const LK *L, MxDev *s, GridSync *gs, double *partA, double *partB,
                             res::PhaseFlags *pf, unsigned long long *mbox, cudaStream_t st)
{
    const int lx = op->lx, ly = op->ly;
    const auto key = std::make_tuple(op->device, lx, ly, variant);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (g_ptuned.count(key)) return;
    }
    if (const char *e = std::getenv("GLINALG_PERSIST_SHAPE")) {  // as GLINALG_TILE
        const int c = std::atoi(e);
        if (c >= 0 && c < kNumPersist && persist_cand_applies(c, lx, ly, variant)) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_ptuned[key] = c;
            return;
        }
    }
    const long n = op->size;
    std::vector<double2> ones(n, cmk(1.0, 0.0));
    double2 *d1 = nullptr;
    if (lib_malloc_async((void **)&d1, sizeof(double2) * n, st) != cudaSuccess) return;
    cudaMemcpyAsync(d1, ones.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, st);
    MxDev h = {};
    h.rsq = (double)n;  // |r|^2 of r = 1
    h.beta = 0.0;
    h.scale = 1.0;
    h.bsq = 1.0;
    h.rmax = 1e300;
    h.max_iter = 16;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = -1;
    float best_ms = 1e30f;
    for (int c = 0; c < kNumPersist; c++) {
        if (!persist_cand_applies(c, lx, ly, variant)) continue;
        const PersistKernel<S, R, LK> pk = persist_cand<S, R, LK>(c, lx, ly);
        if (!pk.ok()) continue;
        float m = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
            k_copy_links<R><<<vgrid(n), 256, 0, st>>>(r, d1, n);
            cudaMemsetAsync(p0, 0, sizeof(S) * n, st);
            cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st);
            k_busy_wait<<<1, 1, 0, st>>>(30000);
            cudaEventRecord(e0, st);
            cudaError_t e = launch_persist(pk, st, L, r, p0, p1, t, xlo, (float)op->mass, 0.f, lx, ly, s, gs,
                                           partA, partB, pf, mbox);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            MxDev back;
            cudaMemcpy(&back, s, sizeof(back), cudaMemcpyDeviceToHost);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess || back.done || back.k != 16) {
                cudaGetLastError();
                m = 1e30f;
                break;
            }
            m = std::min(m, ms);
        }
        if (m < best_ms) {
            best_ms = m;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(d1, st);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_ptuned[key] = best;
}

// ---------------------------------------------------------------- driver

template <class S, class R, class LK>
static glinalg_status run_mixed(const glinalg_operator_s *op, double2 *x, const double2 *b,
                                int max_iter, double eps, double delta, double sigma,
                                glinalg_info *info, cudaStream_t st, const char *name, int variant,
                                int wait_limit_us)
{
    const long n = op->size;
    const int lx = op->lx, ly = op->ly;
    const bool stag = op->kind == GLINALG_OP_STAGGERED_NORMAL;
    Scratch sc(st);
    R *r;
    S *p0, *p1, *t;
    LK *L;
    float2 *xlo;
    double2 *rhi, *tmp64, *Ax;
    double *partials;
    MxDev *s;
    const int nb = reduction_blocks(n);
    const dim3 lblk(kLBX, kLBY), lgrd((lx + kLBX - 1) / kLBX, (ly + kLBY - 1) / kLBY);
    const long max_blocks = std::max<long>(std::max<long>(nb, (long)lgrd.x * lgrd.y), max_tile_blocks(lx, ly));
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.zeros(&p0, n));
    GL_TRY(sc.zeros(&p1, n));
    GL_TRY(sc.alloc(&t, n));
    GL_TRY(sc.alloc(&L, 2 * n));
    GL_TRY(sc.zeros(&xlo, n));
    GL_TRY(sc.alloc(&rhi, n));
    GL_TRY(sc.alloc(&tmp64, n));
    GL_TRY(sc.alloc(&Ax, n));
    // the reliable updates' FP64 passes run register-tiled on a FP64 hopping table where the
    // lattice allows (lx a multiple of 32)
    double2 *H64 = nullptr;
    if (stag && lx % 32 == 0) {
        GL_TRY(sc.alloc(&H64, 2 * (size_t)n));
        GL_TRY(launch_make_hop64(H64, op, st));
    }
    GL_TRY(sc.alloc(&partials, 2 * (size_t)max_blocks));
    GL_TRY(sc.zeros(&s, 1));
    if (stag) k_make_hop<LK><<<vgrid(n), 256, 0, st>>>(L, op->U, lx, ly);
    else k_copy_links<LK><<<vgrid(2 * n), 256, 0, st>>>(L, op->U, 2 * n);
    GL_CUDA(cudaGetLastError());

    StagKernels<S, R, LK> sk{};
    const bool use_persist = stag && persist_enabled() && any_persist_applies(lx, ly, variant);
    GridSync *gs = nullptr;
    res::PhaseFlags *pf = nullptr;
    unsigned long long *mbox = nullptr;
    double *partA = nullptr, *partB = nullptr;
    if (use_persist) {
        GL_TRY(sc.zeros(&gs, 1));
        GL_TRY(sc.zeros(&pf, 1));
        // border mailboxes of the rectangle-resident kernel (the same rectangles for 16 and 32 warps)
        const res::Plan rp = resident_plan(lx, ly, 4);
        const res::Plan rp16 = resident16_plan(lx, ly, sizeof(S), sizeof(LK));
        if (variant == 1 && rp.ok) GL_TRY(sc.zeros(&mbox, res::mbox_words(sm_count(), rp.ty)));
        else if (variant != 1 && rp16.ok) GL_TRY(sc.zeros(&mbox, res::mbox_words(sm_count(), rp16.ty)));
        GL_TRY(sc.alloc(&partA, sm_count()));
        GL_TRY(sc.alloc(&partB, sm_count()));
    }
    if (stag) {
        const int cand = autotune<S, R, LK>(op, variant, r, p0, p1, t, xlo, L, s, partials, st);
        sk = kernels_for<S, R, LK>(cand, lx % 32 == 0);
        if (use_persist)
            autotune_persist<S, R, LK>(op, variant, r, p0, p1, t, xlo, L, s, gs, partA, partB, pf, mbox, st);
        // the tuning runs wrote the work vectors: start from zero again
        GL_CUDA(cudaMemsetAsync(p0, 0, sizeof(S) * n, st));
        GL_CUDA(cudaMemsetAsync(p1, 0, sizeof(S) * n, st));
        GL_CUDA(cudaMemsetAsync(xlo, 0, sizeof(float2) * n, st));
    }

    MxDev h = {};
    h.eps = eps;
    h.delta = delta;
    h.sigma = sigma;
    h.max_iter = max_iter;
    h.scale = 1.0;
    h.wait_ns = wait_limit_us > 0 ? 1000LL * wait_limit_us : (wait_limit_us < 0 ? -1LL : 0LL);
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    GL_TRY(launch_norm2(b, n, partials, &s->cnt[4], &s->bsq, st));

    // The reliable-update sequence, used once for the setup (r = b - A x0) and then inside
    // the outer loop.  On setup the inner "previous residual" is unknown: rsq = 0 there makes
    // beta = 0, so the first direction is the residual itself.
    auto reliable_seq = [&](cudaStream_t cs) -> glinalg_status {
        k_mx_R1<<<vgrid(n), 256, 0, cs>>>(x, xlo, n, s);
        if (H64) {
            GL_TRY(launch_stag64(tmp64, x, H64, op, +1.0, &s->done, cs));
            GL_TRY(launch_stag64(Ax, tmp64, H64, op, -1.0, &s->done, cs));
        } else if (stag) {
            GL_TRY(launch_staggered(op, tmp64, x, +1.0, &s->done, cs));
            GL_TRY(launch_staggered(op, Ax, tmp64, -1.0, &s->done, cs));
        } else {
            GL_TRY(launch_apply(op, Ax, x, nullptr, &s->done, cs));
        }
        k_mx_R2<<<nb, kRedThreads, 0, cs>>>(rhi, b, Ax, x, n, s, partials);
        // the current direction lives in p0 or p1 according to s->parity
        k_mx_R3<S, R><<<nb, kRedThreads, 0, cs>>>(r, p0, p1, rhi, n, s, partials);
        k_mx_R4<S, R><<<vgrid(n), 256, 0, cs>>>(p0, p1, r, n, s);
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    };
    GL_TRY(reliable_seq(st));

    // one inner iteration reading the direction from pold and writing it to pnew
    auto inner = [&](cudaStream_t cs, S *pold, S *pnew, int dir_parity,
                     cudaGraphConditionalHandle hin, int uc) -> glinalg_status {
        if (stag) {
            sk.A<<<sk.grid(lx, ly), sk.block(), 0, cs>>>(r, pold, pnew, t, L, (float)op->mass, (float)sigma,
                                                        lx, ly, s, partials, hin, uc);
            sk.B<<<sk.grid(lx, ly), sk.block(), 0, cs>>>(t, pnew, r, xlo, L, (float)op->mass, (float)sigma,
                                                        lx, ly, dir_parity, s, partials, hin, uc);
        } else {
            const float diag = (float)(4.0 + op->mass + sigma);
            k_lapA<S, R, LK><<<lgrd, lblk, 0, cs>>>(r, pold, pnew, t, L, diag, lx, ly, s, partials, hin, uc);
            k_lapB<S, R><<<lgrd, lblk, 0, cs>>>(t, pnew, r, xlo, lx, ly, dir_parity, s, partials, hin, uc);
        }
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    };

    // Graph: while (!done) { arm inner; while (inner) { A(p0->p1) B ; A(p1->p0) B } ;
    // reliable update ; tail }.  The inner body holds two iterations so that the direction
    // buffers alternate without a copy; B records which buffer holds the current direction
    // and the reliable update moves it back to p0.  Graphs are captured on a private stream
    // (capturing the caller's stream would fail for the legacy default stream).
    cudaStream_t cap_st = capture_stream();
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    glinalg_status status = GLINALG_SUCCESS;
    auto fail = [&](glinalg_status e) {
        if (status == GLINALG_SUCCESS) status = e;
    };
    // Persistent path (staggered operator, large lattices): while (!done) { persistent inner
    // loop ; reliable update ; tail } -- one cooperative kernel per reliable-update cycle.
    bool persisted = false;
    if (use_persist) {
        const PersistKernel<S, R, LK> pk = persist_cand<S, R, LK>(persist_tuned(lx, ly, variant), lx, ly);
        if (pk.ok()) {
            glinalg_status ps = run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
                GL_CUDA(launch_persist(pk, cs, L, r, p0, p1, t, xlo, (float)op->mass, (float)sigma, lx, ly, s,
                                       gs, partA, partB, pf, mbox));
                GL_TRY(reliable_seq(cs));
                k_mx_outer_tail<<<1, 32, 0, cs>>>(s, 0, 0);
                GL_CUDA(cudaGetLastError());
                return GLINALG_SUCCESS;
            });
            if (ps == GLINALG_SUCCESS) persisted = true;
            else cudaGetLastError();  // fall through to the per-kernel path below
        }
    }
    if (persisted) {
        // nothing more to enqueue
    } else if (!use_graphs()) {
        // host-driven: the same kernels in the same order, flags read after every launch pair
        // f[0] = done, f[2] = reliable (MxDev keeps done, status, reliable adjacent)
        static_assert(offsetof(MxDev, reliable) == offsetof(MxDev, done) + 2 * sizeof(int),
                      "flag layout");
        for (long outer = 0;; outer++) {
            int hflags[3];
            GL_CUDA(cudaMemcpyAsync(hflags, &s->done, sizeof(hflags), cudaMemcpyDeviceToHost, st));
            GL_CUDA(cudaStreamSynchronize(st));
            if (hflags[0]) break;
            for (long it = 0;; it++) {
                GL_TRY(inner(st, (it & 1) ? p1 : p0, (it & 1) ? p0 : p1, (it & 1) ? 0 : 1, 0, 0));
                int f[3];
                GL_CUDA(cudaMemcpyAsync(f, &s->done, sizeof(f), cudaMemcpyDeviceToHost, st));
                GL_CUDA(cudaStreamSynchronize(st));
                if (f[0] || f[2]) break;  // done or reliable
            }
            GL_TRY(reliable_seq(st));
            k_mx_outer_tail<<<1, 32, 0, st>>>(s, 0, 0);
            GL_CUDA(cudaGetLastError());
        }
    }
    do {
        if (!use_graphs() || persisted) break;
        cudaGraphConditionalHandle h_out, h_in;
        if (cudaGraphCreate(&g, 0) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        if (cudaGraphConditionalHandleCreate(&h_out, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        cudaGraphNodeParams op_ = {};
        op_.type = cudaGraphNodeTypeConditional;
        op_.conditional.handle = h_out;
        op_.conditional.type = cudaGraphCondTypeWhile;
        op_.conditional.size = 1;
        cudaGraphNode_t n_out;
        if (cudaGraphAddNode(&n_out, g, nullptr, nullptr, 0, &op_) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        cudaGraph_t body_out = op_.conditional.phGraph_out[0];
        if (cudaGraphConditionalHandleCreate(&h_in, body_out, 0, 0) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        // outer body part 1: arm the inner loop
        if (cudaStreamBeginCaptureToGraph(cap_st, body_out, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        k_mx_arm_inner<<<1, 32, 0, cap_st>>>(s, h_in);
        cudaGraph_t cap = nullptr;
        if (cudaStreamEndCapture(cap_st, &cap) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        size_t nn = 0;
        cudaGraphGetNodes(body_out, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(body_out, nodes.data(), &nn);
        cudaGraphNodeParams ip = {};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h_in;
        ip.conditional.type = cudaGraphCondTypeWhile;
        ip.conditional.size = 1;
        cudaGraphNode_t n_in;
        if (cudaGraphAddNode(&n_in, body_out, nodes.data(), nullptr, nn, &ip) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        cudaGraph_t body_in = ip.conditional.phGraph_out[0];
        // inner body: kInnerUnroll iterations, the direction buffers swapped between them
        // (an even count, so every body pass starts from p0)
        if (cudaStreamBeginCaptureToGraph(cap_st, body_in, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        glinalg_status bs = GLINALG_SUCCESS;
        for (int u = 0; u < kInnerUnroll && bs == GLINALG_SUCCESS; u++)
            bs = (u & 1) ? inner(cap_st, p1, p0, 0, h_in, 1) : inner(cap_st, p0, p1, 1, h_in, 1);
        if (cudaStreamEndCapture(cap_st, &cap) != cudaSuccess || bs != GLINALG_SUCCESS) { fail(bs ? bs : GLINALG_ERROR_CUDA); break; }
        // outer body part 2 (after the inner node): reliable update and tail
        if (cudaStreamBeginCaptureToGraph(cap_st, body_out, &n_in, nullptr, 1, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        bs = reliable_seq(cap_st);
        if (bs == GLINALG_SUCCESS) k_mx_outer_tail<<<1, 32, 0, cap_st>>>(s, h_out, 1);
        if (cudaStreamEndCapture(cap_st, &cap) != cudaSuccess || bs != GLINALG_SUCCESS) { fail(bs ? bs : GLINALG_ERROR_CUDA); break; }
        if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
        if (cudaGraphLaunch(ex, st) != cudaSuccess) { fail(GLINALG_ERROR_CUDA); break; }
    } while (0);
    if (status != GLINALG_SUCCESS) {
        cudaError_t e = cudaGetLastError();
        set_last_error(std::string("mixed CG graph: ") + cudaGetErrorString(e));
        cudaStreamSynchronize(st);
        if (ex) cudaGraphExecDestroy(ex);
        if (g) cudaGraphDestroy(g);
        return status;
    }
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    if (h.status == GLINALG_SOLVE_TIMEOUT) {
        // the kernel gave up a bounded wait for other blocks and returned; the context is intact
        info->resSq = 0.0;
        info->iter = h.k;
        info->success = 0;
        info->ops_count = h.k + h.n_reliable;
        info->status = GLINALG_SOLVE_TIMEOUT;
        info->reliable_updates = h.n_reliable;
        set_last_error("a bounded wait of the persistent CG kernel for other blocks ran out");
        return GLINALG_ERROR_INTERNAL;
    }
    info->resSq = h.rsq_true;
    info->iter = h.k;
    info->success = h.status == GLINALG_SOLVE_CONVERGED ? 1 : 0;
    // inner iterations: 1 operator application each; every reliable update: 1 more
    info->ops_count = h.k + h.n_reliable;
    info->status = h.status;
    info->reliable_updates = h.n_reliable;
    info->device_ms = tm.ms();
    const double w = Fmt<S>::bytes, wr = Fmt<R>::bytes, wl = Fmt<LK>::bytes;
    // A: r(wr) p_old(w) links(2wl) -> p'(w) t(w); B: t(w) links(2wl) p'(w) r(2 wr) x_lo(16)
    const double per_iter = stag ? (6.0 * w + 4.0 * wl + 3.0 * wr + 16.0) : (6.0 * w + 2.0 * wl + 3.0 * wr + 16.0);
    // reliable update: x_hi r/w + x_lo r/w, FP64 operator (two passes), r_hi, r_lo, p
    const double per_rel = 16.0 * 2 + 16.0 + 8.0 * 64.0 / 8.0 + 16.0 * 3 + 2 * wr + 4 * w;
    info->gbytes = ((double)h.k * per_iter * n + (double)h.n_reliable * per_rel * n) * 1e-9;
    info->kernel_ms = (double)h.inner_ns * 1e-6;
    info->kernel_gbytes = (double)h.inner_iters * per_iter * n * 1e-9;
    info->kernel_launches = h.inner_launches;
    fill_name(info, name);
    return GLINALG_SUCCESS;
}

// ---------------------------------------------------------------- checkerboarded even system
//
// The FP32 mixed-precision CG on m^2 - D_eo D_oe (+ sigma) with the even fields stored packed
// (half-lattice layout: even site (x, y) at j = y * lx/2 + x/2) and the inner iterations in the
// rectangle-resident kernel k_resident_eo.  The FP64 side keeps x on the full lattice (odd
// sites zero), so that the reliable update's true residual is m^2 x - D_eo D_oe x formed as
// D^dagger (D x) by the FP64 stencils (on an even-only field the two agree at the even sites).

// Full-lattice index of packed even site j.
__device__ __forceinline__ long eo_full_even(long j, int hw, int lx)
{
    const long y = j / hw;
    const long u = j - y * hw;
    return y * lx + 2 * u + (y & 1);
}

// Packed FP32 hopping table: H2[2 j] = h_x, H2[2 j + 1] = h_y of the even site at packed index
// j, the odd sites from 4 nh on (the values of k_make_hop: h_x = -U_x / 2, h_y = -eta(x) U_y / 2).
__global__ void k_eo_pack_hop(float2 *__restrict__ H2, const double2 *__restrict__ U, int lx, int ly)
{
    const long vol = (long)lx * ly, nh = vol / 2;
    const int hw = lx / 2;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol; i += (long)gridDim.x * blockDim.x) {
        const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
        const double eta = (x & 1) ? -1.0 : 1.0;
        const long j = (long)y * hw + (x >> 1) + (((x + y) & 1) ? nh : 0);
        H2[2 * j] = Fmt<float2>::from(cscale(-0.5, U[2 * i]));
        H2[2 * j + 1] = Fmt<float2>::from(cscale(-0.5 * eta, U[2 * i + 1]));
    }
}

// be = b at the even sites, packed.
__global__ void k_eo_gather(double2 *__restrict__ be, const double2 *__restrict__ b, int lx, int ly)
{
    const long nh = (long)lx * ly / 2;
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < nh; j += (long)gridDim.x * blockDim.x)
        be[j] = b[eo_full_even(j, lx / 2, lx)];
}

// R1 on the packed x_lo: x_hi(even site of j) += scale * x_lo[j] ; x_lo = 0
__global__ void k_eo_R1(double2 *__restrict__ x, float2 *__restrict__ xlo, int lx, int ly, const MxDev *s)
{
    if (s->done) return;
    const long nh = (long)lx * ly / 2;
    const double sc = s->scale;
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < nh; j += (long)gridDim.x * blockDim.x) {
        const long i = eo_full_even(j, lx / 2, lx);
        const float2 d = xlo[j];
        const double2 xv = x[i];
        x[i] = cmk(xv.x + sc * (double)d.x, xv.y + sc * (double)d.y);
        xlo[j] = make_float2(0.f, 0.f);
    }
}

// R2 on the even sites: r_hi[j] = b_e[j] - (Ax + sigma x)(even site of j) ; |r_hi|^2
__global__ void __launch_bounds__(kRedThreads)
k_eo_R2(double2 *__restrict__ rhi, const double2 *__restrict__ be, const double2 *__restrict__ Ax,
        const double2 *__restrict__ x, int lx, int ly, MxDev *s, double *partials)
{
    if (s->done) return;
    const long nh = (long)lx * ly / 2;
    const double sg = s->sigma;
    double v[1] = {0.0};
    for (long j = blockIdx.x * (long)kRedThreads + threadIdx.x; j < nh; j += (long)gridDim.x * kRedThreads) {
        const long i = eo_full_even(j, lx / 2, lx);
        const double2 ri = csub(be[j], cadd(Ax[i], cscale(sg, x[i])));
        rhi[j] = ri;
        v[0] += cabs2(ri);
    }
    if (grid_sum<1, kRedThreads>(v, partials, &s->cnt[2]) && threadIdx.x == 0) mx_true_residual(s, v[0], nh);
}

// The rectangle grid of k_resident_eo on this device (512 bytes of the per-block budget kept for
// its static shared memory).
static res::Plan eo_plan(int lx, int ly)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return res::Plan{};
    }
    return reseo::plan(lx, ly, sm_count(), (size_t)std::max(0, optin - 512));
}

using EoKernel = void (*)(const float2 *, float2 *, float2 *, float2 *, float, float, int, int, MxDev *,
                          res::PhaseFlags *, unsigned long long *, int, int);

// The kernel instance for a plan, with its shared memory set and its grid checked against the
// device's co-resident blocks; nullptr when it cannot run.
static EoKernel eo_kernel(const res::Plan &p)
{
    if (!p.ok) return nullptr;
    EoKernel f = p.ny == 8 ? k_resident_eo<8> : (p.ny == 14 ? k_resident_eo<14> : nullptr);
    if (!f) return nullptr;
    int per_sm = 0;
    const void *fp = reinterpret_cast<const void *>(f);
    if (cudaFuncSetAttribute(fp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp, 32 * res::kWX * reseo::kWY, p.smem) !=
            cudaSuccess ||
        per_sm < 1 || p.gx * p.gy > sm_count() * per_sm) {
        cudaGetLastError();
        return nullptr;
    }
    return f;
}

// GLINALG_EO_PACKED=0 keeps the even system on the full-lattice solver.
static bool eo_packed_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("GLINALG_EO_PACKED");
        return !(e && e[0] == '0');
    }();
    return on;
}

static bool eo_packed_applies(const glinalg_operator_s *op)
{
    return eo_packed_enabled() && persist_enabled() && op->kind == GLINALG_OP_STAGGERED_M2MDEODOE &&
           eo_plan(op->lx, op->ly).ok;
}

static glinalg_status run_mixed_eo(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                                   double eps, double delta, double sigma, glinalg_info *info, cudaStream_t st,
                                   int wait_limit_us)
{
    const long n = op->size, nh = n / 2;
    const int lx = op->lx, ly = op->ly;
    const res::Plan pl = eo_plan(lx, ly);
    const EoKernel kern = eo_kernel(pl);
    if (!kern) {
        set_last_error("the checkerboarded resident kernel does not fit this device");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    Scratch sc(st);
    float2 *r, *p0, *xlo, *H2;
    double2 *xf, *be, *rhi, *tmp64, *Ax, *H64;
    double *partials;
    MxDev *s;
    res::PhaseFlags *pf;
    unsigned long long *mbox;
    const int nb = reduction_blocks(n);
    GL_TRY(sc.alloc(&r, nh));
    GL_TRY(sc.zeros(&p0, nh));
    GL_TRY(sc.zeros(&xlo, nh));
    GL_TRY(sc.alloc(&H2, 2 * (size_t)n));
    GL_TRY(sc.alloc(&xf, n));
    GL_TRY(sc.alloc(&be, nh));
    GL_TRY(sc.alloc(&rhi, nh));
    GL_TRY(sc.alloc(&tmp64, n));
    GL_TRY(sc.alloc(&Ax, n));
    GL_TRY(sc.alloc(&H64, 2 * (size_t)n));
    GL_TRY(sc.alloc(&partials, 2 * (size_t)nb));
    GL_TRY(sc.zeros(&s, 1));
    GL_TRY(sc.zeros(&pf, 1));
    GL_TRY(sc.zeros(&mbox, res::mbox_words(pl.gx * pl.gy, pl.ty)));
    k_eo_pack_hop<<<vgrid(n), 256, 0, st>>>(H2, op->U, lx, ly);
    k_eo_gather<<<vgrid(nh), 256, 0, st>>>(be, b, lx, ly);
    GL_CUDA(cudaGetLastError());
    GL_TRY(launch_make_hop64(H64, op, st));
    // x on the full lattice with its odd sites zero (only the even sites come back)
    GL_TRY(launch_even_part(op, xf, x, st));

    MxDev h = {};
    h.eps = eps;
    h.delta = delta;
    h.sigma = sigma;
    h.max_iter = max_iter;
    h.scale = 1.0;
    h.wait_ns = wait_limit_us > 0 ? 1000LL * wait_limit_us : (wait_limit_us < 0 ? -1LL : 0LL);
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    GL_TRY(launch_norm2(be, nh, partials, &s->cnt[4], &s->bsq, st));
    const int nbh = reduction_blocks(nh);
    auto reliable_seq = [&](cudaStream_t cs) -> glinalg_status {
        k_eo_R1<<<vgrid(nh), 256, 0, cs>>>(xf, xlo, lx, ly, s);
        GL_TRY(launch_stag64(tmp64, xf, H64, op, +1.0, &s->done, cs));
        GL_TRY(launch_stag64(Ax, tmp64, H64, op, -1.0, &s->done, cs));
        k_eo_R2<<<nbh, kRedThreads, 0, cs>>>(rhi, be, Ax, xf, lx, ly, s, partials);
        // the resident kernel leaves the direction in p0 (parity 0)
        k_mx_R3<float2, float2><<<nbh, kRedThreads, 0, cs>>>(r, p0, p0, rhi, nh, s, partials);
        k_mx_R4<float2, float2><<<vgrid(nh), 256, 0, cs>>>(p0, p0, r, nh, s);
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    };
    GL_TRY(reliable_seq(st));
    GL_TRY(run_loop(st, &s->done, [&](cudaStream_t cs) -> glinalg_status {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(pl.gx * pl.gy);
        cfg.blockDim = dim3(32, res::kWX * reseo::kWY);
        cfg.dynamicSmemBytes = pl.smem;
        cfg.stream = cs;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        GL_CUDA(cudaLaunchKernelEx(&cfg, kern, (const float2 *)H2, r, p0, xlo, (float)op->mass, (float)sigma, lx, ly,
                                   s, pf, mbox, pl.ty, pl.gx));
        GL_TRY(reliable_seq(cs));
        k_mx_outer_tail<<<1, 32, 0, cs>>>(s, 0, 0);
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    }));
    tm.stop(st);
    GL_TRY(launch_even_into(op, x, xf, st));
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    if (h.status == GLINALG_SOLVE_TIMEOUT) {
        info->resSq = 0.0;
        info->iter = h.k;
        info->success = 0;
        info->ops_count = h.k + h.n_reliable;
        info->status = GLINALG_SOLVE_TIMEOUT;
        info->reliable_updates = h.n_reliable;
        set_last_error("a bounded wait of the persistent CG kernel for other blocks ran out");
        return GLINALG_ERROR_INTERNAL;
    }
    info->resSq = h.rsq_true;
    info->iter = h.k;
    info->success = h.status == GLINALG_SOLVE_CONVERGED ? 1 : 0;
    info->ops_count = h.k + h.n_reliable;
    info->status = h.status;
    info->reliable_updates = h.n_reliable;
    info->device_ms = tm.ms();
    // a streaming iteration on the half lattice: the full-lattice iteration's words per even site
    const double per_iter = 6.0 * 8 + 4.0 * 8 + 3.0 * 8 + 16.0;
    const double per_rel = 16.0 * 2 + 16.0 + 8.0 * 64.0 / 8.0 + 16.0 * 3 + 2 * 8 + 4 * 8;
    info->gbytes = ((double)h.k * per_iter * nh + (double)h.n_reliable * per_rel * n) * 1e-9;
    info->kernel_ms = (double)h.inner_ns * 1e-6;
    info->kernel_gbytes = (double)h.inner_iters * per_iter * nh * 1e-9;
    info->kernel_launches = h.inner_launches;
    fill_name(info, "CG-FP32-EO");
    return GLINALG_SUCCESS;
}

// Mixed-precision CG on m^2 - D_eo D_oe (square_staggered_m2mdeodoe_u1, operators.cpp:566).  On
// even-only fields this operator equals D^dagger D, so the staggered normal solver runs on the
// even parts of b and of the guess.  Only x's even sites are written: the odd sites keep their
// input values, as in the reference's CG, whose operator zeroes them (b's odd sites must be
// zero, as square_staggered_eoprec_prepare makes them; they are not read).
static glinalg_status cg_mixed_even(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                                    double eps, int precision, double delta, double sigma, const Verb &verb,
                                    glinalg_info *info, cudaStream_t st, int wait_limit_us)
{
    Scratch sc(st);
    double2 *be, *xe;
    GL_TRY(sc.alloc(&be, op->size));
    GL_TRY(sc.alloc(&xe, op->size));
    GL_TRY(launch_even_part(op, be, b, st));
    GL_TRY(launch_even_part(op, xe, x, st));
    // D^dagger D on the same links and mass; the view owns no device memory
    glinalg_operator_s view;
    view.kind = GLINALG_OP_STAGGERED_NORMAL;
    view.lx = op->lx;
    view.ly = op->ly;
    view.mass = op->mass;
    view.vol = op->vol;
    view.size = op->size;
    view.device = op->device;
    view.U = op->U;
    const glinalg_status s =
        cg_mixed(&view, xe, be, max_iter, eps, precision, delta, sigma, verb, info, st, wait_limit_us);
    view.U = nullptr;
    GL_TRY(s);
    return launch_even_into(op, x, xe, st);
}

glinalg_status cg_mixed(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter,
                        double eps, int precision, double delta, double sigma, const Verb &verb,
                        glinalg_info *info, cudaStream_t st, int wait_limit_us)
{
    // the even system runs checkerboarded (k_resident_eo) in FP32 where the lattice allows,
    // otherwise on the full-lattice solver
    const bool eo_packed = op->kind == GLINALG_OP_STAGGERED_M2MDEODOE && precision == GLINALG_PREC_SINGLE &&
                           eo_packed_applies(op);
    if (op->kind == GLINALG_OP_STAGGERED_M2MDEODOE && !eo_packed)
        return cg_mixed_even(op, x, b, max_iter, eps, precision, delta, sigma, verb, info, st, wait_limit_us);
    if (!(op->kind == GLINALG_OP_STAGGERED_NORMAL || op->kind == GLINALG_OP_LAPLACE || eo_packed)) {
        set_last_error("mixed-precision CG needs the staggered normal operator, m^2 - D_eo D_oe or the gauge "
                       "Laplacian");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    // default reliable-update trigger: FP32 iterates stay accurate over two orders of magnitude
    // of residual reduction (1024^2, m = 0.01: 6 updates instead of 11, the same 2100
    // iterations); 16-bit iterates need an update after one
    if (!(delta > 0.0 && delta < 1.0)) delta = precision == GLINALG_PREC_SINGLE ? 0.01 : 0.1;
    glinalg_status s;
    switch (precision) {
    case GLINALG_PREC_SINGLE:
        s = eo_packed ? run_mixed_eo(op, x, b, max_iter, eps, delta, sigma, info, st, wait_limit_us)
                      : run_mixed<float2, float2, float2>(op, x, b, max_iter, eps, delta, sigma, info, st, "CG-FP32",
                                                          1, wait_limit_us);
        break;
    case GLINALG_PREC_HALF:
        // FP16 fields, FP32 links (as BF16): with FP16 links the inner operator differs from
        // the FP64 one by the links' rounding, every reliable-update cycle gains only as many
        // orders as that allows, and the 1024^2 solve took 5456 iterations (63 ms) against
        // 2103 (24.7 ms) with FP32 links.
        s = run_mixed<__half2, float2, float2>(op, x, b, max_iter, eps, delta, sigma, info, st, "CG-FP16", 2, wait_limit_us);
        break;
    case GLINALG_PREC_BFLOAT:
        s = run_mixed<__nv_bfloat162, float2, float2>(op, x, b, max_iter, eps, delta, sigma, info, st, "CG-BF16", 3, wait_limit_us);
        break;
    default: set_last_error("unknown precision"); return GLINALG_ERROR_INVALID_VALUE;
    }
    if (s != GLINALG_SUCCESS) return s;
    if (!verb.prints_summary()) return GLINALG_SUCCESS;
    double bsqrt = 0.0;
    {
        // |b| for the summary line
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
    verb.summary(info->name, info->success != 0, info->iter, info->ops_count, std::sqrt(info->resSq) / bsqrt);
    return GLINALG_SUCCESS;
}

// ---------------------------------------------------------------- kernel timing hook

template <class S, class R, class LK>
static glinalg_status profile_inner(const glinalg_operator_s *op, int variant, int n_launch, double ms[2],
                                    double bytes[2])
{
    const long n = op->size;
    const int lx = op->lx, ly = op->ly;
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    R *r;
    S *p0, *p1, *t;
    LK *L;
    float2 *xlo;
    double *partials;
    MxDev *s;
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.zeros(&p0, n));
    GL_TRY(sc.zeros(&p1, n));
    GL_TRY(sc.zeros(&t, n));
    GL_TRY(sc.alloc(&L, 2 * n));
    GL_TRY(sc.zeros(&xlo, n));
    GL_TRY(sc.alloc(&partials, (size_t)max_tile_blocks(lx, ly)));
    GL_TRY(sc.zeros(&s, 1));
    k_make_hop<LK><<<vgrid(n), 256, 0, st>>>(L, op->U, lx, ly);
    GL_CUDA(cudaGetLastError());
    const int cand = autotune<S, R, LK>(op, variant, r, p0, p1, t, xlo, L, s, partials, st);
    auto k = kernels_for<S, R, LK>(cand, lx % 32 == 0);
    MxDev h = {};
    h.beta = 0.5;
    h.scale = 1.0;
    h.rmax = 1e300;
    h.max_iter = 0x7fffffff;
    EventTimer ta, tb;
    double sa = 0.0, sb = 0.0;
    const float mass = (float)op->mass;
    for (int it = 0; it < n_launch + 2; it++) {
        GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));
        S *po = (it & 1) ? p1 : p0, *pn = (it & 1) ? p0 : p1;
        // queue both kernels behind a 50 us busy wait, so the events time the kernels and not
        // the host's launch latency
        k_busy_wait<<<1, 1, 0, st>>>(50000);
        ta.start(st);
        k.A<<<k.grid(lx, ly), k.block(), 0, st>>>(r, po, pn, t, L, mass, 0.f, lx, ly, s, partials, 0, 0);
        ta.stop(st);
        tb.start(st);
        k.B<<<k.grid(lx, ly), k.block(), 0, st>>>(t, pn, r, xlo, L, mass, 0.f, lx, ly, 0, s, partials, 0, 0);
        tb.stop(st);
        GL_CUDA(cudaGetLastError());
        const double a = ta.ms(), b = tb.ms();
        if (it >= 2) {  // two warm-up launches
            sa += a;
            sb += b;
        }
    }
    ms[0] = sa / n_launch;
    ms[1] = sb / n_launch;
    const double w = Fmt<S>::bytes, wr = Fmt<R>::bytes, wl = Fmt<LK>::bytes;
    // A: r, p_old in; p', t out; hopping coefficients (2 per site).  B: t, p in; r in and
    // out; x_lo (FP32) in and out; hopping coefficients.
    bytes[0] = (double)n * (wr + w + 2 * wl + 2 * w);
    bytes[1] = (double)n * (w + w + 2 * wr + 16.0 + 2 * wl);
    return GLINALG_SUCCESS;
}

// Times the tuned persistent inner-loop kernel of op's lattice with CUDA events: n_launch
// launches (after one untimed) of exactly n_iter inner iterations each, on CG for A x = 1 from
// r = 1, p = 0 (the per-iteration work does not depend on the values).  Each launch is queued
// behind a short busy wait so that the events bracket the kernel, not the host's launch latency.
template <class S, class R, class LK>
static glinalg_status profile_persist(const glinalg_operator_s *op, int variant, int n_launch, int n_iter,
                                      double *ms, double *bytes, int *cand_out)
{
    const long n = op->size;
    const int lx = op->lx, ly = op->ly;
    const int cand = persist_tuned(lx, ly, variant);
    if (cand < 0) {
        set_last_error("no persistent inner-loop kernel has been tuned for this lattice and precision "
                       "(run a mixed-precision solve on it first)");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    const PersistKernel<S, R, LK> pk = persist_cand<S, R, LK>(cand, lx, ly);
    if (!pk.ok()) {
        set_last_error("the tuned persistent kernel is not available");
        return GLINALG_ERROR_INTERNAL;
    }
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    R *r;
    S *p0, *p1, *t;
    LK *L;
    float2 *xlo;
    MxDev *s;
    GridSync *gs;
    res::PhaseFlags *pf;
    unsigned long long *mbox = nullptr;
    double *partA, *partB, *ones;
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.zeros(&p0, n));
    GL_TRY(sc.zeros(&p1, n));
    GL_TRY(sc.zeros(&t, n));
    GL_TRY(sc.alloc(&L, 2 * n));
    GL_TRY(sc.zeros(&xlo, n));
    GL_TRY(sc.zeros(&s, 1));
    GL_TRY(sc.zeros(&gs, 1));
    GL_TRY(sc.zeros(&pf, 1));
    GL_TRY(sc.alloc(&partA, sm_count()));
    GL_TRY(sc.alloc(&partB, sm_count()));
    GL_TRY(sc.alloc(&ones, 2 * n));
    if (pk.fr) GL_TRY(sc.zeros(&mbox, res::mbox_words(sm_count(), pk.plan.ty)));
    std::vector<double2> h1(n, cmk(1.0, 0.0));
    GL_CUDA(cudaMemcpyAsync(ones, h1.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, st));
    k_make_hop<LK><<<vgrid(n), 256, 0, st>>>(L, op->U, lx, ly);
    GL_CUDA(cudaGetLastError());
    MxDev h = {};
    h.rsq = (double)n;  // |r|^2 of r = 1
    h.scale = 1.0;
    h.bsq = 1.0;
    h.rmax = 1e300;
    h.max_iter = n_iter;  // delta = eps = 0: the launch runs exactly n_iter iterations
    EventTimer tm;
    double sum = 0.0;
    for (int it = 0; it <= n_launch; it++) {
        k_copy_links<R><<<vgrid(n), 256, 0, st>>>(r, reinterpret_cast<const double2 *>(ones), n);
        GL_CUDA(cudaMemsetAsync(p0, 0, sizeof(S) * n, st));
        GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));
        k_busy_wait<<<1, 1, 0, st>>>(50000);
        tm.start(st);
        GL_CUDA(launch_persist(pk, st, L, r, p0, p1, t, xlo, (float)op->mass, 0.f, lx, ly, s, gs, partA, partB, pf,
                               mbox));
        tm.stop(st);
        MxDev back;
        GL_CUDA(cudaMemcpyAsync(&back, s, sizeof(back), cudaMemcpyDeviceToHost, st));
        GL_CUDA(cudaStreamSynchronize(st));
        if (back.k != n_iter || back.done) {
            set_last_error("the persistent kernel did not run the requested iterations");
            return GLINALG_ERROR_INTERNAL;
        }
        if (it > 0) sum += tm.ms();
    }
    *ms = sum / n_launch;
    const double w = Fmt<S>::bytes, wr = Fmt<R>::bytes, wl = Fmt<LK>::bytes;
    *bytes = (double)n_iter * (6.0 * w + 4.0 * wl + 3.0 * wr + 16.0) * n;  // per launch, as in info->kernel_gbytes
    *cand_out = cand;
    return GLINALG_SUCCESS;
}

int tuned_tile(const glinalg_operator_s *op, int variant)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(std::make_tuple(op->device, op->lx, op->ly, variant));
    return it == g_tuned.end() ? -1 : it->second;
}

int tuned_persist(const glinalg_operator_s *op, int variant)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_ptuned.find(std::make_tuple(op->device, op->lx, op->ly, variant));
    return it == g_ptuned.end() ? -1 : it->second;
}

}  // namespace glinalg

extern "C" glinalg_status glinalg_profile_mixed_kernels(glinalg_operator op, int precision, int n_launch,
                                                        double ms[2], double bytes[2])
{
    using namespace glinalg;
    if (!op || !ms || !bytes || n_launch <= 0)
        return invalid_arg("!op || !ms || !bytes || n_launch <= 0");
    if (op->kind != GLINALG_OP_STAGGERED_NORMAL) return GLINALG_ERROR_UNSUPPORTED_OP;
    GL_TRY(ensure_device());
    switch (precision) {
    case GLINALG_PREC_SINGLE: return profile_inner<float2, float2, float2>(op, 1, n_launch, ms, bytes);
    case GLINALG_PREC_HALF: return profile_inner<__half2, float2, float2>(op, 2, n_launch, ms, bytes);
    case GLINALG_PREC_BFLOAT: return profile_inner<__nv_bfloat162, float2, float2>(op, 3, n_launch, ms, bytes);
    default: return GLINALG_ERROR_INVALID_VALUE;
    }
}

extern "C" glinalg_status glinalg_profile_persist_kernel(glinalg_operator op, int precision, int n_launch,
                                                         int n_iter, double *ms, double *bytes, int *cand)
{
    using namespace glinalg;
    if (!op || !ms || !bytes || !cand || n_launch <= 0 || n_iter <= 0)
        return invalid_arg("!op || !ms || !bytes || !cand || n_launch <= 0 || n_iter <= 0");
    if (op->kind != GLINALG_OP_STAGGERED_NORMAL) return GLINALG_ERROR_UNSUPPORTED_OP;
    GL_TRY(ensure_device());
    switch (precision) {
    case GLINALG_PREC_SINGLE: return profile_persist<float2, float2, float2>(op, 1, n_launch, n_iter, ms, bytes, cand);
    case GLINALG_PREC_HALF: return profile_persist<__half2, float2, float2>(op, 2, n_launch, n_iter, ms, bytes, cand);
    case GLINALG_PREC_BFLOAT:
        return profile_persist<__nv_bfloat162, float2, float2>(op, 3, n_launch, n_iter, ms, bytes, cand);
    default: return GLINALG_ERROR_INVALID_VALUE;
    }
}

extern "C" int glinalg_tuned_tile(glinalg_operator op, int precision)
{
    return op ? glinalg::tuned_tile(op, precision) : -1;
}

extern "C" int glinalg_tuned_persist(glinalg_operator op, int precision)
{
    return op ? glinalg::tuned_persist(op, precision) : -1;
}
