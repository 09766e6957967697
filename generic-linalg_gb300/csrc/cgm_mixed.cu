// cgm_mixed.cu -- multishift CG for many sources of the staggered normal operator in mixed
// precision (glinalg_cg_m_multi with precision GLINALG_PREC_SINGLE).
//
// Phase 1: the multishift recurrence of generic_cg_m.cpp:312-600 for every source at once,
// with the base vectors (r, p, A p) and the operator in FP32, the scalar recurrences (beta,
// alpha, zeta_s, beta_s, alpha_s: complex, as in the reference) in FP64, and the shifted
// solutions x_s accumulated in FP64.  FP32 shifted solutions stop improving once their true
// residuals reach 1e-5..1e-6 of |b| (the rounding of the FP32 updates never enters them; the
// recurrence does not recompute them), so phase 1 stops each shift at max(eps, kPhase1Tol).
// Phase 2: every (source, shift) system is refined from its phase-1 solution by the mixed CG
// with FP64 reliable updates (cg_batch_mixed: all systems advanced together) to the FP64-true
// relative residual eps.  D^dagger D + sigma with mass m is exactly D^dagger D with mass
// sqrt(m^2 + sigma) (D = m + D_hop with D_hop anti-Hermitian, so D^dagger D = m^2 +
// D_hop^dagger D_hop), so each shifted system is a staggered normal system of its own mass.
//
// Blocked shift updates.  Each shift's direction and solution change by
//   x_s -= beta_s p_s;  p_s = zeta_s r + alpha_s p_s
// every iteration, so within a block of kBlk iterations starting at k0 both are linear
// combinations of p_s(k0) and the base residuals r(k0+1) .. r(k0+kBlk) with scalar
// coefficients.  Phase 1 keeps the last kBlk + 1 residuals in a ring, updates only the FP64
// coefficients each iteration (one warp per source, lane = basis vector), and every kBlk
// iterations (or when the source stops) writes x_s and p_s once, in one pass (k_mx_F).  The
// per-iteration shift traffic drops from 4 complex words per live shift to about
// (kBlk + 6 live) / kBlk, and x_s is summed in FP64 at no FP64-pipe cost.
//
// Phase-1 kernels, for all sources at once (grid.y = source), mirroring cgm_batch.cu:
//   C  r(k+1) = r(k) + beta Ap into the ring and |r|^2; in the source's last block: retire
//      converged shifts, alpha, alpha_s, then the shifts' coefficients
//   F  at a block's end: x_s += X_s . basis (FP64), p_s = P_s . basis (FP32)
//   A  p' = r + alpha p, then t = D p'
//   B  Ap = D^dagger t and <p', Ap>; in the source's last block: beta, zeta_s, beta_s
//   tail: sources that stopped (and flushed) are marked finished; all finished ends the loop.
// Sums: FP32 per thread, FP64 across threads and blocks.  The operator uses a FP32 hopping
// table with the 1/2 and eta(x) folded in (exact: powers of two and signs).

#include <algorithm>
#include <cmath>
#include <vector>

#include "solvers.h"
#include "stag_tiles.cuh"

namespace glinalg {
namespace {

constexpr int kMaxMixShifts = 32;
// Phase-1 target: the FP32 shifted solutions' true residuals level off at 1e-5..1e-6 |b|.
constexpr double kPhase1Tol = 1e-6;
constexpr int kBlk = 16;         // iterations per block of shift updates
constexpr int kNB = kBlk + 1;    // basis: p_s at the block's start, then r(k0+1) .. r(k0+kBlk)
constexpr int kRing = kBlk + 1;  // residuals kept: r(k) is in slot k % kRing

int mvec_grid(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

struct MxSrc {  // scalar state of one source (FP64)
    double2 alpha, beta;
    double rsq, bsq;
    int k, done, status, iters, napply, n_rem, n_rem_before, shift_updates;
    int k0;         // first iteration of the current block of shift updates
    int kr;         // the last residual in the ring is r(kr)
    int flush;      // 1: k_mx_F writes x_s and p_s in this pass
    int nflush;     // flushes done (bytes accounting)
    unsigned cnt[3];
};

struct MxArgs {
    MxSrc *src;
    double2 *zeta, *zeta_prev, *beta_s, *alpha_s;  // [q * ns + slot]
    double *shifts;                                 // [q * ns + slot], permuted with the slots
    int *map;                                       // [q * ns + slot] -> caller's shift index
    int *state;                                     // [q * ns + j]: 0 live, 1 retired, 2 written out
    double2 *Pc, *Xc;                               // [(q * ns + j) * kNB]: coefficients of p_s, dx_s
    double2 *X;                                     // [(q * ns + j) * n]: the caller's FP64 solutions
    float2 *Ps;                                     // [(q * ns + j) * n]: p_s at the block's start
    float2 *R;                                      // [(q * kRing + slot) * n]: the residual ring
    float2 *p0, *p1, *t, *Ap;                       // [q * n]
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

__device__ __forceinline__ float2 *ring(const MxArgs &a, int q, int k)
{
    return a.R + ((size_t)q * kRing + (k % kRing)) * a.n;
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
        s->flush = 1;  // write out what this block accumulated
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

// The source's bookkeeping once |r(k+1)|^2 = rn is known (generic_cg_m.cpp:424-513), called by
// every thread of the source's last block: retire converged shifts, alpha, alpha_s; then, on
// warp 0, the shifts' coefficients:
//   x_s -= beta_s p_s  for the shifts live when beta_s was formed,
//   p_s = zeta_s r(k+1) + alpha_s p_s  for the shifts still live.
__device__ void mx_bookkeeping(const MxArgs &a, MxSrc *s, int q, int k, double rn)
{
    __shared__ int sh_nb, sh_na, sh_idx;
    if (threadIdx.x == 0) {
        const double bsqrt = sqrt(s->bsq), srn = sqrt(rn);
        const int o = q * a.ns;
        const int nb = s->n_rem_before;
        if (k % a.rfc == 0) {
            for (int j = 0; j < s->n_rem; j++) {
                if (cabsd(a.zeta[o + j]) * srn < a.eps * bsqrt) {
                    s->n_rem--;
                    const int e = s->n_rem;
                    a.state[o + a.map[o + j]] = 1;
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
        int na = 0;
        if (!isfinite(rn)) {
            s->iters = k + 1;
            s->status = GLINALG_SOLVE_NONFINITE;
            s->done = 1;
        } else if (s->n_rem == 0 || last) {
            s->iters = k + 1;
            s->status = last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED;
            s->done = 1;
        } else {
            const double2 alpha = cmk(rn / s->rsq, 0.0);
            s->alpha = alpha;
            s->rsq = rn;
            for (int j = 0; j < s->n_rem; j++)
                a.alpha_s[o + j] =
                    cdiv(cmul(cmul(alpha, a.zeta[o + j]), a.beta_s[o + j]), cmul(a.zeta_prev[o + j], s->beta));
            s->k = k + 1;
            s->napply++;
            na = s->n_rem;
        }
        const int idx = k + 1 - s->k0;  // basis index of r(k+1)
        s->kr = k + 1;
        if (s->done || idx == kBlk) s->flush = 1;
        sh_nb = nb;
        sh_na = na;
        sh_idx = idx;
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    // warp 0: lane l updates basis coefficient l of every shift
    const int l = threadIdx.x, o = q * a.ns;
    const int nb = sh_nb, na = sh_na, idx = sh_idx;
    if (l >= kNB) return;
    for (int j = 0; j < nb; j++) {
        const size_t c = (size_t)(o + a.map[o + j]) * kNB + l;
        const double2 pc = a.Pc[c];
        a.Xc[c] = csub(a.Xc[c], cmul(a.beta_s[o + j], pc));
        if (j < na) a.Pc[c] = cadd(cmul(a.alpha_s[o + j], pc), l == idx ? a.zeta[o + j] : cmk(0.0, 0.0));
    }
}

// C: r(k+1) = r(k) + beta Ap into the ring, |r|^2, then the source's bookkeeping.
__global__ void __launch_bounds__(kRedThreads) k_mx_C(MxArgs a)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    const int k = s->k;
    const float2 *r = ring(a, q, k);
    float2 *rn_v = ring(a, q, k + 1);
    const float2 *Ap = a.Ap + q * n;
    const float2 bt = f2(s->beta);
    float vf = 0.f;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        const float2 ri = fadd(r[i], fmul(bt, Ap[i]));
        rn_v[i] = ri;
        vf += fn2(ri);
    }
    double v[1] = {(double)vf};
    if (!grid_sum_row<1, kRedThreads>(v, mrow_partials(a, q), &s->cnt[1])) return;
    mx_bookkeeping(a, s, q, k, v[0]);
}

// ---- register-tiled forms (lx a multiple of 32), using <p', A p'> = |D p'|^2 = |t|^2 for the
// Hermitian A = D^dagger D, so that an iteration is two stencil kernels and A p is never stored:
//   At  p' = r + alpha p (formed at every site it is read), t = D p', |t|^2; then beta, zeta_s,
//       beta_s in the source's last block
//   Bt  Ap = D^dagger t, r(k+1) = r(k) + beta Ap into the ring, |r|^2; then the bookkeeping
// A warp owns a tile of 32 columns by kTNY rows; a lane holds its column for rows -1 .. kTNY in
// registers (y-neighbours) and takes x-neighbours from the adjacent lanes by shuffle (lanes 0
// and 31 load across the tile edge).

constexpr int kTNY = 4;                    // rows per warp tile
constexpr int kTWarps = kRedThreads / 32;  // warps per block
// Tiles per warp, at most: a block covers kTWarps * runs tiles of its source, so its reduction
// and its launch serve that many more sites, as long as all sources together still give every
// SM kMinBlocksPerSM blocks.  512^2, 64 sources: the multishift phase takes 158.5 ms with one
// tile a warp, 140.3 with two, 133.4 with four, 137.3 with eight (8-row tiles, two a warp:
// 142.6).
constexpr int kTileRuns = 4;
constexpr int kMinBlocksPerSM = 4;
// Blocks of k_mx_F per source: nb / runs, runs at most kFlushRuns (and again at least
// kMinBlocksPerSM blocks an SM over all sources).  The kernel runs every iteration but
// flushes every kBlk-th; a smaller grid makes the other launches cheap (multishift phase,
// 64 sources: 133.8 ms with nb blocks, 124.2 with nb / 4, 122.5 with nb / 8).
constexpr int kFlushRuns = 8;
// Reliable-update threshold of the refinement: an FP64 true residual whenever the iterated one
// has fallen by this factor.  The refinement starts 1e-5..1e-6 from its tolerance, so three
// orders of magnitude between FP64 updates leave one or two updates per system, each a FP64
// operator pass bound by GB300's FP64 rate.  512^2, 64 sources: 656 ms with 0.1, 584 with the
// single-system default 0.01, 557 with 0.001.
constexpr double kRefineDelta = 1e-3;

__device__ __forceinline__ float2 shfl_dn2(float2 v)
{
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
}
__device__ __forceinline__ float2 shfl_up2f(float2 v)
{
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
}

// Calls body(i, f(i), hs) for the tile's rows below nrow, hs as in hop32; ld(j) gives f at j.
template <class Ld, class Body>
__device__ __forceinline__ void tile32_hops(Ld ld, const float2 *__restrict__ H, int lx, int ly, int x0, int y0,
                                            int nrow, Body body)
{
    const int lane = threadIdx.x & 31;
    const int x = x0 + lane;
    const int xl = x == 0 ? lx - 1 : x - 1, xr = x + 1 == lx ? 0 : x + 1;
    float2 col[kTNY + 2], hyc[kTNY + 1];
#pragma unroll
    for (int j = 0; j < kTNY + 2; j++) {
        int y = y0 - 1 + j;
        y = y < 0 ? y + ly : (y >= ly ? y - ly : y);
        col[j] = ld((long)y * lx + x);
        if (j < kTNY + 1) hyc[j] = H[2 * ((long)y * lx + x) + 1];
    }
#pragma unroll
    for (int q = 0; q < kTNY; q++) {
        if (q >= nrow) break;
        const long row = (long)(y0 + q) * lx;
        const long i = row + x;
        const float2 c = col[q + 1];
        float2 fr = shfl_dn2(c), fl = shfl_up2f(c);
        const float2 hx = H[2 * i];
        float2 hxm = shfl_up2f(hx);
        if (lane == 31) fr = ld(row + xr);
        if (lane == 0) {
            fl = ld(row + xl);
            hxm = H[2 * (row + xl)];
        }
        float2 hs = fmul(hx, fr);
        hs = fsub(hs, fmulc(hxm, fl));
        hs = fadd(hs, fmul(hyc[q + 1], col[q + 2]));
        hs = fsub(hs, fmulc(hyc[q], col[q]));
        body(i, c, hs);
    }
}

__global__ void __launch_bounds__(kRedThreads) k_mx_At(MxArgs a, int setup)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    const int k = s->k;
    const float2 alpha = f2(s->alpha);
    const float2 *r = ring(a, q, k);
    const float2 *pold = ((k & 1) ? a.p0 : a.p1) + q * n;
    float2 *pnew = ((k & 1) ? a.p1 : a.p0) + q * n;
    float2 *t = a.t + q * n;
    const float mass = a.mass;
    const int ntx = a.lx / 32, ntiles = ntx * ((a.ly + kTNY - 1) / kTNY);
    const int warp = threadIdx.x >> 5;
    float acc = 0.f;
    for (int tile = blockIdx.x * kTWarps + warp; tile < ntiles; tile += gridDim.x * kTWarps) {
        const int x0 = (tile % ntx) * 32, y0 = (tile / ntx) * kTNY, nrow = min(kTNY, a.ly - y0);
        if (setup) {
            auto ld = [pnew](long j) { return pnew[j]; };
            tile32_hops(ld, a.H, a.lx, a.ly, x0, y0, nrow, [&](long i, float2 c, float2 hs) {
                const float2 tv = fsub(fscale(mass, c), hs);
                t[i] = tv;
                acc += fn2(tv);
            });
        } else {
            auto ld = [r, pold, alpha](long j) { return fadd(r[j], fmul(alpha, pold[j])); };
            tile32_hops(ld, a.H, a.lx, a.ly, x0, y0, nrow, [&](long i, float2 c, float2 hs) {
                pnew[i] = c;
                const float2 tv = fsub(fscale(mass, c), hs);
                t[i] = tv;
                acc += fn2(tv);
            });
        }
    }
    double v[1] = {(double)acc};
    if (grid_sum_row<1, kRedThreads>(v, mrow_partials(a, q), &s->cnt[0]) && threadIdx.x == 0)
        mx_beta_scalars(a, s, q, v[0], 0.0);
}

__global__ void __launch_bounds__(kRedThreads) k_mx_Bt(MxArgs a)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    const int k = s->k;
    const float2 *r = ring(a, q, k);
    float2 *rn_v = ring(a, q, k + 1);
    const float2 *t = a.t + q * n;
    const float2 bt = f2(s->beta);
    const float mass = a.mass;
    const int ntx = a.lx / 32, ntiles = ntx * ((a.ly + kTNY - 1) / kTNY);
    const int warp = threadIdx.x >> 5;
    float acc = 0.f;
    auto ld = [t](long j) { return t[j]; };
    for (int tile = blockIdx.x * kTWarps + warp; tile < ntiles; tile += gridDim.x * kTWarps) {
        const int x0 = (tile % ntx) * 32, y0 = (tile / ntx) * kTNY, nrow = min(kTNY, a.ly - y0);
        tile32_hops(ld, a.H, a.lx, a.ly, x0, y0, nrow, [&](long i, float2 c, float2 hs) {
            const float2 ap = fadd(fscale(mass, c), hs);
            const float2 rv = fadd(r[i], fmul(bt, ap));
            rn_v[i] = rv;
            acc += fn2(rv);
        });
    }
    double v[1] = {(double)acc};
    if (!grid_sum_row<1, kRedThreads>(v, mrow_partials(a, q), &s->cnt[1])) return;
    mx_bookkeeping(a, s, q, k, v[0]);
}

// F: at the end of a block (or of the source), for every shift not yet written out:
//   x_s += sum_l X_s[l] basis_l (summed in FP32, added in FP64), and for live shifts
//   p_s = sum_l P_s[l] basis_l, with basis_0 = p_s at the block's start and basis_l = r(k0+l).
// The source's last block then resets the coefficients for the next block.
__global__ void __launch_bounds__(kRedThreads) k_mx_F(MxArgs a)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done == 2 || !s->flush) return;
    __shared__ float2 cx[kMaxMixShifts][kNB], cp[kMaxMixShifts][kNB];
    __shared__ int jl[kMaxMixShifts], live[kMaxMixShifts];
    __shared__ int nj, ticket;
    const long n = a.n;
    const int o = q * a.ns;
    const int k0 = s->k0;
    // basis vectors used: r(k0+1) .. r(kend), the residuals of this block in the ring
    const int kend = s->kr;
    const int nbv = min(kend - k0, kBlk);
    if (threadIdx.x == 0) {
        int m = 0;
        for (int j = 0; j < a.ns; j++) {
            const int st = a.state[o + j];
            if (st == 2) continue;
            jl[m] = j;
            live[m] = st == 0 && !s->done;
            m++;
        }
        nj = m;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nj * kNB; e += kRedThreads) {
        const int m = e / kNB, l = e % kNB;
        const size_t c = (size_t)(o + jl[m]) * kNB + l;
        cx[m][l] = f2(a.Xc[c]);
        cp[m][l] = f2(a.Pc[c]);
    }
    __syncthreads();
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
        float2 rv[kBlk];
#pragma unroll
        for (int l = 0; l < kBlk; l++) rv[l] = l < nbv ? ring(a, q, k0 + 1 + l)[i] : make_float2(0.f, 0.f);
        for (int m = 0; m < nj; m++) {
            const size_t f = (size_t)(o + jl[m]) * n + i;
            const float2 p0 = a.Ps[f];
            float2 dx = fmul(cx[m][0], p0), pn = fmul(cp[m][0], p0);
#pragma unroll
            for (int l = 0; l < kBlk; l++) {
                dx = fadd(dx, fmul(cx[m][l + 1], rv[l]));
                pn = fadd(pn, fmul(cp[m][l + 1], rv[l]));
            }
            const double2 xo = a.X[f];
            a.X[f] = make_double2(xo.x + (double)dx.x, xo.y + (double)dx.y);
            if (live[m]) a.Ps[f] = pn;
        }
    }
    // the last block to finish resets the coefficients and opens the next block
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        ticket = atomicAdd(&s->cnt[2], 1u);
    }
    __syncthreads();
    if (ticket != gridDim.x - 1) return;
    __threadfence();
    for (int e = threadIdx.x; e < nj * kNB; e += kRedThreads) {
        const int m = e / kNB, l = e % kNB;
        const size_t c = (size_t)(o + jl[m]) * kNB + l;
        a.Xc[c] = cmk(0.0, 0.0);
        a.Pc[c] = cmk(l == 0 ? 1.0 : 0.0, 0.0);
    }
    if (threadIdx.x == 0) {
        for (int m = 0; m < nj; m++)
            if (!live[m]) a.state[o + jl[m]] = 2;
        s->k0 = kend;
        s->flush = 0;
        s->nflush++;
        s->cnt[2] = 0;
    }
}

// A: p' = r + alpha p at every site of the source, then t = D p'.
// setup = 1: p' = p0 as stored (the source).
__global__ void __launch_bounds__(kRedThreads) k_mx_A(MxArgs a, int setup)
{
    const int q = blockIdx.y;
    MxSrc *s = a.src + q;
    if (s->done) return;
    const long n = a.n;
    const int k = s->k;
    const float2 alpha = f2(s->alpha);
    const float2 *r = ring(a, q, k);
    const float2 *pold = ((k & 1) ? a.p0 : a.p1) + q * n;
    float2 *pnew = ((k & 1) ? a.p1 : a.p0) + q * n;
    const float mass = a.mass;
    for (long i = blockIdx.x * (long)kRedThreads + threadIdx.x; i < n; i += (long)gridDim.x * kRedThreads) {
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

// Sources that stopped and have written their shifts out are finished; all finished ends the
// loop.
__global__ void k_mx_tail(MxArgs a)
{
    if (threadIdx.x != 0) return;
    int fin = 0;
    for (int q = 0; q < a.nrhs; q++) {
        MxSrc *s = a.src + q;
        if (s->done == 1 && !s->flush) s->done = 2;
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

// x_s = 0 (FP64), p_s = b, r(0) = p = b (FP32) (generic_cg_m.cpp:372-391)
__global__ void k_mx_init(MxArgs a)
{
    const int q = blockIdx.y;
    const long n = a.n;
    float2 *r0 = ring(a, q, 0);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 bi = f2(a.b[q * n + i]);
        for (int j = 0; j < a.ns; j++) {
            a.X[((long)q * a.ns + j) * n + i] = make_double2(0.0, 0.0);
            a.Ps[((long)q * a.ns + j) * n + i] = bi;
        }
        r0[i] = bi;
        a.p0[q * n + i] = bi;
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
    GL_TRY(sc.alloc(&a.Ps, (size_t)n_rhs * ns * n));
    GL_TRY(sc.alloc(&a.R, (size_t)n_rhs * kRing * n));
    GL_TRY(sc.zeros(&a.state, (size_t)n_rhs * ns));
    GL_TRY(sc.zeros(&a.Xc, (size_t)n_rhs * ns * kNB));
    GL_TRY(sc.alloc(&a.Pc, (size_t)n_rhs * ns * kNB));
    GL_TRY(sc.alloc(&a.p0, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.p1, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.Ap, (size_t)n_rhs * n));
    GL_TRY(sc.alloc(&a.t, (size_t)n_rhs * n));
    float2 *H;
    GL_TRY(sc.alloc(&H, 2 * (size_t)n));
    a.H = H;
    // the register-tiled kernels (lx a multiple of 32): one block of warps per kTWarps * runs
    // tiles
    const bool tiled = op->lx % 32 == 0;
    const int ntiles = (op->lx / 32) * ((op->ly + kTNY - 1) / kTNY);
    const long min_blocks = (long)kMinBlocksPerSM * sm_count();
    const int runs = (int)std::max(1L, std::min((long)kTileRuns, (long)ntiles * n_rhs / (kTWarps * min_blocks)));
    const int tg = tiled ? (ntiles + kTWarps * runs - 1) / (kTWarps * runs) : 0;
    GL_TRY(sc.alloc(&a.partials, (size_t)n_rhs * 2 * std::max(nb, tg)));
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
        std::vector<double2> pc((size_t)n_rhs * ns * kNB, cmk(0.0, 0.0));
        for (size_t c = 0; c < pc.size(); c += kNB) pc[c] = cmk(1.0, 0.0);
        GL_CUDA(cudaMemcpyAsync(a.Pc, pc.data(), sizeof(double2) * pc.size(), cudaMemcpyHostToDevice, st));
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
    a.X = X;
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
    const int fruns = (int)std::max(1L, std::min((long)kFlushRuns, (long)nb * n_rhs / min_blocks));
    const dim3 fg(std::max(1, nb / fruns), n_rhs);
    k_mx_hop<<<mvec_grid(n), 256, 0, st>>>(H, op->U, op->lx, n);
    k_mx_init<<<vg, 256, 0, st>>>(a);
    k_mx_norms<<<rg, kRedThreads, 0, st>>>(a);
    GL_CUDA(cudaGetLastError());
    if (max_iter > 0 && tiled) {
        const dim3 tgr(tg, n_rhs);
        // setup: t = D b and the first beta
        k_mx_At<<<tgr, kRedThreads, 0, st>>>(a, 1);
        k_mx_tail<<<1, 32, 0, st>>>(a);
        GL_CUDA(cudaGetLastError());
        GL_TRY(run_loop(st, a.all_done, [&](cudaStream_t cs) -> glinalg_status {
            k_mx_Bt<<<tgr, kRedThreads, 0, cs>>>(a);
            k_mx_F<<<fg, kRedThreads, 0, cs>>>(a);
            k_mx_At<<<tgr, kRedThreads, 0, cs>>>(a, 0);
            k_mx_tail<<<1, 32, 0, cs>>>(a);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    } else if (max_iter > 0) {
        // setup: Ap = A b and the first beta
        k_mx_A<<<rg, kRedThreads, 0, st>>>(a, 1);
        k_mx_B<<<rg, kRedThreads, 0, st>>>(a);
        k_mx_tail<<<1, 32, 0, st>>>(a);
        GL_CUDA(cudaGetLastError());
        GL_TRY(run_loop(st, a.all_done, [&](cudaStream_t cs) -> glinalg_status {
            k_mx_C<<<rg, kRedThreads, 0, cs>>>(a);
            k_mx_F<<<fg, kRedThreads, 0, cs>>>(a);
            k_mx_A<<<rg, kRedThreads, 0, cs>>>(a, 0);
            k_mx_B<<<rg, kRedThreads, 0, cs>>>(a);
            k_mx_tail<<<1, 32, 0, cs>>>(a);
            GL_CUDA(cudaGetLastError());
            return GLINALG_SUCCESS;
        }));
    }
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
                                       kRefineDelta, inf2.data(), st);
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
        // phase 1 per iteration: C r, Ap in, r out (3 FP32 words); A r, p in, p', t out, 2 links
        // (6); B t in, Ap out, p' in, 2 links (5); per flush the block's residuals (at most kBlk
        // FP32 words) once, and per shift not yet written out p_s in and out (2 FP32 words) and
        // x_s in and out (2 FP64 words)
        const double words = tiled ? 11.0 : 14.0;  // tiled: A r, p in, p', t out, 2 links; B t in, r in and out, 2 links
        const double gb1 = ((double)h.iters * words * 8.0 + (double)h.nflush * (kBlk * 8.0 + ns * 48.0)) * n * 1e-9;
        info->gbytes = gb1 + gb;
        // the FP32 multishift phase of the whole batch (every source), and its bytes for this source
        info->kernel_ms = ms - ms2;
        info->kernel_gbytes = gb1;
        fill_name(info, "CG-M-FP32");
    }
    return GLINALG_SUCCESS;
}

}  // namespace glinalg
