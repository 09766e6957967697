// cg_batch.cu -- CG with reduced-precision inner iterations and FP64 reliable updates on many
// independent Hermitian systems of different sizes and kinds (staggered D^dagger D and the
// gauge Laplacian), all advanced by the same kernels (glinalg_cg_batch).  The reference solves
// one system per minv_vector_cg call (generic_cg.cpp:278-382).
//
// Per system the algorithm is the single-system mixed solver's (cg_mixed.cu: the same MxDev
// state, the same scalar updates mx_after_A / mx_after_B, the same reliable-update steps and
// the same tile bodies), so each system converges to the same FP64-true tolerance.
//
// Layout: the work vectors of all systems are packed one after another (system s starts at
// site sys[s].off).  Inner kernels work on tiles of one system (32 columns by BY * NY rows,
// numbered system by system); the vector and FP64 kernels on blocks of up to 1024 sites of one
// system.  Every reduction is over the blocks of one system (grid_sum_*_ids with the block's
// index inside its system), so a system's sums do not depend on the other systems.
//
// Control: the graph body is kBatchUnroll inner iterations (A, B) for the systems that are
// iterating, then the reliable-update steps (R1, FP64 operator, R2, R3, R4) for the systems
// that flagged one, then a tail that re-arms those systems and ends the loop when every system
// has stopped.  A system that flags an update during the unrolled iterations waits for the end
// of the pass; its own arithmetic does not depend on the pass structure.  The kernels do not
// launch a block per tile of every system: a list kernel (k_bList) writes the (system, block)
// pairs of the systems that still run (every kListEvery inner iterations, the tiles of the
// systems that are iterating; before the reliable-update steps, the vector blocks of the
// systems that flagged one), and a grid of resident blocks walks that list.  Every kernel still reads its system's flags first and skips a system with
// nothing to do (one that flagged an update or stopped during the pass).  The tile shape of
// the inner kernels is picked for the batch by timing the candidates.

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "mixed_state.cuh"
#include "sites.cuh"

namespace glinalg {

// bounded spin on the device clock (cg_mixed.cu)
__global__ void k_busy_wait(long long ns);

namespace {

// Inner iterations per graph pass.  A system that flags a reliable update idles until the pass
// ends; a longer pass spreads the per-pass kernels (reliable update, tail, loop guard) over more
// iterations.  The 256-system workload: 108 ms with 4, 98 with 8, 92 with 16, 90 with 32.
constexpr int kBatchUnroll = 32;
// Inner iterations between rebuilds of the tile list: a system that flags a reliable update
// leaves the list at the next rebuild instead of the pass's end.  64-source multishift:
// 646 ms rebuilding once a pass, 619 every 4 iterations, 617 every iteration (where the
// uneven batch loses 4 ms to the extra list launches).
constexpr int kListEvery = 4;
constexpr int kVecSites = 1024;  // sites per block of the vector kernels (256 threads x 4)

struct BSys {
    long off;          // first site in the packed work vectors
    long loff;         // first site of its packed link table (systems with the same links share one)
    int lown;          // 1: this system packs the table at loff
    const double2 *U;  // FP64 links (the operator's device copy)
    double2 *x;        // FP64 solution (device)
    const double2 *b;  // source (device)
    double mass;       // staggered: mass; Laplace: the reference's additive mass
    int lx, ly, stag, xs;  // stag: D^dagger D (else Laplace); xs: lx % 32 == 0
    int tb0, ntb, tiles_x;
    int vb0, nvb;
};

template <class S, class R, class LK>
struct BArgs {
    const BSys *sys;
    MxDev *st;
    const int *vblk;  // system of each vector block (the one-off kernels: norms, links)
    R *r;
    S *p0, *p1, *t;
    float2 *xlo;
    LK *L;
    double2 *rhi, *tmp64, *Ax;
    double *tpart, *vpart;
    int *all_done;
    int nsys;
    const int2 *tlist, *vlist;  // (system, tile block) / (system, vector block) pairs to run
    const int *ntl, *nvl;       // their lengths
};

// ---------------------------------------------------------------- Laplace tile bodies
// The arithmetic of k_lapA / k_lapB (cg_mixed.cu), NY rows of column x per thread.

template <class S, class R, class LK, int NY>
__device__ __forceinline__ float lap_tile_A(const R *r, const S *pold, S *pnew, S *Ap, const LK *G,
                                            float beta, float diag, int lx, int ly, int x, int ybase)
{
    float acc = 0.f;
    if (x >= lx) return acc;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int y = ybase + q;
        if (y >= ly) break;
        const int xp = x + 1 == lx ? 0 : x + 1, xm = x == 0 ? lx - 1 : x - 1;
        const int yp = y + 1 == ly ? 0 : y + 1, ym = y == 0 ? ly - 1 : y - 1;
        const long i = (long)y * lx + x;
        auto P = [&](long j) { return fadd(Fmt<R>::ld(r, j), fscale(beta, Fmt<S>::ld(pold, j))); };
        const float2 pc = P(i);
        float2 hs = fmul(Fmt<LK>::ld(G, 2 * i), P((long)y * lx + xp));
        hs = fadd(hs, fmulc(Fmt<LK>::ld(G, 2 * ((long)y * lx + xm)), P((long)y * lx + xm)));
        hs = fadd(hs, fmul(Fmt<LK>::ld(G, 2 * i + 1), P((long)yp * lx + x)));
        hs = fadd(hs, fmulc(Fmt<LK>::ld(G, 2 * ((long)ym * lx + x) + 1), P((long)ym * lx + x)));
        const float2 av = fsub(fscale(diag, pc), hs);
        Fmt<S>::st(pnew, i, pc);
        Fmt<S>::st(Ap, i, av);
        const float2 pq = Fmt<S>::round(pc), aq = Fmt<S>::round(av);
        acc += pq.x * aq.x + pq.y * aq.y;
    }
    return acc;
}

template <class S, class R, int NY>
__device__ __forceinline__ float lap_tile_B(const S *Ap, const S *p, R *r, float2 *xlo, float alpha, int lx,
                                            int ly, int x, int ybase)
{
    float acc = 0.f;
    if (x >= lx) return acc;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int y = ybase + q;
        if (y >= ly) break;
        const long i = (long)y * lx + x;
        const float2 pc = Fmt<S>::ld(p, i);
        xlo[i] = fadd(xlo[i], fscale(alpha, pc));
        const float2 rn = Fmt<R>::round(fsub(Fmt<R>::ld(r, i), fscale(alpha, Fmt<S>::ld(Ap, i))));
        Fmt<R>::st(r, i, rn);
        acc += fn2(rn);
    }
    return acc;
}

// ---------------------------------------------------------------- inner kernels

// A: p' = r + beta p ; t = D p' and |t|^2 (staggered) or Ap = L p' and <p', Ap> (Laplace)
template <class S, class R, class LK, int BY, int NY>
__device__ __forceinline__ void bA_tile(const BArgs<S, R, LK> &a, int sid, int lb)
{
    const BSys sy = a.sys[sid];
    MxDev *s = a.st + sid;
    if (s->done || s->reliable) return;
    const int x = (lb % sy.tiles_x) * 32 + threadIdx.x;
    const int ybase = (lb / sy.tiles_x) * (BY * NY) + threadIdx.y * NY;
    const int par = s->parity;
    const long o = sy.off;
    const S *pold = (par ? a.p1 : a.p0) + o;
    S *pnew = (par ? a.p0 : a.p1) + o;
    const float beta = (float)s->beta;
    float acc[1];
    if (!sy.stag)
        acc[0] = lap_tile_A<S, R, LK, NY>(a.r + o, pold, pnew, a.t + o, a.L + 2 * sy.loff, beta, (float)(4.0 + sy.mass),
                                          sy.lx, sy.ly, x, ybase);
    else if (sy.xs)
        acc[0] = tile_A<S, R, LK, NY, true, false>(a.r + o, pold, pnew, a.t + o, a.L + 2 * sy.loff, beta, (float)sy.mass,
                                                   0.f, sy.lx, sy.ly, threadIdx.x, x, true, ybase);
    else
        acc[0] = tile_A<S, R, LK, NY, false, false>(a.r + o, pold, pnew, a.t + o, a.L + 2 * sy.loff, beta,
                                                    (float)sy.mass, 0.f, sy.lx, sy.ly, threadIdx.x, x, x < sy.lx,
                                                    ybase);
    double out[1];
    if (grid_sum_f_ids<1, 32 * BY>(acc, a.tpart + sy.tb0, &s->cnt[0], out, lb, sy.ntb) && threadIdx.x == 0 &&
        threadIdx.y == 0)
        mx_after_A(s, out[0], 0, 0);
}

// B: Ap = D^dagger t (staggered; Laplace reads Ap from t) ; x_lo += alpha p' ; r -= alpha Ap
template <class S, class R, class LK, int BY, int NY>
__device__ __forceinline__ void bB_tile(const BArgs<S, R, LK> &a, int sid, int lb)
{
    const BSys sy = a.sys[sid];
    MxDev *s = a.st + sid;
    if (s->done || s->reliable) return;
    const int x = (lb % sy.tiles_x) * 32 + threadIdx.x;
    const int ybase = (lb / sy.tiles_x) * (BY * NY) + threadIdx.y * NY;
    const int par = s->parity;  // A wrote the new direction into the other buffer
    const long o = sy.off;
    const S *p = (par ? a.p0 : a.p1) + o;
    const float alpha = (float)s->alpha;
    float acc[1];
    if (!sy.stag)
        acc[0] = lap_tile_B<S, R, NY>(a.t + o, p, a.r + o, a.xlo + o, alpha, sy.lx, sy.ly, x, ybase);
    else if (sy.xs)
        acc[0] = tile_B<S, R, LK, NY, true, false>(a.t + o, p, a.r + o, a.xlo + o, a.L + 2 * sy.loff, alpha,
                                                   (float)sy.mass, 0.f, sy.lx, sy.ly, threadIdx.x, x, true, ybase);
    else
        acc[0] = tile_B<S, R, LK, NY, false, false>(a.t + o, p, a.r + o, a.xlo + o, a.L + 2 * sy.loff, alpha,
                                                    (float)sy.mass, 0.f, sy.lx, sy.ly, threadIdx.x, x, x < sy.lx,
                                                    ybase);
    double out[1];
    if (grid_sum_f_ids<1, 32 * BY>(acc, a.tpart + sy.tb0, &s->cnt[1], out, lb, sy.ntb) && threadIdx.x == 0 &&
        threadIdx.y == 0)
        mx_after_B(s, out[0], 1 - par, 0, 0);
}

// The inner kernels: a grid of resident blocks takes the tiles of the list in order.  Block b
// starts with entry b; while a tile runs, its first thread claims the next entry from the
// launch's counter (zeroed by k_bList), so the tiles in flight stay a narrow window of the
// list, as a launch with one block per tile would keep them: neighbouring tiles share their
// halo rows and the shifted systems of one source their link table in L2.  A tile whose system
// skips returns before any barrier, so the whole block takes the same path through the
// reduction.  MINB: blocks per SM that the register budget must allow (the warps an SM keeps in
// flight: 32 warps need 64 registers a thread).
template <class S, class R, class LK, int BY, int NY, int MINB>
__global__ void __launch_bounds__(32 * BY, MINB) k_bA(BArgs<S, R, LK> a, int *claim)
{
    __shared__ int next;
    const int nt = *a.ntl;
    const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
    for (int v = blockIdx.x; v < nt;) {
        int c = 0;
        if (lead) c = atomicAdd(claim, 1);
        const int2 e = a.tlist[v];
        bA_tile<S, R, LK, BY, NY>(a, e.x, e.y);
        if (lead) next = c + (int)gridDim.x;
        __syncthreads();
        v = next;
        __syncthreads();
    }
}

template <class S, class R, class LK, int BY, int NY, int MINB>
__global__ void __launch_bounds__(32 * BY, MINB) k_bB(BArgs<S, R, LK> a, int *claim)
{
    __shared__ int next;
    const int nt = *a.ntl;
    const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
    for (int v = blockIdx.x; v < nt;) {
        int c = 0;
        if (lead) c = atomicAdd(claim, 1);
        const int2 e = a.tlist[v];
        bB_tile<S, R, LK, BY, NY>(a, e.x, e.y);
        if (lead) next = c + (int)gridDim.x;
        __syncthreads();
        v = next;
        __syncthreads();
    }
}

// Lists the blocks that the next kernels run: mode 0, the tile blocks of every system that is
// iterating (not stopped, no reliable update pending; for the inner kernels); mode 1, the
// vector blocks of every system that runs a reliable update in this pass.  Entries are
// (system, block index inside the system), system by system.  Every block forms the same
// prefix sum of the systems' block counts (1024 systems at a time, blockDim.x = 1024) and
// writes the entries of the systems q with q % gridDim.x == blockIdx.x.  Mode 0 also zeroes
// the nclaim claim counters of the inner kernels.
__global__ void __launch_bounds__(1024) k_bList(const BSys *sys, const MxDev *st, int nsys, int mode, int2 *list,
                                                int *total, int *claims, int nclaim)
{
    if (mode == 0 && blockIdx.x == 0)
        for (int j = threadIdx.x; j < nclaim; j += blockDim.x) claims[j] = 0;
    __shared__ int wsum[32];
    __shared__ int cstart[1024], ccnt[1024];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nsys; c0 += 1024) {
        const int q = c0 + threadIdx.x;
        int cnt = 0;
        if (q < nsys) {
            const bool on = mode == 0 ? !(st[q].done || st[q].reliable) : (st[q].reliable && !st[q].done);
            cnt = on ? (mode == 0 ? sys[q].ntb : sys[q].nvb) : 0;
        }
        int inc = cnt;  // inclusive scan within the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            int w = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const int start = carry + (warp ? wsum[warp - 1] : 0) + inc - cnt;
        cstart[threadIdx.x] = start;
        ccnt[threadIdx.x] = cnt;
        __syncthreads();
        if (threadIdx.x == 1023) carry = start + cnt;
        const int m = min(1024, nsys - c0);
        const int G = gridDim.x;
        for (int j = ((int)blockIdx.x - c0 % G + G) % G; j < m; j += G) {
            const int n = ccnt[j], b = cstart[j];
            for (int e = threadIdx.x; e < n; e += 1024) list[b + e] = make_int2(c0 + j, e);
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *total = carry;
}

// ---------------------------------------------------------------- reliable-update kernels
// One block covers up to kVecSites sites of one system; `upd` is true for systems that run a
// reliable update in this pass.

#define BATCH_VEC_PROLOGUE                                                                  \
    const BSys sy = a.sys[sid];                                                             \
    MxDev *s = a.st + sid;                                                                  \
    if (s->done || !s->reliable) return;                                                    \
    const long n = (long)sy.lx * sy.ly, o = sy.off;                                         \
    const long i0 = (long)lb * kRedThreads + threadIdx.x, di = (long)sy.nvb * kRedThreads;

// R1: x_hi += scale x_lo ; x_lo = 0
template <class S, class R, class LK>
__device__ __forceinline__ void bR1_blk(const BArgs<S, R, LK> &a, int sid, unsigned lb)
{
    BATCH_VEC_PROLOGUE
    const double sc = s->scale;
    for (long i = i0; i < n; i += di) {
        const float2 d = a.xlo[o + i];
        const double2 xv = sy.x[i];
        sy.x[i] = cmk(xv.x + sc * (double)d.x, xv.y + sc * (double)d.y);
        a.xlo[o + i] = make_float2(0.f, 0.f);
    }
}

// FP64 operator on x: staggered pass 1 (tmp = D x) or the Laplacian (Ax = L x)
template <class S, class R, class LK>
__device__ __forceinline__ void bOp1_blk(const BArgs<S, R, LK> &a, int sid, unsigned lb)
{
    BATCH_VEC_PROLOGUE
    const double2 *x = sy.x;
    auto ld = [x](long j) { return x[j]; };
    for (long i = i0; i < n; i += di) {
        if (sy.stag) a.tmp64[o + i] = stag_site(ld, sy.U, sy.mass, sy.lx, sy.ly, +1.0, i);
        else a.Ax[o + i] = lap_site(ld, sy.U, sy.mass, sy.lx, sy.ly, i);
    }
}

// staggered pass 2: Ax = D^dagger tmp
template <class S, class R, class LK>
__device__ __forceinline__ void bOp2_blk(const BArgs<S, R, LK> &a, int sid, unsigned lb)
{
    BATCH_VEC_PROLOGUE
    if (!sy.stag) return;
    const double2 *tm = a.tmp64 + o;
    auto ld = [tm](long j) { return tm[j]; };
    for (long i = i0; i < n; i += di) a.Ax[o + i] = stag_site(ld, sy.U, sy.mass, sy.lx, sy.ly, -1.0, i);
}

// R2: r_hi = b - A x ; |r_hi|^2 -> convergence and the new scale (as k_mx_R2, sigma = 0)
template <class S, class R, class LK>
__device__ __forceinline__ void bR2_blk(const BArgs<S, R, LK> &a, int sid, unsigned lb)
{
    BATCH_VEC_PROLOGUE
    double v[1] = {0.0};
    for (long i = i0; i < n; i += di) {
        const double2 ri = csub(sy.b[i], a.Ax[o + i]);
        a.rhi[o + i] = ri;
        v[0] += cabs2(ri);
    }
    if (!(grid_sum_ids<1, kRedThreads>(v, a.vpart + 2 * sy.vb0, &s->cnt[2], lb, sy.nvb) && threadIdx.x == 0))
        return;
    const double rt = v[0];
    s->rsq_old_true = s->rsq * s->scale * s->scale;
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
    if (rt == 0.0) {  // exactly zero residual: x is exact (as k_mx_R2)
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
    s->pscale = s->scale / new_scale;
    s->scale = new_scale;
    s->rmax = sqrt(rt);
}

// R3: r_lo = r_hi / scale ; p *= pscale ; <r_lo, p>, |r_lo|^2 (as k_mx_R3)
template <class S, class R, class LK>
__device__ __forceinline__ void bR3_blk(const BArgs<S, R, LK> &a, int sid, unsigned lb)
{
    BATCH_VEC_PROLOGUE
    S *plo = (s->parity ? a.p1 : a.p0) + o;
    R *rlo = a.r + o;
    const double inv = 1.0 / s->scale;
    const float f = (float)s->pscale;
    double v[2] = {0.0, 0.0};
    for (long i = i0; i < n; i += di) {
        const double2 rh = a.rhi[o + i];
        Fmt<R>::st(rlo, i, make_float2((float)(rh.x * inv), (float)(rh.y * inv)));
        const float2 pq = fscale(f, Fmt<S>::ld(plo, i));
        Fmt<S>::st(plo, i, pq);
        const float2 rq = Fmt<R>::ld(rlo, i), pr = Fmt<S>::ld(plo, i);
        v[0] += (double)(rq.x * pr.x + rq.y * pr.y);
        v[1] += (double)fn2(rq);
    }
    if (grid_sum_ids<2, kRedThreads>(v, a.vpart + 2 * sy.vb0, &s->cnt[3], lb, sy.nvb) && threadIdx.x == 0) {
        const double rr = v[1];
        s->rp = rr > 0.0 ? v[0] / rr : 0.0;
        const double sc2 = s->scale * s->scale;
        s->beta = s->rsq_old_true > 0.0 ? (rr * sc2) / s->rsq_old_true : 0.0;
        s->rsq = rr;
    }
}

// R4: p0 = p - rp r_lo (the direction is in p0 afterwards)
template <class S, class R, class LK>
__device__ __forceinline__ void bR4_blk(const BArgs<S, R, LK> &a, int sid, unsigned lb)
{
    BATCH_VEC_PROLOGUE
    const S *plo = (s->parity ? a.p1 : a.p0) + o;
    S *p0 = a.p0 + o;
    const R *rlo = a.r + o;
    const float rp = (float)s->rp;
    for (long i = i0; i < n; i += di) Fmt<S>::st(p0, i, fsub(Fmt<S>::ld(plo, i), fscale(rp, Fmt<R>::ld(rlo, i))));
}

// The reliable-update kernels: a grid of resident blocks walks the vector-block list.
#define BATCH_VEC_KERNEL(name, body)                                                        \
    template <class S, class R, class LK>                                                   \
    __global__ void __launch_bounds__(kRedThreads) name(BArgs<S, R, LK> a)                  \
    {                                                                                       \
        const int nv = *a.nvl;                                                              \
        for (int v = blockIdx.x; v < nv; v += gridDim.x) {                                  \
            const int2 e = a.vlist[v];                                                      \
            body<S, R, LK>(a, e.x, (unsigned)e.y);                                          \
            __syncthreads();                                                                \
        }                                                                                   \
    }
BATCH_VEC_KERNEL(k_bR1, bR1_blk)
BATCH_VEC_KERNEL(k_bOp1, bOp1_blk)
BATCH_VEC_KERNEL(k_bOp2, bOp2_blk)
BATCH_VEC_KERNEL(k_bR2, bR2_blk)
BATCH_VEC_KERNEL(k_bR3, bR3_blk)
BATCH_VEC_KERNEL(k_bR4, bR4_blk)
#undef BATCH_VEC_KERNEL

// |b|^2 of every system
template <class S, class R, class LK>
__global__ void __launch_bounds__(kRedThreads) k_bNorm(BArgs<S, R, LK> a)
{
    const int sid = a.vblk[blockIdx.x];
    const BSys sy = a.sys[sid];
    MxDev *s = a.st + sid;
    const unsigned lb = blockIdx.x - sy.vb0;
    const long n = (long)sy.lx * sy.ly;
    double v[1] = {0.0};
    for (long i = (long)lb * kRedThreads + threadIdx.x; i < n; i += (long)sy.nvb * kRedThreads)
        v[0] += cabs2(sy.b[i]);
    if (grid_sum_ids<1, kRedThreads>(v, a.vpart + 2 * sy.vb0, &s->cnt[4], lb, sy.nvb) && threadIdx.x == 0)
        s->bsq = v[0];
}

// r = 1 at every site (the autotuner's input)
template <class S, class R, class LK>
__global__ void __launch_bounds__(kRedThreads) k_bFillR(BArgs<S, R, LK> a)
{
    const int sid = a.vblk[blockIdx.x];
    const BSys sy = a.sys[sid];
    const unsigned lb = blockIdx.x - sy.vb0;
    const long n = (long)sy.lx * sy.ly;
    for (long i = (long)lb * kRedThreads + threadIdx.x; i < n; i += (long)sy.nvb * kRedThreads)
        Fmt<R>::st(a.r + sy.off, i, make_float2(1.f, 0.f));
}

// Links in the inner format: the staggered hopping table (1/2 and eta folded in, as k_make_hop)
// or the Laplacian's links as they are.
template <class S, class R, class LK>
__global__ void __launch_bounds__(kRedThreads) k_bLinks(BArgs<S, R, LK> a)
{
    const int sid = a.vblk[blockIdx.x];
    const BSys sy = a.sys[sid];
    const unsigned lb = blockIdx.x - sy.vb0;
    const long n = (long)sy.lx * sy.ly, o = sy.loff;
    if (!sy.lown) return;
    for (long i = (long)lb * kRedThreads + threadIdx.x; i < n; i += (long)sy.nvb * kRedThreads) {
        if (sy.stag) {
            const int x = (int)(i % sy.lx);
            const double eta = (x & 1) ? -1.0 : 1.0;
            a.L[2 * (o + i)] = Fmt<LK>::from(cscale(-0.5, sy.U[2 * i]));
            a.L[2 * (o + i) + 1] = Fmt<LK>::from(cscale(-0.5 * eta, sy.U[2 * i + 1]));
        } else {
            a.L[2 * (o + i)] = Fmt<LK>::from(sy.U[2 * i]);
            a.L[2 * (o + i) + 1] = Fmt<LK>::from(sy.U[2 * i + 1]);
        }
    }
}

// After the reliable-update steps: systems that ran one go back to iterating (as
// k_mx_outer_tail); when every system has stopped, the loop ends.  setup = 1 after the initial
// residual computation (no outer-iteration count).
__global__ void k_bTail(MxDev *st, int nsys, int *all_done, int setup)
{
    __shared__ int fin;
    if (threadIdx.x == 0) fin = 0;
    __syncthreads();
    int mine = 0;
    for (int q = threadIdx.x; q < nsys; q += blockDim.x) {
        MxDev *s = st + q;
        if (s->reliable && !s->done) {
            if (!setup) {
                s->outer++;
                if (s->outer > s->max_iter + 2) {
                    s->status = GLINALG_SOLVE_MAX_ITER;
                    s->done = 1;
                }
            }
            if (!s->done) {
                s->reliable = 0;
                s->parity = 0;
            }
        }
        mine += s->done != 0;
    }
    atomicAdd(&fin, mine);
    __syncthreads();
    if (threadIdx.x == 0 && fin == nsys) *all_done = 1;
}

// ---------------------------------------------------------------- tile candidates

// Candidates (BY warps of NY rows, blocks per SM): shapes of up to four rows a thread fit 64
// registers without spilling (32 warps an SM); the eight-row shape keeps its own register
// count.  Uneven batch: 84.7 ms with every shape at its own register count (three blocks of
// eight warps for the 8 x 4 shape the autotuner picks), 76.0 with the 64-register bound; a
// 40-register bound on the two-row shapes (48 warps) spills and gives 81.3.
constexpr int kNumBatchTiles = 4;
constexpr int kBatchTileRows[kNumBatchTiles] = {16, 32, 32, 32};  // BY * NY

template <class S, class R, class LK>
struct BKern {
    void (*A)(BArgs<S, R, LK>, int *);
    void (*B)(BArgs<S, R, LK>, int *);
    dim3 block;
};

template <class S, class R, class LK>
BKern<S, R, LK> batch_kernels(int c)
{
    switch (c) {
    case 0: return {k_bA<S, R, LK, 8, 2, 4>, k_bB<S, R, LK, 8, 2, 4>, dim3(32, 8)};
    case 1: return {k_bA<S, R, LK, 8, 4, 4>, k_bB<S, R, LK, 8, 4, 4>, dim3(32, 8)};
    case 2: return {k_bA<S, R, LK, 4, 8, 1>, k_bB<S, R, LK, 4, 8, 1>, dim3(32, 4)};
    default: return {k_bA<S, R, LK, 16, 2, 2>, k_bB<S, R, LK, 16, 2, 2>, dim3(32, 16)};
    }
}

std::mutex g_btune_mu;
std::map<std::tuple<int, int, std::vector<int>>, int> g_btuned;

// Tile-block layout of the batch for candidate c; returns the number of tile blocks.
int layout_tiles(std::vector<BSys> &sys, int c)
{
    const int rows = kBatchTileRows[c];
    int ntb = 0;
    for (BSys &y : sys) {
        y.tiles_x = (y.lx + 31) / 32;
        y.tb0 = ntb;
        y.ntb = y.tiles_x * ((y.ly + rows - 1) / rows);
        ntb += y.ntb;
    }
    return ntb;
}

template <class S, class R, class LK>
glinalg_status run_batch(const glinalg_operator_s *const *ops, int nsys, double2 *const *X,
                         const double2 *const *B, int max_iter, double eps, double delta, int variant,
                         glinalg_info *infos, cudaStream_t st, const char *name)
{
    const int dev = ops[0]->device;
    Scratch sc(st);
    std::vector<BSys> sys(nsys);
    std::vector<int> vblk;
    long N = 0, NL = 0;
    std::vector<int> sig;
    for (int q = 0; q < nsys; q++) {
        const glinalg_operator_s *op = ops[q];
        BSys &y = sys[q];
        y = BSys{};
        y.off = N;
        y.U = op->U;
        y.x = X[q];
        y.b = B[q];
        y.mass = op->mass;
        y.lx = op->lx;
        y.ly = op->ly;
        y.stag = op->kind == GLINALG_OP_STAGGERED_NORMAL;
        y.xs = op->lx % 32 == 0;
        const long n = op->size;
        // one packed link table per distinct (links, kind, lattice): systems that differ only in
        // mass (the shifted systems of a multishift refinement) read the same table
        y.loff = -1;
        for (int e = 0; e < q; e++) {
            const BSys &z = sys[e];
            if (z.lown && z.U == y.U && z.stag == y.stag && z.lx == y.lx && z.ly == y.ly) {
                y.loff = z.loff;
                break;
            }
        }
        if (y.loff < 0) {
            y.loff = NL;
            y.lown = 1;
            NL += n;
        }
        y.vb0 = (int)vblk.size();
        y.nvb = (int)((n + kVecSites - 1) / kVecSites);
        vblk.insert(vblk.end(), y.nvb, q);
        N += n;
        sig.push_back(y.lx);
        sig.push_back(y.ly);
        sig.push_back(y.stag);
    }
    const int nvb = (int)vblk.size();
    BArgs<S, R, LK> a = {};
    GL_TRY(sc.alloc(&a.r, N));
    GL_TRY(sc.zeros(&a.p0, N));
    GL_TRY(sc.zeros(&a.p1, N));
    GL_TRY(sc.alloc(&a.t, N));
    GL_TRY(sc.zeros(&a.xlo, N));
    GL_TRY(sc.alloc(&a.L, 2 * NL));
    GL_TRY(sc.alloc(&a.rhi, N));
    GL_TRY(sc.alloc(&a.tmp64, N));
    GL_TRY(sc.alloc(&a.Ax, N));
    GL_TRY(sc.alloc(&a.vpart, 2 * (size_t)nvb));
    GL_TRY(sc.zeros(&a.st, nsys));
    GL_TRY(sc.zeros(&a.all_done, 1));
    BSys *dsys;
    int *dvblk, *dcounts, *dclaims;  // dclaims: one tile counter per inner-kernel launch of a pass
    int2 *dtlist, *dvlist;
    GL_TRY(sc.alloc(&dsys, nsys));
    GL_TRY(sc.alloc(&dvblk, nvb));
    // the largest tile-block count over the candidates
    int max_tb = 0;
    for (int c = 0; c < kNumBatchTiles; c++) max_tb = std::max(max_tb, layout_tiles(sys, c));
    GL_TRY(sc.alloc(&dtlist, max_tb));
    GL_TRY(sc.alloc(&dvlist, nvb));
    GL_TRY(sc.zeros(&dcounts, 2));
    GL_TRY(sc.zeros(&dclaims, 2 * kBatchUnroll));
    GL_TRY(sc.alloc(&a.tpart, max_tb));
    a.sys = dsys;
    a.vblk = dvblk;
    a.nsys = nsys;
    a.tlist = dtlist;
    a.vlist = dvlist;
    a.ntl = dcounts;
    a.nvl = dcounts + 1;
    GL_CUDA(cudaMemcpyAsync(dvblk, vblk.data(), sizeof(int) * nvb, cudaMemcpyHostToDevice, st));
    auto upload = [&](int c) -> glinalg_status {
        layout_tiles(sys, c);
        GL_CUDA(cudaMemcpyAsync(dsys, sys.data(), sizeof(BSys) * nsys, cudaMemcpyHostToDevice, st));
        return GLINALG_SUCCESS;
    };
    // the list kernels and the resident grids that walk the lists
    const int list_grid = std::max(1, std::min(nsys, 2 * sm_count()));
    auto list_tiles = [&](cudaStream_t cs) {
        k_bList<<<list_grid, 1024, 0, cs>>>(dsys, a.st, nsys, 0, dtlist, dcounts, dclaims, 2 * kBatchUnroll);
    };
    auto list_vec = [&](cudaStream_t cs) {
        k_bList<<<list_grid, 1024, 0, cs>>>(dsys, a.st, nsys, 1, dvlist, dcounts + 1, nullptr, 0);
    };
    auto resident = [&](const void *fn, int threads, int cap) -> int {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        return std::max(1, std::min(cap, per_sm * sm_count()));
    };
    const int vgrid = resident((const void *)k_bOp1<S, R, LK>, kRedThreads, nvb);
    GL_TRY(upload(0));
    k_bLinks<S, R, LK><<<nvb, kRedThreads, 0, st>>>(a);
    GL_CUDA(cudaGetLastError());

    // ---- tile shape for this batch: time two inner iterations of every candidate once
    int cand = -1;
    const auto key = std::make_tuple(dev, variant, sig);
    {
        std::lock_guard<std::mutex> lk(g_btune_mu);
        auto it = g_btuned.find(key);
        if (it != g_btuned.end()) cand = it->second;
    }
    if (const char *e = std::getenv("GLINALG_TILE")) {
        const int c = std::atoi(e);
        if (c >= 0 && c < kNumBatchTiles) cand = c;
    }
    if (cand < 0) {
        std::vector<MxDev> hs(nsys);
        for (int q = 0; q < nsys; q++) {
            hs[q] = MxDev{};
            hs[q].rsq = (double)ops[q]->size;  // |r|^2 of r = 1
            hs[q].scale = 1.0;
            hs[q].bsq = 1.0;
            hs[q].rmax = 1e300;  // delta = eps = 0: no reliable update during the timing
            hs[q].max_iter = 1 << 30;
        }
        cudaEvent_t e0, e1;
        GL_CUDA(cudaEventCreate(&e0));
        GL_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        for (int c = 0; c < kNumBatchTiles; c++) {
            GL_TRY(upload(c));
            const BKern<S, R, LK> k = batch_kernels<S, R, LK>(c);
            const int ntb = sys.back().tb0 + sys.back().ntb;
            const int nth = (int)(k.block.x * k.block.y);
            const int gA = resident((const void *)k.A, nth, ntb), gB = resident((const void *)k.B, nth, ntb);
            float m = 1e30f;
            for (int rep = 0; rep < 3; rep++) {
                // r = 1 everywhere, p = 0, fresh state
                k_bFillR<S, R, LK><<<nvb, kRedThreads, 0, st>>>(a);
                GL_CUDA(cudaMemsetAsync(a.p0, 0, sizeof(S) * N, st));
                GL_CUDA(cudaMemcpyAsync(a.st, hs.data(), sizeof(MxDev) * nsys, cudaMemcpyHostToDevice, st));
                list_tiles(st);
                k_busy_wait<<<1, 1, 0, st>>>(30000);  // keep launch latency out of the events
                GL_CUDA(cudaEventRecord(e0, st));
                for (int it = 0; it < 2; it++) {
                    k.A<<<gA, k.block, 0, st>>>(a, dclaims + 2 * it);
                    k.B<<<gB, k.block, 0, st>>>(a, dclaims + 2 * it + 1);
                }
                GL_CUDA(cudaEventRecord(e1, st));
                GL_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                GL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                m = std::min(m, ms);
            }
            if (m < best) {
                best = m;
                cand = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        std::lock_guard<std::mutex> lk(g_btune_mu);
        g_btuned[key] = cand;
        GL_CUDA(cudaMemsetAsync(a.p0, 0, sizeof(S) * N, st));
        GL_CUDA(cudaMemsetAsync(a.p1, 0, sizeof(S) * N, st));
        GL_CUDA(cudaMemsetAsync(a.xlo, 0, sizeof(float2) * N, st));
    }
    GL_TRY(upload(cand));
    const BKern<S, R, LK> k = batch_kernels<S, R, LK>(cand);
    const int ntb = sys.back().tb0 + sys.back().ntb;
    const int nth = (int)(k.block.x * k.block.y);
    const int gA = resident((const void *)k.A, nth, ntb), gB = resident((const void *)k.B, nth, ntb);

    // ---- initial state: every system starts with a reliable update (r = b - A x0)
    {
        std::vector<MxDev> hs(nsys);
        for (int q = 0; q < nsys; q++) {
            hs[q] = MxDev{};
            hs[q].eps = eps;
            hs[q].delta = delta;
            hs[q].max_iter = max_iter;
            hs[q].scale = 1.0;
            hs[q].reliable = 1;
        }
        GL_CUDA(cudaMemcpyAsync(a.st, hs.data(), sizeof(MxDev) * nsys, cudaMemcpyHostToDevice, st));
    }
    EventTimer tm;
    tm.start(st);
    auto reliable_seq = [&](cudaStream_t cs) -> glinalg_status {
        list_vec(cs);
        k_bR1<S, R, LK><<<vgrid, kRedThreads, 0, cs>>>(a);
        k_bOp1<S, R, LK><<<vgrid, kRedThreads, 0, cs>>>(a);
        k_bOp2<S, R, LK><<<vgrid, kRedThreads, 0, cs>>>(a);
        k_bR2<S, R, LK><<<vgrid, kRedThreads, 0, cs>>>(a);
        k_bR3<S, R, LK><<<vgrid, kRedThreads, 0, cs>>>(a);
        k_bR4<S, R, LK><<<vgrid, kRedThreads, 0, cs>>>(a);
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    };
    k_bNorm<S, R, LK><<<nvb, kRedThreads, 0, st>>>(a);
    GL_TRY(reliable_seq(st));
    k_bTail<<<1, 256, 0, st>>>(a.st, nsys, a.all_done, 1);
    GL_CUDA(cudaGetLastError());
    GL_TRY(run_loop(st, a.all_done, [&](cudaStream_t cs) -> glinalg_status {
        for (int u = 0; u < kBatchUnroll; u++) {
            if (u % kListEvery == 0) list_tiles(cs);
            k.A<<<gA, k.block, 0, cs>>>(a, dclaims + 2 * u);
            k.B<<<gB, k.block, 0, cs>>>(a, dclaims + 2 * u + 1);
        }
        GL_TRY(reliable_seq(cs));
        k_bTail<<<1, 256, 0, cs>>>(a.st, nsys, a.all_done, 0);
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    }));
    tm.stop(st);
    std::vector<MxDev> hs(nsys);
    GL_CUDA(cudaMemcpyAsync(hs.data(), a.st, sizeof(MxDev) * nsys, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    const double w = Fmt<S>::bytes, wr = Fmt<R>::bytes, wl = Fmt<LK>::bytes;
    for (int q = 0; q < nsys; q++) {
        const MxDev &h = hs[q];
        const long n = ops[q]->size;
        glinalg_info *info = &infos[q];
        double *keep = info->resSqmrhs;
        *info = glinalg_info{};
        info->resSqmrhs = keep;
        info->resSq = h.rsq_true;
        info->iter = h.k;
        info->success = h.status == GLINALG_SOLVE_CONVERGED ? 1 : 0;
        info->ops_count = h.k + h.n_reliable;
        info->status = h.status;
        info->reliable_updates = h.n_reliable;
        info->device_ms = tm.ms();
        const bool stg = sys[q].stag;
        const double per_iter = stg ? (6.0 * w + 4.0 * wl + 3.0 * wr + 16.0) : (6.0 * w + 2.0 * wl + 3.0 * wr + 16.0);
        const double per_rel = 16.0 * 2 + 16.0 + 8.0 * 64.0 / 8.0 + 16.0 * 3 + 2 * wr + 4 * w;
        info->gbytes = ((double)h.k * per_iter * n + (double)h.n_reliable * per_rel * n) * 1e-9;
        fill_name(info, name);
    }
    return GLINALG_SUCCESS;
}

}  // namespace

glinalg_status cg_batch_mixed(const glinalg_operator_s *const *ops, int nsys, double2 *const *X,
                              const double2 *const *B, int max_iter, double eps, int precision, double delta,
                              glinalg_info *infos, cudaStream_t st)
{
    // the single-system defaults: 0.01 for FP32 iterates, 0.1 for 16-bit storage
    if (!(delta > 0.0 && delta < 1.0)) delta = precision == GLINALG_PREC_SINGLE ? 0.01 : 0.1;
    switch (precision) {
    case GLINALG_PREC_SINGLE:
        return run_batch<float2, float2, float2>(ops, nsys, X, B, max_iter, eps, delta, 1, infos, st, "CG-FP32");
    case GLINALG_PREC_HALF:
        // FP16 fields, FP32 links, as the single-system FP16 solver
        return run_batch<__half2, float2, float2>(ops, nsys, X, B, max_iter, eps, delta, 2, infos, st, "CG-FP16");
    case GLINALG_PREC_BFLOAT:
        return run_batch<__nv_bfloat162, float2, float2>(ops, nsys, X, B, max_iter, eps, delta, 3, infos, st,
                                                         "CG-BF16");
    default:
        set_last_error("batched mixed-precision CG: precision must be SINGLE, HALF or BFLOAT");
        return GLINALG_ERROR_INVALID_VALUE;
    }
}

}  // namespace glinalg
