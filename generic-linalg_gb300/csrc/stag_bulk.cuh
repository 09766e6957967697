// stag_bulk.cuh -- the persistent inner loop of the mixed-precision CG on the staggered normal
// operator, with every tile staged through shared memory by bulk asynchronous copies (the
// Tensor Memory Accelerator's cp.async.bulk) instead of per-thread loads.
//
// The iteration is the one of k_persist (cg_mixed.cu):
//   A: p' = r + beta p ; t = D p' ; |t|^2 + sigma |p'|^2            -> grid barrier -> alpha
//   B: Ap = D^dagger t + sigma p' ; x_lo += alpha p' ; r -= alpha Ap ; |r|^2 -> barrier -> beta
// with the same per-site arithmetic as tile_A / tile_B (stag_tiles.cuh).
//
// A tile is TY rows x SX columns.  Warp 0 of the block issues the copies of a tile's rows
// (one row segment per lane) into one of kStages shared-memory stages, its lane 0 having armed
// the stage's mbarrier with the number of bytes to expect; the 16 warps compute tile k from its stage while the copies of tiles
// k+1 .. k+kStages-1 are in flight, so the latency of L2 is paid once per phase rather than
// once per row of loads.  Fields read at neighbours (r and p in A, t in B) are copied with a
// 16-byte halo on either side in x and one row above and below; the links with one site to the
// left (one row below for the y-links).  A row segment that crosses x = 0 or x = lx is copied in
// two pieces (periodic lattice).  Every copy starts and ends on a 16-byte boundary: lx and SX
// are multiples of 256 sites and the halos are 16 bytes wide.
//
// Ordering: results are stored with ordinary stores; before the grid barrier every thread
// fences its stores against the async proxy, and warp 0 fences again before it issues the
// copies of the next phase.  Every mbarrier wait is bounded (kBarrierTimeoutNs); a wait that
// runs out raises the grid's error flag, like a barrier timeout.
#pragma once

#include <cstdint>

#include "mixed_state.cuh"

namespace glinalg {
namespace bulk {

constexpr int kStages = 3;    // shared-memory stages in flight
constexpr int kBY = 16;       // warps per block
constexpr int kThreads = 32 * kBY;

// Tile geometry: SX columns x TY rows, two sites per thread.
template <int SX_, int TY_>
struct Geom {
    static constexpr int SX = SX_, TY = TY_;
    static_assert(SX * TY == 2 * kThreads, "two sites per thread");
};
using Geom256x4 = Geom<256, 4>;
using Geom512x2 = Geom<512, 2>;

template <class T>
constexpr int halo() { return 16 / (int)sizeof(T) < 1 ? 1 : 16 / (int)sizeof(T); }
template <class LK>
constexpr int link_halo() { return 16 / (2 * (int)sizeof(LK)) < 1 ? 1 : 16 / (2 * (int)sizeof(LK)); }

// Byte offsets inside one stage.  A: r, p (TY+2 rows with halos), links (TY+1 rows).
// B: t (TY+2 rows with halos), links, then p', r, x_lo of the tile's own sites.
template <class S, class R, class LK, class G>
struct Layout {
    static constexpr int SX = G::SX, TY = G::TY;
    static constexpr int hS = halo<S>(), hR = halo<R>(), hL = link_halo<LK>();
    static constexpr int WS = SX + 2 * hS, WR = SX + 2 * hR, WL = SX + hL;
    static constexpr int LB = 2 * (int)sizeof(LK);  // bytes of one site's link pair
    static constexpr int A_R = 0;
    static constexpr int A_P = A_R + (TY + 2) * WR * (int)sizeof(R);
    static constexpr int A_L = A_P + (TY + 2) * WS * (int)sizeof(S);
    static constexpr int A_END = A_L + (TY + 1) * WL * LB;
    static constexpr int B_T = 0;
    static constexpr int B_L = B_T + (TY + 2) * WS * (int)sizeof(S);
    static constexpr int B_P = B_L + (TY + 1) * WL * LB;
    static constexpr int B_R = B_P + TY * SX * (int)sizeof(S);
    static constexpr int B_X = B_R + TY * SX * (int)sizeof(R);
    static constexpr int B_END = B_X + TY * SX * 8;
    static constexpr int STAGE = ((A_END > B_END ? A_END : B_END) + 127) / 128 * 128;
    static constexpr int SMEM = kStages * STAGE;
    static_assert(A_P % 16 == 0 && A_L % 16 == 0 && B_L % 16 == 0 && B_P % 16 == 0 && B_R % 16 == 0 &&
                      B_X % 16 == 0,
                  "16-byte aligned stage arrays");
};

__device__ __forceinline__ unsigned su32(const void *p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *b, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *b, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity)
{
    if (mbar_test(b, parity)) return true;
    const long long t0 = gtimer();
    while (!mbar_test(b, parity))
        if (gtimer() - t0 > kBarrierTimeoutNs) return false;
    return true;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *b)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(b))
                 : "memory");
}

__device__ __forceinline__ void fence_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Copy elements xs .. xs+cnt-1 (E bytes each, x periodic modulo lx) of the row starting at
// element rowbase of g into dst.
template <int E>
__device__ __forceinline__ void copy_row(char *dst, const char *g, long rowbase, int xs, int cnt, int lx, uint64_t *bar)
{
    int done = 0, pos = xs;
    while (done < cnt) {
        int gx = pos % lx;
        if (gx < 0) gx += lx;
        const int run = min(cnt - done, lx - gx);
        bulk_g2s(dst + (long)done * E, g + (rowbase + gx) * E, (unsigned)(run * E), bar);
        done += run;
        pos += run;
    }
}

__device__ __forceinline__ int wrap_row(int y, int ly) { return y < 0 ? y + ly : (y >= ly ? y - ly : y); }

// The copies of one tile are spread over the 32 lanes of warp 0: lane 0 arms the stage's
// mbarrier with the tile's byte count, then every lane issues the row segments j with
// j % 32 == lane (row segments: A 2*(TY+2) + TY+1, B TY+2 + TY+1 + 3*TY).
template <class S, class R, class LK, class G>
__device__ __forceinline__ void issue_A(char *st, uint64_t *bar, int tile, const R *r, const S *pold, const LK *H,
                                        int lx, int ly, int lane)
{
    using L = Layout<S, R, LK, G>;
    constexpr int SX = G::SX, TY = G::TY;
    const int ntx = lx / SX, x0 = (tile % ntx) * SX, y0 = (tile / ntx) * TY;
    if (lane == 0) mbar_arrive_tx(bar, (unsigned)L::A_END);
    __syncwarp();
    for (int j = lane; j < 3 * TY + 5; j += 32) {
        if (j < 2 * (TY + 2)) {
            const int q = j >> 1;
            const long rb = (long)wrap_row(y0 - 1 + q, ly) * lx;
            if (j & 1)
                copy_row<sizeof(S)>(st + L::A_P + q * L::WS * (int)sizeof(S), (const char *)pold, rb, x0 - L::hS,
                                    L::WS, lx, bar);
            else
                copy_row<sizeof(R)>(st + L::A_R + q * L::WR * (int)sizeof(R), (const char *)r, rb, x0 - L::hR, L::WR,
                                    lx, bar);
        } else {
            const int q = j - 2 * (TY + 2);
            const long rb = (long)wrap_row(y0 - 1 + q, ly) * lx;
            copy_row<L::LB>(st + L::A_L + q * L::WL * L::LB, (const char *)H, rb, x0 - L::hL, L::WL, lx, bar);
        }
    }
}

template <class S, class R, class LK, class G>
__device__ __forceinline__ void issue_B(char *st, uint64_t *bar, int tile, const S *t, const LK *H, const S *pnew,
                                        const R *r, const float2 *xlo, int lx, int ly, int lane)
{
    using L = Layout<S, R, LK, G>;
    constexpr int SX = G::SX, TY = G::TY;
    const int ntx = lx / SX, x0 = (tile % ntx) * SX, y0 = (tile / ntx) * TY;
    if (lane == 0) mbar_arrive_tx(bar, (unsigned)L::B_END);
    __syncwarp();
    for (int j = lane; j < 5 * TY + 3; j += 32) {
        if (j < TY + 2) {
            const long rb = (long)wrap_row(y0 - 1 + j, ly) * lx;
            copy_row<sizeof(S)>(st + L::B_T + j * L::WS * (int)sizeof(S), (const char *)t, rb, x0 - L::hS, L::WS, lx,
                                bar);
        } else if (j < 2 * TY + 3) {
            const int q = j - (TY + 2);
            const long rb = (long)wrap_row(y0 - 1 + q, ly) * lx;
            copy_row<L::LB>(st + L::B_L + q * L::WL * L::LB, (const char *)H, rb, x0 - L::hL, L::WL, lx, bar);
        } else {
            const int u = j - (2 * TY + 3), q = u / 3, f = u % 3;
            const long rb = (long)(y0 + q) * lx;
            if (f == 0)
                copy_row<sizeof(S)>(st + L::B_P + q * SX * (int)sizeof(S), (const char *)pnew, rb, x0, SX, lx, bar);
            else if (f == 1)
                copy_row<sizeof(R)>(st + L::B_R + q * SX * (int)sizeof(R), (const char *)r, rb, x0, SX, lx, bar);
            else
                copy_row<8>(st + L::B_X + q * SX * 8, (const char *)xlo, rb, x0, SX, lx, bar);
        }
    }
}

// The links of site column c (tile coordinates) in smem row q: (h_x, h_y).
template <class LK, int hL, int WL>
__device__ __forceinline__ void link_at(const LK *sl, int q, int c, float2 &hx, float2 &hy)
{
    const int k = 2 * (q * WL + c + hL);
    hx = Fmt<LK>::ld(sl, k);
    hy = Fmt<LK>::ld(sl, k + 1);
}

// A on the two sites of this thread in the tile held by `st`; returns sum |t|^2 + sigma |p'|^2.
template <class S, class R, class LK, class G>
__device__ __forceinline__ float compute_A(const char *st, int tid, int tile, S *pnew, S *t, float beta, float mass,
                                           float sigma, int lx)
{
    using L = Layout<S, R, LK, G>;
    constexpr int SX = G::SX, TY = G::TY;
    const R *sr = (const R *)(st + L::A_R);
    const S *sp = (const S *)(st + L::A_P);
    const LK *sl = (const LK *)(st + L::A_L);
    const int ntx = lx / SX, x0 = (tile % ntx) * SX, y0 = (tile / ntx) * TY;
    const int c = tid % SX;
    auto P = [&](int q, int cc) {
        return fadd(Fmt<R>::ld(sr, q * L::WR + cc + L::hR), fscale(beta, Fmt<S>::ld(sp, q * L::WS + cc + L::hS)));
    };
    float acc = 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int yy = tid / SX + h * (kThreads / SX);
        const float2 pc = P(yy + 1, c), pxp = P(yy + 1, c + 1), pxm = P(yy + 1, c - 1);
        const float2 pyp = P(yy + 2, c), pym = P(yy, c);
        float2 hx, hy, hxm, dum, hym;
        link_at<LK, L::hL, L::WL>(sl, yy + 1, c, hx, hy);
        link_at<LK, L::hL, L::WL>(sl, yy + 1, c - 1, hxm, dum);
        link_at<LK, L::hL, L::WL>(sl, yy, c, dum, hym);
        float2 hs = fmul(hx, pxp);
        hs = fsub(hs, fmulc(hxm, pxm));
        hs = fadd(hs, fmul(hy, pyp));
        hs = fsub(hs, fmulc(hym, pym));
        const float2 tv = fadd(fscale(mass, pc), hs);
        const long i = (long)(y0 + yy) * lx + x0 + c;
        Fmt<S>::st(pnew, i, pc);
        Fmt<S>::st(t, i, tv);
        const float2 pq = Fmt<S>::round(pc), tq = Fmt<S>::round(tv);
        acc += fn2(tq) + sigma * fn2(pq);
    }
    return acc;
}

// B on the two sites of this thread; returns sum |r|^2.
template <class S, class R, class LK, class G>
__device__ __forceinline__ float compute_B(const char *st, int tid, int tile, R *r, float2 *xlo, float alpha,
                                           float mass, float sigma, int lx)
{
    using L = Layout<S, R, LK, G>;
    constexpr int SX = G::SX, TY = G::TY;
    const S *stt = (const S *)(st + L::B_T);
    const LK *sl = (const LK *)(st + L::B_L);
    const S *spn = (const S *)(st + L::B_P);
    const R *srr = (const R *)(st + L::B_R);
    const float2 *sx = (const float2 *)(st + L::B_X);
    const int ntx = lx / SX, x0 = (tile % ntx) * SX, y0 = (tile / ntx) * TY;
    const int c = tid % SX;
    auto T = [&](int q, int cc) { return Fmt<S>::ld(stt, q * L::WS + cc + L::hS); };
    float acc = 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int yy = tid / SX + h * (kThreads / SX);
        const float2 ct = T(yy + 1, c), txp = T(yy + 1, c + 1), txm = T(yy + 1, c - 1);
        const float2 typ = T(yy + 2, c), tym = T(yy, c);
        float2 hx, hy, hxm, dum, hym;
        link_at<LK, L::hL, L::WL>(sl, yy + 1, c, hx, hy);
        link_at<LK, L::hL, L::WL>(sl, yy + 1, c - 1, hxm, dum);
        link_at<LK, L::hL, L::WL>(sl, yy, c, dum, hym);
        float2 hs = fmul(hx, txp);
        hs = fsub(hs, fmulc(hxm, txm));
        hs = fadd(hs, fmul(hy, typ));
        hs = fsub(hs, fmulc(hym, tym));
        const float2 pv = Fmt<S>::ld(spn, yy * SX + c);
        const float2 av = fadd(fsub(fscale(mass, ct), hs), fscale(sigma, pv));
        const float2 xv = fadd(sx[yy * SX + c], fscale(alpha, pv));
        const float2 rv = Fmt<R>::round(fsub(Fmt<R>::ld(srr, yy * SX + c), fscale(alpha, av)));
        const long i = (long)(y0 + yy) * lx + x0 + c;
        xlo[i] = xv;
        Fmt<R>::st(r, i, rv);
        acc += fn2(rv);
    }
    return acc;
}

}  // namespace bulk

// Whether the bulk-copy persistent kernel with geometry G serves this lattice.
template <class G>
inline bool bulk_applies(int lx, int ly, int nblocks)
{
    return lx % G::SX == 0 && ly % G::TY == 0 && ly >= 2 * G::TY && (long)(lx / G::SX) * (ly / G::TY) >= (long)nblocks;
}

template <class S, class R, class LK, class G>
__global__ void __launch_bounds__(bulk::kThreads, 1)
k_persist_bulk(const LK *__restrict__ H, R *r, S *p0, S *p1, S *t, float2 *xlo, float mass, float sigma, int lx,
               int ly, MxDev *s, GridSync *gs, double *partA, double *partB)
{
    using namespace bulk;
    constexpr int SX = G::SX, TY = G::TY;
    extern __shared__ __align__(128) char smem[];
    __shared__ double sm[33];
    __shared__ __align__(8) uint64_t bars[kStages];
    __shared__ int bad;
    // one read of the solve state per block (bad doubles as the flag), so that a block never
    // splits here: block 0 of a launch whose waits ran out may set s->done while other blocks
    // are still starting
    if (threadIdx.x == 0 && threadIdx.y == 0) bad = s->done || s->reliable;
    __syncthreads();
    if (bad) return;
    const long long t_start = gtimer();
    const unsigned nb = gridDim.x;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int ntiles = (lx / SX) * (ly / TY);
    const int my = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)nb + 1 : 0;
    const int stage_bytes = Layout<S, R, LK, G>::STAGE;
    if (tid == 0) {
        for (int q = 0; q < kStages; q++) mbar_init(&bars[q], 1);
        bad = 0;
    }
    __syncthreads();
    unsigned parity = 0;  // bit q: parity of the next completion of stage q
    double rsq = s->rsq, beta = s->beta, rmax = s->rmax, rn = 0.0;
    const double scale = s->scale, delta = s->delta, eps = s->eps, bsqrt = sqrt(s->bsq);
    int k = s->k;
    const int max_iter = s->max_iter;
    int j = 0, status = -1;
    bool reliable = false;

    // One phase over this block's tiles; false if a stage never arrived.
    auto phase = [&](int which, const S *pold, S *pnew, float fb, float fa, float &acc) -> bool {
        if (threadIdx.y == 0) {
            fence_async_global();
            for (int q = 0; q < kStages && q < my; q++) {
                const int tile = (int)blockIdx.x + q * (int)nb;
                if (which == 0)
                    issue_A<S, R, LK, G>(smem + q * stage_bytes, &bars[q], tile, r, pold, H, lx, ly, threadIdx.x);
                else
                    issue_B<S, R, LK, G>(smem + q * stage_bytes, &bars[q], tile, t, H, pnew, r, xlo, lx, ly, threadIdx.x);
            }
        }
        for (int m = 0; m < my; m++) {
            const int q = m % kStages;
            const int tile = (int)blockIdx.x + m * (int)nb;
            const bool arrived = mbar_wait(&bars[q], (parity >> q) & 1u);
            parity ^= 1u << q;
            if (!arrived) bad = 1;
            __syncthreads();
            if (bad) return false;
            const char *st = smem + q * stage_bytes;
            if (which == 0) acc += bulk::compute_A<S, R, LK, G>(st, tid, tile, pnew, t, fb, mass, sigma, lx);
            else acc += bulk::compute_B<S, R, LK, G>(st, tid, tile, r, xlo, fa, mass, sigma, lx);
            __syncthreads();  // every thread is done with stage q
            if (threadIdx.y == 0 && m + kStages < my) {
                fence_async_shared();
                const int nt = (int)blockIdx.x + (m + kStages) * (int)nb;
                if (which == 0)
                    issue_A<S, R, LK, G>(smem + q * stage_bytes, &bars[q], nt, r, pold, H, lx, ly, threadIdx.x);
                else
                    issue_B<S, R, LK, G>(smem + q * stage_bytes, &bars[q], nt, t, H, pnew, r, xlo, lx, ly, threadIdx.x);
            }
        }
        fence_async_global();  // this thread's stores, before the barrier that publishes them
        return true;
    };

    for (;;) {
        const S *pold = (j & 1) ? p1 : p0;
        S *pnew = (j & 1) ? p0 : p1;
        float acc = 0.f;
        if (!phase(0, pold, pnew, (float)beta, 0.f, acc)) { status = GLINALG_SOLVE_TIMEOUT; break; }
        block_partial(acc, partA, sm);
        if (!grid_sync(gs, nb, peer_wait_ns(s))) { status = GLINALG_SOLVE_TIMEOUT; break; }
        const double pAp = grid_total(partA, nb, sm);
        if (!(pAp > 0.0) || !isfinite(pAp)) {
            status = pAp == 0.0 ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
            break;
        }
        const float alpha = (float)(rsq / pAp);
        acc = 0.f;
        if (!phase(1, pold, pnew, 0.f, alpha, acc)) { status = GLINALG_SOLVE_TIMEOUT; break; }
        block_partial(acc, partB, sm);
        if (!grid_sync(gs, nb, peer_wait_ns(s))) { status = GLINALG_SOLVE_TIMEOUT; break; }
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
    if (status == GLINALG_SOLVE_TIMEOUT) {
        cuda::atomic_ref<int, cuda::thread_scope_device> err(gs->error);
        err.store(1, cuda::memory_order_relaxed);
        // copies still in flight land in this block's shared memory: wait for them (bounded)
        if (tid == 0)
            for (int q = 0; q < kStages; q++) mbar_wait(&bars[q], (parity >> q) & 1u);
    }
    if (blockIdx.x == 0 && tid == 0) {
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

}  // namespace glinalg
