// stag_resident_s.cuh -- the inner loop of the mixed-precision CG on the staggered normal
// operator D^dagger D (+ sigma) with 16-bit storage (FP16 or BF16 direction and t, FP16 or FP32
// links) and each block's share of the lattice held on chip.
//
// The FP32 kernel (k_resident) forms t = D p' by the recurrence t = D r + beta t_old, so that its
// first stencil does not wait for beta.  With t stored in 16 bits that recurrence accumulates
// the storage rounding from one iteration to the next and the solve does not converge.  This
// kernel forms t = D p' from the stored p' every iteration, as the streaming 16-bit kernels do
// (stag_tiles.cuh): the rounding of p' and t enters once per iteration.  One inner iteration:
//   U: beta (the previous B's total); p' = r + beta p, stored in 16 bits; export the border of p'.
//   A: t = D p', stored in 16 bits; partial |t|^2 + sigma |p'|^2; export the border of t.
//   B: Ap = D^dagger t + sigma p'; alpha (the total of A); x_lo += alpha p', r -= alpha Ap;
//      partial |r|^2.
// Shared memory holds p' and t (16-bit, each with a one-site ring) and the links (LK); r and
// x_lo stay in registers.  The rectangles, the ring, the mailboxes (p' and t take the two
// fields) and the bounded waits are k_resident's (stag_resident.cuh).  The partial sums of A and
// B go to separate word arrays, each alternating between two slots by iteration: a block
// rewrites a slot two iterations later, after it has waited for a sum that every block joins
// only after reading that slot.
#pragma once

#include "stag_resident.cuh"

namespace glinalg {
namespace ress {

using res::kPW;
using res::kTX;
using res::kWX;

constexpr int kWY = 4;  // warps along y (16 warps a block)
constexpr int kNumNY = 3;
constexpr int kNY[kNumNY] = {4, 8, 14};

// Dynamic shared memory of a rectangle of ty rows: the links (h_x, h_y of the rectangle, h_x of
// the column left of it, h_y of the row below it), then p' and t with their ring.
inline size_t smem_bytes(int ty, size_t s_bytes, size_t lk_bytes)
{
    return lk_bytes * (2 * (size_t)ty * kTX + (size_t)ty + kTX) + s_bytes * 2 * (size_t)(ty + 2) * kPW;
}

inline res::Plan plan(int lx, int ly, int nsm, size_t max_smem, size_t s_bytes, size_t lk_bytes)
{
    res::Plan p;
    if (lx % kTX != 0 || ly < 1 || nsm < 1) return p;
    p.wy = kWY;
    p.gx = lx / kTX;
    const int gy_max = nsm / p.gx;
    if (gy_max < 1) return p;
    p.ty = (ly + gy_max - 1) / gy_max;
    p.gy = (ly + p.ty - 1) / p.ty;
    for (int c = 0; c < kNumNY; c++) {
        if (kNY[c] * kWY >= p.ty) {
            p.ny = kNY[c];
            break;
        }
    }
    if (p.ny == 0) return p;
    p.smem = smem_bytes(p.ty, s_bytes, lk_bytes);
    p.ok = p.smem <= max_smem && 2 * kTX + 2 * p.ty <= 32 * kWX * kWY && p.gx * p.gy <= res::kMaxBlocks;
    return p;
}

template <class T>
__device__ __forceinline__ float2 lds(const T *p)
{
    return Fmt<T>::ld(p, 0);
}

// Hopping sums of the thread's rows from the 16-bit field F (links LK), as res::hop_rows:
//   hs = h_x f(x+1) - h_x(x-1)^* f(x-1) + h_y f(y+1) - h_y(y-1)^* f(y-1);  body(q, f(x, y), hs).
template <int NY, bool FULL, class S, class LK, class Body>
__device__ __forceinline__ void hop_rows_s(const S *__restrict__ F, const LK *__restrict__ HX,
                                           const LK *__restrict__ HY, const LK *__restrict__ HxL,
                                           const LK *__restrict__ HyB, int xl, int yb, int nrow, Body body)
{
    float2 prev = lds(F + yb * kPW + xl + 1), cur = lds(F + (yb + 1) * kPW + xl + 1);
    float2 hyp = yb == 0 ? lds(HyB + xl) : lds(HY + (yb - 1) * kTX + xl);
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        const int yl = yb + q;
        const float2 next = lds(F + (yl + 2) * kPW + xl + 1);
        const float2 xm = lds(F + (yl + 1) * kPW + xl), xp = lds(F + (yl + 1) * kPW + xl + 2);
        const float2 hx = lds(HX + yl * kTX + xl), hy = lds(HY + yl * kTX + xl);
        const float2 hxm = xl ? lds(HX + yl * kTX + xl - 1) : lds(HxL + yl);
        float2 s = fmul(hx, xp);
        s = fsub(s, fmulc(hxm, xm));
        s = fadd(s, fmul(hy, next));
        s = fsub(s, fmulc(hyp, prev));
        body(q, cur, s);
        prev = cur;
        cur = next;
        hyp = hy;
    }
}

// res::post_columns for a 16-bit buffer.
template <class S>
__device__ __forceinline__ void post_columns_s(unsigned long long *mb, unsigned e, const S *F, int wx, int yb, int nrow,
                                               int ty)
{
    if (wx != 0 && wx != kWX - 1) return;
    __syncwarp();
    const int lane = threadIdx.x;
    if (lane < nrow) {
        const int yl = yb + lane;
        const int xl = wx == 0 ? 0 : kTX - 1;
        const float2 v = lds(F + (yl + 1) * kPW + xl + 1);
        res::st_relaxed_2u64(mb + 2 * (2 * kTX + (wx == 0 ? 0 : ty) + yl), res::tag(e, v.x), res::tag(e, v.y));
    }
}

// The word slot of block b for a partial of epoch e (three epochs an iteration).  A's partials
// use PhaseFlags::w, B's the first word of each block's PhaseFlags::w4 entry (the
// single-reduction FP32 kernel's four-partial words, which this kernel never shares a launch
// with); each alternates between its two slots by iteration.
__device__ __forceinline__ unsigned long long *word_A(res::PhaseFlags *pf, unsigned e, int b)
{
    return pf->w[((e - 1) / 3) & 1] + b;
}
__device__ __forceinline__ unsigned long long *word_B(res::PhaseFlags *pf, unsigned e, int b)
{
    return &pf->w4[((e - 1) / 3) & 1][b][0];
}

// res::poll_partial on an explicit word.
__device__ __forceinline__ float poll_word(const unsigned long long *w, unsigned e, res::PhaseFlags *pf, int *err,
                                           long long lim)
{
    const long long t0 = clock64();
    for (unsigned n = 1;; n++) {
        const unsigned long long v = res::ld_relaxed_u64(w);
        if ((unsigned)(v >> 32) == e) return __uint_as_float((unsigned)v);
        if (((n & 63) == 0 || lim == 0) && (clock64() - t0 > lim || res::ld_relaxed_s32(&pf->error) != 0)) {
            atomicExch(&pf->error, 1);
            *err = 1;
            return 0.f;
        }
    }
}

// res::publish_sum to an explicit word.
template <int NW>
__device__ __forceinline__ void publish_word(float acc, unsigned long long *w, unsigned e, float *sm_w)
{
    const int lane = threadIdx.x, warp = threadIdx.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) sm_w[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        float v = lane < NW ? sm_w[lane] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) res::st_relaxed_u64(w, res::tag(e, v));
    }
}

}  // namespace ress

template <int NY, class S, class LK>
__global__ void __launch_bounds__(32 * res::kWX * ress::kWY, 1)
k_resident_s(const LK *__restrict__ H, float2 *r, S *p0, float2 *xlo, float mass, float sigma, int lx, int ly,
             MxDev *s, res::PhaseFlags *pf, unsigned long long *mbox, int ty, int gx)
{
    using namespace res;
    using namespace ress;
    constexpr int NW = kWX * kWY, NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float sm_w[32];
    __shared__ float sm_scalar;
    __shared__ int sm_ctl, sm_err;
    __shared__ ResScalars sc;
    __shared__ float2 sm_hl[kMaxBlocks / 32];
    // one read of the solve state per block, so that a block never splits here
    if (threadIdx.x == 0 && threadIdx.y == 0) sm_ctl = (s->done || s->reliable) ? kResStop : kResGo;
    __syncthreads();
    if (sm_ctl != kResGo) return;
    const long long t_start = gtimer();
    const long long lim = peer_wait_cycles(s);
    const unsigned nb = gridDim.x;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int tid = warp * 32 + lane;
    const int xl = (warp % kWX) * 32 + lane, yb = (warp / kWX) * NY;
    const int bx = blockIdx.x % gx, by = blockIdx.x / gx, gy = (int)nb / gx;
    const int x0 = bx * kTX, y0 = by * ty;
    const int tyb = min(ty, ly - y0);
    const int nrow = min(NY, tyb - yb);
    const int nring = 2 * kTX + 2 * tyb;
    const int nslot = mbox_slots(ty);
    const int nb_l = by * gx + (bx + gx - 1) % gx, nb_r = by * gx + (bx + 1) % gx;
    const int nb_d = ((by + gy - 1) % gy) * gx + bx, nb_u = ((by + 1) % gy) * gx + bx;
    unsigned long long *const Mp = mbox, *const Mt = mbox + 2 * (size_t)nb * nslot;
    // shared memory: links first (the wider type), then p' and t
    LK *const HX = reinterpret_cast<LK *>(smraw);
    LK *const HY = HX + (size_t)ty * kTX;
    LK *const HxL = HY + (size_t)ty * kTX;
    LK *const HyB = HxL + ty;
    S *const P = reinterpret_cast<S *>(HyB + kTX);
    S *const T = P + (ty + 2) * kPW;
    const bool has_ring = tid < nring;
    int rslot = 0, rgi = 0, rsrc = 0;
    if (has_ring) {
        ring_site(tid, tyb, x0, y0, lx, ly, rslot, rgi);
        rsrc = ring_source(tid, ty, tyb, nslot, nb_l, nb_r, nb_d, nb_u);
    }
    unsigned long long *const mbP = Mp + 2 * (size_t)blockIdx.x * nslot;
    unsigned long long *const mbT = Mt + 2 * (size_t)blockIdx.x * nslot;
    const int grow = (y0 + yb) * lx + x0 + xl;
    const int c0 = (yb + 1) * kPW + xl + 1;  // the thread's first row in P and T
    const int qtop = tyb - 1 - yb;
    if (tid == 0) {
        sm_err = 0;
        sc.rsq = (float)s->rsq;
        sc.rmax = (float)fmin(s->rmax, 1e38);
        sc.rn = 0.f;
        sc.beta = (float)s->beta;
        sc.scale = (float)s->scale;
        sc.delta = (float)s->delta;
        sc.stop = (float)(s->eps * sqrt(s->bsq));
        sc.k = s->k;
        sc.max_iter = s->max_iter;
        sc.status = -1;
        sc.reliable = 0;
        sc.iters = 0;
    }

    // ---- entry: r and x_lo into registers, the direction and the links into shared memory
    float2 rv[NY], xv[NY], tmp[NY];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        rv[q] = xv[q] = make_float2(0.f, 0.f);
        if (q < nrow) {
            const int gi = grow + q * lx;
            rv[q] = __ldcg(r + gi);
            xv[q] = __ldcg(xlo + gi);
            P[c0 + q * kPW] = p0[gi];
            HX[(yb + q) * kTX + xl] = H[2 * gi];
            HY[(yb + q) * kTX + xl] = H[2 * gi + 1];
        }
    }
    for (int k = tid; k < tyb + kTX; k += NT) {
        if (k < tyb) {
            const int xm = x0 == 0 ? lx - 1 : x0 - 1;
            HxL[k] = H[2 * ((y0 + k) * lx + xm)];
        } else {
            const int ym = y0 == 0 ? ly - 1 : y0 - 1;
            HyB[k - tyb] = H[2 * (ym * lx + x0 + (k - tyb)) + 1];
        }
    }
    __syncthreads();

    unsigned ep = pf->epoch;
    float fb = (float)s->beta;
    bool first = true;
    for (;;) {
        // ---- U: beta from the previous B's total; p' = r + beta p; export the border of p'
        if (!first) {
            stage_partials(tid < (int)nb ? poll_word(word_B(pf, ep, tid), ep, pf, &sm_err, lim) : 0.f, nb, sm_hl);
            __syncthreads();
            if (tid == 0) {
                const float tot = total_partials(sm_hl, nb);
                int ctl = kResGo;
                sc.rn = tot;
                sc.k++;
                sc.iters++;
                if (sm_err) {
                    sc.status = GLINALG_SOLVE_TIMEOUT;
                    ctl = kResStop;
                } else if (!isfinite(tot)) {
                    sc.status = GLINALG_SOLVE_NONFINITE;
                    ctl = kResStop;
                } else {
                    const float rho = sqrtf(tot) * sc.scale;
                    if (rho > sc.rmax) sc.rmax = rho;
                    if (rho < sc.delta * sc.rmax || rho < sc.stop || sc.k >= sc.max_iter) {
                        sc.reliable = 1;
                        ctl = kResReliable;
                    } else {
                        sc.beta = tot / sc.rsq;
                        sc.rsq = tot;
                        sm_scalar = sc.beta;
                    }
                }
                sm_ctl = ctl;
            }
            __syncthreads();
            if (sm_ctl != kResGo) break;
            fb = sm_scalar;
        }
        first = false;
        const unsigned eU = ++ep;
        {
            float2 vb = make_float2(0.f, 0.f), vt = vb;
#pragma unroll
            for (int q = 0; q < NY; q++) {
                if (q >= nrow) break;
                const float2 pn = Fmt<S>::round(fadd(rv[q], fscale(fb, lds(P + c0 + q * kPW))));
                Fmt<S>::st(P + c0 + q * kPW, 0, pn);
                if (q == 0) vb = pn;
                vt = q == qtop ? pn : vt;
            }
            post_border_rows(mbP, eU, xl, yb, nrow, qtop, tyb, vb, vt);
        }
        post_columns_s(mbP, eU, P, warp % kWX, yb, nrow, ty);
        if (has_ring) Fmt<S>::st(P + rslot, 0, poll_slot(Mp + rsrc, eU, pf, &sm_err, lim));
        __syncthreads();
        // ---- A: t = D p', stored in 16 bits; |t|^2 + sigma |p'|^2; export the border of t
        const unsigned eA = ++ep;
        float acc = 0.f;
        {
            float2 vb = make_float2(0.f, 0.f), vt = vb;
            auto body = [&](int q, float2 cur, float2 hs) {
                const float2 tv = Fmt<S>::round(fadd(fscale(mass, cur), hs));
                tmp[q] = tv;
                if (q == 0) vb = tv;
                vt = q == qtop ? tv : vt;
                acc += fn2(tv) + sigma * fn2(cur);
            };
            if (nrow == NY) hop_rows_s<NY, true>(P, HX, HY, HxL, HyB, xl, yb, nrow, body);
            else if (nrow > 0) hop_rows_s<NY, false>(P, HX, HY, HxL, HyB, xl, yb, nrow, body);
#pragma unroll
            for (int q = 0; q < NY; q++) {
                if (q >= nrow) break;
                Fmt<S>::st(T + c0 + q * kPW, 0, tmp[q]);
            }
            post_border_rows(mbT, eA, xl, yb, nrow, qtop, tyb, vb, vt);
        }
        post_columns_s(mbT, eA, T, warp % kWX, yb, nrow, ty);
        publish_word<NW>(acc, word_A(pf, eA, blockIdx.x), eA, sm_w);
        if (has_ring) Fmt<S>::st(T + rslot, 0, poll_slot(Mt + rsrc, eA, pf, &sm_err, lim));
        __syncthreads();
        // ---- B: Ap = D^dagger t + sigma p'; alpha from the total of A; x_lo += alpha p',
        // r -= alpha Ap
        {
            auto body = [&](int q, float2 cur, float2 hs) {
                tmp[q] = fadd(fsub(fscale(mass, cur), hs), fscale(sigma, lds(P + c0 + q * kPW)));
            };
            if (nrow == NY) hop_rows_s<NY, true>(T, HX, HY, HxL, HyB, xl, yb, nrow, body);
            else if (nrow > 0) hop_rows_s<NY, false>(T, HX, HY, HxL, HyB, xl, yb, nrow, body);
        }
        stage_partials(tid < (int)nb ? poll_word(word_A(pf, eA, tid), eA, pf, &sm_err, lim) : 0.f, nb, sm_hl);
        __syncthreads();
        if (tid == 0) {
            const float tot = total_partials(sm_hl, nb);
            int ctl = kResGo;
            if (sm_err) {
                sc.status = GLINALG_SOLVE_TIMEOUT;
                ctl = kResStop;
            } else if (!(tot > 0.f) || !isfinite(tot)) {
                sc.status = tot == 0.f ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
                ctl = kResStop;
            }
            sm_scalar = sc.rsq / tot;
            sm_ctl = ctl;
        }
        __syncthreads();
        if (sm_ctl != kResGo) break;
        const float alpha = sm_scalar;
        const unsigned eB = ++ep;
        acc = 0.f;
#pragma unroll
        for (int q = 0; q < NY; q++) {
            if (q >= nrow) break;
            xv[q] = fadd(xv[q], fscale(alpha, lds(P + c0 + q * kPW)));
            rv[q] = fsub(rv[q], fscale(alpha, tmp[q]));
            acc += fn2(rv[q]);
        }
        publish_word<NW>(acc, word_B(pf, eB, blockIdx.x), eB, sm_w);
    }
    // ---- exit: r, x_lo and the direction back to global memory (direction in p0)
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (q < nrow) {
            const int gi = grow + q * lx;
            r[gi] = rv[q];
            p0[gi] = P[c0 + q * kPW];
            xlo[gi] = xv[q];
        }
    }
    if (blockIdx.x == 0 && tid == 0) {
        pf->epoch = ep;
        s->k = sc.k;
        s->rmax = sc.rmax;
        s->rsq = sc.rsq;
        s->beta = sc.beta;
        s->rsq_new = sc.rn;
        s->parity = 0;
        if (sc.status >= 0) {
            s->status = sc.status;
            s->done = 1;
        }
        if (sc.reliable) s->reliable = 1;
        s->inner_ns += gtimer() - t_start;
        s->inner_iters += sc.iters;
        s->inner_launches += 1;
    }
}

}  // namespace glinalg
