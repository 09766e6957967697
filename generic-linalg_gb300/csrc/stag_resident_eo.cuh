// stag_resident_eo.cuh -- the inner loop of the FP32 mixed-precision CG on the even system of
// the staggered operator, m^2 - D_eo D_oe (operators.cpp:566-590; the system the reference's
// even/odd solve hands to CG, tests/staggered_pieces/staggered_pieces.cpp:331-346), in a
// checkerboarded (half-lattice) layout with each block's share on chip.
//
// With D = m + H (H the hopping term, which maps each parity to the other), the even system is
// A p_e = m^2 p_e - H (H p_e) restricted to even sites, and <p_e, A p_e> = m^2 |p_e|^2 + |H p_e|^2.
// The even fields (r, p, x_lo) and the odd field t = H p' are stored packed: site (x, y) of a
// parity sits at packed column u = x / 2 of row y, so a row holds lx / 2 sites of each parity.
// In packed coordinates a site's vertical neighbours keep its column, and its horizontal
// neighbours (which have the other parity) sit at
//   odd site (u, y):  u - (y & 1) on the left, u + 1 - (y & 1) on the right;
//   even site (u, y): u - 1 + (y & 1) on the left, u + (y & 1) on the right.
// One inner iteration, as in k_resident, with each stencil needing only the neighbours' borders:
//   A: u_o = H r (odd sites); then beta; t = u_o + beta t_old (= H p'), p' = r + beta p;
//      partial m^2 |p'|^2 + |t|^2 (+ sigma |p'|^2); export the border of t.
//   B: Ap = m^2 p' - H t + sigma p' (even sites); then alpha; x_lo += alpha p', r -= alpha Ap;
//      partial |r|^2; export the border of r.
// Each block owns 128 packed columns (256 lattice columns) by ty rows: r and t with a one-site
// ring, and the hopping coefficients of both parities (with the column left of and the row
// below the rectangle), in shared memory; p' and x_lo in registers.  Half the sites of the
// full-lattice kernel per stencil, the same exchange: border sites and partial sums travel as
// epoch-tagged words (stag_resident.cuh), every wait bounded.
//
// Requirements: lx a multiple of 256, ly even (so that a site keeps its parity across the
// periodic wrap), the rectangle within shared memory.
#pragma once

#include "stag_resident.cuh"

namespace glinalg {
namespace reseo {

using res::kPW;
using res::kTX;
using res::kWX;

// Dynamic shared memory of a rectangle of ty rows: r and t with their ring, h_x of both parities
// with the column left of the rectangle (kTX + 1 a row), h_y of both parities with the row below
// (ty + 1 rows).
inline size_t smem_bytes(int ty)
{
    return 2 * (size_t)(ty + 2) * kPW * sizeof(float2) + 2 * (size_t)ty * (kTX + 1) * sizeof(float2) +
           2 * (size_t)(ty + 1) * kTX * sizeof(float2);
}

// Rows per thread the kernel is instantiated for (4 warps along y).
constexpr int kWY = 4;
constexpr int kNumNY = 2;
constexpr int kNY[kNumNY] = {8, 14};

inline res::Plan plan(int lx, int ly, int nsm, size_t max_smem)
{
    res::Plan p;
    if (lx % (2 * kTX) != 0 || ly < 2 || ly % 2 != 0 || nsm < 1) return p;
    p.wy = kWY;
    p.gx = (lx / 2) / kTX;
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
    p.smem = smem_bytes(p.ty);
    p.ok = p.smem <= max_smem && 2 * kTX + 2 * p.ty <= 32 * kWX * kWY && p.gx * p.gy <= res::kMaxBlocks;
    return p;
}

// The shared-memory view of a rectangle (packed columns xl, rows yl).
struct RectEO {
    float2 *R, *T;     // r (even), t (odd) at [(yl + 1) * kPW + xl + 1], ring included
    float2 *HEx, *HOx; // h_x of the even / odd sites at [yl * (kTX + 1) + xl + 1] (xl = -1: left column)
    float2 *HEy, *HOy; // h_y of the even / odd sites at [(yl + 1) * kTX + xl] (yl = -1: row below)
};

__device__ __forceinline__ int hx_at(int yl, int xl) { return yl * (kTX + 1) + xl + 1; }
__device__ __forceinline__ int hy_at(int yl, int xl) { return (yl + 1) * kTX + xl; }

// Hopping sums of the thread's rows (yb .. yb+nrow-1, column xl) with outputs on the parity
// `odd_out` and inputs from the other parity in F:
//   hs = h_x f(right) - h_x(left)^* f(left) + h_y f(up) - h_y(down)^* f(down)
// (h_x(left): the link of the left neighbour, of the other parity; h_y(down) likewise), so that
// H f = hs at the output sites; body(q, hs).
template <int NY, class Body>
__device__ __forceinline__ void hop_rows_eo(const RectEO &S, const float2 *__restrict__ F, int odd_out, int xl,
                                           int yb, int nrow, int y0, Body body)
{
    const float2 *HXo = odd_out ? S.HOx : S.HEx, *HYo = odd_out ? S.HOy : S.HEy;  // outputs' links
    const float2 *HXi = odd_out ? S.HEx : S.HOx, *HYi = odd_out ? S.HEy : S.HOy;  // inputs' links
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (q >= nrow) break;
        const int yl = yb + q;
        const int py = (y0 + yl) & 1;
        // columns of the left and right neighbours in packed coordinates
        const int xlft = odd_out ? xl - py : xl - 1 + py;
        const int xrgt = xlft + 1;
        const float2 fr = F[(yl + 1) * kPW + xrgt + 1], fl = F[(yl + 1) * kPW + xlft + 1];
        const float2 fu = F[(yl + 2) * kPW + xl + 1], fd = F[yl * kPW + xl + 1];
        const float2 hx = HXo[hx_at(yl, xl)], hxl = HXi[hx_at(yl, xlft)];
        const float2 hy = HYo[hy_at(yl, xl)], hyd = HYi[hy_at(yl - 1, xl)];
        float2 s = fmul(hx, fr);
        s = fsub(s, fmulc(hxl, fl));
        s = fadd(s, fmul(hy, fu));
        s = fsub(s, fmulc(hyd, fd));
        body(q, s);
    }
}

// The pointwise passes after each stencil, over the thread's rows of column xl (T, R: the
// thread's first row in the t and r buffers).  FULL (nrow == NY) drops the per-row guard, and
// the border rows' values come out in vbot (the rectangle's first row, when the thread owns it)
// and vtop (row qtop of the thread), so that the rows carry no branch between them and the
// compiler can interleave their shared-memory loads; the posts follow the pass.
// A: t = u + beta t_old, p' = r + beta p; returns |t|^2 + m2s |p'|^2.
template <int NY, bool FULL>
__device__ __forceinline__ float update_A(float2 *__restrict__ T, const float2 *__restrict__ R, const float2 (&u)[NY],
                                          float2 (&pv)[NY], float beta, float m2s, int nrow, int qtop, float2 &vbot,
                                          float2 &vtop)
{
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        const float2 tv = fadd(u[q], fscale(beta, T[q * kPW]));
        const float2 pn = fadd(R[q * kPW], fscale(beta, pv[q]));
        pv[q] = pn;
        T[q * kPW] = tv;
        if (q == 0) vbot = tv;
        vtop = q == qtop ? tv : vtop;
        acc += fn2(tv) + m2s * fn2(pn);
    }
    return acc;
}

// B: x_lo += alpha p', r -= alpha Ap; returns |r|^2.
template <int NY, bool FULL>
__device__ __forceinline__ float update_B(float2 *__restrict__ R, const float2 (&ap)[NY], const float2 (&pv)[NY],
                                          float2 (&xv)[NY], float alpha, int nrow, int qtop, float2 &vbot, float2 &vtop)
{
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        xv[q] = fadd(xv[q], fscale(alpha, pv[q]));
        const float2 rnv = fsub(R[q * kPW], fscale(alpha, ap[q]));
        R[q * kPW] = rnv;
        if (q == 0) vbot = rnv;
        vtop = q == qtop ? rnv : vtop;
        acc += fn2(rnv);
    }
    return acc;
}

}  // namespace reseo

// The kernel: one cooperative launch per reliable-update cycle, one block of 16 warps (4 across,
// 4 down) per rectangle.  H2: packed hopping table, H2[2 j] = h_x and H2[2 j + 1] = h_y of the even
// site at packed index j = y * (lx / 2) + u, then the same for the odd sites from 2 * nh on
// (nh = lx / 2 * ly); r, p0, xlo: packed even fields (r and the direction in / out, x_lo out).
template <int NY>
__global__ void __launch_bounds__(32 * res::kWX * reseo::kWY, 1)
k_resident_eo(const float2 *__restrict__ H2, float2 *r, float2 *p0, float2 *xlo, float mass, float sigma, int lx,
              int ly, MxDev *s, res::PhaseFlags *pf, unsigned long long *mbox, int ty, int gx)
{
    using namespace res;
    using namespace reseo;
    constexpr int WY = kWY, NW = kWX * WY, NT = 32 * NW;
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
    const int hw = lx / 2;  // packed row width
    const long nh = (long)hw * ly;
    const int xl = (warp % kWX) * 32 + lane, yb = (warp / kWX) * NY;
    const int bx = blockIdx.x % gx, by = blockIdx.x / gx, gy = (int)nb / gx;
    const int x0 = bx * kTX, y0 = by * ty;
    const int tyb = min(ty, ly - y0);
    const int nrow = min(NY, tyb - yb);
    const int nring = 2 * kTX + 2 * tyb;
    const int nslot = mbox_slots(ty);
    const int nb_l = by * gx + (bx + gx - 1) % gx, nb_r = by * gx + (bx + 1) % gx;
    const int nb_d = ((by + gy - 1) % gy) * gx + bx, nb_u = ((by + 1) % gy) * gx + bx;
    unsigned long long *const Mr = mbox, *const Mt = mbox + 2 * (size_t)nb * nslot;
    RectEO S;
    S.R = reinterpret_cast<float2 *>(smraw);
    S.T = S.R + (ty + 2) * kPW;
    S.HEx = S.T + (ty + 2) * kPW;
    S.HOx = S.HEx + (size_t)ty * (kTX + 1);
    S.HEy = S.HOx + (size_t)ty * (kTX + 1);
    S.HOy = S.HEy + (size_t)(ty + 1) * kTX;
    const bool has_ring = tid < nring;
    int rslot = 0, rgi = 0, rsrc = 0;
    if (has_ring) {
        ring_site(tid, tyb, x0, y0, hw, ly, rslot, rgi);
        rsrc = ring_source(tid, ty, tyb, nslot, nb_l, nb_r, nb_d, nb_u);
    }
    unsigned long long *const mbR = Mr + 2 * (size_t)blockIdx.x * nslot;
    unsigned long long *const mbT = Mt + 2 * (size_t)blockIdx.x * nslot;
    const long grow = (long)(y0 + yb) * hw + x0 + xl;  // packed index of the thread's first row
    float2 *const Tt = S.T + (yb + 1) * kPW + xl + 1, *const Rt = S.R + (yb + 1) * kPW + xl + 1;
    const int qtop = tyb - 1 - yb;  // the thread's row that is the rectangle's last (if in range)
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
    const float m2 = mass * mass;

    // ---- entry: r, the links and the direction p of the rectangle on chip (p in registers and,
    // for one stencil, in T with its ring); t_old = H p into T
    float2 pv[NY], tmp[NY], xv[NY];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int yl = yb + q;
        pv[q] = make_float2(0.f, 0.f);
        xv[q] = make_float2(0.f, 0.f);
        if (q < nrow) {
            const long gi = grow + (long)q * hw;
            S.R[(yl + 1) * kPW + xl + 1] = __ldcg(r + gi);
            pv[q] = __ldcg(p0 + gi);
            xv[q] = __ldcg(xlo + gi);
            S.T[(yl + 1) * kPW + xl + 1] = pv[q];
            const float4 he = __ldg(reinterpret_cast<const float4 *>(H2) + gi);
            const float4 ho = __ldg(reinterpret_cast<const float4 *>(H2 + 2 * nh) + gi);
            S.HEx[hx_at(yl, xl)] = make_float2(he.x, he.y);
            S.HEy[hy_at(yl, xl)] = make_float2(he.z, he.w);
            S.HOx[hx_at(yl, xl)] = make_float2(ho.x, ho.y);
            S.HOy[hy_at(yl, xl)] = make_float2(ho.z, ho.w);
        }
    }
    // the column left of the rectangle (h_x of both parities) and the row below (h_y)
    for (int k = tid; k < tyb + kTX; k += NT) {
        if (k < tyb) {
            const int xm = x0 == 0 ? hw - 1 : x0 - 1;
            const long gi = (long)(y0 + k) * hw + xm;
            S.HEx[hx_at(k, -1)] = __ldg(H2 + 2 * gi);
            S.HOx[hx_at(k, -1)] = __ldg(H2 + 2 * nh + 2 * gi);
        } else {
            const int ym = y0 == 0 ? ly - 1 : y0 - 1;
            const long gi = (long)ym * hw + x0 + (k - tyb);
            S.HEy[hy_at(-1, k - tyb)] = __ldg(H2 + 2 * gi + 1);
            S.HOy[hy_at(-1, k - tyb)] = __ldg(H2 + 2 * nh + 2 * gi + 1);
        }
    }
    if (has_ring) {
        S.R[rslot] = __ldcg(r + rgi);
        S.T[rslot] = __ldcg(p0 + rgi);
    }
    __syncthreads();
    hop_rows_eo<NY>(S, S.T, 1, xl, yb, nrow, y0, [&](int q, float2 hs) { tmp[q] = hs; });
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NY; q++)
        if (q < nrow) S.T[(yb + q + 1) * kPW + xl + 1] = tmp[q];

    unsigned ep = pf->epoch;
    float fb = (float)s->beta;
    bool first = true;
    for (;;) {
        // ---- A: u = H r at the odd sites (needs only the ring of r), then beta from the
        // previous phase's total; t = u + beta t_old, p' = r + beta p
        hop_rows_eo<NY>(S, S.R, 1, xl, yb, nrow, y0, [&](int q, float2 hs) { tmp[q] = hs; });
        if (!first) {
            stage_partials(tid < (int)nb ? poll_partial(pf, ep, tid, &sm_err, lim) : 0.f, nb, sm_hl);
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
        const unsigned eA = ++ep;
        float acc;
        {
            float2 vb = make_float2(0.f, 0.f), vt = vb;
            if (nrow == NY) acc = update_A<NY, true>(Tt, Rt, tmp, pv, fb, m2 + sigma, nrow, qtop, vb, vt);
            else acc = update_A<NY, false>(Tt, Rt, tmp, pv, fb, m2 + sigma, nrow, qtop, vb, vt);
            if (yb == 0 && nrow > 0) post_rows(mbT, eA, xl, 0, tyb, vb);
            if (qtop >= 0 && qtop < nrow) post_rows(mbT, eA, xl, tyb - 1, tyb, vt);
        }
        post_columns(mbT, eA, S.T, warp % kWX, yb, nrow, ty);
        publish_sum<NW>(acc, pf, eA, sm_w);
        if (has_ring) S.T[rslot] = poll_slot(Mt + rsrc, eA, pf, &sm_err, lim);
        __syncthreads();
        // ---- B: Ap = m^2 p' - H t + sigma p' at the even sites (needs only the ring of t),
        // then alpha from the total of A; x_lo += alpha p', r -= alpha Ap
        hop_rows_eo<NY>(S, S.T, 0, xl, yb, nrow, y0,
                        [&](int q, float2 hs) { tmp[q] = fsub(fscale(m2 + sigma, pv[q]), hs); });
        stage_partials(tid < (int)nb ? poll_partial(pf, eA, tid, &sm_err, lim) : 0.f, nb, sm_hl);
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
        {
            float2 vb = make_float2(0.f, 0.f), vt = vb;
            if (nrow == NY) acc = update_B<NY, true>(Rt, tmp, pv, xv, alpha, nrow, qtop, vb, vt);
            else acc = update_B<NY, false>(Rt, tmp, pv, xv, alpha, nrow, qtop, vb, vt);
            if (yb == 0 && nrow > 0) post_rows(mbR, eB, xl, 0, tyb, vb);
            if (qtop >= 0 && qtop < nrow) post_rows(mbR, eB, xl, tyb - 1, tyb, vt);
        }
        post_columns(mbR, eB, S.R, warp % kWX, yb, nrow, ty);
        publish_sum<NW>(acc, pf, eB, sm_w);
        if (has_ring) S.R[rslot] = poll_slot(Mr + rsrc, eB, pf, &sm_err, lim);
        __syncthreads();
    }
    // ---- exit: the rectangle's r, x_lo and direction back to global memory (direction in p0)
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (q < nrow) {
            const long gi = grow + (long)q * hw;
            r[gi] = S.R[(yb + q + 1) * kPW + xl + 1];
            p0[gi] = pv[q];
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
