// stag_resident.cuh -- the inner loop of the FP32 mixed-precision CG on the staggered normal
// operator D^dagger D (+ sigma) with each block's share of the lattice held on chip.
//
// One cooperative launch, one block of 16 or 32 warps per SM (4 across, WY down), and every
// block owns one fixed rectangle of the lattice (128 columns by `ty` rows) for the whole launch:
//   shared memory: the hopping coefficients of the rectangle (h_x and h_y arrays) plus the h_x
//                  column left of it and the h_y row below it; the direction p' and t = D p',
//                  each with a one-site ring around the rectangle;
//   registers:     the residual r and the low-precision solution x_lo of the thread's sites
//                  (one column, NY rows).
// Per inner iteration nothing but the rectangle borders leaves the SM:
//   A: p' = r + beta p (own sites from shared memory and registers, the ring from the
//      neighbours' exported r and p'), t = D p', |t|^2 + sigma |p'|^2; export the border of t.
//   -- grid barrier (alpha) --
//   B: import the ring of t, Ap = D^dagger t + sigma p', x_lo += alpha p', r -= alpha Ap,
//      |r|^2; export the border of r and p'.
//   -- grid barrier (beta, or a reliable update is due) --
// The exchange goes through the solve's global r, t and p1 arrays (only border sites are
// written; loads use ld.global.cg).  Both barriers already separate every export from the
// imports that read it and from the next export to the same sites, so no extra
// synchronisation is needed.  The lattice wraps periodically through the same exchange, which
// also covers a rectangle that spans the whole lattice in one direction.
//
// On entry the kernel loads r, x_lo and the direction (p0) of its rectangle; on exit it writes
// them back (the direction to p0, parity 0) for the FP64 reliable update.  The per-site
// arithmetic and its order are those of tile_A / tile_B (stag_tiles.cuh).
#pragma once

#include "mixed_state.cuh"

namespace glinalg {
namespace res {

constexpr int kWX = 4;         // warps along x
constexpr int kTX = 32 * kWX;  // rectangle width (sites)
constexpr int kPW = kTX + 2;   // row pitch of the p' / t buffers (one ring site each side)

// Dynamic shared memory of a rectangle of ty rows.
inline size_t smem_bytes(int ty)
{
    return 2 * (size_t)ty * kTX * sizeof(float2)          // h_x and h_y of the rectangle
           + 2 * (size_t)(ty + 2) * kPW * sizeof(float2)  // p' and t with their ring
           + (size_t)ty * sizeof(float2)                  // h_x of the column left of the rectangle
           + (size_t)kTX * sizeof(float2);                // h_y of the row below it
}

struct Plan {
    int gx = 0, gy = 0, ty = 0, ny = 0, wy = 0;
    size_t smem = 0;
    bool ok = false;
};

// Rows per thread the kernel is instantiated for, by warps along y (4 or 8).
constexpr int kNumNY = 3;
constexpr int kNY4[kNumNY] = {4, 8, 14};
constexpr int kNY8[kNumNY] = {2, 4, 7};

// The rectangle grid for an lx x ly lattice on nsm SMs with wy warps along y: 128-column
// rectangles, as many rows of them as the SMs allow, every rectangle's state within max_smem
// bytes of shared memory.
inline Plan plan(int lx, int ly, int nsm, size_t max_smem, int wy)
{
    Plan p;
    if (lx % kTX != 0 || ly < 1 || nsm < 1 || (wy != 4 && wy != 8)) return p;
    p.wy = wy;
    p.gx = lx / kTX;
    const int gy_max = nsm / p.gx;
    if (gy_max < 1) return p;
    p.ty = (ly + gy_max - 1) / gy_max;
    p.gy = (ly + p.ty - 1) / p.ty;
    const int *ny = wy == 4 ? kNY4 : kNY8;
    for (int c = 0; c < kNumNY; c++) {
        if (ny[c] * wy >= p.ty) {
            p.ny = ny[c];
            break;
        }
    }
    if (p.ny == 0) return p;
    p.smem = smem_bytes(p.ty);
    // one ring site per thread at most (the import loops assume it)
    p.ok = p.smem <= max_smem && 2 * kTX + 2 * p.ty <= 32 * kWX * wy;
    return p;
}

// Ring site k of a rectangle (x0, y0, 128 x tyb): its slot in a p' / t buffer and its lattice
// index.  k < 128: the row below; < 256: the row above; then the column left, the column right.
__device__ __forceinline__ void ring_site(int k, int tyb, int x0, int y0, int lx, int ly, int &slot, int &gi)
{
    int xl, yl;
    if (k < kTX) {
        xl = k;
        yl = -1;
    } else if (k < 2 * kTX) {
        xl = k - kTX;
        yl = tyb;
    } else if (k < 2 * kTX + tyb) {
        xl = -1;
        yl = k - 2 * kTX;
    } else {
        xl = kTX;
        yl = k - 2 * kTX - tyb;
    }
    int gxs = x0 + xl, gys = y0 + yl;
    gxs = gxs < 0 ? gxs + lx : (gxs >= lx ? gxs - lx : gxs);
    gys = gys < 0 ? gys + ly : (gys >= ly ? gys - ly : gys);
    slot = (yl + 1) * kPW + xl + 1;
    gi = gys * lx + gxs;
}

// The shared-memory view of a rectangle.
struct Rect {
    float2 *HX, *HY;  // h_x, h_y at [yl * kTX + xl]
    float2 *P, *T;    // p', t at [(yl + 1) * kPW + xl + 1], ring included
    float2 *HxL;      // h_x at column x0 - 1, [yl]
    float2 *HyB;      // h_y at row y0 - 1, [xl]
};

// Staggered hopping sums of the thread's column (rows yb .. yb+NY-1, only the first nrow
// when !FULL) from the buffer F:
//   hs = h_x(x) f(x+1) - h_x(x-1)^* f(x-1) + h_y(y) f(y+1) - h_y(y-1)^* f(y-1)
// and, per row, body(q, f(x,y), hs).  The pointer arguments are restrict-qualified so that the
// stores of `body` do not hold back the loads of the following rows.
template <int NY, bool FULL, class Body>
__device__ __forceinline__ void hop_rows(const float2 *__restrict__ F, const float2 *__restrict__ HX,
                                         const float2 *__restrict__ HY, const float2 *__restrict__ HxL,
                                         const float2 *__restrict__ HyB, int xl, int yb, int nrow, Body body)
{
    float2 prev = F[yb * kPW + xl + 1], cur = F[(yb + 1) * kPW + xl + 1];
    float2 hyp = yb == 0 ? HyB[xl] : HY[(yb - 1) * kTX + xl];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        const int yl = yb + q;
        const float2 next = F[(yl + 2) * kPW + xl + 1];
        const float2 xm = F[(yl + 1) * kPW + xl], xp = F[(yl + 1) * kPW + xl + 2];
        const float2 hx = HX[yl * kTX + xl], hy = HY[yl * kTX + xl];
        const float2 hxm = *(xl ? HX + yl * kTX + xl - 1 : HxL + yl);
        float2 s = fmul(hx, xp);
        s = fsub(s, fmulc(hxm, xm));
        s = fadd(s, fmul(hy, next));
        s = fsub(s, fmulc(hyp, prev));
        body(q, yl, cur, s);
        prev = cur;
        cur = next;
        hyp = hy;
    }
}

// ---------------------------------------------------------------- phase exchange
//
// Each reduction of the inner loop is also the grid-wide barrier: every block publishes its
// partial sum as one 64-bit word (the phase's epoch in the high half, the FP32 partial in the
// low half) and one warp per block polls all blocks' words with relaxed loads until each
// carries the current epoch, then fences (acquire).  The publishing store follows a
// __syncthreads and a fence (release), so the border sites a block exported before the phase
// are visible to every block that has seen its word.  Words alternate between two arrays by
// phase parity: a block overwrites its word of phase e only in phase e + 2, which it reaches
// after every block has published phase e + 1, i.e. after every block has finished reading
// phase e.  The partials are summed in block order in FP64, so every block holds the same
// total.  Waits are bounded (kBarrierTimeoutNs); a wait that runs out raises the error word,
// which ends the other blocks' waits too.

constexpr int kMaxBlocks = 256;  // one rectangle per SM: above any GB300 SM count
constexpr int kPerLane = kMaxBlocks / 32;

struct PhaseFlags {
    unsigned long long w[2][kMaxBlocks];
    unsigned epoch;  // phases completed by all launches so far
    int error;
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_s32(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Phase exchange, called by every thread of the block with its partial `acc`.  On return the
// grid total is in lane 0 of warp 0 (`total`); the function returns false there when a wait ran
// out.  The caller broadcasts what lane 0 derives from the total and synchronises the block.
template <int NW>
__device__ __forceinline__ bool phase_exchange(float acc, PhaseFlags *pf, unsigned e, unsigned nb, float *sm_w,
                                               double &total)
{
    const int lane = threadIdx.x, warp = threadIdx.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) sm_w[warp] = acc;
    __syncthreads();  // the block's partials and exported border sites are complete
    if (warp != 0) return true;
    float v = lane < NW ? sm_w[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    unsigned long long *W = pf->w[e & 1];
    if (lane == 0) {
        __threadfence();  // release: this block's stores before its word
        st_relaxed_u64(W + blockIdx.x, ((unsigned long long)e << 32) | __float_as_uint(v));
    }
    float vals[kPerLane];
    unsigned pending = 0;
#pragma unroll
    for (int i = 0; i < kPerLane; i++) {
        vals[i] = 0.f;
        if (lane + 32 * i < (int)nb) pending |= 1u << i;
    }
    const long long t0 = gtimer();
    bool ok = true;
    for (;;) {
#pragma unroll
        for (int i = 0; i < kPerLane; i++) {
            if (pending & (1u << i)) {
                const unsigned long long w = ld_relaxed_u64(W + lane + 32 * i);
                if ((unsigned)(w >> 32) == e) {
                    vals[i] = __uint_as_float((unsigned)w);
                    pending &= ~(1u << i);
                }
            }
        }
        if (__all_sync(0xffffffffu, pending == 0)) break;
        const bool give_up = gtimer() - t0 > kBarrierTimeoutNs || ld_relaxed_s32(&pf->error) != 0;
        if (__any_sync(0xffffffffu, give_up)) {
            if (lane == 0) atomicExch(&pf->error, 1);
            ok = false;
            break;
        }
    }
    __threadfence();  // acquire: every block's stores before its word are visible from here
    double part = 0.0;
#pragma unroll
    for (int i = 0; i < kPerLane; i++) part += (double)vals[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    total = part;
    return ok;
}

}  // namespace res

// Control word broadcast by lane 0 of warp 0 after each phase exchange.
enum : int { kResGo = 0, kResReliable = 1, kResStop = 2 };

template <int NY, int WY>
__global__ void __launch_bounds__(32 * res::kWX * WY, 1)
k_resident(const float2 *__restrict__ H, float2 *r, float2 *p0, float2 *p1, float2 *t, float2 *xlo, float mass,
           float sigma, int lx, int ly, MxDev *s, res::PhaseFlags *pf, int ty, int gx)
{
    using namespace res;
    constexpr int NW = kWX * WY, NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float sm_w[32];
    __shared__ float sm_alpha, sm_beta;
    __shared__ int sm_ctl;
    if (s->done || s->reliable) return;
    const long long t_start = gtimer();
    const unsigned nb = gridDim.x;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int tid = warp * 32 + lane;
    const int xl = (warp % kWX) * 32 + lane, yb = (warp / kWX) * NY;
    const int x0 = (blockIdx.x % gx) * kTX, y0 = (blockIdx.x / gx) * ty;
    const int tyb = min(ty, ly - y0);  // rows of this rectangle
    const int nrow = min(NY, tyb - yb);  // rows of this thread (<= 0: none)
    const int nring = 2 * kTX + 2 * tyb;
    Rect R;
    R.HX = reinterpret_cast<float2 *>(smraw);
    R.HY = R.HX + (size_t)ty * kTX;
    R.P = R.HY + (size_t)ty * kTX;
    R.T = R.P + (ty + 2) * kPW;
    R.HxL = R.T + (ty + 2) * kPW;
    R.HyB = R.HxL + ty;

    // ---- entry: the rectangle's state into registers and shared memory
    float2 rv[NY], xv[NY];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int yl = yb + q;
        rv[q] = xv[q] = make_float2(0.f, 0.f);
        if (q < nrow) {
            const int gi = (y0 + yl) * lx + x0 + xl;
            rv[q] = __ldcg(r + gi);
            xv[q] = __ldcg(xlo + gi);
            R.P[(yl + 1) * kPW + xl + 1] = __ldcg(p0 + gi);
            const float4 h = __ldg(reinterpret_cast<const float4 *>(H) + gi);
            R.HX[yl * kTX + xl] = make_float2(h.x, h.y);
            R.HY[yl * kTX + xl] = make_float2(h.z, h.w);
        }
    }
    for (int k = tid; k < tyb + kTX; k += NT) {
        if (k < tyb) {
            const int xm = x0 == 0 ? lx - 1 : x0 - 1;
            R.HxL[k] = __ldg(H + 2 * ((y0 + k) * lx + xm));
        } else {
            const int ym = y0 == 0 ? ly - 1 : y0 - 1;
            R.HyB[k - tyb] = __ldg(H + 2 * (ym * lx + x0 + (k - tyb)) + 1);
        }
    }

    // FP64 recurrence state: used by lane 0 of warp 0 only
    double rsq = s->rsq, rmax = s->rmax, rn = 0.0;
    double beta64 = s->beta;
    const double scale = s->scale;
    const float delta = (float)s->delta, stop = (float)(s->eps * sqrt(s->bsq));
    int k = s->k;
    const int max_iter = s->max_iter;
    const unsigned ebase = pf->epoch;
    int j = 0, status = -1, phases = 0;
    bool reliable = false;
    float fb = (float)s->beta;
    const bool has_ring = tid < nring;
    int rslot = 0, rgi = 0;
    if (has_ring) ring_site(tid, tyb, x0, y0, lx, ly, rslot, rgi);
    const bool border_x = xl == 0 || xl == kTX - 1;
    const int grow = (y0 + yb) * lx + x0 + xl;  // lattice index of the thread's first row
    __syncthreads();
    for (;;) {
        // the neighbours' direction: the launch's input (p0) before their first export to p1
        const float2 *pex = j == 0 ? p0 : p1;
        // ---- A: p' = r + beta p on the rectangle and its ring (the ring loads first, so that
        // their latency overlaps the update of the own sites)
        float2 ra = make_float2(0.f, 0.f), rb = ra;
        if (has_ring) {
            ra = __ldcg(r + rgi);
            rb = __ldcg(pex + rgi);
        }
#pragma unroll
        for (int q = 0; q < NY; q++) {
            if (q < nrow) {
                float2 &pp = R.P[(yb + q + 1) * kPW + xl + 1];
                pp = fadd(rv[q], fscale(fb, pp));
            }
        }
        if (has_ring) R.P[rslot] = fadd(ra, fscale(fb, rb));
        __syncthreads();
        // t = D p' ; |t|^2 + sigma |p'|^2 ; export the border of t
        float acc = 0.f;
        {
            float2 *__restrict__ Tw = R.T;
            auto body = [&](int q, int yl, float2 cur, float2 hs) {
                const float2 tv = fadd(fscale(mass, cur), hs);
                Tw[(yl + 1) * kPW + xl + 1] = tv;
                acc += fn2(tv) + sigma * fn2(cur);
                if (yl == 0 || yl == tyb - 1 || border_x) t[grow + q * lx] = tv;
            };
            if (nrow == NY) hop_rows<NY, true>(R.P, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
            else if (nrow > 0) hop_rows<NY, false>(R.P, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        }
        double tot = 0.0;
        const bool okA = phase_exchange<NW>(acc, pf, ebase + ++phases, nb, sm_w, tot);
        if (tid == 0) {
            int ctl = kResGo;
            if (!okA) {
                status = GLINALG_SOLVE_TIMEOUT;
                ctl = kResStop;
            } else if (!(tot > 0.0) || !isfinite(tot)) {
                status = tot == 0.0 ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
                ctl = kResStop;
            }
            sm_alpha = (float)rsq / (float)tot;
            sm_ctl = ctl;
        }
        __syncthreads();
        if (sm_ctl != kResGo) break;
        const float alpha = sm_alpha;
        // ---- B: the ring of t, then Ap = D^dagger t + sigma p', x_lo += alpha p', r -= alpha Ap
        if (has_ring) R.T[rslot] = __ldcg(t + rgi);
        __syncthreads();
        acc = 0.f;
        {
            const float2 *__restrict__ Pr = R.P;
            auto body = [&](int q, int yl, float2 cur, float2 hs) {
                const float2 pv = Pr[(yl + 1) * kPW + xl + 1];
                const float2 av = fadd(fsub(fscale(mass, cur), hs), fscale(sigma, pv));
                xv[q] = fadd(xv[q], fscale(alpha, pv));
                rv[q] = fsub(rv[q], fscale(alpha, av));
                acc += fn2(rv[q]);
                if (yl == 0 || yl == tyb - 1 || border_x) {
                    r[grow + q * lx] = rv[q];
                    p1[grow + q * lx] = pv;
                }
            };
            if (nrow == NY) hop_rows<NY, true>(R.T, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
            else if (nrow > 0) hop_rows<NY, false>(R.T, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        }
        const bool okB = phase_exchange<NW>(acc, pf, ebase + ++phases, nb, sm_w, tot);
        j++;
        if (tid == 0) {
            int ctl = kResGo;
            rn = tot;
            k++;
            if (!okB) {
                status = GLINALG_SOLVE_TIMEOUT;
                ctl = kResStop;
            } else if (!isfinite(rn)) {
                status = GLINALG_SOLVE_NONFINITE;
                ctl = kResStop;
            } else {
                const float rho = sqrtf((float)rn) * (float)scale;  // true-scale iterated residual
                if (rho > rmax) rmax = rho;
                if (rho < delta * (float)rmax || rho < stop || k >= max_iter) {
                    reliable = true;
                    ctl = kResReliable;
                } else {
                    const float b = (float)rn / (float)rsq;
                    beta64 = b;
                    rsq = rn;
                    sm_beta = b;
                }
            }
            sm_ctl = ctl;
        }
        __syncthreads();
        if (sm_ctl != kResGo) break;
        fb = sm_beta;
    }
    // ---- exit: the rectangle's r, x_lo and direction back to global memory (direction in p0)
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (q < nrow) {
            const int gi = grow + q * lx;
            r[gi] = rv[q];
            xlo[gi] = xv[q];
            p0[gi] = R.P[(yb + q + 1) * kPW + xl + 1];
        }
    }
    if (blockIdx.x == 0 && tid == 0) {
        pf->epoch = ebase + phases;  // every block ran the same phases
        s->k = k;
        s->rmax = rmax;
        s->rsq = rsq;
        s->beta = beta64;
        s->rsq_new = rn;
        s->parity = 0;
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
