// stag_tiles.cuh -- register-tiled stencil kernels for the inner iterations of the
// mixed-precision CG on the staggered normal operator D^dagger D (+ sigma).
//
// Thread block: 32 x BY threads; thread (tx, ty) owns column x = X0 + tx and the NY
// consecutive rows y = Y0 + ty*NY + j, j = 0..NY-1, so a block covers a 32 x (BY*NY) tile.
// The thread loads its column for rows -1..NY (NY+2 values), which gives every y-neighbour
// from registers; x-neighbours come from the adjacent lanes by warp shuffle (only lanes 0
// and 31 load across the warp edge), or by direct loads when lx is not a multiple of 32.
// Row indices are wrapped modulo ly, so partial tiles and lattices smaller than a tile are
// handled; rows past ly are loaded (wrapped) but neither stored nor reduced.
//
// Reductions: each thread sums its rows in FP32, the warp in FP32, the block in FP64, and the
// grid in FP64 (one partial per block, summed by the last block in block order).
#pragma once

#include "common.cuh"

namespace glinalg {

template <class S>
struct Fmt;
template <>
struct Fmt<float2> {
    static __device__ __forceinline__ float2 ld(const float2 *p, long i) { return p[i]; }
    static __device__ __forceinline__ void st(float2 *p, long i, float2 v) { p[i] = v; }
    static __host__ __device__ __forceinline__ float2 from(double2 v) { return make_float2((float)v.x, (float)v.y); }
    static __device__ __forceinline__ float2 round(float2 v) { return v; }
    static constexpr int bytes = 8;
};
template <>
struct Fmt<__half2> {
    static __device__ __forceinline__ float2 ld(const __half2 *p, long i) { return __half22float2(p[i]); }
    static __device__ __forceinline__ void st(__half2 *p, long i, float2 v) { p[i] = __float22half2_rn(v); }
    static __device__ __forceinline__ __half2 from(double2 v) { return __floats2half2_rn((float)v.x, (float)v.y); }
    // the value a store followed by a load would give, without the memory round trip
    static __device__ __forceinline__ float2 round(float2 v) { return __half22float2(__float22half2_rn(v)); }
    static constexpr int bytes = 4;
};
template <>
struct Fmt<__nv_bfloat162> {
    static __device__ __forceinline__ float2 ld(const __nv_bfloat162 *p, long i) { return __bfloat1622float2(p[i]); }
    static __device__ __forceinline__ void st(__nv_bfloat162 *p, long i, float2 v) { p[i] = __float22bfloat162_rn(v); }
    static __device__ __forceinline__ __nv_bfloat162 from(double2 v) { return __floats2bfloat162_rn((float)v.x, (float)v.y); }
    static __device__ __forceinline__ float2 round(float2 v) { return __bfloat1622float2(__float22bfloat162_rn(v)); }
    static constexpr int bytes = 4;
};

__device__ __forceinline__ float2 fadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 fsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 fscale(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
// a * b
__device__ __forceinline__ float2 fmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// conj(a) * b
__device__ __forceinline__ float2 fmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ float fn2(float2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ float2 shfl_down2(float2 v, int d)
{
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ float2 shfl_up2(float2 v, int d)
{
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}

// Grid sum of K floats per thread: FP32 within a warp, FP64 across warps and blocks.
// Returns true in all threads of the last block to arrive; the totals are then in out[]
// of its first thread.  partials: K * (number of blocks) doubles; *counter is 0 on entry
// and left 0.
template <int K, int NT>
__device__ __forceinline__ bool grid_sum_f_ids(float (&vf)[K], double *partials, unsigned *counter,
                                               double (&out)[K], unsigned bid, unsigned nbk);
template <int K, int NT>
__device__ __forceinline__ bool grid_sum_f(float (&vf)[K], double *partials, unsigned *counter,
                                           double (&out)[K])
{
    return grid_sum_f_ids<K, NT>(vf, partials, counter, out, flat_bid(), flat_nblocks());
}

// grid_sum_f over a group of nbk blocks that reduce one problem together; bid is this block's
// index within the group.
template <int K, int NT>
__device__ __forceinline__ bool grid_sum_f_ids(float (&vf)[K], double *partials, unsigned *counter,
                                               double (&out)[K], unsigned bid, unsigned nbk)
{
    __shared__ double sm[K][NT / 32];
    __shared__ unsigned ticket;
    const unsigned tid = flat_tid();
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int j = 0; j < K; j++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vf[j] += __shfl_down_sync(0xffffffffu, vf[j], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < K; j++) sm[j][warp] = (double)vf[j];
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int j = 0; j < K; j++) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; w++) s += sm[j][w];
            partials[(size_t)j * nbk + bid] = s;
        }
        __threadfence();
        ticket = atomicAdd(counter, 1u);
    }
    __syncthreads();
    if (ticket != nbk - 1) return false;
    __threadfence();
    double s[K];
#pragma unroll
    for (int j = 0; j < K; j++) s[j] = 0.0;
    for (unsigned b = tid; b < nbk; b += NT) {
#pragma unroll
        for (int j = 0; j < K; j++) s[j] += __ldcg(partials + (size_t)j * nbk + b);
    }
    block_sum<K, NT>(s);
#pragma unroll
    for (int j = 0; j < K; j++) out[j] = s[j];
    if (tid == 0) *counter = 0u;
    return true;
}

__device__ __forceinline__ int wrapi(int v, int n)
{
    v %= n;
    return v < 0 ? v + n : v;
}

// Loads the tile column of field f (rows -1..NY, wrapped) for a thread, optionally combined
// as a + beta * b (the CG direction update p' = r + beta p) when B is non-null.
template <int NY, class SA, class SB>
__device__ __forceinline__ void load_col(float2 (&c)[NY + 2], const SA *a, const SB *b, float beta,
                                         int x, int ybase, int lx, int ly)
{
#pragma unroll
    for (int j = 0; j < NY + 2; j++) {
        const long i = (long)wrapi(ybase + j - 1, ly) * lx + x;
        float2 v = Fmt<SA>::ld(a, i);
        if (b) v = fadd(v, fscale(beta, Fmt<SB>::ld(b, i)));
        c[j] = v;
    }
}

// Staggered hopping sum at the NY rows of a thread's column:
//   hs_j = h_x(x,y) f(x+1,y) - h_x(x-1,y)^* f(x-1,y) + h_y(x,y) f(x,y+1) - h_y(x,y-1)^* f(x,y-1)
// c: the column of f (rows -1..NY); xm / xp: f at columns x-1 / x+1 for rows 0..NY-1.
template <int NY, class LK>
__device__ __forceinline__ void hop_col(float2 (&hs)[NY], const float2 (&c)[NY + 2],
                                        const float2 (&fxm)[NY], const float2 (&fxp)[NY],
                                        const LK *H, int x, int xm, int ybase, int lx, int ly)
{
    float2 hy_prev = Fmt<LK>::ld(H, 2 * ((long)wrapi(ybase - 1, ly) * lx + x) + 1);
#pragma unroll
    for (int j = 0; j < NY; j++) {
        const long row = (long)wrapi(ybase + j, ly) * lx;
        const float2 hx = Fmt<LK>::ld(H, 2 * (row + x));
        const float2 hy = Fmt<LK>::ld(H, 2 * (row + x) + 1);
        const float2 hxm = Fmt<LK>::ld(H, 2 * (row + xm));
        float2 s = fmul(hx, fxp[j]);
        s = fsub(s, fmulc(hxm, fxm[j]));
        s = fadd(s, fmul(hy, c[j + 2]));
        s = fsub(s, fmulc(hy_prev, c[j]));
        hs[j] = s;
        hy_prev = hy;
    }
}

// x-neighbour columns of the tile column c: by shuffle within the warp when XS (lx a
// multiple of 32), with the two warp-edge lanes computing their outside neighbour through
// `edge(col, j)`; otherwise every lane uses `edge`.
template <int NY, bool XS, class F>
__device__ __forceinline__ void x_neighbours(float2 (&fxm)[NY], float2 (&fxp)[NY],
                                             const float2 (&c)[NY + 2], int lane, int xc, int xm,
                                             int xp, F edge)
{
    // The edge values are loaded by every lane without a branch (lanes 1..30 load their own
    // column, a cache hit, and discard it), so these loads issue together with the others
    // instead of serialising behind divergent single-lane branches.
    const int ecol = lane == 0 ? xm : (lane == 31 ? xp : xc);
    float2 ev[NY];
    if (XS) {
#pragma unroll
        for (int j = 0; j < NY; j++) ev[j] = edge(ecol, j);
    }
#pragma unroll
    for (int j = 0; j < NY; j++) {
        if (XS) {
            float2 up = shfl_down2(c[j + 1], 1);   // value of lane+1 -> column x+1
            float2 dn = shfl_up2(c[j + 1], 1);     // value of lane-1 -> column x-1
            fxp[j] = lane == 31 ? ev[j] : up;
            fxm[j] = lane == 0 ? ev[j] : dn;
        } else {
            fxp[j] = edge(xp, j);
            fxm[j] = edge(xm, j);
        }
    }
}

}  // namespace glinalg

namespace glinalg {

// ---------------------------------------------------------------- tile bodies
//
// One thread's share of a 32 x NY tile: column x, rows ybase .. ybase+NY-1.  CG selects
// ld.global.cg for the fields (needed when other blocks of the same launch write them).

template <class T>
__device__ __forceinline__ float2 ldcg2(const T *p, int i);
template <>
__device__ __forceinline__ float2 ldcg2<float2>(const float2 *p, int i) { return __ldcg(p + i); }
template <>
__device__ __forceinline__ float2 ldcg2<__half2>(const __half2 *p, int i) { return __half22float2(__ldcg(p + i)); }
template <>
__device__ __forceinline__ float2 ldcg2<__nv_bfloat162>(const __nv_bfloat162 *p, int i)
{
    return __bfloat1622float2(__ldcg(p + i));
}

template <bool CG, class T>
__device__ __forceinline__ float2 ldf(const T *p, int i)
{
    if (CG) return ldcg2<T>(p, i);
    return Fmt<T>::ld(p, i);
}

// Both hopping coefficients of a site (h_x, h_y stored adjacently) in one vector load.
template <class LK>
struct LinkPair;
template <>
struct LinkPair<float2> {
    static __device__ __forceinline__ void ld(const float2 *H, int site, float2 &hx, float2 &hy)
    {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(H) + site);
        hx = make_float2(v.x, v.y);
        hy = make_float2(v.z, v.w);
    }
    static __device__ __forceinline__ float2 ldx(const float2 *H, int site) { return __ldg(H + 2 * site); }
};
template <>
struct LinkPair<__half2> {
    static __device__ __forceinline__ void ld(const __half2 *H, int site, float2 &hx, float2 &hy)
    {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(H) + site);
        hx = __half22float2(*reinterpret_cast<const __half2 *>(&v.x));
        hy = __half22float2(*reinterpret_cast<const __half2 *>(&v.y));
    }
    static __device__ __forceinline__ float2 ldx(const __half2 *H, int site) { return __half22float2(__ldg(H + 2 * site)); }
};
template <>
struct LinkPair<__nv_bfloat162> {
    static __device__ __forceinline__ void ld(const __nv_bfloat162 *H, int site, float2 &hx, float2 &hy)
    {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(H) + site);
        hx = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&v.x));
        hy = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&v.y));
    }
    static __device__ __forceinline__ float2 ldx(const __nv_bfloat162 *H, int site)
    {
        return __bfloat1622float2(__ldg(H + 2 * site));
    }
};

// Row offsets y*lx of rows ybase-1 .. ybase+NY, wrapped periodically (a compare and an add
// in the usual case; a modulo only for lattices shorter than a tile).
template <int NY>
__device__ __forceinline__ void row_offsets(int (&off)[NY + 2], int ybase, int lx, int ly)
{
#pragma unroll
    for (int q = 0; q < NY + 2; q++) {
        int y = ybase + q - 1;
        if (y < 0) y += ly;
        if (y >= ly) {
            y -= ly;
            if (y >= ly) y %= ly;
        }
        off[q] = y * lx;
    }
}

// The tile bodies issue every load of the tile first (the column with its halo rows, the
// warp-edge values, both links of every row, and for B the per-site operands), then compute,
// then store: no load waits behind a store that might alias it, so all of a thread's loads
// are in flight together (the kernels are bound by L2 latency, not by instruction issue).

// Kernel-A share: p' = r + beta p_old ; t = D p' = m p' + hop(p') ; stores p', t and returns
// sum |t|^2 + sigma |p'|^2 over the thread's rows (computed from the rounded stored values).
template <class S, class R, class LK, int NY, bool XS, bool CG>
__device__ __forceinline__ float tile_A(const R *r, const S *pold, S *pnew, S *t, const LK *H, float beta,
                                        float mass, float sigma, int lx, int ly, int lane, int x, bool xval,
                                        int ybase)
{
    const int xc = xval ? x : lx - 1;
    const int xp = xc + 1 == lx ? 0 : xc + 1, xm = xc == 0 ? lx - 1 : xc - 1;
    int off[NY + 2];
    row_offsets<NY>(off, ybase, lx, ly);
    // ---- loads
    float2 rr[NY + 2], pp[NY + 2];
#pragma unroll
    for (int q = 0; q < NY + 2; q++) {
        rr[q] = ldf<CG>(r, off[q] + xc);
        pp[q] = ldf<CG>(pold, off[q] + xc);
    }
    float2 erm[NY], epm[NY], erp[NY], epp[NY];
    const int ecol = lane == 0 ? xm : (lane == 31 ? xp : xc);
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (XS) {
            // only the two warp-edge lanes need a value from outside the warp
            erm[q] = epm[q] = make_float2(0.f, 0.f);
            if (lane == 0 || lane == 31) {
                erm[q] = ldf<CG>(r, off[q + 1] + ecol);
                epm[q] = ldf<CG>(pold, off[q + 1] + ecol);
            }
        } else {
            erm[q] = ldf<CG>(r, off[q + 1] + xm);
            epm[q] = ldf<CG>(pold, off[q + 1] + xm);
            erp[q] = ldf<CG>(r, off[q + 1] + xp);
            epp[q] = ldf<CG>(pold, off[q + 1] + xp);
        }
    }
    float2 hx[NY], hy[NY + 1], hxm[NY], dummy;
    LinkPair<LK>::ld(H, off[0] + xc, dummy, hy[0]);
#pragma unroll
    for (int q = 0; q < NY; q++) {
        LinkPair<LK>::ld(H, off[q + 1] + xc, hx[q], hy[q + 1]);
        hxm[q] = LinkPair<LK>::ldx(H, off[q + 1] + xm);
    }
    // ---- compute
    float2 c[NY + 2];
#pragma unroll
    for (int q = 0; q < NY + 2; q++) c[q] = fadd(rr[q], fscale(beta, pp[q]));
    float acc = 0.f;
    float2 pv[NY], tv[NY];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        float2 fxp, fxm;
        if (XS) {
            const float2 ev = fadd(erm[q], fscale(beta, epm[q]));
            const float2 up = shfl_down2(c[q + 1], 1), dn = shfl_up2(c[q + 1], 1);
            fxp = lane == 31 ? ev : up;
            fxm = lane == 0 ? ev : dn;
        } else {
            fxm = fadd(erm[q], fscale(beta, epm[q]));
            fxp = fadd(erp[q], fscale(beta, epp[q]));
        }
        float2 hs = fmul(hx[q], fxp);
        hs = fsub(hs, fmulc(hxm[q], fxm));
        hs = fadd(hs, fmul(hy[q + 1], c[q + 2]));
        hs = fsub(hs, fmulc(hy[q], c[q]));
        pv[q] = c[q + 1];
        tv[q] = fadd(fscale(mass, pv[q]), hs);
        // reduce what is stored, so that alpha matches the rounded vectors
        const float2 pq = Fmt<S>::round(pv[q]), tq = Fmt<S>::round(tv[q]);
        if (xval && ybase + q < ly) acc += fn2(tq) + sigma * fn2(pq);
    }
    // ---- stores
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (xval && ybase + q < ly) {
            const int i = off[q + 1] + x;
            Fmt<S>::st(pnew, i, pv[q]);
            Fmt<S>::st(t, i, tv[q]);
        }
    }
    return acc;
}

// Kernel-B share: Ap = D^dagger t + sigma p' = m t - hop(t) + sigma p' ; x_lo += alpha p' ;
// r -= alpha Ap ; returns sum |r|^2 over the thread's rows.
template <class S, class R, class LK, int NY, bool XS, bool CG>
__device__ __forceinline__ float tile_B(const S *t, const S *p, R *r, float2 *xlo, const LK *H, float alpha,
                                        float mass, float sigma, int lx, int ly, int lane, int x, bool xval,
                                        int ybase)
{
    const int xc = xval ? x : lx - 1;
    const int xp = xc + 1 == lx ? 0 : xc + 1, xm = xc == 0 ? lx - 1 : xc - 1;
    int off[NY + 2];
    row_offsets<NY>(off, ybase, lx, ly);
    // ---- loads
    float2 c[NY + 2];
#pragma unroll
    for (int q = 0; q < NY + 2; q++) c[q] = ldf<CG>(t, off[q] + xc);
    float2 em[NY], ep[NY];
    const int ecol = lane == 0 ? xm : (lane == 31 ? xp : xc);
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (XS) {
            em[q] = make_float2(0.f, 0.f);
            if (lane == 0 || lane == 31) em[q] = ldf<CG>(t, off[q + 1] + ecol);
        } else {
            em[q] = ldf<CG>(t, off[q + 1] + xm);
            ep[q] = ldf<CG>(t, off[q + 1] + xp);
        }
    }
    float2 hx[NY], hy[NY + 1], hxm[NY], dummy;
    LinkPair<LK>::ld(H, off[0] + xc, dummy, hy[0]);
#pragma unroll
    for (int q = 0; q < NY; q++) {
        LinkPair<LK>::ld(H, off[q + 1] + xc, hx[q], hy[q + 1]);
        hxm[q] = LinkPair<LK>::ldx(H, off[q + 1] + xm);
    }
    float2 pv[NY], rv[NY], xv[NY];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int i = off[q + 1] + xc;
        pv[q] = ldf<CG>(p, i);
        rv[q] = ldf<CG>(r, i);
        xv[q] = CG ? __ldcg(xlo + i) : xlo[i];
    }
    // ---- compute
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        float2 fxp, fxm;
        if (XS) {
            const float2 up = shfl_down2(c[q + 1], 1), dn = shfl_up2(c[q + 1], 1);
            fxp = lane == 31 ? em[q] : up;
            fxm = lane == 0 ? em[q] : dn;
        } else {
            fxm = em[q];
            fxp = ep[q];
        }
        float2 hs = fmul(hx[q], fxp);
        hs = fsub(hs, fmulc(hxm[q], fxm));
        hs = fadd(hs, fmul(hy[q + 1], c[q + 2]));
        hs = fsub(hs, fmulc(hy[q], c[q]));
        const float2 av = fadd(fsub(fscale(mass, c[q + 1]), hs), fscale(sigma, pv[q]));
        xv[q] = fadd(xv[q], fscale(alpha, pv[q]));
        rv[q] = Fmt<R>::round(fsub(rv[q], fscale(alpha, av)));
        if (xval && ybase + q < ly) acc += fn2(rv[q]);
    }
    // ---- stores
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (xval && ybase + q < ly) {
            const int i = off[q + 1] + x;
            xlo[i] = xv[q];
            Fmt<R>::st(r, i, rv[q]);
        }
    }
    return acc;
}

}  // namespace glinalg
