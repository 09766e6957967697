// stag_resident.cuh -- the inner loop of the FP32 mixed-precision CG on the staggered normal
// operator D^dagger D (+ sigma) with each block's share of the lattice held on chip.
//
// One cooperative launch, one block of 16 or 32 warps per SM (4 across, WY down), and every
// block owns one fixed rectangle of the lattice (128 columns by `ty` rows) for the whole launch.
// Per inner iteration nothing but the rectangle borders leaves the SM.  The iteration is CG on
// A = D^dagger D + sigma written so that each stencil needs only the neighbours' borders and the
// grid-wide sum it waits for is due only after the stencil (the sum's latency, a few
// microseconds on GB300, hides behind it):
//   A: u = D r; then beta (the total of the previous B); t = u + beta t_old (= D p'),
//      p' = r + beta p, |t|^2 + sigma |p'|^2; export the border of t.
//   B: Ap = D^dagger t + sigma p'; then alpha = |r|^2 / <p', A p'> (the total of A);
//      x_lo += alpha p', r -= alpha Ap, |r|^2; export the border of r.
// Shared memory holds r and t, each with a one-site ring, and the hopping coefficients; the
// direction p' stays in registers.  x_lo stays in registers, in global memory (updated by
// vector reductions in L2) or in tensor memory; in the fastest form the links of each
// thread's sites are in tensor memory too, so that the stencils read only the field from
// shared memory (see the tensor-memory section and k_resident's XM).  Border sites travel
// through epoch-tagged mailboxes in global memory (L2), with no memory fence in the loop (see
// the exchange section below); each border site is posted by the warp that computes it, as
// soon as it is computed.
//
// On entry the kernel loads r and the direction (p0) of its rectangle and computes t_old = D p;
// on exit it writes r, x_lo and the direction (to p0, parity 0) back for the FP64 reliable
// update.  The per-site arithmetic is that of tile_A / tile_B (stag_tiles.cuh) except that
// D p' is formed as D r + beta D p.
#pragma once

#include "mixed_state.cuh"

namespace glinalg {
namespace res {

constexpr int kWX = 4;         // warps along x
constexpr int kTX = 32 * kWX;  // rectangle width (sites)
constexpr int kPW = kTX + 2;   // row pitch of the r / t buffers (one ring site each side)

// Dynamic shared memory of a rectangle of ty rows.
inline size_t smem_bytes(int ty)
{
    return 2 * (size_t)ty * kTX * sizeof(float2)          // h_x and h_y of the rectangle
           + 2 * (size_t)(ty + 2) * kPW * sizeof(float2)  // r and t with their ring
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

// Ring site k of a rectangle (x0, y0, 128 x tyb): its slot in an r / t buffer and its lattice
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
    float2 *F, *T;    // r, t at [(yl + 1) * kPW + xl + 1], ring included
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

// ---------------------------------------------------------------- tensor memory
//
// The kernel does not use the tensor cores, but their accumulator memory (TMEM, 512 columns of
// 128 lanes x 32 bits per SM) is storage outside the register file and the shared-memory pipe.
// A warp reaches only the 32 lanes of its sub-partition (lanes 32 (warp % 4) ..), through
// tcgen05.ld / tcgen05.st of 32-bit columns (shape 32x32b: thread i of the warp reads or writes
// lane 32 (warp % 4) + i).  The block allocates its columns once (one warp, tcgen05.alloc) and
// frees them on every exit path before it returns.

__device__ __forceinline__ unsigned smem_addr(const void *p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }

// Called by one whole warp: allocates ncols columns (a power of two >= 32) and writes their base
// address to *dst (shared memory); gives up the right to allocate again (the block allocates once).
__device__ __forceinline__ void tmem_alloc(unsigned *dst, unsigned ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// Called by the warp that allocated, after every access of the block has completed.
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Two consecutive columns of the thread's lane (issued by the whole warp; the values are valid
// after tmem_wait_ld).
__device__ __forceinline__ void tmem_ld2(unsigned taddr, float2 &v)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(taddr));
}
__device__ __forceinline__ void tmem_st2(unsigned taddr, float2 v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(taddr), "f"(v.x), "f"(v.y) : "memory");
}
// Waits for the thread's outstanding tcgen05.ld; the values pass through the statement so that
// no use of them is scheduled before the wait.
template <int N>
__device__ __forceinline__ void tmem_wait_ld(float2 (&v)[N])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < N; q++) asm volatile("" : "+f"(v[q].x), "+f"(v[q].y));
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld4(unsigned taddr, float4 &v)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_st4(unsigned taddr, float4 v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "f"(v.x), "f"(v.y),
                 "f"(v.z), "f"(v.w)
                 : "memory");
}
// tmem_wait_ld for one row of links (h_x, h_y in a, h_x of the left neighbour in b).
__device__ __forceinline__ void tmem_wait_ld_row(float4 &a, float2 &b)
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    asm volatile("" : "+f"(a.x), "+f"(a.y), "+f"(a.z), "+f"(a.w), "+f"(b.x), "+f"(b.y));
}

// hop_rows with the links of the thread's sites in tensor memory instead of shared memory: tA
// addresses its rows' (h_x, h_y) (4 columns a row), tB its rows' h_x of the left neighbour (2
// columns a row); hyp0 is h_y of the row below the first.  Each row's links are loaded while
// the row before is computed.  Shared memory serves only the field: 3 loads per site, not 6.
template <int NY, bool FULL, class Body>
__device__ __forceinline__ void hop_rows_tm(const float2 *__restrict__ F, unsigned tA, unsigned tB, float2 hyp0,
                                            int xl, int yb, int nrow, Body body)
{
    float2 prev = F[yb * kPW + xl + 1], cur = F[(yb + 1) * kPW + xl + 1];
    float2 hyp = hyp0;
    float4 L;
    float2 Lm;
    tmem_ld4(tA, L);
    tmem_ld2(tB, Lm);
    tmem_wait_ld_row(L, Lm);
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        float4 Ln;
        float2 Lmn;
        if (q + 1 < NY) {
            tmem_ld4(tA + 4 * (q + 1), Ln);
            tmem_ld2(tB + 2 * (q + 1), Lmn);
        }
        const int yl = yb + q;
        const float2 next = F[(yl + 2) * kPW + xl + 1];
        const float2 xm = F[(yl + 1) * kPW + xl], xp = F[(yl + 1) * kPW + xl + 2];
        const float2 hx = make_float2(L.x, L.y), hy = make_float2(L.z, L.w);
        float2 s = fmul(hx, xp);
        s = fsub(s, fmulc(Lm, xm));
        s = fadd(s, fmul(hy, next));
        s = fsub(s, fmulc(hyp, prev));
        body(q, yl, cur, s);
        prev = cur;
        cur = next;
        hyp = hy;
        if (q + 1 < NY) {
            tmem_wait_ld_row(Ln, Lmn);
            L = Ln;
            Lm = Lmn;
        }
    }
}

// ---------------------------------------------------------------- exchange between blocks
//
// Nothing in the inner loop waits for a memory fence.  Every value one block hands to another
// carries the epoch of the phase that produced it, in 64-bit words that are single-copy
// atomic: a border site of r or t goes out as two words (epoch << 32 | float bits of the real
// and of the imaginary part) into the producing block's mailbox, and a block's partial sum as
// one word (epoch << 32 | float bits).  A consumer polls the words it needs with relaxed loads
// until they carry the current epoch, so a value is used only once it has arrived.
//
// Epochs grow by one per phase (two per iteration) across the launches of a solve.  A mailbox
// slot is rewritten two phases later (the same field, the next iteration), and a block reaches
// that write only after the grid-wide sum in between, which every block contributes to only
// after it has read the slot's previous contents (k_resident posts border words from its
// update passes, which come after the wait for that sum); partial-sum words alternate between two
// arrays by phase parity for the same reason.  Every wait is bounded (kSpinCycles by default,
// the caller's limit when the solve sets one: peer_wait_cycles); a wait that runs out raises
// the error word, which ends the waits of every other block too.

constexpr int kMaxBlocks = 256;  // one rectangle per SM: above any GB300 SM count
constexpr int kPerLane = kMaxBlocks / 32;
constexpr long long kSpinCycles = 4000000000LL;  // about 2 s at GB300 clocks

// The solve's bound on a wait, in SM clock cycles (2 per ns: GB300's SM clock is at most
// 2.07 GHz, so the wait lasts at least the requested time): MxDev::wait_ns > 0 converted, the
// default for 0, and 0 (give up at the first poll that finds the data missing) for < 0.
__device__ __forceinline__ long long peer_wait_cycles(const MxDev *s)
{
    return s->wait_ns > 0 ? 2 * s->wait_ns : (s->wait_ns == 0 ? kSpinCycles : 0LL);
}

struct PhaseFlags {
    unsigned long long w[2][kMaxBlocks];  // partial-sum words by phase parity
    // the single-reduction kernel's four partials per block, by iteration parity
    unsigned long long w4[2][kMaxBlocks][4];
    unsigned epoch;                       // phases completed by all launches so far
    int error;
};

// Mailbox slots of a block with ty-row rectangles: bottom row, top row, left column, right column.
__host__ __device__ inline int mbox_slots(int ty) { return 2 * kTX + 2 * ty; }
// 64-bit words of the mailboxes of both fields (r and t) for nb blocks.
inline size_t mbox_words(int nb, int ty) { return 2 * (size_t)nb * mbox_slots(ty) * 2; }

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
__device__ __forceinline__ void ld_relaxed_2u64(const unsigned long long *p, unsigned long long &a,
                                                unsigned long long &b)
{
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}
__device__ __forceinline__ void st_relaxed_2u64(unsigned long long *p, unsigned long long a, unsigned long long b)
{
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
// st_relaxed_2u64 without the memory clobber: for words posted from registers, whose order
// against the thread's plain loads and stores does not matter (volatile statements keep their
// order among themselves, so a post still precedes the thread's later polls).
__device__ __forceinline__ void st_relaxed_2u64_nc(unsigned long long *p, unsigned long long a, unsigned long long b)
{
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b));
}
__device__ __forceinline__ int ld_relaxed_s32(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long tag(unsigned e, float v)
{
    return ((unsigned long long)e << 32) | __float_as_uint(v);
}

// Border slot k of a rectangle (tyb rows): the shared-memory position of the site it carries and
// its slot in the block's mailbox.  Slots: bottom row, top row (kTX each), then the left and
// the right column (ty each, tyb used); a corner site is carried by two slots.
__device__ __forceinline__ void border_slot(int k, int ty, int tyb, int &pos, int &slot)
{
    int xl, yl;
    if (k < kTX) {
        xl = k;
        yl = 0;
        slot = k;
    } else if (k < 2 * kTX) {
        xl = k - kTX;
        yl = tyb - 1;
        slot = k;
    } else if (k < 2 * kTX + tyb) {
        xl = 0;
        yl = k - 2 * kTX;
        slot = 2 * kTX + yl;
    } else {
        xl = kTX - 1;
        yl = k - 2 * kTX - tyb;
        slot = 2 * kTX + ty + yl;
    }
    pos = (yl + 1) * kPW + xl + 1;
}

// Posts site (xl, yl) of a rectangle of tyb rows, value v of epoch e, to the bottom-row and
// top-row border slots that carry it (mb: this block's mailbox within the field), straight from
// the register of the thread that computed it.  yl is the same in the whole warp, so the
// branches do not split it.
__device__ __forceinline__ void post_rows(unsigned long long *mb, unsigned e, int xl, int yl, int tyb, float2 v)
{
    const unsigned long long a = tag(e, v.x), b = tag(e, v.y);
    if (yl == 0) st_relaxed_2u64_nc(mb + 2 * xl, a, b);
    if (yl == tyb - 1) st_relaxed_2u64_nc(mb + 2 * (kTX + xl), a, b);
}

// Posts the left (wx == 0) or right (wx == kWX - 1) column of the warp's rows (yb .. yb+nrow-1)
// of F, epoch e, after the warp has written them to shared memory: lane q posts row yb + q, one
// store instruction for the warp.  Other warps return at once.
__device__ __forceinline__ void post_columns(unsigned long long *mb, unsigned e, const float2 *F, int wx, int yb,
                                             int nrow, int ty)
{
    if (wx != 0 && wx != kWX - 1) return;
    __syncwarp();
    const int lane = threadIdx.x;
    if (lane < nrow) {
        const int yl = yb + lane;
        const int xl = wx == 0 ? 0 : kTX - 1;
        const float2 v = F[(yl + 1) * kPW + xl + 1];
        st_relaxed_2u64(mb + 2 * (2 * kTX + (wx == 0 ? 0 : ty) + yl), tag(e, v.x), tag(e, v.y));
    }
}

// The mailbox word (within a field) that feeds ring site k: the row below comes from the top
// row of the block below, the row above from the bottom row of the block above, the column left
// from the right column of the block to the left, the column right from the left column of the
// block to the right.
__device__ __forceinline__ int ring_source(int k, int ty, int tyb, int nslot, int nb_l, int nb_r, int nb_d,
                                           int nb_u)
{
    int b, slot;
    if (k < kTX) {
        b = nb_d;
        slot = kTX + k;
    } else if (k < 2 * kTX) {
        b = nb_u;
        slot = k - kTX;
    } else if (k < 2 * kTX + tyb) {
        b = nb_l;
        slot = 2 * kTX + ty + (k - 2 * kTX);
    } else {
        b = nb_r;
        slot = 2 * kTX + (k - 2 * kTX - tyb);
    }
    return 2 * (b * nslot + slot);
}

// Polls a mailbox slot until both words carry epoch e; returns the value, or sets *err (and the
// error word) when the wait runs out or another block has raised the error word.
__device__ __forceinline__ float2 poll_slot(const unsigned long long *p, unsigned e, PhaseFlags *pf, int *err,
                                           long long lim)
{
    unsigned long long a, b;
    const long long t0 = clock64();
    for (unsigned n = 1;; n++) {
        ld_relaxed_2u64(p, a, b);
        if ((unsigned)(a >> 32) == e && (unsigned)(b >> 32) == e) break;
        if (((n & 63) == 0 || lim == 0) && (clock64() - t0 > lim || ld_relaxed_s32(&pf->error) != 0)) {
            atomicExch(&pf->error, 1);
            *err = 1;
            break;
        }
    }
    return make_float2(__uint_as_float((unsigned)a), __uint_as_float((unsigned)b));
}

// *p += v, performed in L2 (no value comes back).  No memory clobber: the kernels never read
// x_lo back (the next launch does, after the kernel boundary), so the shared-memory loads and
// stores around the reduction may move past it.
__device__ __forceinline__ void red_add2(float2 *p, float2 v)
{
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(v.x), "f"(v.y));
}

// s + c = a + b exactly (Knuth's TwoSum), for the compensated sums below.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &c)
{
    s = a + b;
    const float bb = s - a;
    c = (a - (s - bb)) + (b - bb);
}

// Called by threads 0 .. nb-1: thread b waits until block b's word carries epoch e and returns
// its partial (0 when the wait runs out, which sets *err).  One word per thread keeps the
// poll's registers few (they count for every thread of the block).
__device__ __forceinline__ float poll_partial(PhaseFlags *pf, unsigned e, int b, int *err, long long lim)
{
    const unsigned long long *w = pf->w[e & 1] + b;
    const long long t0 = clock64();
    for (unsigned n = 1;; n++) {
        const unsigned long long v = ld_relaxed_u64(w);
        if ((unsigned)(v >> 32) == e) return __uint_as_float((unsigned)v);
        if (((n & 63) == 0 || lim == 0) && (clock64() - t0 > lim || ld_relaxed_s32(&pf->error) != 0)) {
            atomicExch(&pf->error, 1);
            *err = 1;
            return 0.f;
        }
    }
}

// Called by every thread right after the polls (thread b < nb holds block b's partial v, the
// others 0): each polling warp sums its 32 partials (compensated FP32, shuffle tree) and lane 0
// stages the pair (sum, error) in sm_hl[warp].  The reduction runs as each warp's polls end, so
// after the barrier only total_partials' short chain remains.
__device__ __forceinline__ void stage_partials(float v, unsigned nb, float2 *sm_hl)
{
    const int lane = threadIdx.x, warp = threadIdx.y;
    if (warp * 32 >= (int)nb) return;
    float hi = v, lo = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o), l2 = __shfl_down_sync(0xffffffffu, lo, o);
        float c;
        two_sum(hi, h2, hi, c);
        lo += l2 + c;
    }
    if (lane == 0) sm_hl[warp] = make_float2(hi, lo);
}

// After the barrier that follows stage_partials: the total over the polling warps in warp order.
// The order of every addition is fixed by the block numbers alone, so every block forms the same
// total.
__device__ __forceinline__ float total_partials(const float2 *sm_hl, unsigned nb)
{
    const int npw = ((int)nb + 31) / 32;
    float2 p[kMaxBlocks / 32];
#pragma unroll
    for (int w = 0; w < kMaxBlocks / 32; w++) p[w] = w < npw ? sm_hl[w] : make_float2(0.f, 0.f);
    float hi = 0.f, lo = 0.f;
#pragma unroll
    for (int w = 0; w < kMaxBlocks / 32; w++) {
        float c;
        two_sum(hi, p[w].x, hi, c);
        lo += p[w].y + c;
    }
    return hi + lo;
}

// Phase A's pointwise pass over the thread's rows: t = u + beta t_old into T and p' = r + beta p;
// returns |t|^2 + sigma |p'|^2.  T and F point at the thread's first row; restrict-qualified,
// so the loads of later rows need not wait for the stores of earlier ones.  FULL (nrow == NY)
// drops the per-row guard, and the values of the rectangle's bottom row (the thread's row 0)
// and top row (the thread's row qtop) come out in vbot / vtop for the caller to post: with no
// branch between the rows, the compiler interleaves their shared-memory loads (the posts inside
// the loop, each under its own test, cost the pass 40% of its time).
template <int NY, bool FULL>
__device__ __forceinline__ float pass_A(float2 *__restrict__ T, const float2 *__restrict__ F, const float2 (&u)[NY],
                                        float2 (&pv)[NY], float beta, float sigma, int nrow, int qtop, float2 &vbot,
                                        float2 &vtop)
{
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        const float2 tv = fadd(u[q], fscale(beta, T[q * kPW]));
        const float2 pn = fadd(F[q * kPW], fscale(beta, pv[q]));
        pv[q] = pn;
        T[q * kPW] = tv;
        if (q == 0) vbot = tv;
        vtop = q == qtop ? tv : vtop;
        acc += fn2(tv) + sigma * fn2(pn);
    }
    return acc;
}

// Phase B's pointwise pass: r -= alpha Ap into R (the thread's first row), x_lo += alpha p' in
// registers (XREG) or in global memory (XGLOB, xg: the thread's first row of x_lo, rows lx
// apart); returns |r|^2.  Border rows as in pass_A.
template <int NY, bool FULL, bool XREG, bool XGLOB, int NX>
__device__ __forceinline__ float pass_B(float2 *__restrict__ R, const float2 (&ap)[NY], const float2 (&pv)[NY],
                                        float2 (&xv)[NX], float2 *xg, int lx, float alpha, int nrow, int qtop,
                                        float2 &vbot, float2 &vtop)
{
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (!FULL && q >= nrow) break;
        if (XREG) xv[q < NX ? q : 0] = fadd(xv[q < NX ? q : 0], fscale(alpha, pv[q]));
        else if (XGLOB) red_add2(xg + (long)q * lx, fscale(alpha, pv[q]));
        const float2 rnv = fsub(R[q * kPW], fscale(alpha, ap[q]));
        R[q * kPW] = rnv;
        if (q == 0) vbot = rnv;
        vtop = q == qtop ? rnv : vtop;
        acc += fn2(rnv);
    }
    return acc;
}

// Posts the rectangle's bottom row (vbot, when the thread's first row is row 0) and top row
// (vtop, the thread's row qtop) after a pointwise pass.
__device__ __forceinline__ void post_border_rows(unsigned long long *mb, unsigned e, int xl, int yb, int nrow,
                                                 int qtop, int tyb, float2 vbot, float2 vtop)
{
    if (yb == 0 && nrow > 0) post_rows(mb, e, xl, 0, tyb, vbot);
    if (qtop >= 0 && qtop < nrow) post_rows(mb, e, xl, tyb - 1, tyb, vtop);
}

// Publishes the block's partial sum of phase e (every thread passes its `acc`): FP32 sums within warps and across the block's warps, one
// tagged word written by thread 0.
template <int NW>
__device__ __forceinline__ void publish_sum(float acc, PhaseFlags *pf, unsigned e, float *sm_w)
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
        if (lane == 0) st_relaxed_u64(pf->w[e & 1] + blockIdx.x, tag(e, v));
    }
}

// Publishes the four partial sums of a block (FP32 within warps and across the block's warps;
// thread 0 writes two tagged 128-bit words), then the border of F (thread k < nborder posts
// border slot k from shared memory).
template <int NW>
__device__ __forceinline__ void publish4(float4 acc, PhaseFlags *pf, unsigned e, float4 *sm_w4, const float2 *F,
                                         unsigned long long *M, int nborder, int bpos, int bslot)
{
    const int lane = threadIdx.x, warp = threadIdx.y, tid = warp * 32 + lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_down_sync(0xffffffffu, acc.z, o);
        acc.w += __shfl_down_sync(0xffffffffu, acc.w, o);
    }
    if (lane == 0) sm_w4[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        float4 v = lane < NW ? sm_w4[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, o);
            v.y += __shfl_down_sync(0xffffffffu, v.y, o);
            v.z += __shfl_down_sync(0xffffffffu, v.z, o);
            v.w += __shfl_down_sync(0xffffffffu, v.w, o);
        }
        if (lane == 0) {
            unsigned long long *w = pf->w4[(e >> 1) & 1][blockIdx.x];
            st_relaxed_2u64(w, tag(e, v.x), tag(e, v.y));
            st_relaxed_2u64(w + 2, tag(e, v.z), tag(e, v.w));
        }
    }
    if (tid < nborder) {
        const float2 v = F[bpos];
        st_relaxed_2u64(M + 2 * bslot, tag(e, v.x), tag(e, v.y));
    }
}

// Posts the border of F (thread k < nborder posts border slot k), with no partial sum.
__device__ __forceinline__ void publish_border(unsigned e, const float2 *F, unsigned long long *M, int nborder,
                                               int bpos, int bslot)
{
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (tid < nborder) {
        const float2 v = F[bpos];
        st_relaxed_2u64(M + 2 * bslot, tag(e, v.x), tag(e, v.y));
    }
}

// Thread b waits until block b's four partial words carry epoch e and stages them.
__device__ __forceinline__ void poll_partial4(PhaseFlags *pf, unsigned e, int b, float4 *sm_part4, int *err,
                                              long long lim)
{
    const unsigned long long *w = pf->w4[(e >> 1) & 1][b];
    const long long t0 = clock64();
    for (unsigned n = 1;; n++) {
        unsigned long long a0, a1, a2, a3;
        ld_relaxed_2u64(w, a0, a1);
        ld_relaxed_2u64(w + 2, a2, a3);
        if ((unsigned)(a0 >> 32) == e && (unsigned)(a1 >> 32) == e && (unsigned)(a2 >> 32) == e &&
            (unsigned)(a3 >> 32) == e) {
            sm_part4[b] = make_float4(__uint_as_float((unsigned)a0), __uint_as_float((unsigned)a1),
                                      __uint_as_float((unsigned)a2), __uint_as_float((unsigned)a3));
            return;
        }
        if (((n & 63) == 0 || lim == 0) && (clock64() - t0 > lim || ld_relaxed_s32(&pf->error) != 0)) {
            atomicExch(&pf->error, 1);
            *err = 1;
            sm_part4[b] = make_float4(0.f, 0.f, 0.f, 0.f);
            return;
        }
    }
}

// Compensated sums of the four components of the staged partials, in block order (warp 0),
// the four chains interleaved; the totals are in lane 0.
__device__ __forceinline__ float4 sum_partials4(const float4 *sm_part4, unsigned nb)
{
    const int lane = threadIdx.x;
    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int b = lane; b < (int)nb; b += 32) {
        const float4 v = sm_part4[b];
        float c;
        two_sum(hi.x, v.x, hi.x, c);
        lo.x += c;
        two_sum(hi.y, v.y, hi.y, c);
        lo.y += c;
        two_sum(hi.z, v.z, hi.z, c);
        lo.z += c;
        two_sum(hi.w, v.w, hi.w, c);
        lo.w += c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float c;
        float h2 = __shfl_down_sync(0xffffffffu, hi.x, o), l2 = __shfl_down_sync(0xffffffffu, lo.x, o);
        two_sum(hi.x, h2, hi.x, c);
        lo.x += l2 + c;
        h2 = __shfl_down_sync(0xffffffffu, hi.y, o);
        l2 = __shfl_down_sync(0xffffffffu, lo.y, o);
        two_sum(hi.y, h2, hi.y, c);
        lo.y += l2 + c;
        h2 = __shfl_down_sync(0xffffffffu, hi.z, o);
        l2 = __shfl_down_sync(0xffffffffu, lo.z, o);
        two_sum(hi.z, h2, hi.z, c);
        lo.z += l2 + c;
        h2 = __shfl_down_sync(0xffffffffu, hi.w, o);
        l2 = __shfl_down_sync(0xffffffffu, lo.w, o);
        two_sum(hi.w, h2, hi.w, c);
        lo.w += l2 + c;
    }
    return make_float4(hi.x + lo.x, hi.y + lo.y, hi.z + lo.z, hi.w + lo.w);
}

// Blocks of the single-reduction kernel: a GB300 has 152 SMs (the four partials of each block
// are staged in static shared memory, which shares the per-block budget with the rectangle).
constexpr int kMaxBlocks1 = 160;

}  // namespace res

// Control word broadcast by lane 0 of warp 0 after each grid-wide total.
enum : int { kResGo = 0, kResReliable = 1, kResStop = 2 };

// The scalar recurrence of a block, kept in shared memory and used by thread 0 only (so that
// it occupies no registers in the other threads), in FP32: the inner iteration's scalars are
// FP32, and the FP64 state is written back at exit.
struct ResScalars {
    float rsq, rmax, rn, beta, scale, delta, stop;
    int k, max_iter, status, reliable, iters;
};

// Where x_lo of the thread's sites lives for the launch (XM):
//   kXGlobal: every update goes to global memory as a vector reduction (fire-and-forget, no
//             register and no round trip; each site has one writer, so the additions happen in
//             program order);
//   kXReg:    in registers;
//   kXTmem:   in tensor memory, two columns per row of the thread (loaded, updated and stored
//             back once per iteration), so that it takes neither registers across the stencils
//             nor the load/store pipe;
//   kXTmemL:  as kXTmem, and the links of the thread's sites are in tensor memory as well
//             (hop_rows_tm), so that the stencils read only the field from shared memory.
//             Columns (per sub-partition lane): (h_x, h_y) of the rows at 0 .. 255 (4 NY per
//             warp), h_x of the left neighbours at 256 .. 383 (2 NY per warp), x_lo at 384 ..
//             511 (2 NY per warp); 512 in all.
enum : int { kXGlobal = 0, kXReg = 1, kXTmem = 2, kXTmemL = 3 };

// Tensor-memory columns of a block with WY warps along y and NY rows per thread (the WY warps
// of one sub-partition take 2 NY columns each): a power of two, at least 32.
__host__ __device__ constexpr unsigned res_tmem_cols(int NY, int WY)
{
    return 2 * NY * WY <= 32 ? 32u : (2 * NY * WY <= 64 ? 64u : (2 * NY * WY <= 128 ? 128u : (2 * NY * WY <= 256 ? 256u : 512u)));
}

template <int NY, int WY, int XM>
__global__ void __launch_bounds__(32 * res::kWX * WY, 1)
k_resident(const float2 *__restrict__ H, float2 *r, float2 *p0, float2 *xlo, float mass, float sigma, int lx, int ly,
           MxDev *s, res::PhaseFlags *pf, unsigned long long *mbox, int ty, int gx)
{
    using namespace res;
    constexpr int NW = kWX * WY, NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float sm_w[32];
    __shared__ float sm_scalar;
    __shared__ int sm_ctl, sm_err;
    __shared__ ResScalars sc;
    __shared__ float2 sm_hl[kMaxBlocks / 32];
    __shared__ unsigned sm_taddr;
    constexpr bool XREG = XM == kXReg, XTM = XM == kXTmem || XM == kXTmemL, LTM = XM == kXTmemL;
    constexpr unsigned kTmemCols = LTM ? 512u : res_tmem_cols(NY, WY);
    static_assert(!LTM || (4 * NY * WY <= 256 && 2 * NY * WY <= 128), "tensor-memory layout");
    // one read of the solve state per block, so that a block never splits here: block 0 of a
    // launch whose waits ran out may set s->done while other blocks are still starting
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
    const int tyb = min(ty, ly - y0);  // rows of this rectangle
    const int nrow = min(NY, tyb - yb);  // rows of this thread (<= 0: none)
    const int nring = 2 * kTX + 2 * tyb;
    const int nslot = mbox_slots(ty);
    // the blocks owning the ring: left, right, below, above (periodic)
    const int nb_l = by * gx + (bx + gx - 1) % gx, nb_r = by * gx + (bx + 1) % gx;
    const int nb_d = ((by + gy - 1) % gy) * gx + bx, nb_u = ((by + 1) % gy) * gx + bx;
    unsigned long long *const Mr = mbox, *const Mt = mbox + 2 * (size_t)nb * nslot;
    Rect R;
    R.HX = reinterpret_cast<float2 *>(smraw);
    R.HY = R.HX + (size_t)ty * kTX;
    R.F = R.HY + (size_t)ty * kTX;
    R.T = R.F + (ty + 2) * kPW;
    R.HxL = R.T + (ty + 2) * kPW;
    R.HyB = R.HxL + ty;
    float2 *const Rr = R.F;
    const bool has_ring = tid < nring;
    int rslot = 0, rgi = 0, rsrc = 0;
    if (has_ring) {
        ring_site(tid, tyb, x0, y0, lx, ly, rslot, rgi);
        rsrc = ring_source(tid, ty, tyb, nslot, nb_l, nb_r, nb_d, nb_u);
    }
    // this block's mailboxes (border sites are posted by the threads that compute them)
    unsigned long long *const mbR = Mr + 2 * (size_t)blockIdx.x * nslot;
    unsigned long long *const mbT = Mt + 2 * (size_t)blockIdx.x * nslot;
    const int grow = (y0 + yb) * lx + x0 + xl;      // lattice index of the thread's first row
    const int qtop = tyb - 1 - yb;                  // the thread's row that is the rectangle's last
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

    // ---- entry: r, links and the direction p of the rectangle on chip (p in registers and,
    // for one stencil, in T with its ring); t_old = D p into T
    if (XTM) {
        if (warp == 0) tmem_alloc(&sm_taddr, kTmemCols);
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
    }
    // the thread's first x_lo column: its sub-partition's lanes, its warp's 2 NY columns
    const unsigned tlane = XTM ? sm_taddr + ((unsigned)(32 * (warp % 4)) << 16) : 0u;
    const unsigned xcol = tlane + (LTM ? 384u : 0u) + (unsigned)(2 * NY * (warp / 4));
    // the links of the thread's rows: (h_x, h_y), and h_x of the left neighbour
    const unsigned tA = tlane + (unsigned)(4 * NY * (warp / 4));
    const unsigned tB = tlane + 256u + (unsigned)(2 * NY * (warp / 4));
    float2 pv[NY], tmp[NY], xv[XREG ? NY : 1];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int yl = yb + q;
        pv[q] = make_float2(0.f, 0.f);
        if (XREG) xv[q] = make_float2(0.f, 0.f);
        if (q < nrow) {
            const int gi = grow + q * lx;
            Rr[(yl + 1) * kPW + xl + 1] = __ldcg(r + gi);
            pv[q] = __ldcg(p0 + gi);
            if (XREG) xv[q] = __ldcg(xlo + gi);
            if (XTM) tmp[q] = __ldcg(xlo + gi);
            R.T[(yl + 1) * kPW + xl + 1] = pv[q];
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
    if (XTM) {
#pragma unroll
        for (int q = 0; q < NY; q++) tmem_st2(xcol + 2 * q, q < nrow ? tmp[q] : make_float2(0.f, 0.f));
    }
    if (has_ring) {
        Rr[rslot] = __ldcg(r + rgi);
        R.T[rslot] = __ldcg(p0 + rgi);
    }
    __syncthreads();
    if (LTM) {  // the links of the thread's rows into tensor memory (zeros past the rectangle)
#pragma unroll
        for (int q = 0; q < NY; q++) {
            const int yl = yb + q;
            const bool in = q < nrow;
            const float2 hx = in ? R.HX[yl * kTX + xl] : make_float2(0.f, 0.f);
            const float2 hy = in ? R.HY[yl * kTX + xl] : make_float2(0.f, 0.f);
            const float2 hxm = in ? (xl ? R.HX[yl * kTX + xl - 1] : R.HxL[yl]) : make_float2(0.f, 0.f);
            tmem_st4(tA + 4 * q, make_float4(hx.x, hx.y, hy.x, hy.y));
            tmem_st2(tB + 2 * q, hxm);
        }
        tmem_wait_st();
    }
    {
        auto body = [&](int q, int, float2 cur, float2 hs) { tmp[q] = fadd(fscale(mass, cur), hs); };
        if (nrow == NY) hop_rows<NY, true>(R.T, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        else if (nrow > 0) hop_rows<NY, false>(R.T, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NY; q++)
        if (q < nrow) R.T[(yb + q + 1) * kPW + xl + 1] = tmp[q];

    unsigned ep = pf->epoch;  // epoch of the last phase published (every launch continues it)
    float fb = (float)s->beta;
    bool first = true;
    for (;;) {
        // ---- A: u = D r (needs only the ring of r), then beta from the previous phase's total;
        // t = u + beta t_old (= D p'), p' = r + beta p
        {
            auto body = [&](int q, int, float2 cur, float2 hs) { tmp[q] = fadd(fscale(mass, cur), hs); };
            if (LTM) {
                if (nrow > 0) {  // (yb < tyb: the row below the first is in range)
                    const float2 hyp0 = yb == 0 ? R.HyB[xl] : R.HY[(yb - 1) * kTX + xl];
                    if (nrow == NY) hop_rows_tm<NY, true>(Rr, tA, tB, hyp0, xl, yb, nrow, body);
                    else hop_rows_tm<NY, false>(Rr, tA, tB, hyp0, xl, yb, nrow, body);
                }
            } else {
                if (nrow == NY) hop_rows<NY, true>(Rr, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
                else if (nrow > 0) hop_rows<NY, false>(Rr, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
            }
        }
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
                    const float rho = sqrtf(tot) * sc.scale;  // true-scale iterated residual
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
            const int c0 = (yb + 1) * kPW + xl + 1;
            float2 vb = make_float2(0.f, 0.f), vt = vb;
            if (nrow == NY) acc = pass_A<NY, true>(R.T + c0, Rr + c0, tmp, pv, fb, sigma, nrow, qtop, vb, vt);
            else acc = pass_A<NY, false>(R.T + c0, Rr + c0, tmp, pv, fb, sigma, nrow, qtop, vb, vt);
            post_border_rows(mbT, eA, xl, yb, nrow, qtop, tyb, vb, vt);
        }
        post_columns(mbT, eA, R.T, warp % kWX, yb, nrow, ty);
        publish_sum<NW>(acc, pf, eA, sm_w);
        if (has_ring) R.T[rslot] = poll_slot(Mt + rsrc, eA, pf, &sm_err, lim);
        __syncthreads();
        // ---- B: Ap = D^dagger t + sigma p' (needs only the ring of t), then alpha from the
        // total of A; x_lo += alpha p', r -= alpha Ap
        {
            auto body = [&](int q, int, float2 cur, float2 hs) {
                tmp[q] = fadd(fsub(fscale(mass, cur), hs), fscale(sigma, pv[q]));
            };
            if (LTM) {
                if (nrow > 0) {  // (yb < tyb: the row below the first is in range)
                    const float2 hyp0 = yb == 0 ? R.HyB[xl] : R.HY[(yb - 1) * kTX + xl];
                    if (nrow == NY) hop_rows_tm<NY, true>(R.T, tA, tB, hyp0, xl, yb, nrow, body);
                    else hop_rows_tm<NY, false>(R.T, tA, tB, hyp0, xl, yb, nrow, body);
                }
            } else {
                if (nrow == NY) hop_rows<NY, true>(R.T, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
                else if (nrow > 0) hop_rows<NY, false>(R.T, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
            }
        }
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
        acc = 0.f;
        if (XTM) {
            float2 xt[NY];
            tmem_wait_st();
#pragma unroll
            for (int q = 0; q < NY; q++) tmem_ld2(xcol + 2 * q, xt[q]);
            tmem_wait_ld(xt);
#pragma unroll
            for (int q = 0; q < NY; q++) tmem_st2(xcol + 2 * q, fadd(xt[q], fscale(alpha, pv[q])));
        }
        {
            const int c0 = (yb + 1) * kPW + xl + 1;
            float2 vb = make_float2(0.f, 0.f), vt = vb;
            if (nrow == NY)
                acc = pass_B<NY, true, XREG, !XREG && !XTM>(Rr + c0, tmp, pv, xv, xlo + grow, lx, alpha, nrow, qtop,
                                                           vb, vt);
            else
                acc = pass_B<NY, false, XREG, !XREG && !XTM>(Rr + c0, tmp, pv, xv, xlo + grow, lx, alpha, nrow, qtop,
                                                            vb, vt);
            post_border_rows(mbR, eB, xl, yb, nrow, qtop, tyb, vb, vt);
        }
        post_columns(mbR, eB, Rr, warp % kWX, yb, nrow, ty);
        publish_sum<NW>(acc, pf, eB, sm_w);
        if (has_ring) Rr[rslot] = poll_slot(Mr + rsrc, eB, pf, &sm_err, lim);
        __syncthreads();
    }
    // ---- exit: the rectangle's r, x_lo and direction back to global memory (direction in p0)
    if (XTM) {  // x_lo out of tensor memory (into tmp), then the columns are freed
        tmem_wait_st();
#pragma unroll
        for (int q = 0; q < NY; q++) tmem_ld2(xcol + 2 * q, tmp[q]);
        tmem_wait_ld(tmp);
    }
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (q < nrow) {
            const int gi = grow + q * lx;
            r[gi] = Rr[(yb + q + 1) * kPW + xl + 1];
            p0[gi] = pv[q];
            if (XREG) xlo[gi] = xv[q];
            if (XTM) xlo[gi] = tmp[q];
        }
    }
    if (XTM) {
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
        if (warp == 0) tmem_dealloc(sm_taddr, kTmemCols);
    }
    if (blockIdx.x == 0 && tid == 0) {
        pf->epoch = ep;  // every block ran the same phases
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

// ---------------------------------------------------------------- single-reduction form
//
// k_resident1 runs the same CG on A = D^dagger D + sigma with one grid-wide sum per iteration
// instead of two.  Iteration k, from r_k, the previous direction p and s = A p:
//   A: u = D r_k (ring of r); partials gamma = |r_k|^2, delta = <r_k, A r_k> = |u|^2 + sigma
//      |r_k|^2, rho = Re <r_k, s>, pi = Re <p, s>; export the border of u.
//   B: w = A r_k = D^dagger u + sigma r_k (ring of u); then the four totals: beta =
//      gamma / gamma_old, <p', A p'> = delta + 2 beta rho + beta^2 pi for p' = r_k + beta p
//      (an identity of the Hermitian A, with no orthogonality assumed), alpha = gamma / <p', A p'>;
//      p' = r_k + beta p, s' = w + beta s, x_lo += alpha p', r -= alpha s'; export the border of r.
// The stopping tests run on gamma where the two-sum kernel runs them (after the residual's
// total, before the direction is updated), so the state at exit is the same: r, the previous
// direction, x_lo, and beta / rsq as that kernel leaves them.  On entry s = A p is formed from
// the direction p with two stencils (the ring of D p computed from global memory).
//
// Measured at 1024^2 (m = 0.01, 2100 inner iterations): 10.9 us per iteration with 16 warps
// against 8.5 us for k_resident.  The third per-site vector (s) takes the 16-warp kernel to
// its 128-register limit (with spills, whose reloads go to L2 here, since shared memory leaves
// 28 KB of L1), and the 32-warp kernel spills more; the saved grid-wide sum does not make up for
// it.  The autotuner keeps both as candidates.
//
// Exchange: u and r borders go through the two mailboxes as in k_resident; a slot is rewritten
// one iteration later, and a block gets there only after the neighbour that reads the slot has
// posted its next border, which it does after reading the slot.  The partial words alternate
// by iteration between two arrays; a block rewrites an array only after the next iteration's
// sum, which every block joins only after it has read the array.

template <int NY, int WY>
__global__ void __launch_bounds__(32 * res::kWX * WY, 1)
k_resident1(const float2 *__restrict__ H, float2 *r, float2 *p0, float2 *xlo, float mass, float sigma, int lx, int ly,
            MxDev *s, res::PhaseFlags *pf, unsigned long long *mbox, int ty, int gx)
{
    using namespace res;
    constexpr int NW = kWX * WY, NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float4 sm_w4[32];
    __shared__ float sm_alpha, sm_beta;
    __shared__ int sm_ctl, sm_err;
    __shared__ ResScalars sc;
    __shared__ float4 sm_part4[kMaxBlocks1];
    // one read of the solve state per block, so that a block never splits here: block 0 of a
    // launch whose waits ran out may set s->done while other blocks are still starting
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
    unsigned long long *const Mr = mbox, *const Mu = mbox + 2 * (size_t)nb * nslot;
    Rect R;
    R.HX = reinterpret_cast<float2 *>(smraw);
    R.HY = R.HX + (size_t)ty * kTX;
    R.F = R.HY + (size_t)ty * kTX;
    R.T = R.F + (ty + 2) * kPW;
    R.HxL = R.T + (ty + 2) * kPW;
    R.HyB = R.HxL + ty;
    float2 *const Rr = R.F, *const Ru = R.T;
    const bool has_ring = tid < nring;
    int rslot = 0, rgi = 0, rsrc = 0;
    if (has_ring) {
        ring_site(tid, tyb, x0, y0, lx, ly, rslot, rgi);
        rsrc = ring_source(tid, ty, tyb, nslot, nb_l, nb_r, nb_d, nb_u);
    }
    const int nborder = nring;
    int bpos = 0, bslot = 0;
    if (tid < nborder) {
        border_slot(tid, ty, tyb, bpos, bslot);
        bslot += (int)blockIdx.x * nslot;
    }
    const int grow = (y0 + yb) * lx + x0 + xl;
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

    // ---- entry: r, links and the direction p on chip; s = A p (D p into the u buffer with its
    // ring, then D^dagger of it)
    float2 pv[NY], sv[NY], tmp[NY];
#pragma unroll
    for (int q = 0; q < NY; q++) {
        const int yl = yb + q;
        pv[q] = make_float2(0.f, 0.f);
        sv[q] = make_float2(0.f, 0.f);
        if (q < nrow) {
            const int gi = grow + q * lx;
            Rr[(yl + 1) * kPW + xl + 1] = __ldcg(r + gi);
            pv[q] = __ldcg(p0 + gi);
            Ru[(yl + 1) * kPW + xl + 1] = pv[q];
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
    float2 dp_ring = make_float2(0.f, 0.f);
    if (has_ring) {
        Rr[rslot] = __ldcg(r + rgi);
        Ru[rslot] = __ldcg(p0 + rgi);
        // D p at the ring site, from global memory
        const int gyy = rgi / lx, gxx = rgi - gyy * lx;
        const int xp = gxx + 1 == lx ? 0 : gxx + 1, xm = gxx == 0 ? lx - 1 : gxx - 1;
        const int yp = gyy + 1 == ly ? 0 : gyy + 1, ym = gyy == 0 ? ly - 1 : gyy - 1;
        const float2 pc = __ldcg(p0 + rgi);
        float2 hs = fmul(__ldg(H + 2 * rgi), __ldcg(p0 + gyy * lx + xp));
        hs = fsub(hs, fmulc(__ldg(H + 2 * (gyy * lx + xm)), __ldcg(p0 + gyy * lx + xm)));
        hs = fadd(hs, fmul(__ldg(H + 2 * rgi + 1), __ldcg(p0 + yp * lx + gxx)));
        hs = fsub(hs, fmulc(__ldg(H + 2 * (ym * lx + gxx) + 1), __ldcg(p0 + ym * lx + gxx)));
        dp_ring = fadd(fscale(mass, pc), hs);
    }
    __syncthreads();
    {
        auto body = [&](int q, int, float2 cur, float2 hs) { tmp[q] = fadd(fscale(mass, cur), hs); };
        if (nrow == NY) hop_rows<NY, true>(Ru, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        else if (nrow > 0) hop_rows<NY, false>(Ru, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NY; q++)
        if (q < nrow) Ru[(yb + q + 1) * kPW + xl + 1] = tmp[q];
    if (has_ring) Ru[rslot] = dp_ring;
    __syncthreads();
    {
        auto body = [&](int q, int, float2 cur, float2 hs) {
            sv[q] = fadd(fsub(fscale(mass, cur), hs), fscale(sigma, pv[q]));
        };
        if (nrow == NY) hop_rows<NY, true>(Ru, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        else if (nrow > 0) hop_rows<NY, false>(Ru, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
    }
    __syncthreads();

    unsigned ep = pf->epoch;
    bool first = true;
    for (;;) {
        // ---- A: u = D r and the four partials; export the border of u
        {
            auto body = [&](int q, int, float2 cur, float2 hs) { tmp[q] = fadd(fscale(mass, cur), hs); };
            if (nrow == NY) hop_rows<NY, true>(Rr, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
            else if (nrow > 0) hop_rows<NY, false>(Rr, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        }
        const unsigned eA = ++ep;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int q = 0; q < NY; q++) {
            if (q < nrow) {
                const int c = (yb + q + 1) * kPW + xl + 1;
                const float2 rv = Rr[c];
                const float r2 = fn2(rv);
                acc.x += r2;
                acc.y += fn2(tmp[q]) + sigma * r2;
                acc.z += rv.x * sv[q].x + rv.y * sv[q].y;
                acc.w += pv[q].x * sv[q].x + pv[q].y * sv[q].y;
                Ru[c] = tmp[q];
            }
        }
        publish4<NW>(acc, pf, eA, sm_w4, Ru, Mu, nborder, bpos, bslot);
        if (has_ring) Ru[rslot] = poll_slot(Mu + rsrc, eA, pf, &sm_err, lim);
        __syncthreads();
        // ---- B: w = D^dagger u + sigma r, then the totals, the scalars and the updates
        {
            auto body = [&](int q, int yl, float2 cur, float2 hs) {
                tmp[q] = fadd(fsub(fscale(mass, cur), hs), fscale(sigma, Rr[(yl + 1) * kPW + xl + 1]));
            };
            if (nrow == NY) hop_rows<NY, true>(Ru, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
            else if (nrow > 0) hop_rows<NY, false>(Ru, R.HX, R.HY, R.HxL, R.HyB, xl, yb, nrow, body);
        }
        if (tid < (int)nb) poll_partial4(pf, eA, tid, sm_part4, &sm_err, lim);
        __syncthreads();
        if (warp == 0) {
            const float4 tot = sum_partials4(sm_part4, nb);
            const float g = tot.x, d = tot.y, rh = tot.z, pi = tot.w;
            if (lane == 0) {
                int ctl = kResGo;
                if (sm_err) {
                    sc.status = GLINALG_SOLVE_TIMEOUT;
                    ctl = kResStop;
                } else if (!isfinite(g)) {
                    sc.status = GLINALG_SOLVE_NONFINITE;
                    ctl = kResStop;
                } else if (!first) {
                    sc.rn = g;
                    sc.k++;
                    sc.iters++;
                    const float rho = sqrtf(g) * sc.scale;  // true-scale iterated residual
                    if (rho > sc.rmax) sc.rmax = rho;
                    if (rho < sc.delta * sc.rmax || rho < sc.stop || sc.k >= sc.max_iter) {
                        sc.reliable = 1;
                        ctl = kResReliable;
                    }
                }
                if (ctl == kResGo) {
                    const float beta = first ? sc.beta : g / sc.rsq;
                    const float pap = d + 2.f * beta * rh + beta * beta * pi;  // <p', A p'>
                    if (!(pap > 0.f) || !isfinite(pap)) {
                        sc.status = pap == 0.f ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
                        ctl = kResStop;
                    } else {
                        sc.beta = beta;
                        sc.rsq = g;
                        sm_beta = beta;
                        sm_alpha = g / pap;
                    }
                }
                sm_ctl = ctl;
            }
        }
        __syncthreads();
        if (sm_ctl != kResGo) break;
        first = false;
        const float alpha = sm_alpha, beta = sm_beta;
        const unsigned eB = ++ep;
#pragma unroll
        for (int q = 0; q < NY; q++) {
            if (q < nrow) {
                const int c = (yb + q + 1) * kPW + xl + 1;
                const float2 rv = Rr[c];
                const float2 pn = fadd(rv, fscale(beta, pv[q]));
                const float2 sn = fadd(tmp[q], fscale(beta, sv[q]));
                pv[q] = pn;
                sv[q] = sn;
                red_add2(xlo + grow + q * lx, fscale(alpha, pn));
                Rr[c] = fsub(rv, fscale(alpha, sn));
            }
        }
        __syncthreads();
        publish_border(eB, Rr, Mr, nborder, bpos, bslot);
        if (has_ring) Rr[rslot] = poll_slot(Mr + rsrc, eB, pf, &sm_err, lim);
        __syncthreads();
    }
    // ---- exit: r, the direction (to p0) back to global memory; x_lo is already there
#pragma unroll
    for (int q = 0; q < NY; q++) {
        if (q < nrow) {
            const int gi = grow + q * lx;
            r[gi] = Rr[(yb + q + 1) * kPW + xl + 1];
            p0[gi] = pv[q];
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
