// cg64_fused.cu -- the FP64 CG on the staggered normal operator D^dagger D as one persistent
// cooperative kernel: the whole solve is a single launch, each iteration two fused passes over
// the lattice separated by grid-wide sums.
//
// The recurrence is the reference's CG (generic_cg.cpp:278-382) on A = D^dagger D, with two
// exact rewritings that let each pass need the neighbours of only one field that the previous
// pass finished:
//   - <p, A p> = |D p|^2 (A = D^dagger D), so alpha = |r|^2 / |t|^2 with t = D p;
//   - t = D p' for p' = r + beta p is formed as D r + beta t_old (D is linear), so the stencil
//     of the first pass reads r, not the direction that pass is writing.
// Iteration k:
//   A: u = D r; t = u + beta t; p = r + beta p; partial |t|^2        -> grid sum -> alpha
//   B: Ap = D^dagger t; x += alpha p; r -= alpha Ap; partial |r|^2   -> grid sum -> beta, stop
// with beta = 0 on the first pass (t = D r, p = r).  It stops as the reference does: on the
// iterated residual, sqrt|r|^2 < eps |b|, or after max_iter iterations.
//
// Arithmetic: GB300 runs FP64 at 1/64 of the FP32 rate, and at 1024^2 every field of the
// iteration fits in L2, so the FP64 pipe bounds this kernel, not HBM.  The per-site work is
// kept to fused multiply-adds: the 1/2 and the staggered phase eta(x) are folded into a FP64
// hopping table (H[2i] = 1/2 U_x(i), H[2i+1] = 1/2 eta(x) U_y(i), built once per solve), the
// four link products accumulate into one complex sum (16 DFMA), and alpha and beta are real.
// About 48 FP64 instructions per site and iteration (A: 18 stencil + 2 + 2 + 2; B: 18 + 2 +
// 2 + 2).
//
// Layout: a warp owns a tile of 32 columns by NY rows; its lanes hold their column for rows
// -1 .. NY in registers (y-neighbours), x-neighbours come by warp shuffle with lanes 0 and 31
// loading across the tile edge.  Tiles are dealt to warps in order; lx must be a multiple of
// 32, ly is any size (rows past ly are neither stored nor summed).
//
// Grid-wide sums: every block writes its partial, passes a generation barrier (bounded wait,
// MxDev-style limit), and sums all partials in block order, so every block holds the same
// totals and takes the same branch.

#include "mixed_state.cuh"
#include "solver_util.h"
#include "solvers.h"

#include <cmath>
#include <cstdlib>
#include <vector>

namespace glinalg {
namespace {

constexpr int kC64Warps = 8;   // warps per block
constexpr int kC64NY = 2;      // rows per warp tile

struct C64Dev {
    double bsq, rsq, eps;
    int max_iter;
    int iters, status, done;  // results
    double rsq_last;
    long long wait_ns;        // bound on the grid-barrier waits (0: default, < 0: none)
    double *hist;             // |r| / |b| per iteration (verbosity), hist_cap entries
    int hist_cap;
};

__global__ void k_make_hop64(double2 *__restrict__ H, const double2 *__restrict__ U, int lx, int ly)
{
    const long n = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % lx);
        const double ey = (x & 1) ? -0.5 : 0.5;
        const double2 ux = U[2 * i], uy = U[2 * i + 1];
        H[2 * i] = make_double2(0.5 * ux.x, 0.5 * ux.y);
        H[2 * i + 1] = make_double2(ey * uy.x, ey * uy.y);
    }
}

__device__ __forceinline__ double2 shfl_down_d2(double2 v)
{
    return make_double2(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
}
__device__ __forceinline__ double2 shfl_up_d2(double2 v)
{
    return make_double2(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
}

// acc += a * b and acc -= conj(a) * b, as fused multiply-adds.
__device__ __forceinline__ void fma_mul(double2 &acc, double2 a, double2 b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void fms_mulc(double2 &acc, double2 a, double2 b)
{
    acc.x = fma(-a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(-a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// Hopping sums of one warp tile: calls body(q, i, f(x,y), hs) for rows q < nrow with
//   hs = H_x f(x+1) - H_x(x-1)^* f(x-1) + H_y f(y+1) - H_y(y-1)^* f(y-1)
// so that D f = m f - hs and D^dagger f = m f + hs.
template <class Body>
__device__ __forceinline__ void tile_hops(const double2 *__restrict__ F, const double2 *__restrict__ H, int lx,
                                          int ly, int x0, int y0, int nrow, Body body)
{
    const int lane = threadIdx.x;
    const int x = x0 + lane;
    const int xl = x == 0 ? lx - 1 : x - 1, xr = x + 1 == lx ? 0 : x + 1;
    double2 col[kC64NY + 2], hyc[kC64NY + 1];
#pragma unroll
    for (int j = 0; j < kC64NY + 2; j++) {
        int y = y0 - 1 + j;
        y = y < 0 ? y + ly : (y >= ly ? y - ly : y);
        col[j] = __ldcg(F + (long)y * lx + x);
        if (j < kC64NY + 1) hyc[j] = __ldg(H + 2 * ((long)y * lx + x) + 1);
    }
#pragma unroll
    for (int q = 0; q < kC64NY; q++) {
        if (q >= nrow) break;
        const long row = (long)(y0 + q) * lx;
        const long i = row + x;
        const double2 c = col[q + 1];
        double2 fr = shfl_down_d2(c), fl = shfl_up_d2(c);
        const double2 hx = __ldg(H + 2 * i);
        double2 hxm = shfl_up_d2(hx);
        if (lane == 31) fr = __ldcg(F + row + xr);
        if (lane == 0) {
            fl = __ldcg(F + row + xl);
            hxm = __ldg(H + 2 * (row + xl));
        }
        double2 hs = make_double2(0.0, 0.0);
        fma_mul(hs, hx, fr);
        fms_mulc(hs, hxm, fl);
        fma_mul(hs, hyc[q + 1], col[q + 2]);
        fms_mulc(hs, hyc[q], col[q]);
        body(q, i, c, hs);
    }
}

// Block partial of one double per thread, written to part[blockIdx.x].
__device__ __forceinline__ void block_partial64(double v, double *part, double *sm)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) sm[threadIdx.y] = v;
    __syncthreads();
    if (threadIdx.y == 0) {
        double w = threadIdx.x < blockDim.y ? sm[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
        if (threadIdx.x == 0) part[blockIdx.x] = w;
    }
}

__global__ void __launch_bounds__(32 * kC64Warps, 2)
k_cg64(const double2 *__restrict__ H, double2 *r, double2 *t, double2 *p, double2 *x, double mass, int lx,
       int ly, C64Dev *s, GridSync *gs, double *partA, double *partB)
{
    __shared__ double sm[33];
    const unsigned nb = gridDim.x;
    const int ntx = lx / 32, nty = (ly + kC64NY - 1) / kC64NY, ntiles = ntx * nty;
    const int gw = blockIdx.x * kC64Warps + threadIdx.y, nw = nb * kC64Warps;
    const long long lim = s->wait_ns > 0 ? s->wait_ns : (s->wait_ns == 0 ? kBarrierTimeoutNs : 0LL);
    const double bsqrt = sqrt(s->bsq), eps = s->eps;
    const int max_iter = s->max_iter;
    double rsq = s->rsq, beta = 0.0, rn = rsq;
    int k = 0, status = -1;
    for (;;) {
        // ---- A: t = D r + beta t ; p = r + beta p ; |t|^2
        double acc = 0.0;
        for (int tile = gw; tile < ntiles; tile += nw) {
            const int x0 = (tile % ntx) * 32, y0 = (tile / ntx) * kC64NY;
            tile_hops(r, H, lx, ly, x0, y0, min(kC64NY, ly - y0), [&](int, long i, double2 c, double2 hs) {
                const double2 to = t[i], po = p[i];
                double2 tn, pn;
                tn.x = fma(beta, to.x, fma(mass, c.x, -hs.x));
                tn.y = fma(beta, to.y, fma(mass, c.y, -hs.y));
                pn.x = fma(beta, po.x, c.x);
                pn.y = fma(beta, po.y, c.y);
                t[i] = tn;
                p[i] = pn;
                acc = fma(tn.x, tn.x, fma(tn.y, tn.y, acc));
            });
        }
        block_partial64(acc, partA, sm);
        if (!grid_sync(gs, nb, lim)) { status = GLINALG_SOLVE_TIMEOUT; break; }
        const double pAp = grid_total(partA, nb, sm);
        if (!(pAp > 0.0) || !isfinite(pAp)) {
            status = pAp == 0.0 ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
            break;
        }
        const double alpha = rsq / pAp;
        // ---- B: Ap = D^dagger t ; x += alpha p ; r -= alpha Ap ; |r|^2
        acc = 0.0;
        for (int tile = gw; tile < ntiles; tile += nw) {
            const int x0 = (tile % ntx) * 32, y0 = (tile / ntx) * kC64NY;
            tile_hops(t, H, lx, ly, x0, y0, min(kC64NY, ly - y0), [&](int, long i, double2 c, double2 hs) {
                const double2 ap = make_double2(fma(mass, c.x, hs.x), fma(mass, c.y, hs.y));
                const double2 pi = p[i], xi = x[i], ri = r[i];
                x[i] = make_double2(fma(alpha, pi.x, xi.x), fma(alpha, pi.y, xi.y));
                const double2 rr = make_double2(fma(-alpha, ap.x, ri.x), fma(-alpha, ap.y, ri.y));
                r[i] = rr;
                acc = fma(rr.x, rr.x, fma(rr.y, rr.y, acc));
            });
        }
        block_partial64(acc, partB, sm);
        if (!grid_sync(gs, nb, lim)) { status = GLINALG_SOLVE_TIMEOUT; break; }
        rn = grid_total(partB, nb, sm);
        if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0 && k < s->hist_cap)
            s->hist[k] = sqrt(rn) / bsqrt;
        const bool last = k == max_iter - 1;
        k++;
        if (!isfinite(rn)) { status = GLINALG_SOLVE_NONFINITE; break; }
        if (sqrt(rn) < eps * bsqrt || last) {
            status = last ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED;
            break;
        }
        beta = rn / rsq;
        rsq = rn;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
        s->iters = k;
        s->status = status;
        s->rsq_last = rn;
        s->done = 1;
    }
}

// One FP64 staggered pass out = D in (sign +1) or D^dagger in (sign -1), register-tiled like
// the fused CG's passes (16 FMAs per site with the hopping table).  done: optional device flag;
// when it is set the kernel writes nothing (used inside solver loops).
__global__ void __launch_bounds__(32 * kC64Warps)
k_stag64(double2 *__restrict__ out, const double2 *__restrict__ in, const double2 *__restrict__ H, double mass,
         int lx, int ly, double sign, const int *done)
{
    if (done && *done) return;
    const int ntx = lx / 32, nty = (ly + kC64NY - 1) / kC64NY, ntiles = ntx * nty;
    const int gw = blockIdx.x * kC64Warps + threadIdx.y, nw = gridDim.x * kC64Warps;
    for (int tile = gw; tile < ntiles; tile += nw) {
        const int x0 = (tile % ntx) * 32, y0 = (tile / ntx) * kC64NY;
        tile_hops(in, H, lx, ly, x0, y0, min(kC64NY, ly - y0), [&](int, long i, double2 c, double2 hs) {
            out[i] = make_double2(fma(mass, c.x, -sign * hs.x), fma(mass, c.y, -sign * hs.y));
        });
    }
}

int vgrid64(long n)
{
    long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

int cg64_grid()
{
    static int grid = [] {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg64, 32 * kC64Warps, 0) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return per_sm * sm_count();
    }();
    return grid;
}

}  // namespace

glinalg_status launch_make_hop64(double2 *H, const glinalg_operator_s *op, cudaStream_t st)
{
    k_make_hop64<<<vgrid64(op->vol), 256, 0, st>>>(H, op->U, op->lx, op->ly);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_stag64(double2 *out, const double2 *in, const double2 *H, const glinalg_operator_s *op,
                             double sign, const int *done, cudaStream_t st)
{
    const int ntiles = (op->lx / 32) * ((op->ly + kC64NY - 1) / kC64NY);
    const int grid = (ntiles + kC64Warps - 1) / kC64Warps;
    k_stag64<<<grid, dim3(32, kC64Warps), 0, st>>>(out, in, H, op->mass, op->lx, op->ly, sign, done);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

bool cg64_fused_applies(const glinalg_operator_s *op, double sigma)
{
    static const bool on = [] {
        const char *e = std::getenv("GLINALG_FP64_FUSED");
        return !(e && e[0] == '0');
    }();
    return on && op->kind == GLINALG_OP_STAGGERED_NORMAL && sigma == 0.0 && op->lx % 32 == 0 && op->ly >= 2 &&
           cg64_grid() > 0;
}

glinalg_status cg64_fused(const glinalg_operator_s *op, double2 *x, const double2 *b, int max_iter, double eps,
                          const Verb &verb, glinalg_info *info, cudaStream_t st, int wait_limit_us)
{
    const long n = op->size;
    const int grid = cg64_grid();
    Scratch sc(st);
    double2 *H, *r, *t, *p, *tmp;
    double *partA, *partB, *partials, *hist, *truersq;
    C64Dev *s;
    GridSync *gs;
    const int hist_cap = verb.level == 3 ? (max_iter > 0 ? max_iter : 1) : 0;
    const int nbr = reduction_blocks(n);
    GL_TRY(sc.alloc(&H, 2 * (size_t)n));
    GL_TRY(sc.alloc(&r, n));
    GL_TRY(sc.zeros(&t, n));
    GL_TRY(sc.zeros(&p, n));
    GL_TRY(sc.alloc(&tmp, n));
    GL_TRY(sc.alloc(&partA, grid));
    GL_TRY(sc.alloc(&partB, grid));
    GL_TRY(sc.alloc(&partials, 2 * (size_t)nbr));
    GL_TRY(sc.alloc(&hist, hist_cap ? hist_cap : 1));
    GL_TRY(sc.alloc(&truersq, 1));
    GL_TRY(sc.zeros(&s, 1));
    GL_TRY(sc.zeros(&gs, 1));
    unsigned *cnt;
    GL_TRY(sc.zeros(&cnt, 4));
    C64Dev h = {};
    h.eps = eps;
    h.max_iter = max_iter;
    h.hist = hist;
    h.hist_cap = hist_cap;
    h.wait_ns = wait_limit_us > 0 ? 1000LL * wait_limit_us : (wait_limit_us < 0 ? -1LL : 0LL);
    GL_CUDA(cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st));

    EventTimer tm;
    tm.start(st);
    k_make_hop64<<<vgrid64(n), 256, 0, st>>>(H, op->U, op->lx, op->ly);
    GL_CUDA(cudaGetLastError());
    // setup (generic_cg.cpp:303-321): |b|, r = b - A x, |r|^2
    GL_TRY(launch_norm2(b, n, partials, &cnt[0], &s->bsq, st));
    GL_TRY(launch_apply_sigma(op, t, x, tmp, 0.0, nullptr, st));
    GL_TRY(launch_sub(r, b, t, n, st));
    GL_CUDA(cudaMemsetAsync(t, 0, sizeof(double2) * n, st));
    GL_TRY(launch_norm2(r, n, partials, &cnt[1], &s->rsq, st));
    int iters = 1, status = GLINALG_SOLVE_MAX_ITER;
    if (max_iter > 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(32, kC64Warps);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        GL_CUDA(cudaLaunchKernelEx(&cfg, k_cg64, (const double2 *)H, r, t, p, x, op->mass, op->lx, op->ly, s, gs,
                                   partA, partB));
    }
    // true residual (generic_cg.cpp:366-367)
    GL_TRY(launch_apply_sigma(op, t, x, tmp, 0.0, nullptr, st));
    GL_TRY(launch_diffnorm2(t, b, n, partials, &cnt[2], truersq, st));
    tm.stop(st);
    GL_CUDA(cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
    double tr = 0.0;
    GL_CUDA(cudaMemcpyAsync(&tr, truersq, sizeof(double), cudaMemcpyDeviceToHost, st));
    std::vector<double> hh(hist_cap);
    if (hist_cap) GL_CUDA(cudaMemcpyAsync(hh.data(), hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    if (max_iter > 0) {
        iters = h.iters;
        status = h.status;
    } else {  // the loop never runs: k stays 0 (generic_cg.cpp:356-364)
        status = (0 == max_iter - 1) ? GLINALG_SOLVE_MAX_ITER : GLINALG_SOLVE_CONVERGED;
    }
    info->resSq = tr;
    info->iter = iters;
    info->success = status == GLINALG_SOLVE_CONVERGED ? 1 : 0;
    // setup A x, the first A p, one A p per further iteration, the true-residual check
    info->ops_count = max_iter > 0 ? iters + 2 : 2;
    info->status = status;
    info->device_ms = tm.ms();
    info->kernel_launches = max_iter > 0 ? 1 : 0;
    // per iteration: A reads r (stencil), 2 links, t, p and writes t, p; B reads t (stencil),
    // 2 links, p, x, r and writes x, r: 16 complex words
    info->gbytes = ((double)iters * 16.0 * 16.0 * n + 4 * apply_bytes(op)) * 1e-9;
    fill_name(info, "CG");
    if (status == GLINALG_SOLVE_TIMEOUT) {
        set_last_error("a bounded wait of the fused FP64 CG kernel for other blocks ran out");
        return GLINALG_ERROR_INTERNAL;
    }
    const double bsqrt = std::sqrt(h.bsq);
    for (int k = 0; k < std::min(iters, hist_cap); k++) verb.resid("CG", k + 1, 2 + k, hh[k]);
    verb.summary("CG", info->success != 0, iters, info->ops_count, std::sqrt(tr) / bsqrt);
    return GLINALG_SUCCESS;
}

}  // namespace glinalg
