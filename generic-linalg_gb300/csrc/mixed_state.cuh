// mixed_state.cuh -- device state of a mixed-precision CG solve with FP64 reliable updates
// and the scalar updates that follow each inner kernel's reduction (cg_mixed.cu, cg_batch.cu).
#pragma once

#include <cuda/atomic>

#include "solvers.h"
#include "stag_tiles.cuh"

namespace glinalg {

struct MxDev {
    double rsq;        // |r_lo|^2 at the start of the current inner iteration (scaled units)
    double rsq_new;
    double alpha, beta;
    double scale;      // r_true ~= scale * r_lo
    double rmax;       // largest true-scale iterated residual since the last update
    double bsq, eps, delta, sigma;
    double rp;         // <r, p> / |r|^2 for the re-orthogonalisation
    double pscale;     // old scale / new scale, applied to p at a reliable update
    double rsq_true;   // last FP64 true residual
    double rsq_old_true;
    int k, max_iter, done, status, reliable, n_reliable, outer;
    int parity;        // which p buffer (0 or 1) holds the current direction
    unsigned cnt[6];
    long long inner_ns;  // device time spent in the persistent inner-loop kernel
    int inner_iters;     // iterations it ran
    int inner_launches;
    long long wait_ns;   // bound on each wait for other blocks: 0 = the default, < 0 = none
};

__device__ __forceinline__ void mx_stop_inner(cudaGraphConditionalHandle cond, int use_cond)
{
    if (use_cond) cudaGraphSetConditional(cond, 0);
}

// After the reduction of A: alpha = rsq / <p, A p>, or stop on breakdown.
__device__ __forceinline__ void mx_after_A(MxDev *s, double pAp, cudaGraphConditionalHandle cond,
                                           int use_cond)
{
    if (!(pAp > 0.0) || !isfinite(pAp)) {
        s->status = pAp == 0.0 ? GLINALG_SOLVE_BREAKDOWN : GLINALG_SOLVE_NONFINITE;
        s->done = 1;
        mx_stop_inner(cond, use_cond);
        return;
    }
    s->alpha = s->rsq / pAp;
}

// After the reduction of B: beta for the next iteration, or flag a reliable update (which
// also covers convergence of the iterated residual and the iteration cap).
__device__ __forceinline__ void mx_after_B(MxDev *s, double rn, int dir_parity,
                                           cudaGraphConditionalHandle cond, int use_cond)
{
    const int k = s->k;
    s->parity = dir_parity;
    s->rsq_new = rn;
    s->k = k + 1;
    if (!isfinite(rn)) {
        s->status = GLINALG_SOLVE_NONFINITE;
        s->done = 1;
        mx_stop_inner(cond, use_cond);
        return;
    }
    const double rho = sqrt(rn) * s->scale;  // true-scale iterated residual
    if (rho > s->rmax) s->rmax = rho;
    const double bsqrt = sqrt(s->bsq);
    if (rho < s->delta * s->rmax || rho < s->eps * bsqrt || k + 1 >= s->max_iter) {
        s->reliable = 1;
        mx_stop_inner(cond, use_cond);
        return;
    }
    s->beta = rn / s->rsq;
    s->rsq = rn;
}

// ---------------------------------------------------------------- persistent-kernel helpers

struct GridSync {
    unsigned arrive;
    unsigned gen;
    int error;
    int pad;
};

__device__ __forceinline__ long long gtimer()
{
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bound on one barrier wait; a wait that runs out raises g->error (the solve then reports
// GLINALG_SOLVE_TIMEOUT) instead of spinning on.
constexpr long long kBarrierTimeoutNs = 2000000000LL;

// The bound, in ns, on a persistent kernel's waits for other blocks (grid barriers, mailbox
// polls) during this solve: MxDev::wait_ns if positive, the default if 0, and none at all (give
// up at the first check that finds the data missing) if negative.  Waits of a block on its own
// asynchronous copies keep the fixed kBarrierTimeoutNs.
__device__ __forceinline__ long long peer_wait_ns(const MxDev *s)
{
    return s->wait_ns > 0 ? s->wait_ns : (s->wait_ns == 0 ? kBarrierTimeoutNs : 0LL);
}

// Grid-wide barrier for a co-resident grid (generation counter; acquire/release atomics at
// device scope).  Returns false in every thread of the block once any block has given up
// waiting.
__device__ __forceinline__ bool grid_sync(GridSync *g, unsigned nblocks, long long lim_ns = kBarrierTimeoutNs)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(g->gen), arr(g->arrive);
        cuda::atomic_ref<int, cuda::thread_scope_device> err(g->error);
        const unsigned my = gen.load(cuda::memory_order_acquire);
        int good = 1;
        const unsigned a = arr.fetch_add(1u, cuda::memory_order_acq_rel);
        if (a == nblocks - 1) {
            arr.store(0u, cuda::memory_order_relaxed);
            gen.fetch_add(1u, cuda::memory_order_release);
        } else {
            const long long t0 = gtimer();
            while (gen.load(cuda::memory_order_acquire) == my) {
                if (err.load(cuda::memory_order_relaxed)) { good = 0; break; }
                if (gtimer() - t0 > lim_ns) {
                    err.store(1, cuda::memory_order_relaxed);
                    good = 0;
                    break;
                }
            }
        }
        if (err.load(cuda::memory_order_relaxed)) good = 0;
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Sum of the per-block partials in block order, identical in every block; all threads get it.
__device__ __forceinline__ double grid_total(const double *part, unsigned nb, double *sm)
{
    __syncthreads();
    if (threadIdx.y == 0) {
        double v = 0.0;
        for (unsigned b = threadIdx.x; b < nb; b += 32) v += __ldcg(part + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) sm[32] = v;
    }
    __syncthreads();
    return sm[32];
}

// Block sum of one float per thread (FP32 within warps, FP64 across the 32 warps) written to
// part[blockIdx.x] by the block's first thread.
__device__ __forceinline__ void block_partial(float acc, double *part, double *sm)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) sm[threadIdx.y] = (double)acc;
    __syncthreads();
    if (threadIdx.y == 0) {
        double v = threadIdx.x < blockDim.y ? sm[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) part[blockIdx.x] = v;
    }
}

}  // namespace glinalg
