// mixed_state.cuh -- device state of a mixed-precision CG solve with FP64 reliable updates
// and the scalar updates that follow each inner kernel's reduction (cg_mixed.cu, cg_batch.cu).
#pragma once

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

}  // namespace glinalg
