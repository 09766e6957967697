// common.cuh -- shared device helpers: complex arithmetic on double2/float2, block and
// single-pass grid reductions, error plumbing.  All kernels of the library include this.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <string>

#include "glinalg.h"

namespace glinalg {

// ---------------------------------------------------------------- errors

// Last error message of the calling host thread (set by the C-ABI layer).
void set_last_error(const std::string &msg);

#define GL_CUDA(expr)                                                                     \
    do {                                                                                  \
        cudaError_t _e = (expr);                                                          \
        if (_e != cudaSuccess) {                                                          \
            ::glinalg::set_last_error(std::string(#expr) + ": " + cudaGetErrorString(_e)); \
            return _e == cudaErrorMemoryAllocation ? GLINALG_ERROR_OUT_OF_MEMORY          \
                                                   : GLINALG_ERROR_CUDA;                  \
        }                                                                                 \
    } while (0)

// Rejects an argument: records the message for glinalg_last_error() and returns
// GLINALG_ERROR_INVALID_VALUE.
inline glinalg_status invalid_arg(const char *msg)
{
    set_last_error(std::string("invalid argument: ") + msg);
    return GLINALG_ERROR_INVALID_VALUE;
}

#define GL_TRY(expr)                              \
    do {                                          \
        glinalg_status _s = (expr);               \
        if (_s != GLINALG_SUCCESS) return _s;     \
    } while (0)

// ---------------------------------------------------------------- complex helpers

__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__host__ __device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }

// Complex division a / b by Smith's algorithm (R. L. Smith, "Algorithm 116: Complex
// division", CACM 5(8), 1962): divide through by the larger component of b so that no
// intermediate overflows for representable quotients.
__host__ __device__ inline double2 cdiv(double2 a, double2 b)
{
    if (fabs(b.y) <= fabs(b.x)) {
        double r = b.y / b.x;
        double d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    } else {
        double r = b.x / b.y;
        double d = b.y + b.x * r;
        return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
    }
}
__host__ __device__ __forceinline__ double cabsd(double2 a) { return hypot(a.x, a.y); }

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ---------------------------------------------------------------- reductions

constexpr int kRedThreads = 256;

template <int K>
struct Vec {
    double v[K];
};

__device__ __forceinline__ unsigned flat_tid()
{
    return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
}
__device__ __forceinline__ unsigned flat_bid() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ __forceinline__ unsigned flat_nblocks() { return gridDim.x * gridDim.y * gridDim.z; }

// Sum K doubles over the block (NT threads, any block shape); the result is valid in the
// block's first thread.  Fixed shuffle tree and fixed warp order, so the result depends only
// on the inputs' positions.
template <int K, int NT>
__device__ __forceinline__ void block_sum(double (&v)[K])
{
    __shared__ double sm[K][NT / 32];
    const unsigned tid = flat_tid();
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int j = 0; j < K; j++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < K; j++) sm[j][warp] = v[j];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int j = 0; j < K; j++) {
            double s = (lane < NT / 32) ? sm[j][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            v[j] = s;
        }
    }
    __syncthreads();
}

// Single-pass grid reduction: every block stores its partial, the last block to arrive
// sums all partials in block order (deterministic for a fixed grid) and returns true in
// all of its threads with the total in its first thread's v.  counter must be 0 on entry
// and is reset to 0 by the last block.  partials holds K * (number of blocks) doubles.
template <int K, int NT>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double *partials, unsigned *counter)
{
    __shared__ unsigned ticket;
    const unsigned tid = flat_tid(), bid = flat_bid(), nbk = flat_nblocks();
    block_sum<K, NT>(v);
    if (tid == 0) {
#pragma unroll
        for (int j = 0; j < K; j++) partials[(size_t)j * nbk + bid] = v[j];
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
    for (int j = 0; j < K; j++) v[j] = s[j];
    if (tid == 0) *counter = 0u;
    return true;
}

template <int K, int NT>
__device__ __forceinline__ bool grid_sum_ids(double (&v)[K], double *partials, unsigned *counter,
                                             unsigned bid, unsigned nbk);
// grid_sum for grids whose rows (blockIdx.y) are independent problems: sums over the blocks
// of this block's row only (1D blocks of NT threads).  partials and counter belong to the row.
template <int K, int NT>
__device__ __forceinline__ bool grid_sum_row(double (&v)[K], double *partials, unsigned *counter)
{
    return grid_sum_ids<K, NT>(v, partials, counter, blockIdx.x, gridDim.x);
}

// grid_sum over a group of nbk blocks that reduce one problem together (1D blocks of NT
// threads); bid is this block's index within the group.  partials and counter belong to the
// group.
template <int K, int NT>
__device__ __forceinline__ bool grid_sum_ids(double (&v)[K], double *partials, unsigned *counter,
                                             unsigned bid, unsigned nbk)
{
    __shared__ unsigned ticket;
    const unsigned tid = threadIdx.x;
    block_sum<K, NT>(v);
    if (tid == 0) {
#pragma unroll
        for (int j = 0; j < K; j++) partials[(size_t)j * nbk + bid] = v[j];
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
    for (int j = 0; j < K; j++) v[j] = s[j];
    if (tid == 0) *counter = 0u;
    return true;
}

// Grid used by every reduction kernel over n elements (fixed for a given n, so reductions
// are reproducible run to run).
int reduction_blocks(long n);
int sm_count();

inline int blocks_for(long n, int nt) { return (int)((n + nt - 1) / nt); }

}  // namespace glinalg
