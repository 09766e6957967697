// probe.cu -- measured on-chip bandwidth, the denominator of the on-chip roofline of the
// rectangle-resident CG kernel (whose iteration moves its fields through shared memory, not
// HBM).  One block of 1024 threads per SM (twice over, 2 x 32 KB of shared memory per SM)
// streams 128-bit loads out of shared memory, each warp reading 512 consecutive bytes, so every
// load instruction is four conflict-free wavefronts; the sums go to a global word only if a
// sentinel shows up, so no load can be dropped.

#include "operator.h"

namespace glinalg {
namespace {

constexpr int kProbeThreads = 1024;
constexpr int kProbeElems = 2048;  // float4 in shared memory: 32 KB
constexpr int kProbeUnroll = 8;

__global__ void __launch_bounds__(kProbeThreads) k_smem_read(float *sink, int reps)
{
    __shared__ float4 buf[kProbeElems];
    for (int i = threadIdx.x; i < kProbeElems; i += blockDim.x)
        buf[i] = make_float4((float)i, 1.f, 2.f, 3.f);
    __syncthreads();
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    // the kProbeUnroll loads of a pass read kProbeUnroll distinct addresses (offsets k * 256
    // within the 2048-entry buffer), so none can be merged with another
    unsigned idx = threadIdx.x;
    for (int r = 0; r < reps; r++) {
#pragma unroll
        for (int k = 0; k < kProbeUnroll; k += 2) {
            const float4 v = buf[(idx + k * (kProbeElems / kProbeUnroll)) & (kProbeElems - 1)];
            const float4 w = buf[(idx + (k + 1) * (kProbeElems / kProbeUnroll)) & (kProbeElems - 1)];
            a0.x += v.x; a0.y += v.y; a0.z += v.z; a0.w += v.w;
            a1.x += w.x; a1.y += w.y; a1.z += w.z; a1.w += w.w;
        }
        idx += 32;  // a new address each pass, so no load is loop-invariant
    }
    const float s = a0.x + a0.y + a0.z + a0.w + a1.x + a1.y + a1.z + a1.w;
    if (s == -1.0f) sink[blockIdx.x] = s;
}

}  // namespace
}  // namespace glinalg

using namespace glinalg;

extern "C" glinalg_status glinalg_probe_smem_bandwidth(double *gbs, double *ms)
{
    if (!gbs) return invalid_arg("gbs == NULL");
    GL_TRY(ensure_device());
    int dev = 0, nsm = 0;
    GL_CUDA(cudaGetDevice(&dev));
    GL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = lib_stream();
    float *sink = nullptr;
    GL_CUDA(lib_malloc_async((void **)&sink, sizeof(float) * 2 * nsm, st));
    const int grid = 2 * nsm, reps = 4096;
    cudaEvent_t e0, e1;
    GL_CUDA(cudaEventCreate(&e0));
    GL_CUDA(cudaEventCreate(&e1));
    k_smem_read<<<grid, kProbeThreads, 0, st>>>(sink, 64);  // warm-up
    GL_CUDA(cudaEventRecord(e0, st));
    const int n_launch = 5;
    for (int i = 0; i < n_launch; i++) k_smem_read<<<grid, kProbeThreads, 0, st>>>(sink, reps);
    GL_CUDA(cudaEventRecord(e1, st));
    GL_CUDA(cudaGetLastError());
    GL_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    GL_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    GL_CUDA(cudaFreeAsync(sink, st));
    GL_CUDA(cudaStreamSynchronize(st));
    const double bytes = (double)n_launch * grid * kProbeThreads * (double)reps * kProbeUnroll * sizeof(float4);
    *gbs = bytes / (t * 1e-3) / 1e9;
    if (ms) *ms = t / n_launch;
    return GLINALG_SUCCESS;
}
