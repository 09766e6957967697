// noalloc.cu -- an entry point that allocates no device memory: the staggered normal
// operator lhs = D^dagger D rhs on caller-provided device buffers, with the intermediate
// field D rhs held in a fixed array compiled into this library instead of a per-call
// allocation.
//
// Who needs it: callers that must not allocate device memory while they run -- a host
// application that reserves all of HBM for its own pools up front, a code path running
// under a memory budget or inside another framework's allocator where a stray cudaMalloc
// fails or fragments the pool, or latency-critical loops where an allocation (and the
// implicit synchronisation cudaMalloc / cudaFree can cause) is not acceptable.  Every other
// entry point of this library allocates its work fields per call.
//
// The array (kNoAllocSites complex<double> values, 4 MiB) lives in this library's device
// image: every GPU that loads the library holds it until the process exits.  Its device
// address is looked up once per device (cudaGetSymbolAddress), on the first call made with
// that device current; make that first call before any stream capture.  The call only
// enqueues its two kernels on the caller's stream and returns; lhs is complete once that
// stream has reached them.  All calls share the one array: calls whose work overlaps on the
// GPU (different streams, or different host threads) race on it and must be serialised by
// the caller.  The array keeps the previous
// call's contents; this operator overwrites every entry it reads before reading it, so
// nothing needs clearing.

#include <mutex>

#include "operator.h"

namespace glinalg {

// FP64 staggered D (sign = +1) / D^dagger (sign = -1), defined in operators.cu.
__global__ void k_staggered(double2 *__restrict__ out, const double2 *__restrict__ in,
                            const double2 *__restrict__ U, double mass, int lx, int ly,
                            double sign, const int *__restrict__ done);

namespace {

constexpr long kNoAllocSites = GLINALG_NOALLOC_MAX_SITES;

// The scratch field.  In host code `g_noalloc_scratch` names a host-side stand-in, not the
// device array: only the address from cudaGetSymbolAddress may be passed to kernels.
static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocSites];

std::mutex g_mu;
void *g_ptr[64] = {};

// Device address of the scratch array on the current device (looked up once per device).
glinalg_status scratch_address(double2 **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return GLINALG_ERROR_NO_DEVICE;
    }
    if (dev < 0 || dev >= 64) {
        set_last_error("device index out of range for the no-allocation scratch table");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            set_last_error(std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(e));
            return GLINALG_ERROR_CUDA;
        }
        g_ptr[dev] = p;
    }
    *out = (double2 *)g_ptr[dev];
    return GLINALG_SUCCESS;
}

}  // namespace
}  // namespace glinalg

using namespace glinalg;

extern "C" glinalg_status glinalg_staggered_normal_apply_noalloc(const double *links, double mass, int lx,
                                                                 int ly, double *lhs, const double *rhs,
                                                                 void *stream)
{
    if (!links || !lhs || !rhs || lx <= 0 || ly <= 0) {
        set_last_error("null pointer or non-positive lattice extent");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    const long vol = (long)lx * ly;
    if (vol > kNoAllocSites) {
        set_last_error("lattice of " + std::to_string(vol) + " sites exceeds the no-allocation scratch of " +
                       std::to_string(kNoAllocSites) + " sites (GLINALG_NOALLOC_MAX_SITES)");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    double2 *scratch = nullptr;
    GL_TRY(scratch_address(&scratch));
    cudaStream_t st = (cudaStream_t)stream;
    const int nt = 256;
    const int grid = (int)((vol + nt - 1) / nt);
    k_staggered<<<grid, nt, 0, st>>>(scratch, (const double2 *)rhs, (const double2 *)links, mass, lx, ly, +1.0,
                                    nullptr);
    k_staggered<<<grid, nt, 0, st>>>((double2 *)lhs, scratch, (const double2 *)links, mass, lx, ly, -1.0,
                                    nullptr);
    // no synchronisation here: the work is ordered on the caller's stream, and the caller waits
    // on that stream (or an event recorded after the call) before reading lhs
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}
