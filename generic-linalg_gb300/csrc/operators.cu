// operators.cu -- device operator objects and the FP64 operator kernels:
//   staggered D / D^dagger / D^dagger D   (operators.cpp:184-239, :372-441, :444-453)
//   gauge Laplacian                       (operators.cpp:73-120)
//   generic stencil_2d apply / _eo / _oe  (coarse_stencil.cpp:12-172, :395-460, :560-625)
//   staggered stencil builders            (operators_stencil.cpp:14-63, :120-169)
// plus the library's device/stream bookkeeping and the BLAS-1 entry points.
//
// The FP64 kernels keep the reference's accumulation order per output site (hopping terms
// in the order +x, -x, +y, -y, then the 1/2 and the mass) so that results agree with the
// reference to rounding.  Fields are site-major double2 (16-byte loads per site).

#include <mutex>
#include <vector>

#include "operator.h"
#include "sites.cuh"

namespace glinalg {

// ---------------------------------------------------------------- device bookkeeping

namespace {
std::mutex g_mu;
cudaStream_t g_stream[64] = {};
int g_sms[64] = {};
}  // namespace

glinalg_status ensure_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_last_error("no CUDA device available");
        return GLINALG_ERROR_NO_DEVICE;
    }
    return GLINALG_SUCCESS;
}

static int cur_dev()
{
    int d = 0;
    cudaGetDevice(&d);
    return d < 64 ? d : 0;
}

static cudaStream_t g_user_stream[64] = {};
static bool g_has_user_stream[64] = {};

cudaStream_t lib_stream()
{
    int d = cur_dev();
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_has_user_stream[d]) return g_user_stream[d];
    if (!g_stream[d]) cudaStreamCreateWithFlags(&g_stream[d], cudaStreamNonBlocking);
    return g_stream[d];
}

// The library's stream-ordered memory pool of each device.  It keeps the memory that calls
// free (release threshold: unlimited), so that a repeated solve takes its work vectors from the
// pool instead of mapping and unmapping device memory on every call (about 0.5 ms of a 1024^2
// solve with the default pool, which returns freed memory at every synchronisation);
// glinalg_release_memory() hands it back.
static cudaMemPool_t g_pool[64] = {};
static bool g_pool_made[64] = {};

static cudaMemPool_t pool_of(int d)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_pool_made[d]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = d;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) == cudaSuccess) {
            unsigned long long keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            g_pool[d] = pool;
        } else {
            cudaGetLastError();  // fall back to the device's default pool
        }
        g_pool_made[d] = true;
    }
    return g_pool[d];
}

cudaError_t lib_malloc_async(void **p, size_t bytes, cudaStream_t st)
{
    const cudaMemPool_t pool = pool_of(cur_dev());
    return pool ? cudaMallocFromPoolAsync(p, bytes, pool, st) : cudaMallocAsync(p, bytes, st);
}

static cudaStream_t g_capture[64] = {};

cudaStream_t capture_stream()
{
    int d = cur_dev();
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_capture[d]) cudaStreamCreateWithFlags(&g_capture[d], cudaStreamNonBlocking);
    return g_capture[d];
}

void set_user_stream(cudaStream_t s, bool use)
{
    int d = cur_dev();
    std::lock_guard<std::mutex> lk(g_mu);
    g_user_stream[d] = s;
    g_has_user_stream[d] = use;
}

int sm_count()
{
    int d = cur_dev();
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_sms[d]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
        g_sms[d] = v > 0 ? v : 1;
    }
    return g_sms[d];
}

int reduction_blocks(long n)
{
    long b = (n + kRedThreads - 1) / kRedThreads;
    long cap = (long)sm_count() * 4;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

bool is_staggered(int k)
{
    return k == GLINALG_OP_STAGGERED || k == GLINALG_OP_STAGGERED_DAGGER ||
           k == GLINALG_OP_STAGGERED_NORMAL;
}
bool is_stencil(int k)
{
    return (k >= GLINALG_OP_STENCIL && k <= GLINALG_OP_STENCIL_OE) || k == GLINALG_OP_STENCIL_M2MDEODOE ||
           (k >= GLINALG_OP_STENCIL_TB && k <= GLINALG_OP_STENCIL_DAGGER_TB);
}
bool is_hermitian(int k)
{
    return k == GLINALG_OP_STAGGERED_NORMAL || k == GLINALG_OP_LAPLACE || k == GLINALG_OP_STAGGERED_M2MDEODOE ||
           k == GLINALG_OP_STENCIL_M2MDEODOE;
}
bool needs_tmp(int k)
{
    return k == GLINALG_OP_STAGGERED_NORMAL || k == GLINALG_OP_STAGGERED_M2MDEODOE ||
           k == GLINALG_OP_STENCIL_M2MDEODOE || (k >= GLINALG_OP_STENCIL_M2MDTBDBT && k <= GLINALG_OP_STENCIL_DAGGER_TB);
}

double apply_bytes(const glinalg_operator_s *op)
{
    // per output site: in + out + links (2 per site) as stored; the normal operator is two
    // passes.  Stencil: clover + 4 hops (+8 two-link) Nc x Nc per site plus in/out.
    const double w = 16.0;
    if (needs_tmp(op->kind)) return 8.0 * w * op->vol;  // two passes (even/odd: zeros at one parity)
    if (is_stencil(op->kind)) {
        double nc = op->nc;
        double terms = 1 + 4 + (op->two_link ? 8 : 0);
        return w * op->vol * (2 * nc + nc * nc * terms);
    }
    return 4.0 * w * op->vol;
}

// ---------------------------------------------------------------- kernels

// square_staggered_u1 (sign = +1) and square_staggered_dagger_u1 (sign = -1), FP64,
// one site per thread.
__global__ void k_staggered(double2 *__restrict__ out, const double2 *__restrict__ in,
                            const double2 *__restrict__ U, double mass, int lx, int ly,
                            double sign, const int *__restrict__ done)
{
    if (done && *done) return;
    const long vol = (long)lx * ly;
    auto ld = [in](long j) { return in[j]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol;
         i += (long)gridDim.x * blockDim.x)
        out[i] = stag_site(ld, U, mass, lx, ly, sign, i);
}

// square_laplace_u1, FP64.
__global__ void k_laplace(double2 *__restrict__ out, const double2 *__restrict__ in,
                          const double2 *__restrict__ U, double mass, int lx, int ly,
                          const int *__restrict__ done)
{
    if (done && *done) return;
    const long vol = (long)lx * ly;
    auto ld = [in](long j) { return in[j]; };
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol;
         i += (long)gridDim.x * blockDim.x)
        out[i] = lap_site(ld, U, mass, lx, ly, i);
}

// apply_stencil_2d (parity 0), _eo (parity 1: even output sites, hopping only), _oe
// (parity 2), _tb (parity 3: top half of the colours out, bottom half in; clover, hopping and
// two-link, no shifts; coarse_stencil.cpp:725) and _bt (parity 4, :1120).  One (site,
// colour-row) element per thread.  NC > 0 fixes the colour count
// at compile time; NC == 0 reads it from nc_rt.
template <int NC>
__global__ void k_stencil(double2 *__restrict__ out, const double2 *__restrict__ in,
                          const double2 *__restrict__ clov, const double2 *__restrict__ hop,
                          const double2 *__restrict__ two, double2 shift, double2 eo_shift,
                          double2 dof_shift, int lx, int ly, int nc_rt, int parity,
                          const int *__restrict__ done, const double2 *__restrict__ comb_r = nullptr,
                          double2 comb_s2 = double2{0.0, 0.0})
{
    if (done && *done) return;
    const int nc = NC > 0 ? NC : nc_rt;
    const long lsize = (long)lx * ly * nc;
    const bool has_shift = shift.x != 0.0 || shift.y != 0.0;
    const bool has_eo = eo_shift.x != 0.0 || eo_shift.y != 0.0;
    const bool has_dof = dof_shift.x != 0.0 || dof_shift.y != 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < lsize;
         i += (long)gridDim.x * blockDim.x) {
        const int color = (int)(i % nc);
        const long site = i / nc;
        const int y = (int)(site / lx), x = (int)(site - (long)y * lx);
        const bool even = ((x + y) & 1) == 0;
        if ((parity == 1 && !even) || (parity == 2 && even) || (parity == 3 && color >= nc / 2) ||
            (parity == 4 && color < nc / 2)) {
            out[i] = comb_r ? csub(cmul(comb_s2, comb_r[i]), out[i]) : cmk(0.0, 0.0);
            continue;
        }
        // tb (3) reads the bottom half of the input colours, bt (4) the top half
        const int c0 = parity == 3 ? nc / 2 : 0, c1 = parity == 4 ? nc / 2 : nc;
        const bool full = parity == 0 || parity >= 3;  // clover and two-link terms included
        double2 acc = cmk(0.0, 0.0);
        if (full) {
            for (int c = c0; c < c1; c++)
                acc = cadd(acc, cmul(clov[c + (long)nc * i], in[site * nc + c]));
        }
        // hopping directions {+x, +y, -x, -y}
        const int hxs[4] = {1, 0, -1, 0}, hys[4] = {0, 1, 0, -1};
#pragma unroll
        for (int d = 0; d < 4; d++) {
            int xx = x + hxs[d], yy = y + hys[d];
            xx = xx < 0 ? xx + lx : (xx >= lx ? xx - lx : xx);
            yy = yy < 0 ? yy + ly : (yy >= ly ? yy - ly : yy);
            const long nb = ((long)yy * lx + xx) * nc;
            const double2 *h = hop + (long)d * nc * lsize + (long)nc * i;
            for (int c = c0; c < c1; c++) acc = cadd(acc, cmul(h[c], in[nb + c]));
        }
        if (full && two != nullptr) {
            // two-link directions {+2x, +x+y, +2y, -x+y, -2x, -x-y, -2y, +x-y}
            const int txs[8] = {2, 1, 0, -1, -2, -1, 0, 1}, tys[8] = {0, 1, 2, 1, 0, -1, -2, -1};
#pragma unroll
            for (int d = 0; d < 8; d++) {
                int xx = (x + txs[d] + 2 * lx) % lx, yy = (y + tys[d] + 2 * ly) % ly;
                const long nb = ((long)yy * lx + xx) * nc;
                const double2 *h = two + (long)d * nc * lsize + (long)nc * i;
                for (int c = c0; c < c1; c++) acc = cadd(acc, cmul(h[c], in[nb + c]));
            }
        }
        if (parity == 0) {
            const double2 r = in[i];
            if (has_shift) acc = cadd(acc, cmul(shift, r));
            if (has_eo) acc = cadd(acc, cmul(cscale(even ? 1.0 : -1.0, eo_shift), r));
            if (has_dof) acc = cadd(acc, cmul(cscale(color < nc / 2 ? 1.0 : -1.0, dof_shift), r));
        }
        // combined form: out = (s2 r - out) - acc, the last step of m^2 - A - B
        out[i] = comb_r ? csub(csub(cmul(comb_s2, comb_r[i]), out[i]), acc) : acc;
    }
}

// out += sigma * in
__global__ void k_axpy_real(double2 *__restrict__ out, const double2 *__restrict__ in,
                            double sigma, long n, const int *__restrict__ done)
{
    if (done && *done) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        double2 o = out[i];
        out[i] = cadd(o, cscale(sigma, in[i]));
    }
}

// get_square_staggered_u1_stencil (dagger = 0) / get_square_staggered_dagger_u1_stencil.
__global__ void k_staggered_stencil(double2 *__restrict__ hop, const double2 *__restrict__ U,
                                    int lx, int ly, double s)
{
    const long vol = (long)lx * ly;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < vol;
         i += (long)gridDim.x * blockDim.x) {
        const int y = (int)(i / lx), x = (int)(i - (long)y * lx);
        const double eta = (double)(1 - 2 * (x & 1));
        const long imx = (long)y * lx + wrap_m(x, lx);
        const long imy = (long)wrap_m(y, ly) * lx + x;
        hop[i] = cscale(-0.5 * s, U[2 * i]);
        hop[i + vol] = cscale((-0.5 * s) * eta, U[2 * i + 1]);
        hop[i + 2 * vol] = cscale(0.5 * s, cconj(U[2 * imx]));
        hop[i + 3 * vol] = cscale((0.5 * s) * eta, cconj(U[2 * imy + 1]));
    }
}

// ---------------------------------------------------------------- launchers

static int grid_for(long n, int nt)
{
    long b = (n + nt - 1) / nt;
    long cap = (long)sm_count() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

glinalg_status launch_staggered(const glinalg_operator_s *op, double2 *out, const double2 *in,
                                double sign, const int *done, cudaStream_t st)
{
    const int nt = 256;
    k_staggered<<<grid_for(op->vol, nt), nt, 0, st>>>(out, in, op->U, op->mass, op->lx, op->ly,
                                                      sign, done);
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_apply(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs,
                            double2 *tmp, const int *done, cudaStream_t st)
{
    const int nt = 256;
    switch (op->kind) {
    case GLINALG_OP_STAGGERED: return launch_staggered(op, lhs, rhs, +1.0, done, st);
    case GLINALG_OP_STAGGERED_DAGGER: return launch_staggered(op, lhs, rhs, -1.0, done, st);
    case GLINALG_OP_STAGGERED_NORMAL:
        if (!tmp) return GLINALG_ERROR_INTERNAL;
        GL_TRY(launch_staggered(op, tmp, rhs, +1.0, done, st));
        return launch_staggered(op, lhs, tmp, -1.0, done, st);
    case GLINALG_OP_LAPLACE:
        k_laplace<<<grid_for(op->vol, nt), nt, 0, st>>>(lhs, rhs, op->U, op->mass, op->lx,
                                                        op->ly, done);
        GL_CUDA(cudaGetLastError());
        return GLINALG_SUCCESS;
    case GLINALG_OP_STENCIL:
    case GLINALG_OP_STENCIL_EO:
    case GLINALG_OP_STENCIL_OE: return launch_stencil_parity(op, lhs, rhs, op->kind - GLINALG_OP_STENCIL, done, st);
    case GLINALG_OP_STAGGERED_DEO:
    case GLINALG_OP_STAGGERED_DOE:
    case GLINALG_OP_STAGGERED_M2MDEODOE:
    case GLINALG_OP_STENCIL_M2MDEODOE: return launch_eo_apply(op, lhs, rhs, tmp, done, st);
    case GLINALG_OP_STENCIL_TB: return launch_stencil_parity(op, lhs, rhs, 3, done, st);
    case GLINALG_OP_STENCIL_BT: return launch_stencil_parity(op, lhs, rhs, 4, done, st);
    case GLINALG_OP_STENCIL_M2MDTBDBT:
    case GLINALG_OP_STENCIL_NORMAL_EO:
    case GLINALG_OP_STENCIL_NORMAL_TB:
    case GLINALG_OP_STENCIL_DAGGER_EO:
    case GLINALG_OP_STENCIL_DAGGER_TB: return launch_coarse_piece(op, lhs, rhs, tmp, done, st);
    default: return GLINALG_ERROR_UNSUPPORTED_OP;
    }
}

glinalg_status launch_stencil_parity(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs, int parity,
                                     const int *done, cudaStream_t st, const double2 *comb_r, double2 comb_s2)
{
    const int nt = 256;
    const int g = grid_for(op->size, nt);
#define GL_STENCIL(NCT, NCR)                                                                                       \
    k_stencil<NCT><<<g, nt, 0, st>>>(lhs, rhs, op->clover, op->hopping, op->two_link, op->shift, op->eo_shift,     \
                                     op->dof_shift, op->lx, op->ly, NCR, parity, done, comb_r, comb_s2)
    if (op->nc == 1) GL_STENCIL(1, 1);
    else if (op->nc == 2) GL_STENCIL(2, 2);
    else if (op->nc == 4) GL_STENCIL(4, 4);
    else if (op->nc == 8) GL_STENCIL(8, 8);
    else GL_STENCIL(0, op->nc);
#undef GL_STENCIL
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

glinalg_status launch_apply_sigma(const glinalg_operator_s *op, double2 *lhs, const double2 *rhs,
                                  double2 *tmp, double sigma, const int *done, cudaStream_t st)
{
    GL_TRY(launch_apply(op, lhs, rhs, tmp, done, st));
    if (sigma != 0.0) {
        k_axpy_real<<<grid_for(op->size, 256), 256, 0, st>>>(lhs, rhs, sigma, op->size, done);
        GL_CUDA(cudaGetLastError());
    }
    return GLINALG_SUCCESS;
}

glinalg_status launch_apply_shifted(const glinalg_operator_s *op, double2 *lhs,
                                    const double2 *rhs, double2 *tmp, double sigma,
                                    cudaStream_t st)
{
    return launch_apply_sigma(op, lhs, rhs, tmp, sigma, nullptr, st);
}

}  // namespace glinalg

using namespace glinalg;

// The operator's arrays go back to the library's pool.  The device is synchronised first, as
// cudaFree would: work of any stream that still reads them has finished.
glinalg_operator_s::~glinalg_operator_s()
{
    if (!U && !clover && !hopping && !two_link) return;  // a view that owns nothing
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaDeviceSynchronize();
    const cudaStream_t st = lib_stream();
    for (void *p : {(void *)U, (void *)clover, (void *)hopping, (void *)two_link})
        if (p) cudaFreeAsync(p, st);
    cudaSetDevice(prev);
}

// ---------------------------------------------------------------- C-ABI: operators

static glinalg_status upload(double2 **dst, const double *src, long n_complex, int dev_ptrs,
                             cudaStream_t st)
{
    GL_CUDA(lib_malloc_async((void **)dst, sizeof(double2) * (size_t)n_complex, st));
    GL_CUDA(cudaMemcpyAsync(*dst, src, sizeof(double2) * (size_t)n_complex,
                            dev_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_operator_create(const glinalg_op_desc *d, glinalg_operator *out)
{
    if (!d || !out) return invalid_arg("!d || !out");
    *out = nullptr;
    if (d->lx <= 0 || d->ly <= 0) return invalid_arg("d->lx <= 0 || d->ly <= 0");
    if (d->kind < GLINALG_OP_STAGGERED || d->kind > GLINALG_OP_STENCIL_DAGGER_TB)
        return GLINALG_ERROR_UNSUPPORTED_OP;
    const bool sten = is_stencil(d->kind);
    if (sten && (d->nc <= 0 || !d->clover || !d->hopping))
        return invalid_arg("sten && (d->nc <= 0 || !d->clover || !d->hopping)");
    if (d->kind == GLINALG_OP_STENCIL_M2MDEODOE && d->nc != 1) {
        set_last_error("the stencil form of m^2 - D_eo D_oe needs nc = 1 (a staggered stencil)");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    if (!sten && !d->links) return invalid_arg("!sten && !d->links");
    GL_TRY(ensure_device());
    auto *op = new glinalg_operator_s();
    op->kind = d->kind;
    op->lx = d->lx;
    op->ly = d->ly;
    op->nc = sten ? d->nc : 1;
    op->mass = d->mass;
    op->vol = (long)d->lx * d->ly;
    op->size = op->vol * op->nc;
    cudaGetDevice(&op->device);
    cudaStream_t st = lib_stream();
    const int dp = d->flags & GLINALG_PTR_DEVICE;
    glinalg_status s = GLINALG_SUCCESS;
    if (!sten) {
        s = upload(&op->U, d->links, 2 * op->vol, dp, st);
    } else {
        const long cc = op->vol * op->nc * op->nc;
        s = upload(&op->clover, d->clover, cc, dp, st);
        if (s == GLINALG_SUCCESS) s = upload(&op->hopping, d->hopping, 4 * cc, dp, st);
        if (s == GLINALG_SUCCESS && d->two_link) s = upload(&op->two_link, d->two_link, 8 * cc, dp, st);
        op->shift = cmk(d->shift[0], d->shift[1]);
        op->eo_shift = cmk(d->eo_shift[0], d->eo_shift[1]);
        op->dof_shift = cmk(d->dof_shift[0], d->dof_shift[1]);
    }
    if (s == GLINALG_SUCCESS) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_last_error(cudaGetErrorString(e));
            s = GLINALG_ERROR_CUDA;
        }
    }
    if (s != GLINALG_SUCCESS) {
        delete op;
        return s;
    }
    *out = op;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_release_memory(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (int d = 0; d < 64; d++) {
        if (!g_pool[d]) continue;
        if (cudaMemPoolTrimTo(g_pool[d], 0) != cudaSuccess) {
            const cudaError_t e = cudaGetLastError();
            set_last_error(std::string("cudaMemPoolTrimTo: ") + cudaGetErrorString(e));
            return GLINALG_ERROR_CUDA;
        }
    }
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_set_stream(void *stream, int use)
{
    GL_TRY(ensure_device());
    set_user_stream((cudaStream_t)stream, use != 0);
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_operator_destroy(glinalg_operator op)
{
    delete op;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_operator_set_mass(glinalg_operator op, double mass)
{
    if (!op) return invalid_arg("!op");
    op->mass = mass;
    return GLINALG_SUCCESS;
}

extern "C" long glinalg_operator_size(glinalg_operator op) { return op ? op->size : 0; }

extern "C" glinalg_status glinalg_operator_apply(glinalg_operator op, double *lhs,
                                                 const double *rhs, int flags)
{
    if (!op || !lhs || !rhs) return invalid_arg("!op || !lhs || !rhs");
    cudaStream_t st = lib_stream();
    const size_t bytes = sizeof(double2) * (size_t)op->size;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    double2 *d_in = nullptr, *d_out = nullptr, *d_tmp = nullptr;
    glinalg_status s = GLINALG_SUCCESS;
    auto fail = [&](cudaError_t e) {
        set_last_error(cudaGetErrorString(e));
        s = e == cudaErrorMemoryAllocation ? GLINALG_ERROR_OUT_OF_MEMORY : GLINALG_ERROR_CUDA;
    };
    cudaError_t e = cudaSuccess;
    if (!dev) {
        e = lib_malloc_async((void **)&d_in, bytes, st);
        if (e == cudaSuccess) e = lib_malloc_async((void **)&d_out, bytes, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, rhs, bytes, cudaMemcpyHostToDevice, st);
    } else {
        d_in = (double2 *)rhs;
        d_out = (double2 *)lhs;
    }
    if (e == cudaSuccess && needs_tmp(op->kind))
        e = lib_malloc_async((void **)&d_tmp, bytes, st);
    if (e != cudaSuccess) fail(e);
    if (s == GLINALG_SUCCESS) s = launch_apply(op, d_out, d_in, d_tmp, nullptr, st);
    if (s == GLINALG_SUCCESS && !dev) {
        e = cudaMemcpyAsync(lhs, d_out, bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) fail(e);
    }
    if (d_tmp) cudaFreeAsync(d_tmp, st);
    if (!dev) {
        if (d_in) cudaFreeAsync(d_in, st);
        if (d_out) cudaFreeAsync(d_out, st);
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess && s == GLINALG_SUCCESS) fail(e);
    return s;
}

extern "C" glinalg_status glinalg_staggered_stencil(const double *links, int lx, int ly,
                                                    double mass, int dagger, double *hopping_out,
                                                    double *shift_out, int flags)
{
    if (!links || !hopping_out || lx <= 0 || ly <= 0)
        return invalid_arg("!links || !hopping_out || lx <= 0 || ly <= 0");
    GL_TRY(ensure_device());
    cudaStream_t st = lib_stream();
    const long vol = (long)lx * ly;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    double2 *dU = (double2 *)links, *dH = (double2 *)hopping_out;
    if (!dev) {
        GL_CUDA(lib_malloc_async((void **)&dU, sizeof(double2) * 2 * vol, st));
        GL_CUDA(lib_malloc_async((void **)&dH, sizeof(double2) * 4 * vol, st));
        GL_CUDA(cudaMemcpyAsync(dU, links, sizeof(double2) * 2 * vol, cudaMemcpyHostToDevice, st));
    }
    k_staggered_stencil<<<grid_for(vol, 256), 256, 0, st>>>(dH, dU, lx, ly, dagger ? -1.0 : 1.0);
    GL_CUDA(cudaGetLastError());
    if (!dev) {
        GL_CUDA(cudaMemcpyAsync(hopping_out, dH, sizeof(double2) * 4 * vol, cudaMemcpyDeviceToHost, st));
        cudaFreeAsync(dU, st);
        cudaFreeAsync(dH, st);
    }
    GL_CUDA(cudaStreamSynchronize(st));
    if (shift_out) {
        shift_out[0] = mass;
        shift_out[1] = 0.0;
    }
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_operator_stencil_get(glinalg_operator op, double *clover, double *hopping,
                                                       int flags)
{
    if (!op) return invalid_arg("!op");
    if (!is_stencil(op->kind) || !op->clover || !op->hopping) {
        set_last_error("not a stencil operator");
        return GLINALG_ERROR_UNSUPPORTED_OP;
    }
    cudaStream_t st = lib_stream();
    const size_t cc = sizeof(double2) * (size_t)op->vol * op->nc * op->nc;
    const cudaMemcpyKind k = (flags & GLINALG_PTR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (clover) GL_CUDA(cudaMemcpyAsync(clover, op->clover, cc, k, st));
    if (hopping) GL_CUDA(cudaMemcpyAsync(hopping, op->hopping, 4 * cc, k, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}
