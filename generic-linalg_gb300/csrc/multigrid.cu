// multigrid.cu -- the transfer operators and the Galerkin coarse operator of the reference's
// algebraic multigrid (multigrid/aa_mg/mg_complex.cpp): block_normalize (:191),
// block_orthonormalize (:259), prolong (:372), restrict (:421) and
// generate_coarse_from_fine_stencil (:827).
//
// One level maps a fine lattice lx x ly with nc_f dof per site onto (lx/bx) x (ly/by) coarse
// sites with nc_c dof.  The nc_c null vectors are stored as the reference stores them,
// P[c][f] with fine index f = (y*lx + x)*nc_f + dof, and P_c restricted to a block is the
// coarse basis vector of that block and colour.  Kernels give one output element to one
// thread and accumulate each sum in the reference's order (block rows, block columns, dof),
// so results agree with the reference to rounding of fused multiply-adds.
//
// The coarse operator is formed directly, not by probing: entry (a, b) of the coarse clover
// at block X sums conj(P_a(s)) A(s, t) P_b(t) over fine sites s in X and stencil neighbours
// t of s in X; a coarse hopping entry sums the fine hops of one direction that leave X
// through that face.  On even coarse extents this is exactly what the reference's probing
// computes; on odd ones the probing mixes terms of different coarse sites and this form
// keeps the Galerkin product P^dagger A P.  As in the reference, the fine stencil's two-link
// terms do not enter.

#include <vector>

#include "operator.h"
#include "solver_util.h"

struct glinalg_mg_level_s {
    int lx = 0, ly = 0, nc_f = 0, bx = 0, by = 0, nc_c = 0;
    int xc = 0, yc = 0;
    long fsize = 0, csize = 0;
    double2 *P = nullptr;  // nc_c * fsize
    ~glinalg_mg_level_s()
    {
        if (P) cudaFree(P);
    }
};

namespace glinalg {

namespace {

struct Lv {
    int lx, ly, nc_f, bx, by, nc_c, xc, yc;
    long fsize;
    const double2 *P;
};

Lv lv_of(const glinalg_mg_level_s *l)
{
    return Lv{l->lx, l->ly, l->nc_f, l->bx, l->by, l->nc_c, l->xc, l->yc, l->fsize, l->P};
}

// prolong (mg_complex.cpp:372-418): fine(f) = sum_c P_c(f) coarse(X(f), c), c ascending
__global__ void k_prolong(double2 *__restrict__ fine, const double2 *__restrict__ coarse, Lv v)
{
    for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < v.fsize; f += (long)gridDim.x * blockDim.x) {
        const long s = f / v.nc_f;
        const int y = (int)(s / v.lx), x = (int)(s - (long)y * v.lx);
        const long X = (long)(y / v.by) * v.xc + x / v.bx;
        double2 acc = cmk(0.0, 0.0);
        for (int c = 0; c < v.nc_c; c++) acc = cadd(acc, cmul(v.P[(long)c * v.fsize + f], coarse[X * v.nc_c + c]));
        fine[f] = acc;
    }
}

// restrict (mg_complex.cpp:421-467): coarse(X, c) = sum over the block of conj(P_c(f)) fine(f).
// Threads run colour-major (consecutive threads take consecutive blocks of one null vector), so
// a warp reads a contiguous stretch of that vector and of the fine field.
__global__ void k_restrict(double2 *__restrict__ coarse, const double2 *__restrict__ fine, Lv v)
{
    const long vc = (long)v.xc * v.yc, csize = vc * v.nc_c;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < csize; t += (long)gridDim.x * blockDim.x) {
        const int c = (int)(t / vc);
        const long X = t - (long)c * vc;
        const long i = X * v.nc_c + c;
        const int yc = (int)(X / v.xc), xc = (int)(X - (long)yc * v.xc);
        const double2 *p = v.P + (long)c * v.fsize;
        double2 acc = cmk(0.0, 0.0);
        for (int y = yc * v.by; y < yc * v.by + v.by; y++)
            for (int x = xc * v.bx; x < xc * v.bx + v.bx; x++)
                for (int d = 0; d < v.nc_f; d++) {
                    const long f = ((long)y * v.lx + x) * v.nc_f + d;
                    acc = cadd(acc, cmul(cconj(p[f]), fine[f]));
                }
        coarse[i] = acc;
    }
}

__device__ double block_norm(const Lv &v, const double2 *p, int xc, int yc)
{
    double n = 0.0;
    for (int y = yc * v.by; y < yc * v.by + v.by; y++)
        for (int x = xc * v.bx; x < xc * v.bx + v.bx; x++)
            for (int d = 0; d < v.nc_f; d++) n += cabs2(p[((long)y * v.lx + x) * v.nc_f + d]);
    return sqrt(n);
}

__device__ void block_scale(const Lv &v, double2 *p, int xc, int yc, double norm)
{
    for (int y = yc * v.by; y < yc * v.by + v.by; y++)
        for (int x = xc * v.bx; x < xc * v.bx + v.bx; x++)
            for (int d = 0; d < v.nc_f; d++) {
                const long f = ((long)y * v.lx + x) * v.nc_f + d;
                p[f] = cmk(p[f].x / norm, p[f].y / norm);
            }
}

// block_normalize (mg_complex.cpp:191-257): one thread per (coarse site, vector)
__global__ void k_block_normalize(double2 *P, Lv v)
{
    const long n = (long)v.xc * v.yc * v.nc_c;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % v.nc_c);
        const long X = i / v.nc_c;
        const int yc = (int)(X / v.xc), xc = (int)(X - (long)yc * v.xc);
        double2 *p = P + (long)c * v.fsize;
        block_scale(v, p, xc, yc, block_norm(v, p, xc, yc));
    }
}

// block_orthonormalize (mg_complex.cpp:259-369): one thread per coarse site, modified
// Gram-Schmidt in the reference's order (normalise vector k-1, then project vector k against
// vectors 0..k-1); the final block_normalize is a separate launch
__global__ void k_block_orthogonalize(double2 *P, Lv v)
{
    const long n = (long)v.xc * v.yc;
    for (long X = blockIdx.x * (long)blockDim.x + threadIdx.x; X < n; X += (long)gridDim.x * blockDim.x) {
        const int yc = (int)(X / v.xc), xc = (int)(X - (long)yc * v.xc);
        for (int k = 1; k < v.nc_c; k++) {
            double2 *prev = P + (long)(k - 1) * v.fsize, *cur = P + (long)k * v.fsize;
            block_scale(v, prev, xc, yc, block_norm(v, prev, xc, yc));
            for (int m = 0; m < k; m++) {
                const double2 *pm = P + (long)m * v.fsize;
                double2 dot = cmk(0.0, 0.0);
                for (int y = yc * v.by; y < yc * v.by + v.by; y++)
                    for (int x = xc * v.bx; x < xc * v.bx + v.bx; x++)
                        for (int d = 0; d < v.nc_f; d++) {
                            const long f = ((long)y * v.lx + x) * v.nc_f + d;
                            dot = cadd(dot, cmul(cconj(pm[f]), cur[f]));
                        }
                for (int y = yc * v.by; y < yc * v.by + v.by; y++)
                    for (int x = xc * v.bx; x < xc * v.bx + v.bx; x++)
                        for (int d = 0; d < v.nc_f; d++) {
                            const long f = ((long)y * v.lx + x) * v.nc_f + d;
                            cur[f] = csub(cur[f], cmul(dot, pm[f]));
                        }
            }
        }
    }
}

struct FineSt {
    const double2 *clover, *hopping;
    double2 shift, eo_shift, dof_shift;
    bool with_shifts;
};

// Coarse clover and hopping entries (a, b) of block X: one thread per (X, a, b).
__global__ void k_coarse_stencil(double2 *__restrict__ cclov, double2 *__restrict__ chop, Lv v, FineSt fs)
{
    const int nc = v.nc_c, nf = v.nc_f;
    const long vc = (long)v.xc * v.yc, csize = vc * nc, fsize = v.fsize;
    const long n = vc * nc * nc;
    const int hx[4] = {1, 0, -1, 0}, hy[4] = {0, 1, 0, -1};
    const bool has_shift = fs.with_shifts && (fs.shift.x != 0.0 || fs.shift.y != 0.0);
    const bool has_eo = fs.with_shifts && (fs.eo_shift.x != 0.0 || fs.eo_shift.y != 0.0);
    const bool has_dof = fs.with_shifts && (fs.dof_shift.x != 0.0 || fs.dof_shift.y != 0.0);
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int b = (int)(t % nc);
        const long ia = t / nc;  // X * nc + a
        const int a = (int)(ia % nc);
        const long X = ia / nc;
        const int yc = (int)(X / v.xc), xc = (int)(X - (long)yc * v.xc);
        const double2 *Pa = v.P + (long)a * fsize, *Pb = v.P + (long)b * fsize;
        double2 acc[5] = {cmk(0, 0), cmk(0, 0), cmk(0, 0), cmk(0, 0), cmk(0, 0)};
        for (int y = yc * v.by; y < yc * v.by + v.by; y++) {
            for (int x = xc * v.bx; x < xc * v.bx + v.bx; x++) {
                const long s = (long)y * v.lx + x;
                for (int al = 0; al < nf; al++) {
                    const long fi = s * nf + al;
                    const double2 pa = cconj(Pa[fi]);
                    // clover and shifts: (A_0 P_b)(s, al)
                    double2 w = cmk(0.0, 0.0);
                    for (int be = 0; be < nf; be++) w = cadd(w, cmul(fs.clover[be + (long)nf * fi], Pb[s * nf + be]));
                    const double2 pb = Pb[fi];
                    if (has_shift) w = cadd(w, cmul(fs.shift, pb));
                    if (has_eo) w = cadd(w, cmul(cscale(((x + y) & 1) == 0 ? 1.0 : -1.0, fs.eo_shift), pb));
                    if (has_dof) w = cadd(w, cmul(cscale(al < nf / 2 ? 1.0 : -1.0, fs.dof_shift), pb));
                    acc[0] = cadd(acc[0], cmul(pa, w));
                    // the four hops: within the block -> clover, across a face -> that face's slot
                    for (int d = 0; d < 4; d++) {
                        int xx = x + hx[d], yy = y + hy[d];
                        xx = xx < 0 ? xx + v.lx : (xx >= v.lx ? xx - v.lx : xx);
                        yy = yy < 0 ? yy + v.ly : (yy >= v.ly ? yy - v.ly : yy);
                        const long tt = (long)yy * v.lx + xx;
                        const bool inside = (xx / v.bx == xc) && (yy / v.by == yc);
                        const bool wraps_self = (d % 2 == 0) ? v.xc == 1 : v.yc == 1;
                        const double2 *h = fs.hopping + (long)d * nf * fsize + (long)nf * fi;
                        double2 u = cmk(0.0, 0.0);
                        for (int be = 0; be < nf; be++) u = cadd(u, cmul(h[be], Pb[tt * nf + be]));
                        const int slot = (inside || wraps_self) ? 0 : 1 + d;
                        acc[slot] = cadd(acc[slot], cmul(pa, u));
                    }
                }
            }
        }
        const long e = (long)b + (long)nc * ia;
        cclov[e] = acc[0];
        for (int d = 0; d < 4; d++) chop[e + (long)d * nc * csize] = acc[1 + d];
    }
}

int grid(long n)
{
    const long g = (n + 255) / 256, cap = (long)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

glinalg_status check_level(glinalg_mg_level l)
{
    if (!l || !l->P) {
        set_last_error("null multigrid level");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    return GLINALG_SUCCESS;
}

}  // namespace

}  // namespace glinalg

using namespace glinalg;

extern "C" glinalg_status glinalg_mg_level_create(int lx, int ly, int nc_fine, int bx, int by, int nc_coarse,
                                                  const double *null_vectors, int flags, glinalg_mg_level *out)
{
    if (!out || !null_vectors) return invalid_arg("!out || !null_vectors");
    *out = nullptr;
    if (lx <= 0 || ly <= 0 || nc_fine <= 0 || bx <= 0 || by <= 0 || nc_coarse <= 0 || lx % bx || ly % by) {
        set_last_error("the block sizes must divide the lattice extents");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    GL_TRY(ensure_device());
    auto *l = new glinalg_mg_level_s();
    l->lx = lx;
    l->ly = ly;
    l->nc_f = nc_fine;
    l->bx = bx;
    l->by = by;
    l->nc_c = nc_coarse;
    l->xc = lx / bx;
    l->yc = ly / by;
    l->fsize = (long)lx * ly * nc_fine;
    l->csize = (long)l->xc * l->yc * nc_coarse;
    const size_t bytes = sizeof(double2) * (size_t)nc_coarse * l->fsize;
    cudaError_t e = cudaMalloc((void **)&l->P, bytes);
    if (e == cudaSuccess)
        e = cudaMemcpy(l->P, null_vectors, bytes, (flags & GLINALG_PTR_DEVICE) ? cudaMemcpyDeviceToDevice
                                                                              : cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_last_error(std::string("mg level: ") + cudaGetErrorString(e));
        delete l;
        return e == cudaErrorMemoryAllocation ? GLINALG_ERROR_OUT_OF_MEMORY : GLINALG_ERROR_CUDA;
    }
    *out = l;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_level_destroy(glinalg_mg_level l)
{
    delete l;
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_get_null_vectors(glinalg_mg_level l, double *out, int flags)
{
    GL_TRY(check_level(l));
    if (!out) return invalid_arg("!out");
    cudaStream_t st = lib_stream();
    GL_CUDA(cudaMemcpyAsync(out, l->P, sizeof(double2) * (size_t)l->nc_c * l->fsize,
                            (flags & GLINALG_PTR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_block_normalize(glinalg_mg_level l)
{
    GL_TRY(check_level(l));
    cudaStream_t st = lib_stream();
    k_block_normalize<<<grid(l->csize), 256, 0, st>>>(l->P, lv_of(l));
    GL_CUDA(cudaGetLastError());
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_block_orthonormalize(glinalg_mg_level l)
{
    GL_TRY(check_level(l));
    cudaStream_t st = lib_stream();
    k_block_orthogonalize<<<grid((long)l->xc * l->yc), 128, 0, st>>>(l->P, lv_of(l));
    k_block_normalize<<<grid(l->csize), 256, 0, st>>>(l->P, lv_of(l));
    GL_CUDA(cudaGetLastError());
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

namespace glinalg {

glinalg_status mg_prolong(const glinalg_mg_level_s *l, double2 *fine, const double2 *coarse, cudaStream_t st)
{
    k_prolong<<<grid(l->fsize), 256, 0, st>>>(fine, coarse, lv_of(l));
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

long mg_level_fine_size(const glinalg_mg_level_s *l) { return l->fsize; }
long mg_level_coarse_size(const glinalg_mg_level_s *l) { return l->csize; }

glinalg_status mg_restrict(const glinalg_mg_level_s *l, double2 *coarse, const double2 *fine, cudaStream_t st)
{
    k_restrict<<<grid(l->csize), 128, 0, st>>>(coarse, fine, lv_of(l));
    GL_CUDA(cudaGetLastError());
    return GLINALG_SUCCESS;
}

}  // namespace glinalg

static glinalg_status mg_transfer(glinalg_mg_level l, double *out, const double *in, int flags, bool up)
{
    GL_TRY(check_level(l));
    if (!out || !in) return invalid_arg("!out || !in");
    cudaStream_t st = lib_stream();
    Scratch sc(st);
    const long n_in = up ? l->csize : l->fsize, n_out = up ? l->fsize : l->csize;
    const bool dev = flags & GLINALG_PTR_DEVICE;
    double2 *d_in = (double2 *)in, *d_out = (double2 *)out;
    if (!dev) {
        GL_TRY(sc.alloc(&d_in, n_in));
        GL_TRY(sc.alloc(&d_out, n_out));
        GL_CUDA(cudaMemcpyAsync(d_in, in, sizeof(double2) * n_in, cudaMemcpyHostToDevice, st));
    }
    if (up) GL_TRY(mg_prolong(l, d_out, d_in, st));
    else GL_TRY(mg_restrict(l, d_out, d_in, st));
    if (!dev) GL_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double2) * n_out, cudaMemcpyDeviceToHost, st));
    GL_CUDA(cudaStreamSynchronize(st));
    return GLINALG_SUCCESS;
}

extern "C" glinalg_status glinalg_mg_prolong(glinalg_mg_level l, double *fine, const double *coarse, int flags)
{
    return mg_transfer(l, fine, coarse, flags, true);
}

extern "C" glinalg_status glinalg_mg_restrict(glinalg_mg_level l, double *coarse, const double *fine, int flags)
{
    return mg_transfer(l, coarse, fine, flags, false);
}

extern "C" glinalg_status glinalg_mg_coarse_stencil(glinalg_mg_level l, glinalg_operator fine, int ignore_shifts,
                                                    glinalg_operator *coarse_out)
{
    GL_TRY(check_level(l));
    if (!fine || !coarse_out) return invalid_arg("!fine || !coarse_out");
    *coarse_out = nullptr;
    if (fine->kind != GLINALG_OP_STENCIL || fine->nc != l->nc_f || fine->lx != l->lx || fine->ly != l->ly) {
        set_last_error("the fine operator must be a stencil (GLINALG_OP_STENCIL) on the level's fine lattice");
        return GLINALG_ERROR_INVALID_VALUE;
    }
    cudaStream_t st = lib_stream();
    auto *op = new glinalg_operator_s();
    op->kind = GLINALG_OP_STENCIL;
    op->lx = l->xc;
    op->ly = l->yc;
    op->nc = l->nc_c;
    op->vol = (long)l->xc * l->yc;
    op->size = l->csize;
    cudaGetDevice(&op->device);
    const long cc = op->vol * op->nc * op->nc;
    // (operator arrays come from the library's pool: the operator's destructor returns them there)
    cudaError_t e = lib_malloc_async((void **)&op->clover, sizeof(double2) * cc, st);
    if (e == cudaSuccess) e = lib_malloc_async((void **)&op->hopping, sizeof(double2) * 4 * cc, st);
    if (e != cudaSuccess) {
        set_last_error(std::string("coarse stencil: ") + cudaGetErrorString(e));
        delete op;
        return e == cudaErrorMemoryAllocation ? GLINALG_ERROR_OUT_OF_MEMORY : GLINALG_ERROR_CUDA;
    }
    FineSt fs{fine->clover, fine->hopping, fine->shift, fine->eo_shift, fine->dof_shift, ignore_shifts == 0};
    k_coarse_stencil<<<grid(cc), 128, 0, st>>>(op->clover, op->hopping, lv_of(l), fs);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(std::string("coarse stencil: ") + cudaGetErrorString(e));
        delete op;
        return GLINALG_ERROR_CUDA;
    }
    *coarse_out = op;
    return GLINALG_SUCCESS;
}
