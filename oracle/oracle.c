/*
 * oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 * Plain C99 with double _Complex.  GCC lowers complex * and / to the same C99 Annex G
 * sequences (__muldc3 / __divdc3 on the NaN path and for division) that libstdc++'s
 * std::complex<double> uses, so with -O2 -ffp-contract=off this file reproduces the
 * reference's floating-point operation order.  The ordering of every accumulation below is
 * deliberate: it follows the cited reference loop term by term.
 */
#include "oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <pthread.h>
#include <stdatomic.h>

typedef double _Complex cplx;

#define CX(p) ((cplx *)(p))
#define CCX(p) ((const cplx *)(p))

static inline cplx mk(double re, double im) { cplx z; __real__ z = re; __imag__ z = im; return z; }

/* ---------------------------------------------------------------- site-loop threads
 *
 * The reference is single-threaded.  Its site loops (operator applications, axpy-type
 * updates) compute every site independently, so spreading them over threads changes no bit
 * of any result.  Its reductions (dot, norm) are serial left-to-right sums; they stay serial,
 * in that order, on the calling thread.  par_ordered() overlaps such a sum with the parallel
 * pass that produces its terms: workers take fixed-size chunks in increasing order, and the
 * calling thread adds up each chunk, in order, once it is finished.  orc_set_threads(n) sets
 * the number of threads (default 1: the plain serial oracle).  A child process made by fork()
 * starts with no workers and recreates them on its first parallel loop. */

typedef void (*range_fn)(void *ctx, long lo, long hi);
typedef void (*task_fn)(void *ctx, int id, int parts);

#define ORC_MAX_THREADS 256
static struct {
    pthread_mutex_t mu;
    pthread_cond_t go, done;
    int nthreads;        /* threads used by a loop, the caller included */
    int nworkers;        /* workers started */
    unsigned long gen;   /* bumped per task */
    int pending;         /* workers still running the current task */
    task_fn fn;
    void *ctx;
    int parts;
} pool = {PTHREAD_MUTEX_INITIALIZER, PTHREAD_COND_INITIALIZER, PTHREAD_COND_INITIALIZER, 1, 0, 0, 0,
          NULL, NULL, 1};

/* generation current when worker j was started (under the pool lock, before the task that
 * started it bumped the generation), so a worker never misses that task */
static unsigned long worker_start_gen[ORC_MAX_THREADS];

static void *pool_worker(void *arg)
{
    int id = (int)(long)arg; /* 1 .. nworkers */
    pthread_mutex_lock(&pool.mu);
    unsigned long seen = worker_start_gen[id];
    for (;;) {
        while (pool.gen == seen) pthread_cond_wait(&pool.go, &pool.mu);
        seen = pool.gen;
        task_fn fn = pool.fn;
        void *ctx = pool.ctx;
        int parts = pool.parts;
        pthread_mutex_unlock(&pool.mu);
        if (id < parts) fn(ctx, id, parts);
        pthread_mutex_lock(&pool.mu);
        if (--pool.pending == 0) pthread_cond_signal(&pool.done);
    }
    return NULL;
}

static void pool_after_fork_child(void)
{
    pthread_mutex_init(&pool.mu, NULL);
    pthread_cond_init(&pool.go, NULL);
    pthread_cond_init(&pool.done, NULL);
    pool.nworkers = 0;
    pool.pending = 0;
}

void orc_set_threads(int n)
{
    static int atfork_done = 0;
    if (n < 1) n = 1;
    if (n > ORC_MAX_THREADS) n = ORC_MAX_THREADS;
    pthread_mutex_lock(&pool.mu);
    if (!atfork_done) {
        pthread_atfork(NULL, NULL, pool_after_fork_child);
        atfork_done = 1;
    }
    pool.nthreads = n;
    pthread_mutex_unlock(&pool.mu);
}

int orc_get_threads(void) { return pool.nthreads; }

/* Starts fn(ctx, id, parts) on workers id = 1 .. parts-1 and returns parts (the caller is
 * part 0 and runs its own share); pool_wait() then waits for the workers. */
static int pool_start(task_fn fn, void *ctx)
{
    int t = pool.nthreads;
    pthread_mutex_lock(&pool.mu);
    while (pool.nworkers < t - 1) {
        pthread_t th;
        worker_start_gen[pool.nworkers + 1] = pool.gen;
        if (pthread_create(&th, NULL, pool_worker, (void *)(long)(pool.nworkers + 1)) != 0) break;
        pthread_detach(th);
        pool.nworkers++;
    }
    int parts = pool.nworkers + 1 < t ? pool.nworkers + 1 : t;
    pool.fn = fn;
    pool.ctx = ctx;
    pool.parts = parts;
    pool.pending = pool.nworkers;
    pool.gen++;
    pthread_cond_broadcast(&pool.go);
    pthread_mutex_unlock(&pool.mu);
    return parts;
}

static void pool_wait(void)
{
    pthread_mutex_lock(&pool.mu);
    while (pool.pending > 0) pthread_cond_wait(&pool.done, &pool.mu);
    pthread_mutex_unlock(&pool.mu);
}

typedef struct {
    long n;
    range_fn fn;
    void *ctx;
} range_task_args;

static void range_task(void *ctx, int id, int parts)
{
    const range_task_args *r = (const range_task_args *)ctx;
    long lo = r->n * id / parts, hi = r->n * (id + 1) / parts;
    if (hi > lo) r->fn(r->ctx, lo, hi);
}

/* fn(ctx, lo, hi) over [0, n) split into contiguous ranges, one per thread. */
static void par_range(long n, range_fn fn, void *ctx)
{
    if (pool.nthreads <= 1 || n < 4096) {
        fn(ctx, 0, n);
        return;
    }
    range_task_args r = {n, fn, ctx};
    int parts = pool_start(range_task, &r);
    range_task(&r, 0, parts);
    pool_wait();
}

#define ORC_CHUNK 8192L
#define ORC_MAX_CHUNKS 65536L
static _Atomic unsigned long chunk_done[ORC_MAX_CHUNKS];
static unsigned long ordered_gen = 0;

typedef struct {
    long n, chunk, nch;
    range_fn work;
    void *ctx;
    _Atomic long next;
    unsigned long gen;
} ordered_args;

static void ordered_task(void *ctx, int id, int parts)
{
    ordered_args *o = (ordered_args *)ctx;
    (void)id;
    (void)parts;
    for (;;) {
        long c = atomic_fetch_add_explicit(&o->next, 1, memory_order_relaxed);
        if (c >= o->nch) break;
        long lo = c * o->chunk, hi = lo + o->chunk < o->n ? lo + o->chunk : o->n;
        o->work(o->ctx, lo, hi);
        atomic_store_explicit(&chunk_done[c], o->gen, memory_order_release);
    }
}

/* work(ctx, lo, hi) over [0, n) on the workers, chunk by chunk in increasing order, while the
 * calling thread runs sum(ctx, lo, hi) over the same chunks strictly in order, each once its
 * work is finished.  With one thread: work then sum per chunk, in order. */
static void par_ordered(long n, range_fn work, range_fn sum, void *ctx)
{
    long chunk = ORC_CHUNK;
    while ((n + chunk - 1) / chunk > ORC_MAX_CHUNKS) chunk *= 2;
    long nch = (n + chunk - 1) / chunk;
    if (pool.nthreads <= 1 || nch < 2) {
        for (long c = 0; c < nch; c++) {
            long lo = c * chunk, hi = lo + chunk < n ? lo + chunk : n;
            work(ctx, lo, hi);
            sum(ctx, lo, hi);
        }
        return;
    }
    ordered_args o;
    o.n = n;
    o.chunk = chunk;
    o.nch = nch;
    o.work = work;
    o.ctx = ctx;
    atomic_init(&o.next, 0);
    o.gen = ++ordered_gen;
    pool_start(ordered_task, &o);
    for (long c = 0; c < nch; c++) {
        long lo = c * chunk, hi = lo + chunk < n ? lo + chunk : n;
        while (atomic_load_explicit(&chunk_done[c], memory_order_acquire) != o.gen) {
            /* a worker holds this chunk; take an unclaimed one meanwhile if any is left */
            long d = atomic_fetch_add_explicit(&o.next, 1, memory_order_relaxed);
            if (d < nch) {
                long dlo = d * chunk, dhi = dlo + chunk < n ? dlo + chunk : n;
                work(ctx, dlo, dhi);
                atomic_store_explicit(&chunk_done[d], o.gen, memory_order_release);
            }
        }
        sum(ctx, lo, hi);
    }
    pool_wait();
}

/* ---------------------------------------------------------------- operators */

/* operator_utils/operators.cpp:184-239 (square_staggered_u1): hopping with eta_x = 1,
 * eta_y = (-1)^x, then 0.5 * sum, then + mass*psi.  sign = +1 for D, -1 for D^dagger
 * (operators.cpp:372-441 flips every hopping sign and keeps the mass). */
typedef struct {
    cplx *lhs;
    const cplx *rhs, *U;
    double mass, sign;
    int lx, ly;
} site_args;

static void staggered_range(void *ctx, long lo, long hi)
{
    const site_args *a = (const site_args *)ctx;
    cplx *lhs = a->lhs;
    const cplx *rhs = a->rhs, *U = a->U;
    const double mass = a->mass, sign = a->sign;
    const int lx = a->lx, ly = a->ly;
    /* the coordinates advance with i instead of being recomputed with % per site */
    int x = (int)(lo % lx), y = (int)(lo / lx);
    for (long i = lo; i < hi; i++) {
        double eta1 = (double)(1 - 2 * (x % 2));
        int xp = x + 1 == lx ? 0 : x + 1, xm = x == 0 ? lx - 1 : x - 1;
        int yp = y + 1 == ly ? 0 : y + 1, ym = y == 0 ? ly - 1 : y - 1;
        cplx acc = 0.0;
        cplx t;
        t = U[(long)y * lx * 2 + x * 2] * rhs[(long)y * lx + xp];
        acc = (sign > 0) ? acc - t : acc + t;
        t = conj(U[(long)y * lx * 2 + xm * 2]) * rhs[(long)y * lx + xm];
        acc = (sign > 0) ? acc + t : acc - t;
        t = (eta1 * U[(long)y * lx * 2 + x * 2 + 1]) * rhs[(long)yp * lx + x];
        acc = (sign > 0) ? acc - t : acc + t;
        t = (eta1 * conj(U[(long)ym * lx * 2 + x * 2 + 1])) * rhs[(long)ym * lx + x];
        acc = (sign > 0) ? acc + t : acc - t;
        acc = 0.5 * acc;
        acc = acc + mass * rhs[i];
        lhs[i] = acc;
        if (++x == lx) {
            x = 0;
            y++;
        }
    }
}

static void staggered_apply(cplx *lhs, const cplx *rhs, const cplx *U, double mass, int lx,
                            int ly, double sign)
{
    site_args a = {lhs, rhs, U, mass, sign, lx, ly};
    par_range((long)lx * ly, staggered_range, &a);
}

/* operator_utils/operators.cpp:73-120 (square_laplace_u1): lhs = (4+mass) psi
 * - sum_mu [U_mu(x) psi(x+mu) + U_mu(x-mu)^* psi(x-mu)], accumulated in the order
 * +x, -x, +y, -y, then the diagonal. */
static void laplace_range(void *ctx, long lo, long hi)
{
    const site_args *a = (const site_args *)ctx;
    cplx *lhs = a->lhs;
    const cplx *rhs = a->rhs, *U = a->U;
    const double mass = a->mass;
    const int lx = a->lx, ly = a->ly;
    int x = (int)(lo % lx), y = (int)(lo / lx);
    for (long i = lo; i < hi; i++) {
        int xp = x + 1 == lx ? 0 : x + 1, xm = x == 0 ? lx - 1 : x - 1;
        int yp = y + 1 == ly ? 0 : y + 1, ym = y == 0 ? ly - 1 : y - 1;
        cplx acc = 0.0;
        acc = acc - U[(long)y * lx * 2 + x * 2] * rhs[(long)y * lx + xp];
        acc = acc - conj(U[(long)y * lx * 2 + xm * 2]) * rhs[(long)y * lx + xm];
        acc = acc - U[(long)y * lx * 2 + x * 2 + 1] * rhs[(long)yp * lx + x];
        acc = acc - conj(U[(long)ym * lx * 2 + x * 2 + 1]) * rhs[(long)ym * lx + x];
        acc = acc + (4 + mass) * rhs[i];
        lhs[i] = acc;
        if (++x == lx) {
            x = 0;
            y++;
        }
    }
}

static void laplace_apply(cplx *lhs, const cplx *rhs, const cplx *U, double mass, int lx, int ly)
{
    site_args a = {lhs, rhs, U, mass, 0.0, lx, ly};
    par_range((long)lx * ly, laplace_range, &a);
}

/* stencil_2d/coarse_stencil.cpp:12-172 (apply_stencil_2d, DIR_ALL), :395-460 (_eo) and
 * :560-625 (_oe), :725-1117 (_tb) and :1120-1512 (_bt).  parity: 0 = full stencil, 1 = even
 * output sites only (hopping only), 2 = odd output sites only (hopping only), 3 = top half
 * of the colours out, bottom half in (clover, hopping and two-link, no shifts), 4 = bottom
 * out, top in.  Site parity is even when x+y is even
 * (lattice/lattice.h:128-139). */
static void stencil_apply(const orc_op *op, cplx *lhs, const cplx *rhs, int parity)
{
    const int lx = op->lx, ly = op->ly, nc = op->nc;
    const long vol = (long)lx * ly;
    const long lsize = vol * nc;
    const cplx *clov = CCX(op->clover), *hop = CCX(op->hopping), *two = CCX(op->two_link);
    const cplx shift = mk(op->shift[0], op->shift[1]);
    const cplx eo_shift = mk(op->eo_shift[0], op->eo_shift[1]);
    const cplx dof_shift = mk(op->dof_shift[0], op->dof_shift[1]);
    /* neighbour offsets in the reference's order: hopping {+x,+y,-x,-y}, two-link
     * {+2x,+x+y,+2y,-x+y,-2x,-x-y,-2y,+x-y} (coarse_stencil.h:44-54). */
    static const int hx[4] = {1, 0, -1, 0}, hy[4] = {0, 1, 0, -1};
    static const int tx[8] = {2, 1, 0, -1, -2, -1, 0, 1}, ty[8] = {0, 1, 2, 1, 0, -1, -2, -1};

    for (long i = 0; i < lsize; i++) {
        int color = (int)(i % nc);
        long site = i / nc;
        int x = (int)(site % lx), y = (int)(site / lx);
        int even = ((x + y) % 2) == 0;
        cplx acc = 0.0;
        if (parity == 1 && !even) { lhs[i] = 0.0; continue; }
        if (parity == 2 && even) { lhs[i] = 0.0; continue; }
        if (parity == 3 && color >= nc / 2) { lhs[i] = 0.0; continue; }
        if (parity == 4 && color < nc / 2) { lhs[i] = 0.0; continue; }
        /* tb (3) reads the bottom half of the input colours, bt (4) the top half */
        const int c0 = parity == 3 ? nc / 2 : 0, c1 = parity == 4 ? nc / 2 : nc;
        if (parity == 0 || parity >= 3)
            for (int c = c0; c < c1; c++) acc += clov[c + (long)nc * i] * rhs[site * nc + c];
        for (int d = 0; d < 4; d++) {
            int xx = (x + hx[d] + lx) % lx, yy = (y + hy[d] + ly) % ly;
            long nb = ((long)yy * lx + xx) * nc;
            for (int c = c0; c < c1; c++)
                acc += hop[c + (long)nc * i + (long)d * nc * lsize] * rhs[nb + c];
        }
        if ((parity == 0 || parity >= 3) && two != NULL) {
            for (int d = 0; d < 8; d++) {
                int xx = (x + tx[d] + 2 * lx) % lx, yy = (y + ty[d] + 2 * ly) % ly;
                long nb = ((long)yy * lx + xx) * nc;
                for (int c = c0; c < c1; c++)
                    acc += two[c + (long)nc * i + (long)d * nc * lsize] * rhs[nb + c];
            }
        }
        if (parity == 0) {
            if (cabs(shift) != 0.0) acc += shift * rhs[i];
            if (cabs(eo_shift) != 0.0) acc += ((even ? 1.0 : -1.0) * eo_shift) * rhs[i];
            if (cabs(dof_shift) != 0.0) acc += ((color < nc / 2 ? 1.0 : -1.0) * dof_shift) * rhs[i];
        }
        lhs[i] = acc;
    }
}

/* operator_utils/operators.cpp:455-497 (square_staggered_deo_u1) and :499-541
 * (square_staggered_doe_u1): the hopping part of square_staggered_u1 (no mass) at the even
 * (odd = 0) or odd (odd = 1) output sites, in the reference's order +x, -x, +y, -y, then the
 * factor 1/2; sites of the other parity are zeroed. */
static void hop_parity_range(void *ctx, long lo, long hi)
{
    const site_args *a = (const site_args *)ctx;
    cplx *lhs = a->lhs;
    const cplx *rhs = a->rhs, *U = a->U;
    const int lx = a->lx, ly = a->ly, odd = (int)a->sign;
    for (long i = lo; i < hi; i++) {
        int x = (int)(i % lx), y = (int)(i / lx);
        double eta1 = (double)(1 - 2 * (x % 2));
        lhs[i] = 0.0;
        if ((x + y) % 2 != odd) continue;
        int xp = (x + 1) % lx, xm = (x + lx - 1) % lx;
        int yp = (y + 1) % ly, ym = (y + ly - 1) % ly;
        cplx acc = 0.0;
        acc = acc - U[(long)y * lx * 2 + x * 2] * rhs[(long)y * lx + xp];
        acc = acc + conj(U[(long)y * lx * 2 + xm * 2]) * rhs[(long)y * lx + xm];
        acc = acc - (eta1 * U[(long)y * lx * 2 + x * 2 + 1]) * rhs[(long)yp * lx + x];
        acc = acc + (eta1 * conj(U[(long)ym * lx * 2 + x * 2 + 1])) * rhs[(long)ym * lx + x];
        lhs[i] = 0.5 * acc;
    }
}

/* (site loop spread over the pool; each site is independent, so the result is the serial
 * loop's bit for bit) */
static void staggered_hop_parity(cplx *lhs, const cplx *rhs, const cplx *U, int lx, int ly, int odd)
{
    site_args a = {lhs, rhs, U, 0.0, (double)odd, lx, ly};
    par_range((long)lx * ly, hop_parity_range, &a);
}

static int site_even(long i, int lx) { return ((i % lx) + (i / lx)) % 2 == 0; }

/* operators.cpp:566-589 (square_staggered_m2mdeodoe_u1): tmp = D_oe rhs; lhs = D_eo tmp;
 * lhs = m*m rhs - lhs on even sites (odd sites stay zero).  The stencil form
 * (operators_stencil.cpp:195-216, apply_square_staggered_m2mdeodoe_stencil) uses
 * apply_stencil_2d_oe / _eo and shift*shift. */
static void m2m_even_range(void *ctx, long lo, long hi)
{
    const site_args *a = (const site_args *)ctx;
    const double m2 = a->mass * a->mass;
    for (long i = lo; i < hi; i++)
        if (site_even(i, a->lx)) a->lhs[i] = m2 * a->rhs[i] - a->lhs[i];
}

static void m2mdeodoe_apply(const orc_op *op, cplx *lhs, const cplx *rhs)
{
    const long v = (long)op->lx * op->ly;
    /* the intermediate D_oe rhs, kept between calls (the oracle is driven from one thread) */
    static cplx *tmp = NULL;
    static long tmp_n = 0;
    if (tmp_n < v) {
        free(tmp);
        tmp = (cplx *)malloc(sizeof(cplx) * v);
        tmp_n = tmp ? v : 0;
        if (!tmp) return;
    }
    if (op->kind == ORC_STAGGERED_M2MDEODOE) {
        staggered_hop_parity(tmp, rhs, CCX(op->links), op->lx, op->ly, 1);
        staggered_hop_parity(lhs, tmp, CCX(op->links), op->lx, op->ly, 0);
        site_args a = {lhs, rhs, NULL, op->mass, 0.0, op->lx, op->ly};
        par_range(v, m2m_even_range, &a);
    } else {
        const cplx shift = mk(op->shift[0], op->shift[1]);
        stencil_apply(op, tmp, rhs, 2);
        stencil_apply(op, lhs, tmp, 1);
        for (long i = 0; i < v; i++)
            if (site_even(i, op->lx)) lhs[i] = (shift * shift) * rhs[i] - lhs[i];
    }
}

/* operators.cpp:543-563 (square_staggered_eoprec_prepare) and operators_stencil.cpp:179-193
 * (apply_square_staggered_eoprec_prepare_stencil): rhs_e = D_eo rhs (odd sites zeroed), then
 * rhs_e = m rhs - rhs_e on even sites (the stencil form: shift rhs - rhs_e). */
void orc_eoprec_prepare(const orc_op *op, double *rhs_e_, const double *rhs_)
{
    cplx *rhs_e = CX(rhs_e_);
    const cplx *rhs = CCX(rhs_);
    const long v = (long)op->lx * op->ly;
    if (op->kind == ORC_STAGGERED_M2MDEODOE) {
        staggered_hop_parity(rhs_e, rhs, CCX(op->links), op->lx, op->ly, 0);
        for (long i = 0; i < v; i++)
            if (site_even(i, op->lx)) rhs_e[i] = op->mass * rhs[i] - rhs_e[i];
    } else {
        const cplx shift = mk(op->shift[0], op->shift[1]);
        stencil_apply(op, rhs_e, rhs, 1);
        for (long i = 0; i < v; i++)
            if (site_even(i, op->lx)) rhs_e[i] = shift * rhs[i] - rhs_e[i];
    }
}

/* operators.cpp:592-620 (square_staggered_eoprec_reconstruct) and operators_stencil.cpp:218-236
 * (apply_square_staggered_eoprec_reconstruct_stencil): lhs_full = D_oe lhs_e; odd sites
 * become inv_mass (rhs_o - lhs_full) with inv_mass = 1/m (the stencil form: 1/Re(shift)), even
 * sites copy lhs_e. */
void orc_eoprec_reconstruct(const orc_op *op, double *lhs_full_, const double *lhs_e_, const double *rhs_o_)
{
    cplx *lhs_full = CX(lhs_full_);
    const cplx *lhs_e = CCX(lhs_e_), *rhs_o = CCX(rhs_o_);
    const long v = (long)op->lx * op->ly;
    double inv_mass;
    if (op->kind == ORC_STAGGERED_M2MDEODOE) {
        inv_mass = 1.0 / op->mass;
        staggered_hop_parity(lhs_full, lhs_e, CCX(op->links), op->lx, op->ly, 1);
    } else {
        inv_mass = 1.0 / op->shift[0];
        stencil_apply(op, lhs_full, lhs_e, 2);
    }
    for (long i = 0; i < v; i++) {
        if (!site_even(i, op->lx)) lhs_full[i] = inv_mass * (rhs_o[i] - lhs_full[i]);
        else lhs_full[i] = lhs_e[i];
    }
}

/* The stencil operators of multigrid/aa_mg/mg_complex.cpp:1228-1375, nc = lattice colours:
 *   m^2 - D_tb D_bt (top rows; bottom zeroed)           :1228-1249
 *   m^2 - D_eo D_oe - D_oe D_eo                          :1277-1302
 *   m^2 - D_tb D_bt - D_bt D_tb                          :1305-1330
 *   epsilon D epsilon (epsilon = +1 on even sites)       :1335-1352
 *   sigma3 D sigma3 (sigma3 = +1 on the top colours)     :1355-1372
 * with m = the stencil's shift (complex, squared as shift * shift). */
static void coarse_pieces_apply(const orc_op *op, cplx *lhs, const cplx *rhs)
{
    const int nc = op->nc;
    const long n = (long)op->lx * op->ly * nc;
    const cplx shift = mk(op->shift[0], op->shift[1]);
    cplx *tmp = (cplx *)calloc(n, sizeof(cplx));
    cplx *tmp2 = (cplx *)calloc(n, sizeof(cplx));
    long i;
    switch (op->kind) {
    case ORC_STENCIL_M2MDTBDBT:
        stencil_apply(op, tmp, rhs, 4);
        stencil_apply(op, lhs, tmp, 3);
        for (i = 0; i < n; i++)
            if ((int)(i % nc) < nc / 2) lhs[i] = shift * shift * rhs[i] - lhs[i];
        break;
    case ORC_STENCIL_NORMAL_EO:
    case ORC_STENCIL_NORMAL_TB: {
        const int a = op->kind == ORC_STENCIL_NORMAL_EO ? 1 : 3, b = op->kind == ORC_STENCIL_NORMAL_EO ? 2 : 4;
        stencil_apply(op, tmp2, rhs, a);
        stencil_apply(op, lhs, tmp2, b);
        stencil_apply(op, tmp2, rhs, b);
        stencil_apply(op, tmp, tmp2, a);
        for (i = 0; i < n; i++) lhs[i] = shift * shift * rhs[i] - lhs[i] - tmp[i];
        break;
    }
    case ORC_STENCIL_DAGGER_EO:
    case ORC_STENCIL_DAGGER_TB: {
        /* lattice_epsilon / lattice_sigma3 (lattice/lattice_functions.h:11-55) */
        const int eo = op->kind == ORC_STENCIL_DAGGER_EO;
        for (int pass = 0; pass < 2; pass++) {
            const cplx *src = pass == 0 ? rhs : tmp;
            for (i = 0; i < n; i++) {
                long site = i / nc;
                int x = (int)(site % op->lx), y = (int)(site / op->lx);
                int plus = eo ? ((x + y) % 2 == 0) : (nc % 2 != 0 || (int)(i % nc) < nc / 2);
                lhs[i] = plus ? src[i] : -src[i];
            }
            if (pass == 0) stencil_apply(op, tmp, lhs, 0);
        }
        break;
    }
    default: break;
    }
    free(tmp);
    free(tmp2);
}

/* apply_square_staggered_tbprec_prepare_stencil / _reconstruct_stencil
 * (mg_complex.cpp:1211-1225 / :1252-1274): rhs_t = m rhs - D_tb rhs on the top colours
 * (bottom zeroed); lhs_full = lhs_t on the top colours, (rhs_b - D_bt lhs_t) / Re(m) on the
 * bottom ones. */
void orc_tbprec_prepare(const orc_op *op, double *rhs_t_, const double *rhs_)
{
    cplx *rhs_t = CX(rhs_t_);
    const cplx *rhs = CCX(rhs_);
    const long n = (long)op->lx * op->ly * op->nc;
    const cplx shift = mk(op->shift[0], op->shift[1]);
    stencil_apply(op, rhs_t, rhs, 3);
    for (long i = 0; i < n; i++)
        if ((int)(i % op->nc) < op->nc / 2) rhs_t[i] = shift * rhs[i] - rhs_t[i];
}

void orc_tbprec_reconstruct(const orc_op *op, double *lhs_full_, const double *lhs_t_, const double *rhs_b_)
{
    cplx *lhs_full = CX(lhs_full_);
    const cplx *lhs_t = CCX(lhs_t_), *rhs_b = CCX(rhs_b_);
    const long n = (long)op->lx * op->ly * op->nc;
    const double inv_mass = 1.0 / op->shift[0];
    stencil_apply(op, lhs_full, lhs_t, 4);
    for (long i = 0; i < n; i++) {
        if ((int)(i % op->nc) >= op->nc / 2) lhs_full[i] = inv_mass * (rhs_b[i] - lhs_full[i]);
        else lhs_full[i] = lhs_t[i];
    }
}

long orc_op_size(const orc_op *op)
{
    long v = (long)op->lx * op->ly;
    if ((op->kind >= ORC_STENCIL && op->kind <= ORC_STENCIL_OE) || op->kind >= ORC_STENCIL_TB) v *= op->nc;
    return v;
}

void orc_apply(const orc_op *op, double *lhs, const double *rhs)
{
    const cplx *U = CCX(op->links);
    switch (op->kind) {
    case ORC_STAGGERED:
        staggered_apply(CX(lhs), CCX(rhs), U, op->mass, op->lx, op->ly, +1.0);
        break;
    case ORC_STAGGERED_DAGGER:
        staggered_apply(CX(lhs), CCX(rhs), U, op->mass, op->lx, op->ly, -1.0);
        break;
    case ORC_STAGGERED_NORMAL: {
        /* operators.cpp:444-453: tmp = D rhs; lhs = D^dagger tmp. */
        long v = (long)op->lx * op->ly;
        cplx *tmp = (cplx *)malloc(sizeof(cplx) * v);
        staggered_apply(tmp, CCX(rhs), U, op->mass, op->lx, op->ly, +1.0);
        staggered_apply(CX(lhs), tmp, U, op->mass, op->lx, op->ly, -1.0);
        free(tmp);
        break;
    }
    case ORC_LAPLACE:
        laplace_apply(CX(lhs), CCX(rhs), U, op->mass, op->lx, op->ly);
        break;
    case ORC_STENCIL: stencil_apply(op, CX(lhs), CCX(rhs), 0); break;
    case ORC_STENCIL_EO: stencil_apply(op, CX(lhs), CCX(rhs), 1); break;
    case ORC_STENCIL_OE: stencil_apply(op, CX(lhs), CCX(rhs), 2); break;
    case ORC_STAGGERED_DEO: staggered_hop_parity(CX(lhs), CCX(rhs), U, op->lx, op->ly, 0); break;
    case ORC_STAGGERED_DOE: staggered_hop_parity(CX(lhs), CCX(rhs), U, op->lx, op->ly, 1); break;
    case ORC_STAGGERED_M2MDEODOE:
    case ORC_STENCIL_M2MDEODOE: m2mdeodoe_apply(op, CX(lhs), CCX(rhs)); break;
    case ORC_STENCIL_TB: stencil_apply(op, CX(lhs), CCX(rhs), 3); break;
    case ORC_STENCIL_BT: stencil_apply(op, CX(lhs), CCX(rhs), 4); break;
    case ORC_STENCIL_M2MDTBDBT:
    case ORC_STENCIL_NORMAL_EO:
    case ORC_STENCIL_NORMAL_TB:
    case ORC_STENCIL_DAGGER_EO:
    case ORC_STENCIL_DAGGER_TB: coarse_pieces_apply(op, CX(lhs), CCX(rhs)); break;
    default: break;
    }
}

/* operator_utils/operators_stencil.cpp:14-63 (get_square_staggered_u1_stencil) and
 * :120-169 (get_square_staggered_dagger_u1_stencil): hopping = {-1/2 U_x(x),
 * -1/2 eta U_y(x), +1/2 U_x(x-x)^*, +1/2 eta U_y(x-y)^*}, negated for the dagger. */
void orc_staggered_stencil(double *hopping, const double *links, int lx, int ly, int dagger)
{
    cplx *H = CX(hopping);
    const cplx *U = CCX(links);
    const long vol = (long)lx * ly;
    const double s = dagger ? -1.0 : 1.0;
    for (long i = 0; i < vol; i++) {
        int x = (int)(i % lx), y = (int)(i / lx);
        int eta1 = 1 - 2 * (x % 2);
        long im_x = (long)y * lx + (x - 1 + lx) % lx;
        long im_y = (long)((y - 1 + ly) % ly) * lx + x;
        H[i] = (-0.5 * s) * U[2 * i];
        H[i + vol] = ((-0.5 * s) * eta1) * U[2 * i + 1];
        H[i + 2 * vol] = (0.5 * s) * conj(U[2 * im_x]);
        H[i + 3 * vol] = ((0.5 * s) * eta1) * conj(U[2 * im_y + 1]);
    }
}

/* ---------------------------------------------------------------- BLAS-1 */

/* generic_vector.h:102-114: res = sum conj(a_i) b_i, serial left to right. */
static cplx cdot(const cplx *a, const cplx *b, long n)
{
    cplx r = 0.0;
    for (long i = 0; i < n; i++) r = r + conj(a[i]) * b[i];
    return r;
}

/* generic_vector.h:132-145 */
static double cnorm2(const cplx *a, long n)
{
    double r = 0.0;
    for (long i = 0; i < n; i++) r = r + creal(conj(a[i]) * a[i]);
    return r;
}

/* generic_vector.h:160-169 */
static double cdiffnorm2(const cplx *a, const cplx *b, long n)
{
    double r = 0.0;
    for (long i = 0; i < n; i++) r = r + creal(conj(a[i] - b[i]) * (a[i] - b[i]));
    return r;
}

void orc_dot(const double *a, const double *b, long n, double out[2])
{
    cplx r = cdot(CCX(a), CCX(b), n);
    out[0] = creal(r);
    out[1] = cimag(r);
}
double orc_norm2sq(const double *a, long n) { return cnorm2(CCX(a), n); }
double orc_diffnorm2sq(const double *a, const double *b, long n) { return cdiffnorm2(CCX(a), CCX(b), n); }

/* libstdc++'s real / complex constructs complex(x, 0) and divides (operator/(T, complex)). */
static inline cplx rdivc(double x, cplx y) { return mk(x, 0.0) / y; }
/* libstdc++'s complex / real divides each component (complex::operator/=(T)). */
static inline cplx cdivr(cplx x, double y) { return mk(creal(x) / y, cimag(x) / y); }

static void record(double *hist, int cap, int k, double v)
{
    if (hist != NULL && k >= 0 && k < cap) hist[k] = v;
}

static void set_name(orc_info *info, const char *name)
{
    strncpy(info->name, name, sizeof(info->name) - 1);
    info->name[sizeof(info->name) - 1] = 0;
}

/* Site-parallel forms of the solvers' update loops.  Each writes the same expression, in the
 * same operation order, as the serial loop it replaces. */
typedef struct {
    cplx *x, *r, *p;
    const cplx *Ap;
    cplx a;
    cplx **xs, **ps;          /* multishift: per-shift solution and direction vectors */
    const cplx *as, *bs;      /* multishift: per-shift scalars */
    int ns;
} upd_args;

/* x = x + a p; r = r - a Ap (generic_cg.cpp:320-324) */
static void upd_xr_range(void *ctx, long lo, long hi)
{
    const upd_args *u = (const upd_args *)ctx;
    for (long i = lo; i < hi; i++) {
        u->x[i] = u->x[i] + u->a * u->p[i];
        u->r[i] = u->r[i] - u->a * u->Ap[i];
    }
}

/* p = r + a p (generic_cg.cpp:343-346; generic_cg_m.cpp:515-518) */
static void upd_p_range(void *ctx, long lo, long hi)
{
    const upd_args *u = (const upd_args *)ctx;
    for (long i = lo; i < hi; i++) u->p[i] = u->r[i] + u->a * u->p[i];
}

/* r = r + a Ap (generic_cg_m.cpp:424-427) */
static void upd_r_range(void *ctx, long lo, long hi)
{
    const upd_args *u = (const upd_args *)ctx;
    for (long i = lo; i < hi; i++) u->r[i] = u->r[i] + u->a * u->Ap[i];
}

/* every live shift n: x_n = x_n - bs[n] p_n (generic_cg_m.cpp:410-413) */
static void upd_shift_x_range(void *ctx, long lo, long hi)
{
    const upd_args *u = (const upd_args *)ctx;
    for (int n = 0; n < u->ns; n++) {
        cplx *x = u->xs[n];
        const cplx *ps = u->ps[n];
        const cplx b = u->bs[n];
        for (long i = lo; i < hi; i++) x[i] = x[i] - b * ps[i];
    }
}

/* every live shift n: p_n = as[n] r + bs[n] p_n (generic_cg_m.cpp:505-512; as = zeta_s,
 * bs = alpha_s) */
static void upd_shift_p_range(void *ctx, long lo, long hi)
{
    const upd_args *u = (const upd_args *)ctx;
    for (int n = 0; n < u->ns; n++) {
        cplx *ps = u->ps[n];
        const cplx z = u->as[n], a = u->bs[n];
        for (long i = lo; i < hi; i++) ps[i] = z * u->r[i] + a * ps[i];
    }
}

/* The CG's reductions fused with the passes that produce their terms (par_ordered): the
 * terms are formed and added in the serial loops' order, so the sums are those of cdot and
 * cnorm2 bit for bit. */
typedef struct {
    site_args st;          /* the D^dagger pass of D^dagger D */
    const cplx *a, *b;     /* dot: sum conj(a_i) b_i */
    cplx dot;
    upd_args *upd;         /* the x / r update */
    double nrm;            /* norm: sum |r_i|^2 */
} fused_args;

static void fused_stag_work(void *ctx, long lo, long hi) { staggered_range(&((fused_args *)ctx)->st, lo, hi); }

static void fused_dot_sum(void *ctx, long lo, long hi)
{
    fused_args *f = (fused_args *)ctx;
    cplx r = f->dot;
    for (long i = lo; i < hi; i++) r = r + conj(f->a[i]) * f->b[i];
    f->dot = r;
}

static void fused_xr_work(void *ctx, long lo, long hi) { upd_xr_range(((fused_args *)ctx)->upd, lo, hi); }

static void fused_norm_sum(void *ctx, long lo, long hi)
{
    fused_args *f = (fused_args *)ctx;
    const cplx *r_ = f->upd->r;
    double r = f->nrm;
    for (long i = lo; i < hi; i++) r = r + creal(conj(r_[i]) * r_[i]);
    f->nrm = r;
}

/* Ap = op(p) and returns <p, Ap> (cdot order).  The staggered normal operator runs its D^dagger
 * pass with the dot fused in; other operators apply, then reduce. */
static cplx apply_dot(const orc_op *op, cplx *Ap, const cplx *p, long size, cplx *tmp)
{
    if (op->kind != ORC_STAGGERED_NORMAL || tmp == NULL) {
        orc_apply(op, (double *)Ap, (const double *)p);
        return cdot(p, Ap, size);
    }
    staggered_apply(tmp, p, CCX(op->links), op->mass, op->lx, op->ly, +1.0);
    fused_args f;
    site_args st = {Ap, tmp, CCX(op->links), op->mass, -1.0, op->lx, op->ly};
    f.st = st;
    f.a = p;
    f.b = Ap;
    f.dot = 0.0;
    par_ordered(size, fused_stag_work, fused_dot_sum, &f);
    return f.dot;
}

/* x += alpha p; r -= alpha Ap, and returns |r|^2 (cnorm2 order). */
static double update_xr_norm(upd_args *u, long size)
{
    fused_args f;
    f.upd = u;
    f.nrm = 0.0;
    par_ordered(size, fused_xr_work, fused_norm_sum, &f);
    return f.nrm;
}

/* ---------------------------------------------------------------- CG */

/* generic_cg.cpp:278-382 (complex minv_vector_cg). */
void orc_cg(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
            double eps, orc_info *info, double *hist, int hist_cap)
{
    cplx *phi = CX(phi_);
    const cplx *phi0 = CCX(phi0_);
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta;
    double rsq, rsqNew = 0.0, bsqrt, truersq;
    int k, ops = 0;
    long i;

    cplx *tmp = (op->kind == ORC_STAGGERED_NORMAL) ? (cplx *)malloc(sizeof(cplx) * size) : NULL;
    cplx pAp;

    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)p, (const double *)phi); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - p[i];
    memcpy(p, r, sizeof(cplx) * size);
    /* <p, Ap> is formed with Ap (below and at the end of each iteration) rather than at the
     * top of the next iteration: p and Ap do not change in between */
    pAp = apply_dot(op, Ap, p, size, tmp); ops++;
    rsq = cnorm2(r, size);
    upd_args upd = {phi, r, p, Ap, 0.0, NULL, NULL, NULL, NULL, 0};

    for (k = 0; k < max_iter; k++) {
        alpha = rdivc(rsq, pAp);
        upd.a = alpha;
        rsqNew = update_xr_norm(&upd, size);
        record(hist, hist_cap, k, sqrt(rsqNew) / bsqrt);
        if (sqrt(rsqNew) < eps * bsqrt || k == max_iter - 1) break;
        beta = mk(rsqNew / rsq, 0.0);
        rsq = rsqNew;
        upd.a = beta;
        par_range(size, upd_p_range, &upd);
        pAp = apply_dot(op, Ap, p, size, tmp); ops++;
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    k++;
    orc_apply(op, (double *)Ap, (const double *)phi); ops++;
    truersq = cdiffnorm2(Ap, phi0, size);
    free(r); free(p); free(Ap); free(tmp);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "CG");
}

/* Restart driver shared by CG / BiCGstab / GCR: generic_cg.cpp:387-427,
 * generic_bicgstab.cpp:345-385, generic_gcr.cpp:337-378. */
typedef void (*orc_solver_fn)(const orc_op *, double *, const double *, long, int, double,
                              orc_info *, double *, int);

static void restart_driver(orc_solver_fn fn, const char *base, const orc_op *op, double *phi,
                           const double *phi0, long size, int max_iter, double res,
                           int restart_freq, orc_info *info)
{
    double bsqrt = sqrt(cnorm2(CCX(phi0), size));
    int iter = 0, ops = 0;
    orc_info inner;
    memset(&inner, 0, sizeof(inner));
    do {
        fn(op, phi, phi0, size, restart_freq, res, &inner, NULL, 0);
        iter += inner.iter;
        ops += inner.ops_count;
    } while (iter < max_iter && inner.success == 0 && sqrt(inner.resSq) / bsqrt > res);
    *info = inner;
    info->iter = iter;
    info->ops_count = ops;
    info->success = (sqrt(inner.resSq) / bsqrt > res) ? 0 : 1;
    char nm[32];
    snprintf(nm, sizeof(nm), "%s(%d)", base, restart_freq);
    set_name(info, nm);
}

void orc_cg_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                    double eps, int restart_freq, orc_info *info)
{
    restart_driver(orc_cg, "CG", op, phi, phi0, size, max_iter, eps, restart_freq, info);
}

/* ---------------------------------------------------------------- BiCGstab */

/* generic_bicgstab.cpp:205-341 (complex minv_vector_bicgstab). */
void orc_bicgstab(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
                  double eps, orc_info *info, double *hist, int hist_cap)
{
    cplx *phi = CX(phi_);
    const cplx *phi0 = CCX(phi0_);
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *r0 = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx *s = (cplx *)calloc(size, sizeof(cplx));
    cplx *As = (cplx *)calloc(size, sizeof(cplx));
    cplx rho, rhoNew, alpha, beta, omega;
    double rsq, bsqrt, truersq;
    int k, ops = 0;
    long i;

    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)Ap, (const double *)phi); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - Ap[i];
    memcpy(r0, r, sizeof(cplx) * size);
    memcpy(p, r, sizeof(cplx) * size);
    rho = cdot(r0, r, size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;

    for (k = 0; k < max_iter; k++) {
        alpha = rho / cdot(r0, Ap, size);
        for (i = 0; i < size; i++) s[i] = r[i] - alpha * Ap[i];
        orc_apply(op, (double *)As, (const double *)s); ops++;
        omega = cdot(As, s, size) / cdot(As, As, size);
        for (i = 0; i < size; i++) phi[i] = phi[i] + alpha * p[i] + omega * s[i];
        for (i = 0; i < size; i++) r[i] = s[i] - omega * As[i];
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);
        if (sqrt(rsq) < eps * bsqrt || k == max_iter - 1) break;
        rhoNew = cdot(r0, r, size);
        beta = rhoNew / rho * (alpha / omega);
        rho = rhoNew;
        for (i = 0; i < size; i++) p[i] = r[i] + beta * (p[i] - omega * Ap[i]);
        orc_apply(op, (double *)Ap, (const double *)p); ops++;
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    k++;
    orc_apply(op, (double *)Ap, (const double *)phi); ops++;
    truersq = cdiffnorm2(Ap, phi0, size);
    free(r); free(r0); free(p); free(Ap); free(s); free(As);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "BiCGStab");
}

void orc_bicgstab_restart(const orc_op *op, double *phi, const double *phi0, long size,
                          int max_iter, double eps, int restart_freq, orc_info *info)
{
    restart_driver(orc_bicgstab, "BiCGStab", op, phi, phi0, size, max_iter, eps, restart_freq, info);
}

/* ---------------------------------------------------------------- GCR */

/* generic_gcr.cpp:202-333 (complex minv_vector_gcr): every search direction p_i and A p_i
 * is kept and the new direction is A-orthogonalised against all of them. */
void orc_gcr(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
             double eps, orc_info *info, double *hist, int hist_cap)
{
    cplx *phi = CX(phi_);
    const cplx *phi0 = CCX(phi0_);
    cplx *x = (cplx *)calloc(size, sizeof(cplx));
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ar = (cplx *)calloc(size, sizeof(cplx));
    int cap = (max_iter > 0 ? max_iter : 1) + 1;
    cplx **ps = (cplx **)calloc(cap, sizeof(cplx *));
    cplx **Aps = (cplx **)calloc(cap, sizeof(cplx *));
    int nstore = 0;
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta_ij;
    double rsq, bsqrt, truersq = 0.0;
    int k, ops = 0, ii;
    long i;

    memcpy(x, phi, sizeof(cplx) * size);
    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)p, (const double *)x); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - p[i];
    memcpy(p, r, sizeof(cplx) * size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;

    for (k = 0; k < max_iter; k++) {
        ps[nstore] = p;
        Aps[nstore] = Ap;
        nstore++;
        alpha = cdivr(cdot(Ap, r, size), cnorm2(Ap, size));
        for (i = 0; i < size; i++) {
            x[i] = x[i] + alpha * p[i];
            r[i] = r[i] - alpha * Ap[i];
        }
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);
        if (sqrt(rsq) < eps * bsqrt || k == max_iter - 1) break;
        orc_apply(op, (double *)Ar, (const double *)r); ops++;
        p = (cplx *)malloc(sizeof(cplx) * size);
        memcpy(p, r, sizeof(cplx) * size);
        Ap = (cplx *)malloc(sizeof(cplx) * size);
        memcpy(Ap, Ar, sizeof(cplx) * size);
        for (ii = 0; ii <= k; ii++) {
            beta_ij = cdivr(-cdot(Aps[ii], Ar, size), cnorm2(Aps[ii], size));
            for (i = 0; i < size; i++) {
                p[i] += beta_ij * ps[ii][i];
                Ap[i] += beta_ij * Aps[ii][i];
            }
        }
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    k++;
    /* the true-residual check reuses a scratch vector (generic_gcr.cpp:303-305) */
    cplx *chk = (cplx *)calloc(size, sizeof(cplx));
    orc_apply(op, (double *)chk, (const double *)x); ops++;
    for (i = 0; i < size; i++) truersq += creal(conj(chk[i] - phi0[i]) * (chk[i] - phi0[i]));
    memcpy(phi, x, sizeof(cplx) * size);
    free(chk);
    /* when the loop ran zero times the initial p / Ap were never stored */
    if (nstore == 0) { free(p); free(Ap); }
    for (ii = 0; ii < nstore; ii++) { free(ps[ii]); free(Aps[ii]); }
    free(ps); free(Aps); free(x); free(r); free(Ar);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "GCR");
}

void orc_gcr_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                     double eps, int restart_freq, orc_info *info)
{
    restart_driver(orc_gcr, "GCR", op, phi, phi0, size, max_iter, eps, restart_freq, info);
}

/* ---------------------------------------------------------------- CG-M */

/* generic_cg_m.cpp:312-600 (complex minv_vector_cg_m, Jegerlehner hep-lat/9612014).
 * Converged shifts are swapped to the tail (:434-486) and the order is restored at the
 * end (:533-558); here the permutation acts on local index tables, which is observably the
 * same as the reference's in-place permutation of the caller's phi[] and shifts[]. */
void orc_cg_m(const orc_op *op, double *phi_all, const double *phi0_, int n_shift, long size,
              int resid_freq_check, int max_iter, double eps, const double *shifts_in,
              int worst_first, orc_info *info, double *resSqmrhs, double *hist, int hist_cap)
{
    const cplx *phi0 = CCX(phi0_);
    cplx **phi = (cplx **)malloc(sizeof(cplx *) * n_shift);
    cplx **p_s = (cplx **)malloc(sizeof(cplx *) * n_shift);
    cplx *alpha_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *beta_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *zeta_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *zeta_s_prev = (cplx *)malloc(sizeof(cplx) * n_shift);
    double *shifts = (double *)malloc(sizeof(double) * n_shift);
    int *mapping = (int *)malloc(sizeof(int) * n_shift);
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta, beta_prev, tmp;
    double rsq, rsqNew = 0.0, bsqrt;
    int k, n, n_shift_rem = n_shift, ops = 0;
    long i;

    for (n = 0; n < n_shift; n++) {
        phi[n] = CX(phi_all) + (long)n * size;
        p_s[n] = (cplx *)malloc(sizeof(cplx) * size);
        mapping[n] = n;
        shifts[n] = shifts_in[n];
        beta_s[n] = zeta_s[n] = zeta_s_prev[n] = 1.0;
        alpha_s[n] = 0.0;
    }
    beta = 1.0;
    alpha = 0.0;
    bsqrt = sqrt(cnorm2(phi0, size));
    for (n = 0; n < n_shift; n++) {
        memcpy(p_s[n], phi0, sizeof(cplx) * size);
        memset(phi[n], 0, sizeof(cplx) * size);
    }
    memcpy(p, phi0, sizeof(cplx) * size);
    memcpy(r, phi0, sizeof(cplx) * size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;
    rsq = cnorm2(r, size);
    upd_args mupd = {NULL, r, p, Ap, 0.0, phi, p_s, NULL, NULL, 0};

    for (k = 0; k < max_iter; k++) {
        beta_prev = beta;
        beta = rdivc(-rsq, cdot(p, Ap, size));
        for (n = 0; n < n_shift_rem; n++) {
            tmp = zeta_s[n];
            zeta_s[n] = (zeta_s[n] * zeta_s_prev[n] * beta_prev) /
                        (beta * alpha * (zeta_s_prev[n] - zeta_s[n]) +
                         zeta_s_prev[n] * beta_prev * (mk(1.0, 0.0) - shifts[n] * beta));
            zeta_s_prev[n] = tmp;
            beta_s[n] = beta * zeta_s[n] / zeta_s_prev[n];
        }
        mupd.ns = n_shift_rem;
        mupd.bs = beta_s;
        par_range(size, upd_shift_x_range, &mupd);
        mupd.a = beta;
        par_range(size, upd_r_range, &mupd);
        rsqNew = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsqNew) / bsqrt);

        if (k % resid_freq_check == 0) {
            for (n = 0; n < n_shift_rem; n++) {
                if (cabs(zeta_s[n]) * sqrt(rsqNew) < eps * bsqrt) {
                    n_shift_rem--;
                    if (n_shift_rem != n) {
                        int ti = mapping[n_shift_rem]; mapping[n_shift_rem] = mapping[n]; mapping[n] = ti;
                        cplx *tp = phi[n_shift_rem]; phi[n_shift_rem] = phi[n]; phi[n] = tp;
                        tp = p_s[n_shift_rem]; p_s[n_shift_rem] = p_s[n]; p_s[n] = tp;
                        cplx tc;
                        tc = alpha_s[n_shift_rem]; alpha_s[n_shift_rem] = alpha_s[n]; alpha_s[n] = tc;
                        tc = beta_s[n_shift_rem]; beta_s[n_shift_rem] = beta_s[n]; beta_s[n] = tc;
                        tc = zeta_s[n_shift_rem]; zeta_s[n_shift_rem] = zeta_s[n]; zeta_s[n] = tc;
                        tc = zeta_s_prev[n_shift_rem]; zeta_s_prev[n_shift_rem] = zeta_s_prev[n]; zeta_s_prev[n] = tc;
                        double td = shifts[n_shift_rem]; shifts[n_shift_rem] = shifts[n]; shifts[n] = td;
                        n--;
                    }
                }
            }
        }
        if ((worst_first && cabs(zeta_s[0]) * sqrt(rsqNew) < eps * bsqrt) || n_shift_rem == 0 ||
            k == max_iter - 1)
            break;

        alpha = mk(rsqNew / rsq, 0.0);
        rsq = rsqNew;
        for (n = 0; n < n_shift_rem; n++)
            alpha_s[n] = alpha * zeta_s[n] * beta_s[n] / (zeta_s_prev[n] * beta);
        mupd.ns = n_shift_rem;
        mupd.as = zeta_s;
        mupd.bs = alpha_s;
        par_range(size, upd_shift_p_range, &mupd);
        mupd.a = alpha;
        par_range(size, upd_p_range, &mupd);
        orc_apply(op, (double *)Ap, (const double *)p); ops++;
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    k++;

    /* undo the permutation (generic_cg_m.cpp:533-558) */
    for (n = 0; n < n_shift; n++) {
        if (mapping[n] != n) {
            for (int m = n + 1; m < n_shift; m++) {
                if (mapping[m] == n) {
                    cplx *tp = phi[m]; phi[m] = phi[n]; phi[n] = tp;
                    double td = shifts[m]; shifts[m] = shifts[n]; shifts[n] = td;
                    mapping[m] = mapping[n];
                    mapping[n] = n;
                    n--;
                    break;
                }
            }
        }
    }
    /* explicit residuals of every shifted system (generic_cg_m.cpp:561-572) */
    for (n = 0; n < n_shift; n++) {
        memset(Ap, 0, sizeof(cplx) * size);
        orc_apply(op, (double *)Ap, (const double *)phi[n]); ops++;
        for (i = 0; i < size; i++) Ap[i] = Ap[i] + (shifts[n] * phi[n][i]);
        if (resSqmrhs) resSqmrhs[n] = cdiffnorm2(Ap, phi0, size);
    }
    for (n = 0; n < n_shift; n++) free(p_s[n]);
    free(p_s); free(phi); free(alpha_s); free(beta_s); free(zeta_s); free(zeta_s_prev);
    free(shifts); free(mapping); free(r); free(p); free(Ap);
    info->resSq = 0.0; /* the reference leaves resSq at its initial 0 (generic_cg_m.cpp:596) */
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "CG-M");
}

/* ---------------------------------------------------------------- force */

/* dS/dtheta_mu(s) for S = phi^dagger (D^dagger D + sigma)^-1 phi.  With X the solution and
 * Y = D X, dS/dtheta = -2 Re(Y^dagger dD X).  The link U_x(s) enters D at row s as
 * -1/2 U psi(s+x) and at row s+x as +1/2 U^* psi(s) (operators.cpp:215-218); for U_y the
 * same with eta(s) = (-1)^x (operators.cpp:221-224).  dU/dtheta = iU, so
 * dS/dtheta_x(s) = -Im( Y(s)^* U X(s+x) + Y(s+x)^* U^* X(s) ), and eta(s) times the same
 * for y. */
void orc_staggered_force(const double *links, double mass, int lx, int ly, const double *X_,
                         const double *Y_, double *out)
{
    (void)mass;
    const cplx *U = CCX(links), *X = CCX(X_), *Y = CCX(Y_);
    for (long i = 0; i < (long)lx * ly; i++) {
        int x = (int)(i % lx), y = (int)(i / lx);
        long ixp = (long)y * lx + (x + 1) % lx;
        long iyp = (long)((y + 1) % ly) * lx + x;
        double eta1 = (double)(1 - 2 * (x % 2));
        cplx ux = U[2 * i], uy = U[2 * i + 1];
        cplx fx = conj(Y[i]) * ux * X[ixp] + conj(Y[ixp]) * conj(ux) * X[i];
        cplx fy = conj(Y[i]) * uy * X[iyp] + conj(Y[iyp]) * conj(uy) * X[i];
        out[2 * i] = -cimag(fx);
        out[2 * i + 1] = -eta1 * cimag(fy);
    }
}

/* ================================================================ sibling Krylov solvers */

/* ---------------------------------------------------------------- CR */

/* generic_cr.cpp:198-323 (complex minv_vector_cr): conjugate residual, A Hermitian. */
void orc_cr(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
            double eps, orc_info *info, double *hist, int hist_cap)
{
    const cplx *phi0 = CCX(phi0_);
    cplx *x = (cplx *)calloc(size, sizeof(cplx));
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ar = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta;
    double rsq, bsqrt, truersq, Apsq;
    int k, ops = 0;
    long i;

    memcpy(x, phi_, sizeof(cplx) * size);
    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)p, (const double *)x); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - p[i];
    memcpy(p, r, sizeof(cplx) * size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;
    memcpy(Ar, Ap, sizeof(cplx) * size);
    Apsq = cnorm2(Ap, size);

    for (k = 0; k < max_iter; k++) {
        alpha = cdivr(cdot(Ap, r, size), Apsq);
        for (i = 0; i < size; i++) {
            x[i] = x[i] + alpha * p[i];
            r[i] = r[i] - alpha * Ap[i];
        }
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);
        if (sqrt(rsq) < eps * bsqrt || k == max_iter - 1) break;
        orc_apply(op, (double *)Ar, (const double *)r); ops++;
        beta = cdivr(-cdot(Ap, Ar, size), Apsq);
        for (i = 0; i < size; i++) {
            p[i] = r[i] + beta * p[i];
            Ap[i] = Ar[i] + beta * Ap[i];
        }
        Apsq = cnorm2(Ap, size);
    }
    /* the reference tests k == max_iter here (generic_cr.cpp:287), not max_iter - 1 */
    info->success = (k == max_iter) ? 0 : 1;
    k++;
    orc_apply(op, (double *)p, (const double *)x); ops++;
    truersq = cdiffnorm2(p, phi0, size);
    memcpy(phi_, x, sizeof(cplx) * size);
    free(x); free(r); free(Ar); free(p); free(Ap);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "CR");
}

/* generic_cr.cpp:326-366 (complex minv_vector_cr_restart) */
void orc_cr_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                    double eps, int restart_freq, orc_info *info)
{
    restart_driver(orc_cr, "CR", op, phi, phi0, size, max_iter, eps, restart_freq, info);
}

/* ---------------------------------------------------------------- MinRes */

/* generic_minres.cpp:130-231 (complex minv_vector_minres with omega, printed as "MR_<omega>"):
 * x += omega alpha r, r -= omega alpha A r with alpha = <Ar, r> / |Ar|^2. */
void orc_minres(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
                double eps, double omega, orc_info *info, double *hist, int hist_cap)
{
    const cplx *phi0 = CCX(phi0_);
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *x = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha;
    double rsq, truersq, bsqrt;
    int k, ops = 0;
    long i;

    memcpy(x, phi_, sizeof(cplx) * size);
    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)p, phi_); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - p[i];
    for (k = 0; k < max_iter; k++) {
        orc_apply(op, (double *)p, (const double *)r); ops++;
        alpha = cdivr(cdot(p, r, size), cnorm2(p, size));
        alpha = alpha * omega;
        for (i = 0; i < size; i++) {
            x[i] = x[i] + alpha * r[i];
            r[i] = r[i] - alpha * p[i];
        }
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);
        if (sqrt(rsq) < eps * bsqrt) break;
    }
    info->success = (k == max_iter) ? 0 : 1;
    orc_apply(op, (double *)p, (const double *)x); ops++;
    truersq = cdiffnorm2(p, phi0, size);
    memcpy(phi_, x, sizeof(cplx) * size);
    free(p); free(r); free(x);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "Minimum Residual (MinRes)");
}

/* ---------------------------------------------------------------- CR-M */

/* generic_cr_m.cpp:323-622 (complex minv_vector_cr_m): multishift conjugate residual.  The
 * shift bookkeeping (retire, swap, restore) is the one of CG-M. */
void orc_cr_m(const orc_op *op, double *phi_all, const double *phi0_, int n_shift, long size,
              int resid_freq_check, int max_iter, double eps, const double *shifts_in,
              int worst_first, orc_info *info, double *resSqmrhs, double *hist, int hist_cap)
{
    const cplx *phi0 = CCX(phi0_);
    cplx **phi = (cplx **)malloc(sizeof(cplx *) * n_shift);
    cplx **p_s = (cplx **)malloc(sizeof(cplx *) * n_shift);
    cplx *alpha_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *beta_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *zeta_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *zeta_s_prev = (cplx *)malloc(sizeof(cplx) * n_shift);
    double *shifts = (double *)malloc(sizeof(double) * n_shift);
    int *mapping = (int *)malloc(sizeof(int) * n_shift);
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ar = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta, beta_prev, tmp;
    double rsq, bsqrt, Apsq;
    int k, n, n_shift_rem = n_shift, ops = 0;
    long i;

    for (n = 0; n < n_shift; n++) {
        phi[n] = CX(phi_all) + (long)n * size;
        p_s[n] = (cplx *)malloc(sizeof(cplx) * size);
        mapping[n] = n;
        shifts[n] = shifts_in[n];
        beta_s[n] = zeta_s[n] = zeta_s_prev[n] = 1.0;
        alpha_s[n] = 0.0;
    }
    beta = 1.0;
    alpha = 0.0;
    bsqrt = sqrt(cnorm2(phi0, size));
    for (n = 0; n < n_shift; n++) {
        memcpy(p_s[n], phi0, sizeof(cplx) * size);
        memset(phi[n], 0, sizeof(cplx) * size);
    }
    memcpy(p, phi0, sizeof(cplx) * size);
    memcpy(r, phi0, sizeof(cplx) * size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;
    memcpy(Ar, Ap, sizeof(cplx) * size);
    Apsq = cnorm2(Ap, size);
    rsq = cnorm2(r, size);

    for (k = 0; k < max_iter; k++) {
        beta_prev = beta;
        beta = cdivr(-cdot(Ap, r, size), Apsq);
        for (n = 0; n < n_shift_rem; n++) {
            tmp = zeta_s[n];
            zeta_s[n] = (zeta_s[n] * zeta_s_prev[n] * beta_prev) /
                        (beta * alpha * (zeta_s_prev[n] - zeta_s[n]) +
                         zeta_s_prev[n] * beta_prev * (1.0 - shifts[n] * beta));
            zeta_s_prev[n] = tmp;
            beta_s[n] = beta * zeta_s[n] / zeta_s_prev[n];
            for (i = 0; i < size; i++) phi[n][i] = phi[n][i] - beta_s[n] * p_s[n][i];
        }
        for (i = 0; i < size; i++) r[i] = r[i] + beta * Ap[i];
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);

        if (k % resid_freq_check == 0) {
            for (n = 0; n < n_shift_rem; n++) {
                if (cabs(zeta_s[n]) * sqrt(rsq) < eps * bsqrt) {
                    n_shift_rem--;
                    if (n_shift_rem != n) {
                        int ti = mapping[n_shift_rem]; mapping[n_shift_rem] = mapping[n]; mapping[n] = ti;
                        cplx *tp = phi[n_shift_rem]; phi[n_shift_rem] = phi[n]; phi[n] = tp;
                        tp = p_s[n_shift_rem]; p_s[n_shift_rem] = p_s[n]; p_s[n] = tp;
                        cplx tc;
                        tc = alpha_s[n_shift_rem]; alpha_s[n_shift_rem] = alpha_s[n]; alpha_s[n] = tc;
                        tc = beta_s[n_shift_rem]; beta_s[n_shift_rem] = beta_s[n]; beta_s[n] = tc;
                        tc = zeta_s[n_shift_rem]; zeta_s[n_shift_rem] = zeta_s[n]; zeta_s[n] = tc;
                        tc = zeta_s_prev[n_shift_rem]; zeta_s_prev[n_shift_rem] = zeta_s_prev[n]; zeta_s_prev[n] = tc;
                        double td = shifts[n_shift_rem]; shifts[n_shift_rem] = shifts[n]; shifts[n] = td;
                        n--;
                    }
                }
            }
        }
        if ((worst_first && cabs(zeta_s[0]) * sqrt(rsq) < eps * bsqrt) || n_shift_rem == 0 ||
            k == max_iter - 1)
            break;

        orc_apply(op, (double *)Ar, (const double *)r); ops++;
        alpha = cdivr(-cdot(Ap, Ar, size), Apsq);
        for (n = 0; n < n_shift_rem; n++) {
            alpha_s[n] = alpha * zeta_s[n] * beta_s[n] / (zeta_s_prev[n] * beta);
            for (i = 0; i < size; i++) p_s[n][i] = zeta_s[n] * r[i] + alpha_s[n] * p_s[n][i];
        }
        for (i = 0; i < size; i++) {
            p[i] = r[i] + alpha * p[i];
            Ap[i] = Ar[i] + alpha * Ap[i];
        }
        Apsq = cnorm2(Ap, size);
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    k++;

    for (n = 0; n < n_shift; n++) {
        if (mapping[n] != n) {
            for (int m = n + 1; m < n_shift; m++) {
                if (mapping[m] == n) {
                    cplx *tp = phi[m]; phi[m] = phi[n]; phi[n] = tp;
                    double td = shifts[m]; shifts[m] = shifts[n]; shifts[n] = td;
                    mapping[m] = mapping[n];
                    mapping[n] = n;
                    n--;
                    break;
                }
            }
        }
    }
    for (n = 0; n < n_shift; n++) {
        memset(Ap, 0, sizeof(cplx) * size);
        orc_apply(op, (double *)Ap, (const double *)phi[n]); ops++;
        for (i = 0; i < size; i++) Ap[i] = Ap[i] + (shifts[n] * phi[n][i]);
        if (resSqmrhs) resSqmrhs[n] = cdiffnorm2(Ap, phi0, size);
    }
    for (n = 0; n < n_shift; n++) free(p_s[n]);
    free(p_s); free(phi); free(alpha_s); free(beta_s); free(zeta_s); free(zeta_s_prev);
    free(shifts); free(mapping); free(r); free(Ar); free(p); free(Ap);
    info->resSq = 0.0;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "CR-M");
}

/* ---------------------------------------------------------------- BiCGstab-l */

/* generic_bicgstab_l.cpp:317-561 (complex minv_vector_bicgstab_l): l BiCG steps, then a
 * minimal-residual polynomial of degree l by modified Gram-Schmidt (Sleijpen & Fokkema). */
void orc_bicgstab_l(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
                    double eps, int l, orc_info *info, double *hist, int hist_cap)
{
    cplx *phi = CX(phi_);
    const cplx *phi0 = CCX(phi0_);
    cplx *r0 = (cplx *)calloc(size, sizeof(cplx));
    cplx **r = (cplx **)malloc(sizeof(cplx *) * (l + 1));
    cplx **u = (cplx **)malloc(sizeof(cplx *) * (l + 1));
    double *sigma = (double *)calloc(l + 1, sizeof(double));
    cplx *gamma = (cplx *)calloc(l + 1, sizeof(cplx));
    cplx *gamma_p = (cplx *)calloc(l + 1, sizeof(cplx));
    cplx *gamma_pp = (cplx *)calloc(l + 1, sizeof(cplx));
    cplx *tau = (cplx *)calloc((size_t)(l + 1) * (l + 1), sizeof(cplx));
#define TAU(a, b) tau[(a) * (l + 1) + (b)]
    cplx rho0, rho1, alpha, omega, beta;
    double bsqrt, truersq;
    int k, i, j, ops = 0;
    long h;
    char nm[32];

    for (i = 0; i <= l; i++) {
        r[i] = (cplx *)calloc(size, sizeof(cplx));
        u[i] = (cplx *)calloc(size, sizeof(cplx));
    }
    rho0 = 1.0;
    alpha = 0.0;
    omega = 1.0;
    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)u[0], (const double *)phi); ops++;
    for (h = 0; h < size; h++) r[0][h] = phi0[h] - u[0][h];
    sigma[0] = cnorm2(r[0], size);
    memcpy(r0, r[0], sizeof(cplx) * size);
    memset(u[0], 0, sizeof(cplx) * size);

    for (k = 0; k < max_iter; k += l) {
        rho0 *= -omega;
        for (j = 0; j < l; j++) {
            rho1 = cdot(r0, r[j], size);
            beta = alpha * rho1 / rho0;
            rho0 = rho1;
            for (i = 0; i <= j; i++)
                for (h = 0; h < size; h++) u[i][h] = r[i][h] - beta * u[i][h];
            orc_apply(op, (double *)u[j + 1], (const double *)u[j]); ops++;
            alpha = rho0 / cdot(r0, u[j + 1], size);
            for (i = 0; i <= j; i++)
                for (h = 0; h < size; h++) r[i][h] = r[i][h] - alpha * u[i + 1][h];
            orc_apply(op, (double *)r[j + 1], (const double *)r[j]); ops++;
            for (h = 0; h < size; h++) phi[h] = phi[h] + alpha * u[0][h];
        }
        for (j = 1; j <= l; j++) {
            for (i = 1; i < j; i++) {
                TAU(i, j) = cdivr(cdot(r[i], r[j], size), sigma[i]);
                for (h = 0; h < size; h++) r[j][h] = r[j][h] - TAU(i, j) * r[i][h];
            }
            sigma[j] = cnorm2(r[j], size);
            gamma_p[j] = cdivr(cdot(r[j], r[0], size), sigma[j]);
        }
        gamma[l] = gamma_p[l];
        omega = gamma[l];
        for (j = l - 1; j > 0; j--) {
            gamma[j] = gamma_p[j];
            for (i = j + 1; i <= l; i++) gamma[j] = gamma[j] - TAU(j, i) * gamma[i];
        }
        for (j = 1; j < l; j++) {
            gamma_pp[j] = gamma[j + 1];
            for (i = j + 1; i < l; i++) gamma_pp[j] = gamma_pp[j] + TAU(j, i) * gamma[i + 1];
        }
        for (h = 0; h < size; h++) {
            phi[h] = phi[h] + gamma[1] * r[0][h];
            u[0][h] = u[0][h] - gamma[l] * u[l][h];
            r[0][h] = r[0][h] - gamma_p[l] * r[l][h];
        }
        for (j = 1; j < l; j++) {
            for (h = 0; h < size; h++) {
                u[0][h] = u[0][h] - gamma[j] * u[j][h];
                phi[h] = phi[h] + gamma_pp[j] * r[j][h];
                r[0][h] = r[0][h] - gamma_p[j] * r[j][h];
            }
        }
        sigma[0] = cnorm2(r[0], size);
        record(hist, hist_cap, k / l, sqrt(sigma[0]) / bsqrt);
        if (sqrt(sigma[0]) < eps * bsqrt) break;
    }
#undef TAU
    info->success = (k >= max_iter - 1) ? 0 : 1;
    k++;
    orc_apply(op, (double *)u[0], (const double *)phi); ops++;
    truersq = cdiffnorm2(u[0], phi0, size);
    for (i = 0; i <= l; i++) { free(r[i]); free(u[i]); }
    free(r); free(u); free(r0); free(sigma); free(gamma); free(gamma_p); free(gamma_pp); free(tau);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    snprintf(nm, sizeof(nm), "BiCGStab-%d", l);
    set_name(info, nm);
}

/* generic_bicgstab_l.cpp:564-604 */
void orc_bicgstab_l_restart(const orc_op *op, double *phi, const double *phi0, long size,
                            int max_iter, double eps, int restart_freq, int l, orc_info *info)
{
    double bsqrt = sqrt(cnorm2(CCX(phi0), size));
    int iter = 0, ops = 0;
    orc_info inner;
    memset(&inner, 0, sizeof(inner));
    do {
        orc_bicgstab_l(op, phi, phi0, size, restart_freq, eps, l, &inner, NULL, 0);
        iter += inner.iter;
        ops += inner.ops_count;
    } while (iter < max_iter && inner.success == 0 && sqrt(inner.resSq) / bsqrt > eps);
    *info = inner;
    info->iter = iter;
    info->ops_count = ops;
    info->success = (sqrt(inner.resSq) / bsqrt > eps) ? 0 : 1;
    char nm[64];
    snprintf(nm, sizeof(nm), "BiCGStab-%d(%d)", l, restart_freq);
    set_name(info, nm);
}

/* ---------------------------------------------------------------- BiCGstab-M */

/* generic_bicgstab_m.cpp:402-774 (complex minv_vector_bicgstab_m): multishift BiCGstab
 * (Jegerlehner, hep-lat/9612014).  The shadow vector is conj(b), so <wdag, v> = sum b_i v_i. */
void orc_bicgstab_m(const orc_op *op, double *phi_all, const double *phi0_, int n_shift, long size,
                    int resid_freq_check, int max_iter, double eps, const double *shifts_in,
                    int worst_first, orc_info *info, double *resSqmrhs, double *hist, int hist_cap)
{
    const cplx *phi0 = CCX(phi0_);
    cplx **phi = (cplx **)malloc(sizeof(cplx *) * n_shift);
    cplx **s_s = (cplx **)malloc(sizeof(cplx *) * n_shift);
    cplx *alpha_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *beta_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *zeta_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *zeta_s_prev = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *chi_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *rho_s = (cplx *)malloc(sizeof(cplx) * n_shift);
    cplx *rho_s_prev = (cplx *)malloc(sizeof(cplx) * n_shift);
    double *shifts = (double *)malloc(sizeof(double) * n_shift);
    int *mapping = (int *)malloc(sizeof(int) * n_shift);
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *r_prev = (cplx *)calloc(size, sizeof(cplx));
    cplx *s = (cplx *)calloc(size, sizeof(cplx));
    cplx *As = (cplx *)calloc(size, sizeof(cplx));
    cplx *w = (cplx *)calloc(size, sizeof(cplx));
    cplx *Aw = (cplx *)calloc(size, sizeof(cplx));
    cplx *wdag = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta, beta_prev, psi, delta, delta_prev, chi, tmp;
    double rsqNew, bsqrt;
    int k, n, n_shift_rem = n_shift, ops = 0, breakdown = 0;
    long i;

    for (n = 0; n < n_shift; n++) {
        phi[n] = CX(phi_all) + (long)n * size;
        s_s[n] = (cplx *)malloc(sizeof(cplx) * size);
        mapping[n] = n;
        shifts[n] = shifts_in[n];
        beta_s[n] = zeta_s[n] = zeta_s_prev[n] = rho_s[n] = rho_s_prev[n] = 1.0;
        alpha_s[n] = chi_s[n] = 0.0;
    }
    beta = 1.0;
    alpha = 0.0;
    bsqrt = sqrt(cnorm2(phi0, size));
    for (n = 0; n < n_shift; n++) {
        memcpy(s_s[n], phi0, sizeof(cplx) * size);
        memset(phi[n], 0, sizeof(cplx) * size);
    }
    memcpy(s, phi0, sizeof(cplx) * size);
    memcpy(r, phi0, sizeof(cplx) * size);
    memcpy(r_prev, r, sizeof(cplx) * size);
    orc_apply(op, (double *)As, (const double *)s); ops++;
    for (i = 0; i < size; i++) wdag[i] = conj(r[i]);
    delta = delta_prev = cdot(wdag, r, size);
    psi = cdot(wdag, As, size) / delta;

    for (k = 0; k < max_iter; k++) {
        beta_prev = beta;
        beta = rdivc(-1.0, psi);
        for (i = 0; i < size; i++) w[i] = r[i] + beta * As[i];
        orc_apply(op, (double *)Aw, (const double *)w); ops++;
        chi = cdivr(cdot(Aw, w, size), cnorm2(Aw, size));
        memcpy(r_prev, r, sizeof(cplx) * size);
        for (i = 0; i < size; i++) r[i] = w[i] - chi * Aw[i];
        for (n = 0; n < n_shift_rem; n++) {
            tmp = zeta_s[n];
            zeta_s[n] = (zeta_s[n] * zeta_s_prev[n] * beta_prev) /
                        (beta * alpha * (zeta_s_prev[n] - zeta_s[n]) +
                         zeta_s_prev[n] * beta_prev * (1.0 - shifts[n] * beta));
            zeta_s_prev[n] = tmp;
            beta_s[n] = beta * zeta_s[n] / zeta_s_prev[n];
            chi_s[n] = chi / (1.0 + chi * shifts[n]);
            tmp = rho_s[n];
            rho_s[n] = rho_s[n] / (1.0 + chi * shifts[n]);
            rho_s_prev[n] = tmp;
            for (i = 0; i < size; i++)
                phi[n][i] = phi[n][i] - beta_s[n] * s_s[n][i] + chi_s[n] * rho_s_prev[n] * zeta_s[n] * w[i];
        }
        rsqNew = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsqNew) / bsqrt);
        if (k % resid_freq_check == 0) {
            for (n = 0; n < n_shift_rem; n++) {
                if (cabs(zeta_s[n] * rho_s[n]) * sqrt(rsqNew) < eps * bsqrt) {
                    n_shift_rem--;
                    if (n_shift_rem != n) {
                        int e = n_shift_rem;
                        int ti = mapping[e]; mapping[e] = mapping[n]; mapping[n] = ti;
                        cplx *tp = phi[e]; phi[e] = phi[n]; phi[n] = tp;
                        tp = s_s[e]; s_s[e] = s_s[n]; s_s[n] = tp;
                        cplx tc;
                        tc = alpha_s[e]; alpha_s[e] = alpha_s[n]; alpha_s[n] = tc;
                        tc = beta_s[e]; beta_s[e] = beta_s[n]; beta_s[n] = tc;
                        tc = zeta_s[e]; zeta_s[e] = zeta_s[n]; zeta_s[n] = tc;
                        tc = zeta_s_prev[e]; zeta_s_prev[e] = zeta_s_prev[n]; zeta_s_prev[n] = tc;
                        tc = chi_s[e]; chi_s[e] = chi_s[n]; chi_s[n] = tc;
                        tc = rho_s[e]; rho_s[e] = rho_s[n]; rho_s[n] = tc;
                        tc = rho_s_prev[e]; rho_s_prev[e] = rho_s_prev[n]; rho_s_prev[n] = tc;
                        double td = shifts[e]; shifts[e] = shifts[n]; shifts[n] = td;
                        n--;
                    }
                }
            }
        }
        if ((worst_first && (cabs(zeta_s[0] * rho_s[0]) * sqrt(rsqNew) < eps * bsqrt)) ||
            rsqNew != rsqNew || n_shift_rem == 0 || k == max_iter - 1)
            break;
        delta_prev = delta;
        delta = cdot(wdag, r, size);
        alpha = -beta * delta / (delta_prev * chi);
        for (n = 0; n < n_shift_rem; n++)
            alpha_s[n] = alpha * zeta_s[n] * beta_s[n] / (zeta_s_prev[n] * beta);
        for (i = 0; i < size; i++) s[i] = r[i] + alpha * (s[i] - chi * As[i]);
        for (n = 0; n < n_shift_rem; n++) {
            if (fabs(shifts[n]) != 0.0) {
                for (i = 0; i < size; i++)
                    s_s[n][i] = zeta_s[n] * rho_s[n] * r[i] +
                                alpha_s[n] * (s_s[n][i] - chi_s[n] / beta_s[n] *
                                                              (zeta_s[n] * rho_s_prev[n] * w[i] -
                                                               zeta_s_prev[n] * rho_s_prev[n] * r_prev[i]));
            } else {
                memcpy(s_s[n], s, sizeof(cplx) * size);
            }
        }
        orc_apply(op, (double *)As, (const double *)s); ops++;
        psi = cdot(wdag, As, size) / delta;
        if (cabs(psi) == 0) {
            breakdown = 1;
            break;
        }
    }
    info->success = (k == max_iter - 1 || breakdown) ? 0 : 1;
    k++;
    for (n = 0; n < n_shift; n++) {
        if (mapping[n] != n) {
            for (int m = n + 1; m < n_shift; m++) {
                if (mapping[m] == n) {
                    cplx *tp = phi[m]; phi[m] = phi[n]; phi[n] = tp;
                    double td = shifts[m]; shifts[m] = shifts[n]; shifts[n] = td;
                    mapping[m] = mapping[n];
                    mapping[n] = n;
                    n--;
                    break;
                }
            }
        }
    }
    for (n = 0; n < n_shift; n++) {
        memset(As, 0, sizeof(cplx) * size);
        orc_apply(op, (double *)As, (const double *)phi[n]); ops++;
        for (i = 0; i < size; i++) As[i] = As[i] + (shifts[n] * phi[n][i]);
        if (resSqmrhs) resSqmrhs[n] = cdiffnorm2(As, phi0, size);
    }
    for (n = 0; n < n_shift; n++) free(s_s[n]);
    free(s_s); free(phi); free(alpha_s); free(beta_s); free(zeta_s); free(zeta_s_prev);
    free(chi_s); free(rho_s); free(rho_s_prev); free(shifts); free(mapping);
    free(r); free(r_prev); free(s); free(As); free(w); free(Aw); free(wdag);
    info->resSq = 0.0;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "BICGSTAB-M");
}

/* ---------------------------------------------------------------- preconditioned solvers */

/* generic_precond.cpp:34-77: identity_preconditioner copies; minres_preconditioner runs n_step
 * iterations of minv_vector_minres (omega 1) and gcr_preconditioner n_step iterations of
 * minv_vector_gcr, both from the guess in lhs (the callers zero it). */
static void precond_apply(const orc_precond *pc, cplx *lhs, const cplx *rhs, long size)
{
    orc_info tmp;
    memset(&tmp, 0, sizeof(tmp));
    switch (pc->kind) {
    case ORC_PRECOND_MINRES:
        orc_minres(pc->op, (double *)lhs, (const double *)rhs, size, pc->n_step, pc->rel_res, 1.0, &tmp, NULL, 0);
        break;
    case ORC_PRECOND_GCR:
        orc_gcr(pc->op, (double *)lhs, (const double *)rhs, size, pc->n_step, pc->rel_res, &tmp, NULL, 0);
        break;
    default:
        memcpy(lhs, rhs, sizeof(cplx) * size);
        break;
    }
}

/* generic_cg_flex_precond.cpp:223-364 (complex minv_vector_cg_flex_precond): flexible CG,
 * each new direction A-orthogonalised against every stored one. */
void orc_fpcg(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
              double eps, const orc_precond *pc, orc_info *info, double *hist, int hist_cap)
{
    cplx *phi = CX(phi_);
    const cplx *phi0 = CCX(phi0_);
    const int cap = (max_iter > 0 ? max_iter : 0) + 1;
    cplx **p_store = (cplx **)calloc(cap, sizeof(cplx *));
    cplx **Ap_store = (cplx **)calloc(cap, sizeof(cplx *));
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *z = (cplx *)calloc(size, sizeof(cplx));
    cplx *Az = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta_ij;
    double rsq, bsqrt, truersq;
    int k, ii, ops = 0, nstore = 0;
    long i;

    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)p, (const double *)phi); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - p[i];
    precond_apply(pc, z, r, size);
    memcpy(p, z, sizeof(cplx) * size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;
    for (k = 0; k < max_iter; k++) {
        p_store[nstore] = p;
        Ap_store[nstore] = Ap;
        nstore++;
        alpha = cdot(p, r, size) / cdot(p, Ap, size);
        for (i = 0; i < size; i++) {
            phi[i] = phi[i] + alpha * p[i];
            r[i] = r[i] - alpha * Ap[i];
        }
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);
        if (sqrt(rsq) < eps * bsqrt || k == max_iter - 1) break;
        memset(z, 0, sizeof(cplx) * size);
        precond_apply(pc, z, r, size);
        orc_apply(op, (double *)Az, (const double *)z); ops++;
        p = (cplx *)malloc(sizeof(cplx) * size);
        memcpy(p, z, sizeof(cplx) * size);
        Ap = (cplx *)malloc(sizeof(cplx) * size);
        memcpy(Ap, Az, sizeof(cplx) * size);
        for (ii = 0; ii <= k; ii++) {
            beta_ij = -cdot(Ap_store[ii], z, size) / cdot(p_store[ii], Ap_store[ii], size);
            for (i = 0; i < size; i++) {
                p[i] += beta_ij * p_store[ii][i];
                Ap[i] += beta_ij * Ap_store[ii][i];
            }
        }
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    k++;
    orc_apply(op, (double *)Az, (const double *)phi); ops++;
    truersq = cdiffnorm2(Az, phi0, size);
    for (ii = 0; ii < nstore; ii++) { free(p_store[ii]); free(Ap_store[ii]); }
    if (nstore == 0) { free(p); free(Ap); }
    free(p_store); free(Ap_store); free(r); free(z); free(Az);
    info->resSq = truersq;
    info->iter = k;
    info->ops_count = ops;
    set_name(info, "Flexibly Preconditioned CG");
}

/* generic_cg_flex_precond.cpp:367-415: the restarted driver adds one application for the
 * final true residual to ops_count after printing the summary. */
void orc_fpcg_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                      double eps, int restart_freq, const orc_precond *pc, orc_info *info)
{
    double bsqrt = sqrt(cnorm2(CCX(phi0), size));
    int iter = 0, ops = 0;
    orc_info inner;
    memset(&inner, 0, sizeof(inner));
    do {
        orc_fpcg(op, phi, phi0, size, restart_freq, eps, pc, &inner, NULL, 0);
        iter += inner.iter;
        ops += inner.ops_count;
    } while (iter < max_iter && inner.success == 0 && sqrt(inner.resSq) / bsqrt > eps);
    cplx *Aphi = (cplx *)calloc(size, sizeof(cplx));
    orc_apply(op, (double *)Aphi, phi); ops++;
    inner.resSq = cdiffnorm2(Aphi, CCX(phi0), size);
    free(Aphi);
    *info = inner;
    info->iter = iter;
    info->ops_count = ops;
    info->success = (sqrt(info->resSq) / bsqrt > eps) ? 0 : 1;
    char nm[64];
    snprintf(nm, sizeof(nm), "Flexibly Preconditioned Restarted CG(%d)", restart_freq);
    set_name(info, nm);
}

/* generic_gcr_var_precond.cpp:220-366 (complex minv_vector_gcr_var_precond): GCR with a
 * preconditioner that may change between iterations. */
void orc_vpgcr(const orc_op *op, double *phi_, const double *phi0_, long size, int max_iter,
               double eps, const orc_precond *pc, orc_info *info, double *hist, int hist_cap)
{
    const cplx *phi0 = CCX(phi0_);
    const int cap = (max_iter > 0 ? max_iter : 0) + 1;
    cplx **p_store = (cplx **)calloc(cap, sizeof(cplx *));
    cplx **Ap_store = (cplx **)calloc(cap, sizeof(cplx *));
    cplx *x = (cplx *)calloc(size, sizeof(cplx));
    cplx *r = (cplx *)calloc(size, sizeof(cplx));
    cplx *z = (cplx *)calloc(size, sizeof(cplx));
    cplx *Az = (cplx *)calloc(size, sizeof(cplx));
    cplx *p = (cplx *)calloc(size, sizeof(cplx));
    cplx *Ap = (cplx *)calloc(size, sizeof(cplx));
    cplx alpha, beta_ij;
    double rsq, bsqrt, truersq;
    int k, ii, ops = 0, nstore = 0;
    long i;

    memcpy(x, phi_, sizeof(cplx) * size);
    bsqrt = sqrt(cnorm2(phi0, size));
    orc_apply(op, (double *)p, (const double *)x); ops++;
    for (i = 0; i < size; i++) r[i] = phi0[i] - p[i];
    precond_apply(pc, z, r, size);
    memcpy(p, z, sizeof(cplx) * size);
    orc_apply(op, (double *)Ap, (const double *)p); ops++;
    for (k = 0; k < max_iter; k++) {
        p_store[nstore] = p;
        Ap_store[nstore] = Ap;
        nstore++;
        alpha = cdivr(cdot(Ap, r, size), cnorm2(Ap, size));
        for (i = 0; i < size; i++) {
            x[i] = x[i] + alpha * p[i];
            r[i] = r[i] - alpha * Ap[i];
        }
        rsq = cnorm2(r, size);
        record(hist, hist_cap, k, sqrt(rsq) / bsqrt);
        if (sqrt(rsq) < eps * bsqrt || k == max_iter - 1) break;
        memset(z, 0, sizeof(cplx) * size);
        precond_apply(pc, z, r, size);
        orc_apply(op, (double *)Az, (const double *)z); ops++;
        p = (cplx *)malloc(sizeof(cplx) * size);
        memcpy(p, z, sizeof(cplx) * size);
        Ap = (cplx *)malloc(sizeof(cplx) * size);
        memcpy(Ap, Az, sizeof(cplx) * size);
        for (ii = 0; ii <= k; ii++) {
            beta_ij = cdivr(-cdot(Ap_store[ii], Az, size), cnorm2(Ap_store[ii], size));
            for (i = 0; i < size; i++) {
                p[i] += beta_ij * p_store[ii][i];
                Ap[i] += beta_ij * Ap_store[ii][i];
            }
        }
    }
    info->success = (k == max_iter - 1) ? 0 : 1;
    orc_apply(op, (double *)Az, (const double *)x); ops++;
    truersq = cdiffnorm2(Az, phi0, size);
    memcpy(phi_, x, sizeof(cplx) * size);
    for (ii = 0; ii < nstore; ii++) { free(p_store[ii]); free(Ap_store[ii]); }
    if (nstore == 0) { free(p); free(Ap); }
    free(p_store); free(Ap_store); free(x); free(r); free(z); free(Az);
    info->resSq = truersq;
    info->iter = nstore; /* the reference reports the number of stored directions (:350-362) */
    info->ops_count = ops;
    set_name(info, "Variably Preconditioned GCR");
}

/* generic_gcr_var_precond.cpp:369-411 */
void orc_vpgcr_restart(const orc_op *op, double *phi, const double *phi0, long size, int max_iter,
                       double eps, int restart_freq, const orc_precond *pc, orc_info *info)
{
    double bsqrt = sqrt(cnorm2(CCX(phi0), size));
    int iter = 0, ops = 0;
    orc_info inner;
    memset(&inner, 0, sizeof(inner));
    do {
        orc_vpgcr(op, phi, phi0, size, restart_freq, eps, pc, &inner, NULL, 0);
        iter += inner.iter;
        ops += inner.ops_count;
    } while (iter < max_iter && inner.success == 0 && sqrt(inner.resSq) / bsqrt > eps);
    *info = inner;
    info->iter = iter;
    info->ops_count = ops;
    info->success = (sqrt(inner.resSq) / bsqrt > eps) ? 0 : 1;
    char nm[64];
    snprintf(nm, sizeof(nm), "Variably Preconditioned Restarted GCR(%d)", restart_freq);
    set_name(info, nm);
}

/* ================================================================ gauge-field utilities */

#define ORC_PI 3.14159265358979323846

/* u1_utils.cpp:190-207 (get_plaquette_u1): average of U_x(x) U_y(x+x) U_x(x+y)^* U_y(x)^*,
 * summed in site order. */
void orc_plaquette_u1(const double *links, int lx, int ly, double out[2])
{
    const cplx *U = CCX(links);
    cplx plaq = 0.0, tmp;
    for (int y = 0; y < ly; y++) {
        for (int x = 0; x < lx; x++) {
            tmp = U[2 * lx * y + 2 * x] * U[2 * lx * y + 2 * ((x + 1) % lx) + 1] *
                  conj(U[2 * lx * ((y + 1) % ly) + 2 * x]) * conj(U[2 * lx * y + 2 * x + 1]);
            plaq += tmp;
        }
    }
    plaq = cdivr(plaq, (double)(lx * ly));
    out[0] = creal(plaq);
    out[1] = cimag(plaq);
}

/* u1_utils.cpp:210-226 (get_topo_u1): sum over plaquettes of arg(w), divided by 2 pi. */
double orc_topo_u1(const double *links, int lx, int ly)
{
    const cplx *U = CCX(links);
    double top = 0.0;
    for (int y = 0; y < ly; y++) {
        for (int x = 0; x < lx; x++) {
            cplx w = U[y * lx * 2 + x * 2 + 0] * U[y * lx * 2 + ((x + 1) % lx) * 2 + 1] *
                     conj(U[((y + 1) % ly) * lx * 2 + x * 2 + 0]) * conj(U[y * lx * 2 + x * 2 + 1]);
            top += carg(w);
        }
    }
    return 0.5 * top / ORC_PI;
}

/* u1_utils.cpp:128-142 (apply_gauge_trans_u1): U_mu(x) = g(x) U_mu(x) g(x + mu)^*, in place,
 * in site order. */
void orc_gauge_trans_u1(double *links, const double *trans, int lx, int ly)
{
    cplx *U = CX(links);
    const cplx *g = CCX(trans);
    for (int y = 0; y < ly; y++) {
        for (int x = 0; x < lx; x++) {
            U[2 * lx * y + 2 * x] = g[lx * y + x] * U[2 * lx * y + 2 * x] * conj(g[lx * y + (x + 1) % lx]);
            U[2 * lx * y + 2 * x + 1] = g[lx * y + x] * U[2 * lx * y + 2 * x + 1] * conj(g[lx * ((y + 1) % ly) + x]);
        }
    }
}

/* std::polar(1.0, theta) of libstdc++: (cos theta, sin theta). */
static inline cplx polar1(double th) { return mk(cos(th), sin(th)); }

/* u1_utils.cpp:145-187 (apply_ape_smear_u1): n_iter sweeps of U + alpha (sum of the two
 * staples), each projected back onto U(1) by its phase. */
void orc_ape_smear_u1(double *smeared_, const double *links, int lx, int ly, double alpha, int n_iter)
{
    const long n2 = 2L * lx * ly;
    cplx *S = CX(smeared_);
    cplx *T = (cplx *)malloc(sizeof(cplx) * n2);
    memcpy(T, links, sizeof(cplx) * n2);
    for (int it = 0; it < n_iter; it++) {
        for (int y = 0; y < ly; y++) {
            const int yp = (y + 1) % ly, ym = (y - 1 + ly) % ly;
            for (int x = 0; x < lx; x++) {
                const int xp = (x + 1) % lx, xm = (x - 1 + lx) % lx;
                cplx v = T[y * lx * 2 + x * 2 + 0];
                v += alpha * T[y * lx * 2 + x * 2 + 1] * T[yp * lx * 2 + x * 2 + 0] * conj(T[y * lx * 2 + xp * 2 + 1]);
                v += alpha * conj(T[ym * lx * 2 + x * 2 + 1]) * T[ym * lx * 2 + x * 2 + 0] * T[ym * lx * 2 + xp * 2 + 1];
                S[y * lx * 2 + x * 2 + 0] = v;
                v = T[y * lx * 2 + x * 2 + 1];
                v += alpha * conj(T[y * lx * 2 + xm * 2 + 0]) * T[y * lx * 2 + xm * 2 + 1] * T[yp * lx * 2 + xm * 2 + 0];
                v += alpha * T[y * lx * 2 + x * 2 + 0] * T[y * lx * 2 + xp * 2 + 1] * conj(T[yp * lx * 2 + x * 2 + 0]);
                S[y * lx * 2 + x * 2 + 1] = v;
            }
        }
        for (long i = 0; i < n2; i++) T[i] = polar1(carg(S[i]));
    }
    memcpy(S, T, sizeof(cplx) * n2);
    free(T);
}

/* ================================================================ multigrid transfer */

/* Fine index of (coarse site (xc, yc), fine offset (x, y) in the block, dof). */
static inline long mg_fine_index(const orc_mg_level *lv, int x, int y, int dof)
{
    return ((long)y * lv->lx + x) * lv->nc_f + dof;
}

/* mg_complex.cpp:191-257 (block_normalize): every null vector normalised on every block. */
void orc_mg_block_normalize(orc_mg_level *lv)
{
    const int xc_n = lv->lx / lv->bx, yc_n = lv->ly / lv->by;
    const long fsize = (long)lv->lx * lv->ly * lv->nc_f;
    const long csize = (long)xc_n * yc_n * lv->nc_c;
    for (long i = 0; i < csize; i++) {
        const int cd = (int)(i % lv->nc_c);
        const long t = i / lv->nc_c;
        const int xc = (int)(t % xc_n), yc = (int)(t / xc_n);
        cplx *v = CX(lv->null_vectors) + (long)cd * fsize;
        double norm = 0.0;
        for (int y = yc * lv->by; y < yc * lv->by + lv->by; y++)
            for (int x = xc * lv->bx; x < xc * lv->bx + lv->bx; x++)
                for (int d = 0; d < lv->nc_f; d++) {
                    const cplx z = v[mg_fine_index(lv, x, y, d)];
                    norm += creal(conj(z) * z);
                }
        norm = sqrt(norm);
        for (int y = yc * lv->by; y < yc * lv->by + lv->by; y++)
            for (int x = xc * lv->bx; x < xc * lv->bx + lv->bx; x++)
                for (int d = 0; d < lv->nc_f; d++) v[mg_fine_index(lv, x, y, d)] = cdivr(v[mg_fine_index(lv, x, y, d)], norm);
    }
}

/* mg_complex.cpp:259-369 (block_orthonormalize): per block, modified Gram-Schmidt in the
 * reference's order (normalise vector k-1, then project vector k against 0..k-1), then
 * block_normalize. */
void orc_mg_block_orthonormalize(orc_mg_level *lv)
{
    const int xc_n = lv->lx / lv->bx, yc_n = lv->ly / lv->by;
    const long fsize = (long)lv->lx * lv->ly * lv->nc_f;
    cplx *V = CX(lv->null_vectors);
    for (long i = 0; i < (long)xc_n * yc_n; i++) {
        const int xc = (int)(i % xc_n), yc = (int)(i / xc_n);
        const int x0 = xc * lv->bx, y0 = yc * lv->by;
        for (int cd = 1; cd < lv->nc_c; cd++) {
            cplx *prev = V + (long)(cd - 1) * fsize, *cur = V + (long)cd * fsize;
            double norm = 0.0;
            for (int y = y0; y < y0 + lv->by; y++)
                for (int x = x0; x < x0 + lv->bx; x++)
                    for (int d = 0; d < lv->nc_f; d++) {
                        const cplx z = prev[mg_fine_index(lv, x, y, d)];
                        norm += creal(conj(z) * z);
                    }
            norm = sqrt(norm);
            for (int y = y0; y < y0 + lv->by; y++)
                for (int x = x0; x < x0 + lv->bx; x++)
                    for (int d = 0; d < lv->nc_f; d++) {
                        const long f = mg_fine_index(lv, x, y, d);
                        prev[f] = cdivr(prev[f], norm);
                    }
            for (int m = 0; m < cd; m++) {
                const cplx *vm = V + (long)m * fsize;
                cplx dot = 0.0;
                for (int y = y0; y < y0 + lv->by; y++)
                    for (int x = x0; x < x0 + lv->bx; x++)
                        for (int d = 0; d < lv->nc_f; d++) {
                            const long f = mg_fine_index(lv, x, y, d);
                            dot += conj(vm[f]) * cur[f];
                        }
                for (int y = y0; y < y0 + lv->by; y++)
                    for (int x = x0; x < x0 + lv->bx; x++)
                        for (int d = 0; d < lv->nc_f; d++) {
                            const long f = mg_fine_index(lv, x, y, d);
                            cur[f] -= dot * vm[f];
                        }
            }
        }
    }
    orc_mg_block_normalize(lv);
}

/* mg_complex.cpp:372-418 (prolong): fine = sum over coarse dof of null_vector * coarse. */
void orc_mg_prolong(const orc_mg_level *lv, double *fine_, const double *coarse_)
{
    const int xc_n = lv->lx / lv->bx, yc_n = lv->ly / lv->by;
    const long fsize = (long)lv->lx * lv->ly * lv->nc_f;
    const long csize = (long)xc_n * yc_n * lv->nc_c;
    cplx *fine = CX(fine_);
    const cplx *coarse = CCX(coarse_);
    memset(fine, 0, sizeof(cplx) * fsize);
    for (long i = 0; i < csize; i++) {
        const int cd = (int)(i % lv->nc_c);
        const long t = i / lv->nc_c;
        const int xc = (int)(t % xc_n), yc = (int)(t / xc_n);
        const cplx *v = CCX(lv->null_vectors) + (long)cd * fsize;
        for (int y = yc * lv->by; y < yc * lv->by + lv->by; y++)
            for (int x = xc * lv->bx; x < xc * lv->bx + lv->bx; x++)
                for (int d = 0; d < lv->nc_f; d++) {
                    const long f = mg_fine_index(lv, x, y, d);
                    fine[f] += v[f] * coarse[i];
                }
    }
}

/* mg_complex.cpp:421-467 (restrict): coarse = P^dagger fine. */
void orc_mg_restrict(const orc_mg_level *lv, double *coarse_, const double *fine_)
{
    const int xc_n = lv->lx / lv->bx, yc_n = lv->ly / lv->by;
    const long fsize = (long)lv->lx * lv->ly * lv->nc_f;
    const long csize = (long)xc_n * yc_n * lv->nc_c;
    cplx *coarse = CX(coarse_);
    const cplx *fine = CCX(fine_);
    memset(coarse, 0, sizeof(cplx) * csize);
    for (long i = 0; i < csize; i++) {
        const int cd = (int)(i % lv->nc_c);
        const long t = i / lv->nc_c;
        const int xc = (int)(t % xc_n), yc = (int)(t / xc_n);
        const cplx *v = CCX(lv->null_vectors) + (long)cd * fsize;
        for (int y = yc * lv->by; y < yc * lv->by + lv->by; y++)
            for (int x = xc * lv->bx; x < xc * lv->bx + lv->bx; x++)
                for (int d = 0; d < lv->nc_f; d++) {
                    const long f = mg_fine_index(lv, x, y, d);
                    coarse[i] += conj(v[f]) * fine[f];
                }
    }
}

/* One direction of apply_stencil_2d (stencil_2d::sdir, coarse_stencil.cpp:164-235): dir 0 =
 * clover and shifts, 1..4 = hopping +x, +y, -x, -y. */
static void stencil_apply_dir(const orc_op *op, cplx *lhs, const cplx *rhs, int dir)
{
    const int lx = op->lx, ly = op->ly, nc = op->nc;
    const long lsize = (long)lx * ly * nc;
    const cplx *clov = CCX(op->clover), *hop = CCX(op->hopping);
    const cplx shift = mk(op->shift[0], op->shift[1]);
    const cplx eo_shift = mk(op->eo_shift[0], op->eo_shift[1]);
    const cplx dof_shift = mk(op->dof_shift[0], op->dof_shift[1]);
    static const int hx[4] = {1, 0, -1, 0}, hy[4] = {0, 1, 0, -1};
    for (long i = 0; i < lsize; i++) {
        const int color = (int)(i % nc);
        const long site = i / nc;
        const int x = (int)(site % lx), y = (int)(site / lx);
        cplx acc = 0.0;
        if (dir == 0) {
            for (int c = 0; c < nc; c++) acc += clov[c + (long)nc * i] * rhs[site * nc + c];
            if (cabs(shift) != 0.0) acc += shift * rhs[i];
            if (cabs(eo_shift) != 0.0) acc += (((x + y) % 2 == 0 ? 1.0 : -1.0) * eo_shift) * rhs[i];
            if (cabs(dof_shift) != 0.0) acc += ((color < nc / 2 ? 1.0 : -1.0) * dof_shift) * rhs[i];
        } else {
            const int d = dir - 1;
            const int xx = (x + hx[d] + lx) % lx, yy = (y + hy[d] + ly) % ly;
            const long nb = ((long)yy * lx + xx) * nc;
            for (int c = 0; c < nc; c++) acc += hop[c + (long)nc * i + (long)d * nc * lsize] * rhs[nb + c];
        }
        lhs[i] = acc;
    }
}

/* mg_complex.cpp:827-1199 (generate_coarse_from_fine_stencil): P^dagger A_dir P probed with
 * unit coarse vectors, the clover first, then per coarse colour the +x, -x, +y, -y hopping
 * terms on even and odd coarse rows / columns, accumulated in that order.  The probing reads
 * each direction's neighbours on coarse sites of the other parity, so the coarse extents
 * must be even (the reference's requirement). */
void orc_mg_coarse_stencil(const orc_mg_level *lv, const orc_op *fine, int ignore_shifts, double *clover_,
                           double *hopping_)
{
    const int xc_n = lv->lx / lv->bx, yc_n = lv->ly / lv->by, nc = lv->nc_c;
    const long vc = (long)xc_n * yc_n, csize = vc * nc;
    const long fsize = (long)lv->lx * lv->ly * lv->nc_f;
    cplx *clover = CX(clover_), *hopping = CX(hopping_);
    cplx *t_rhs = (cplx *)calloc(csize, sizeof(cplx)), *t_lhs = (cplx *)calloc(csize, sizeof(cplx));
    cplx *Pr = (cplx *)calloc(fsize, sizeof(cplx)), *APr = (cplx *)calloc(fsize, sizeof(cplx));
    orc_op f = *fine;
    if (ignore_shifts) {
        f.shift[0] = f.shift[1] = f.eo_shift[0] = f.eo_shift[1] = f.dof_shift[0] = f.dof_shift[1] = 0.0;
    }
    memset(clover, 0, sizeof(cplx) * vc * nc * nc);
    memset(hopping, 0, sizeof(cplx) * 4 * vc * nc * nc);
#define PROBE(dir)                                                  \
    do {                                                            \
        orc_mg_prolong(lv, (double *)Pr, (const double *)t_rhs);    \
        stencil_apply_dir(&f, APr, Pr, dir);                        \
        orc_mg_restrict(lv, (double *)t_lhs, (const double *)APr);  \
    } while (0)
    for (int color = 0; color < nc; color++) {
        memset(t_rhs, 0, sizeof(cplx) * csize);
        for (long i = 0; i < vc; i++) t_rhs[i * nc + color] = 1.0;
        PROBE(0);
        for (long i = 0; i < csize; i++) clover[color + (long)nc * i] += t_lhs[i];
    }
    /* direction (1..4), its hopping slot, whether it runs along y */
    static const int dirs[4] = {1, 3, 2, 4}, slot[4] = {0, 2, 1, 3}, alongy[4] = {0, 0, 1, 1};
    for (int color = 0; color < nc; color++) {
        for (int k = 0; k < 4; k++) {
            for (int par = 0; par < 2; par++) {
                memset(t_rhs, 0, sizeof(cplx) * csize);
                for (long s = 0; s < vc; s++) {
                    const int xc = (int)(s % xc_n), yc = (int)(s / xc_n);
                    const int p = alongy[k] ? (yc % 2) : (int)(s % 2);
                    (void)xc;
                    if (p == par) t_rhs[s * nc + color] = 1.0;
                }
                PROBE(dirs[k]);
                for (long i = 0; i < csize; i++) {
                    const long s = i / nc;
                    const int xc = (int)(s % xc_n), yc = (int)(s / xc_n);
                    const int p = alongy[k] ? (yc % 2) : (xc % 2);
                    if (p == par) clover[color + (long)nc * i] += t_lhs[i];
                    else hopping[color + (long)nc * i + (long)slot[k] * nc * csize] += t_lhs[i];
                }
            }
        }
    }
#undef PROBE
    free(t_rhs); free(t_lhs); free(Pr); free(APr);
}
