// ref_driver.cpp -- extern "C" wrappers around the reference's own C++ code
// (TEST INFRASTRUCTURE ONLY).
//
// oracle/Makefile compiles this file together with the reference's unmodified sources,
// read in place from the reference checkout, into oracle/_ref/libref_oracle.so.  The
// library is used in this container to pin the C oracle (oracle.c) and to write the golden
// fixtures under tests/golden/.  Nothing in the product links it.
//
// Complex fields cross the boundary as interleaved (re, im) doubles, which is the memory
// layout of std::complex<double> arrays.

#include <complex>
#include <cstring>
#include <fstream>
#include <vector>
#include <random>
#include <sstream>
#include <iostream>
#include <string>

#include "generic_vector.h"
#include "inverter_struct.h"
#include "verbosity.h"
#include "generic_cg.h"
#include "generic_cg_m.h"
#include "generic_bicgstab.h"
#include "generic_gcr.h"
#include "generic_cr.h"
#include "generic_cr_m.h"
#include "generic_minres.h"
#include "generic_bicgstab_l.h"
#include "generic_bicgstab_m.h"
#include "generic_cg_flex_precond.h"
#include "generic_gcr_var_precond.h"
#include "generic_precond.h"
#include "lattice.h"
#include "operators.h"
#include "coarse_stencil.h"
#include "operators_stencil.h"
#include "u1_utils.h"
#include "mg_complex.h"

using cd = std::complex<double>;
typedef void (*mv_fn)(cd *, cd *, void *);

namespace {

// One operator as the reference sees it: a callback and its extra_info.
struct RefOp {
    int kind;
    staggered_u1_op stag;
    Lattice *lat = nullptr;
    stencil_2d *st = nullptr;
    mv_fn fn = nullptr;
    void *extra = nullptr;
    long size = 0;
    ~RefOp()
    {
        delete st;
        delete lat;
    }
};

// kind: 0 D, 1 D^dagger, 2 D^dagger D, 3 gauge Laplacian, 4 stencil, 5 stencil_eo,
// 6 stencil_oe, 7 D_eo, 8 D_oe, 9 m^2 - D_eo D_oe, 10 its stencil form, 11 stencil_tb,
// 12 stencil_bt, 13 m^2 - D_tb D_bt, 14 normal_eo, 15 normal_tb, 16 dagger_eo, 17 dagger_tb
// (same numbering as oracle.h).
RefOp *make_op(int kind, int lx, int ly, int nc, double mass, const double *links,
               const double *clover, const double *hopping, const double *two_link,
               const double *shifts6)
{
    RefOp *o = new RefOp();
    o->kind = kind;
    o->stag.lattice = (cd *)links;
    o->stag.mass = mass;
    o->stag.x_fine = lx;
    o->stag.y_fine = ly;
    o->stag.Nc = 1;
    o->stag.wilson_coeff = 0.0;
    o->size = (long)lx * ly;
    switch (kind) {
    case 0: o->fn = square_staggered_u1; break;
    case 1: o->fn = square_staggered_dagger_u1; break;
    case 2: o->fn = square_staggered_normal_u1; break;
    case 3: o->fn = square_laplace_u1; break;
    case 7: o->fn = square_staggered_deo_u1; break;
    case 8: o->fn = square_staggered_doe_u1; break;
    case 9: o->fn = square_staggered_m2mdeodoe_u1; break;
    default: {
        int dims[2] = {lx, ly};
        o->lat = new Lattice(2, dims, nc);
        o->st = new stencil_2d(o->lat, two_link ? 2 : 1);
        long v = (long)lx * ly * nc * nc;
        std::memcpy(o->st->clover, clover, sizeof(cd) * v);
        std::memcpy(o->st->hopping, hopping, sizeof(cd) * v * 4);
        if (two_link) std::memcpy(o->st->two_link, two_link, sizeof(cd) * v * 8);
        if (shifts6) {
            o->st->shift = cd(shifts6[0], shifts6[1]);
            o->st->eo_shift = cd(shifts6[2], shifts6[3]);
            o->st->dof_shift = cd(shifts6[4], shifts6[5]);
        }
        o->st->generated = true;
        switch (kind) {
        case 4: o->fn = apply_stencil_2d; break;
        case 5: o->fn = apply_stencil_2d_eo; break;
        case 6: o->fn = apply_stencil_2d_oe; break;
        case 10: o->fn = apply_square_staggered_m2mdeodoe_stencil; break;
        case 11: o->fn = apply_stencil_2d_tb; break;
        case 12: o->fn = apply_stencil_2d_bt; break;
        case 13: o->fn = apply_square_staggered_m2mdtbdbt_stencil; break;
        case 14: o->fn = apply_square_staggered_normal_eo_stencil; break;
        case 15: o->fn = apply_square_staggered_normal_tb_stencil; break;
        case 16: o->fn = apply_square_staggered_dagger_eo_stencil; break;
        default: o->fn = apply_square_staggered_dagger_tb_stencil; break;
        }
        o->size = (long)lx * ly * nc;
        break;
    }
    }
    o->extra = o->st ? (void *)o->st : (void *)&o->stag;
    return o;
}

void fill_info(const inversion_info &inv, double *out4, char *name, int name_cap)
{
    out4[0] = inv.resSq;
    out4[1] = inv.iter;
    out4[2] = inv.success ? 1.0 : 0.0;
    out4[3] = inv.ops_count;
    if (name && name_cap > 0) {
        std::strncpy(name, inv.name.c_str(), name_cap - 1);
        name[name_cap - 1] = 0;
    }
}

// Runs fn with std::cout redirected into log (if given), so the verbosity lines the
// reference prints can be stored as fixtures.
template <typename F>
void with_log(char *log, int log_cap, F fn)
{
    std::ostringstream ss;
    std::streambuf *old = nullptr;
    if (log) old = std::cout.rdbuf(ss.rdbuf());
    fn();
    if (log) {
        std::cout.rdbuf(old);
        std::string s = ss.str();
        std::strncpy(log, s.c_str(), log_cap - 1);
        log[log_cap - 1] = 0;
    }
}

inversion_verbose_struct make_verb(int level, const char *prefix)
{
    inversion_verbose_struct v;
    v.verbosity = (inversion_verbose_level)level;
    v.verb_prefix = prefix ? prefix : "";
    v.precond_verbosity = VERB_NONE;
    v.precond_verb_prefix = "";
    return v;
}

}  // namespace

extern "C" {

// Inputs the way the reference's tests make them: one std::mt19937(seed), then
// rand_gauge_u1 (u1_utils.cpp:79-87), then n_src gaussian vectors (generic_vector.h:48-60).
void ref_make_inputs(unsigned seed, int lx, int ly, double *links, double *src, int n_src,
                     long src_len)
{
    std::mt19937 gen(seed);
    if (links) rand_gauge_u1((cd *)links, lx, ly, gen);
    for (int n = 0; n < n_src; n++) gaussian<double>((cd *)src + (long)n * src_len, (int)src_len, gen);
}

void ref_gauss_gauge(unsigned seed, int lx, int ly, double beta, double *links)
{
    std::mt19937 gen(seed);
    gauss_gauge_u1((cd *)links, lx, ly, gen, beta);
}

void ref_read_gauge(const char *path, int lx, int ly, double *links)
{
    read_gauge_u1((cd *)links, lx, ly, std::string(path));
}

void ref_apply(int kind, int lx, int ly, int nc, double mass, const double *links,
               const double *clover, const double *hopping, const double *two_link,
               const double *shifts6, double *lhs, const double *rhs)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> in((const cd *)rhs, (const cd *)rhs + o->size);
    o->fn((cd *)lhs, in.data(), o->extra);
    delete o;
}

void ref_staggered_stencil(int lx, int ly, double mass, const double *links, int dagger,
                           double *hopping_out, double *shift_out)
{
    int dims[2] = {lx, ly};
    Lattice lat(2, dims, 1);
    stencil_2d st(&lat, 1);
    staggered_u1_op s;
    s.lattice = (cd *)links;
    s.mass = mass;
    s.x_fine = lx;
    s.y_fine = ly;
    s.Nc = 1;
    s.wilson_coeff = 0.0;
    if (dagger) get_square_staggered_dagger_u1_stencil(&st, &s);
    else get_square_staggered_u1_stencil(&st, &s);
    std::memcpy(hopping_out, st.hopping, sizeof(cd) * (long)lx * ly * 4);
    shift_out[0] = st.shift.real();
    shift_out[1] = st.shift.imag();
}

// Even/odd preconditioning steps for kind 9 (square_staggered_eoprec_prepare /
// _reconstruct, operators.cpp:543 / :592) or kind 10 (the stencil forms,
// operators_stencil.cpp:181 / :220).
void ref_eoprec_prepare(int kind, int lx, int ly, int nc, double mass, const double *links,
                        const double *clover, const double *hopping, const double *two_link,
                        const double *shifts6, double *rhs_e, const double *rhs)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> in((const cd *)rhs, (const cd *)rhs + o->size);
    if (kind == 9) square_staggered_eoprec_prepare((cd *)rhs_e, in.data(), o->extra);
    else apply_square_staggered_eoprec_prepare_stencil((cd *)rhs_e, in.data(), o->st);
    delete o;
}

void ref_eoprec_reconstruct(int kind, int lx, int ly, int nc, double mass, const double *links,
                            const double *clover, const double *hopping, const double *two_link,
                            const double *shifts6, double *lhs_full, const double *lhs_e,
                            const double *rhs_o)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> e((const cd *)lhs_e, (const cd *)lhs_e + o->size);
    std::vector<cd> b((const cd *)rhs_o, (const cd *)rhs_o + o->size);
    if (kind == 9) square_staggered_eoprec_reconstruct((cd *)lhs_full, e.data(), b.data(), o->extra);
    else apply_square_staggered_eoprec_reconstruct_stencil((cd *)lhs_full, e.data(), b.data(), o->st);
    delete o;
}

// solver: 0 CG, 1 BiCGstab, 2 GCR; restart_freq > 0 selects the restarted variant.
void ref_solve(int solver, int restart_freq, int kind, int lx, int ly, int nc, double mass,
               const double *links, const double *clover, const double *hopping,
               const double *two_link, const double *shifts6, double *phi, const double *phi0,
               int max_iter, double eps, int verbosity, const char *prefix, double *info4,
               char *name, int name_cap, char *log, int log_cap)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> b((const cd *)phi0, (const cd *)phi0 + o->size);
    inversion_verbose_struct verb = make_verb(verbosity, prefix);
    inversion_info inv;
    with_log(log, log_cap, [&]() {
        cd *x = (cd *)phi;
        int sz = (int)o->size;
        if (solver == 0)
            inv = restart_freq > 0
                      ? minv_vector_cg_restart(x, b.data(), sz, max_iter, eps, restart_freq, o->fn, o->extra, &verb)
                      : minv_vector_cg(x, b.data(), sz, max_iter, eps, o->fn, o->extra, &verb);
        else if (solver == 1)
            inv = restart_freq > 0
                      ? minv_vector_bicgstab_restart(x, b.data(), sz, max_iter, eps, restart_freq, o->fn, o->extra, &verb)
                      : minv_vector_bicgstab(x, b.data(), sz, max_iter, eps, o->fn, o->extra, &verb);
        else
            inv = restart_freq > 0
                      ? minv_vector_gcr_restart(x, b.data(), sz, max_iter, eps, restart_freq, o->fn, o->extra, &verb)
                      : minv_vector_gcr(x, b.data(), sz, max_iter, eps, o->fn, o->extra, &verb);
    });
    fill_info(inv, info4, name, name_cap);
    delete o;
}

// Multishift CG (generic_cg_m.cpp:312).  phi holds n_shift vectors back to back.
void ref_cg_m(int kind, int lx, int ly, int nc, double mass, const double *links,
              const double *clover, const double *hopping, const double *two_link,
              const double *shifts6, double *phi, const double *phi0, int n_shift,
              int resid_freq_check, int max_iter, double eps, double *shifts, int worst_first,
              int verbosity, const char *prefix, double *info4, double *resSqmrhs, char *log,
              int log_cap)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> b((const cd *)phi0, (const cd *)phi0 + o->size);
    std::vector<cd *> ptrs(n_shift);
    for (int n = 0; n < n_shift; n++) ptrs[n] = (cd *)phi + (long)n * o->size;
    inversion_verbose_struct verb = make_verb(verbosity, prefix);
    inversion_info inv;
    with_log(log, log_cap, [&]() {
        inv = minv_vector_cg_m(ptrs.data(), b.data(), n_shift, (int)o->size, resid_freq_check,
                               max_iter, eps, shifts, o->fn, o->extra, worst_first != 0, &verb);
    });
    fill_info(inv, info4, nullptr, 0);
    for (int n = 0; n < n_shift; n++) resSqmrhs[n] = inv.resSqmrhs[n];
    delete o;
}

// Sibling solvers.  solver: 3 CR, 4 MinRes (param = omega), 5 BiCGstab-l (l = iparam),
// 6 flexibly preconditioned CG, 7 variably preconditioned GCR; restart_freq > 0 selects the
// restarted variant (CR, BiCGstab-l, FPCG, VPGCR).  The preconditioner (6, 7) is
// identity_preconditioner (pkind 0), minres_preconditioner (1) or gcr_preconditioner (2) with
// n_step iterations to rel_res on the same operator (generic_precond.cpp).
void ref_solve2(int solver, int restart_freq, int kind, int lx, int ly, int nc, double mass,
                const double *links, const double *clover, const double *hopping,
                const double *two_link, const double *shifts6, double *phi, const double *phi0,
                int max_iter, double eps, int iparam, double param, int pkind, int n_step,
                double rel_res, int verbosity, const char *prefix, int pverbosity,
                const char *pprefix, double *info4, char *name, int name_cap, char *log,
                int log_cap)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> b((const cd *)phi0, (const cd *)phi0 + o->size);
    inversion_verbose_struct verb = make_verb(verbosity, prefix);
    verb.precond_verbosity = (inversion_verbose_level)pverbosity;
    verb.precond_verb_prefix = pprefix ? pprefix : "";
    minres_precond_struct_complex mps;
    gcr_precond_struct_complex gps;
    mps.n_step = gps.n_step = n_step;
    mps.rel_res = gps.rel_res = rel_res;
    mps.matrix_vector = gps.matrix_vector = o->fn;
    mps.matrix_extra_data = gps.matrix_extra_data = o->extra;
    typedef void (*pc_fn)(cd *, cd *, int, void *, inversion_verbose_struct *);
    pc_fn pfn_id = identity_preconditioner, pfn_mr = minres_preconditioner, pfn_gcr = gcr_preconditioner;
    pc_fn pfn = pkind == 1 ? pfn_mr : pkind == 2 ? pfn_gcr : pfn_id;
    void *pinfo = pkind == 1 ? (void *)&mps : pkind == 2 ? (void *)&gps : nullptr;
    inversion_info inv;
    with_log(log, log_cap, [&]() {
        cd *x = (cd *)phi;
        int sz = (int)o->size;
        switch (solver) {
        case 3:
            inv = restart_freq > 0
                      ? minv_vector_cr_restart(x, b.data(), sz, max_iter, eps, restart_freq, o->fn, o->extra, &verb)
                      : minv_vector_cr(x, b.data(), sz, max_iter, eps, o->fn, o->extra, &verb);
            break;
        case 4: inv = minv_vector_minres(x, b.data(), sz, max_iter, eps, param, o->fn, o->extra, &verb); break;
        case 5:
            inv = restart_freq > 0
                      ? minv_vector_bicgstab_l_restart(x, b.data(), sz, max_iter, eps, restart_freq, iparam, o->fn, o->extra, &verb)
                      : minv_vector_bicgstab_l(x, b.data(), sz, max_iter, eps, iparam, o->fn, o->extra, &verb);
            break;
        case 6:
            inv = restart_freq > 0
                      ? minv_vector_cg_flex_precond_restart(x, b.data(), sz, max_iter, eps, restart_freq, o->fn, o->extra, pfn, pinfo, &verb)
                      : minv_vector_cg_flex_precond(x, b.data(), sz, max_iter, eps, o->fn, o->extra, pfn, pinfo, &verb);
            break;
        default:
            inv = restart_freq > 0
                      ? minv_vector_gcr_var_precond_restart(x, b.data(), sz, max_iter, eps, restart_freq, o->fn, o->extra, pfn, pinfo, &verb)
                      : minv_vector_gcr_var_precond(x, b.data(), sz, max_iter, eps, o->fn, o->extra, pfn, pinfo, &verb);
            break;
        }
    });
    fill_info(inv, info4, name, name_cap);
    delete o;
}

// Multishift CR (solver 0, generic_cr_m.cpp:312) or BiCGstab-M (solver 1,
// generic_bicgstab_m.cpp:398).  phi holds n_shift vectors back to back.
void ref_multishift2(int solver, int kind, int lx, int ly, int nc, double mass, const double *links,
                     const double *clover, const double *hopping, const double *two_link,
                     const double *shifts6, double *phi, const double *phi0, int n_shift,
                     int resid_freq_check, int max_iter, double eps, double *shifts, int worst_first,
                     int verbosity, const char *prefix, double *info4, double *resSqmrhs, char *log,
                     int log_cap)
{
    RefOp *o = make_op(kind, lx, ly, nc, mass, links, clover, hopping, two_link, shifts6);
    std::vector<cd> b((const cd *)phi0, (const cd *)phi0 + o->size);
    std::vector<cd *> ptrs(n_shift);
    for (int n = 0; n < n_shift; n++) ptrs[n] = (cd *)phi + (long)n * o->size;
    inversion_verbose_struct verb = make_verb(verbosity, prefix);
    inversion_info inv;
    with_log(log, log_cap, [&]() {
        if (solver == 0)
            inv = minv_vector_cr_m(ptrs.data(), b.data(), n_shift, (int)o->size, resid_freq_check,
                                   max_iter, eps, shifts, o->fn, o->extra, worst_first != 0, &verb);
        else
            inv = minv_vector_bicgstab_m(ptrs.data(), b.data(), n_shift, (int)o->size, resid_freq_check,
                                         max_iter, eps, shifts, o->fn, o->extra, worst_first != 0, &verb);
    });
    fill_info(inv, info4, nullptr, 0);
    for (int n = 0; n < n_shift; n++) resSqmrhs[n] = inv.resSqmrhs[n];
    delete o;
}

// Gauge-field utilities (u1_utils.cpp).
void ref_plaquette(const double *links, int lx, int ly, double *out2)
{
    cd p = get_plaquette_u1((cd *)links, lx, ly);
    out2[0] = p.real();
    out2[1] = p.imag();
}

double ref_topo(const double *links, int lx, int ly) { return get_topo_u1((cd *)links, lx, ly); }

// rand_trans_u1 from std::mt19937(seed), then apply_gauge_trans_u1 in place.
void ref_gauge_trans(unsigned seed, double *links, double *trans, int lx, int ly)
{
    std::mt19937 gen(seed);
    rand_trans_u1((cd *)trans, lx, ly, gen);
    apply_gauge_trans_u1((cd *)links, (cd *)trans, lx, ly);
}

void ref_ape_smear(double *smeared, const double *links, int lx, int ly, double alpha, int n_iter)
{
    std::vector<cd> in((const cd *)links, (const cd *)links + 2L * lx * ly);
    apply_ape_smear_u1((cd *)smeared, in.data(), lx, ly, alpha, n_iter);
}

void ref_write_gauge(const char *path, const double *links, int lx, int ly)
{
    // write_gauge_u1 opens with ios::in|ios::out|ios::trunc, which needs the file to exist
    { std::ofstream touch(path); }
    write_gauge_u1((cd *)links, lx, ly, std::string(path));
}

void ref_unit_gauge(double *links, int lx, int ly) { unit_gauge_u1((cd *)links, lx, ly); }

// Top/bottom preconditioning steps of a coarse stencil (mg_complex.cpp:1211, :1252).
void ref_tbprec(int step, int lx, int ly, int nc, const double *clover, const double *hopping,
                const double *shifts6, double *out, const double *a, const double *b)
{
    RefOp *o = make_op(13, lx, ly, nc, 0.0, nullptr, clover, hopping, nullptr, shifts6);
    std::vector<cd> va((const cd *)a, (const cd *)a + o->size);
    if (step == 0) {
        apply_square_staggered_tbprec_prepare_stencil((cd *)out, va.data(), o->st);
    } else {
        std::vector<cd> vb((const cd *)b, (const cd *)b + o->size);
        apply_square_staggered_tbprec_reconstruct_stencil((cd *)out, va.data(), vb.data(), o->st);
    }
    delete o;
}

namespace {
// A one-level mg_operator_struct_complex (mg_complex.h) at level 0 over the given null vectors.
struct RefMg {
    mg_operator_struct_complex s;
    int bx[1], by[1], nv[1];
    Lattice *lat[2];
    cd **vecs_level[1];
    std::vector<cd *> vecs;
    RefMg(int lx, int ly, int nc_f, int bxs, int bys, int nc_c, double *null_vectors)
    {
        int df[2] = {lx, ly}, dc[2] = {lx / bxs, ly / bys};
        lat[0] = new Lattice(2, df, nc_f);
        lat[1] = new Lattice(2, dc, nc_c);
        bx[0] = bxs;
        by[0] = bys;
        nv[0] = nc_c;
        const long fsize = (long)lx * ly * nc_f;
        for (int c = 0; c < nc_c; c++) vecs.push_back((cd *)null_vectors + c * fsize);
        vecs_level[0] = vecs.data();
        s.x_fine = lx;
        s.y_fine = ly;
        s.n_refine = 1;
        s.blocksize_x = bx;
        s.blocksize_y = by;
        s.Nc = nc_f;
        s.latt = lat;
        s.stencils = nullptr;
        s.have_dagger_stencil = false;
        s.dagger_stencils = nullptr;
        s.n_vectors = nv;
        s.null_vectors = vecs_level;
        s.curr_level = 0;
        s.curr_dof_fine = nc_f;
        s.curr_x_fine = lx;
        s.curr_y_fine = ly;
        s.curr_fine_size = (int)fsize;
        s.curr_dof_coarse = nc_c;
        s.curr_x_coarse = dc[0];
        s.curr_y_coarse = dc[1];
        s.curr_coarse_size = dc[0] * dc[1] * nc_c;
        s.dslash_count = nullptr;
    }
    ~RefMg()
    {
        delete lat[0];
        delete lat[1];
    }
};
}  // namespace

// op: 0 block_normalize, 1 block_orthonormalize (null_vectors in place)
void ref_mg_block(int op, int lx, int ly, int nc_f, int bx, int by, int nc_c, double *null_vectors)
{
    RefMg m(lx, ly, nc_f, bx, by, nc_c, null_vectors);
    if (op == 0) block_normalize(&m.s);
    else block_orthonormalize(&m.s);
}

// dir: 0 prolong (coarse -> fine), 1 restrict (fine -> coarse)
void ref_mg_transfer(int dir, int lx, int ly, int nc_f, int bx, int by, int nc_c, double *null_vectors,
                     double *out, const double *in)
{
    RefMg m(lx, ly, nc_f, bx, by, nc_c, null_vectors);
    const long n_in = dir == 0 ? (long)m.s.curr_coarse_size : (long)m.s.curr_fine_size;
    std::vector<cd> v((const cd *)in, (const cd *)in + n_in);
    if (dir == 0) prolong((cd *)out, v.data(), &m.s);
    else restrict((cd *)out, v.data(), &m.s);
}

// generate_coarse_from_fine_stencil for a fine stencil (clover, hopping, shifts; no two-link)
void ref_mg_coarse(int lx, int ly, int nc_f, int bx, int by, int nc_c, double *null_vectors,
                   const double *fclover, const double *fhopping, const double *shifts6, int ignore_shifts,
                   double *cclover, double *chopping)
{
    RefMg m(lx, ly, nc_f, bx, by, nc_c, null_vectors);
    stencil_2d fine(m.lat[0], 1);
    const long vf = (long)lx * ly * nc_f * nc_f;
    std::memcpy(fine.clover, fclover, sizeof(cd) * vf);
    std::memcpy(fine.hopping, fhopping, sizeof(cd) * vf * 4);
    fine.shift = cd(shifts6[0], shifts6[1]);
    fine.eo_shift = cd(shifts6[2], shifts6[3]);
    fine.dof_shift = cd(shifts6[4], shifts6[5]);
    fine.generated = true;
    stencil_2d coarse(m.lat[1], 1);
    generate_coarse_from_fine_stencil(&coarse, &fine, &m.s, ignore_shifts != 0);
    const long vc = (long)(lx / bx) * (ly / by) * nc_c * nc_c;
    std::memcpy(cclover, coarse.clover, sizeof(cd) * vc);
    std::memcpy(chopping, coarse.hopping, sizeof(cd) * vc * 4);
}

// An outer flexible solve (outer 0: minv_vector_cg_flex_precond, 1: minv_vector_gcr_var_precond)
// of the staggered operator on lx x ly (stencil form, shift = mass) preconditioned by the
// reference's mg_preconditioner (mg_complex.cpp:514) over n_refine levels.  Level l blocks
// bs[l] x bs[l] with nvec[l] null vectors taken from nv (Gaussian inputs, concatenated per
// level), block-orthonormalised and turned into Galerkin coarse stencils here, as the
// reference's driver does after its null-vector generation.  smoother: minv_inverter;
// inner: inner_solver; mlevel: mg_multilevel_type.
void ref_mg_solve(int outer, int lx, int ly, double mass, const double *links, int n_refine, const int *bs,
                  const int *nvec, double *nv, int smoother, const int *n_pre, const int *n_post, int inner,
                  int n_max, int n_restart, const double *rel_res, int mlevel, double *phi, const double *phi0,
                  int max_iter, double eps, double *info4, char *log, int log_cap)
{
    const int L = n_refine + 1;
    std::vector<Lattice *> lat(L);
    std::vector<stencil_2d *> sten(L);
    std::vector<int> bx(n_refine), by(n_refine), nvs(n_refine);
    std::vector<cd **> vecs(n_refine);
    int dims[2] = {lx, ly}, nc = 1;
    lat[0] = new Lattice(2, dims, 1);
    for (int l = 0; l < n_refine; l++) {
        bx[l] = by[l] = bs[l];
        nvs[l] = nvec[l];
        dims[0] /= bs[l];
        dims[1] /= bs[l];
        lat[l + 1] = new Lattice(2, dims, nvec[l]);
    }
    staggered_u1_op stag;
    stag.lattice = (cd *)links;
    stag.mass = mass;
    stag.x_fine = lx;
    stag.y_fine = ly;
    stag.Nc = 1;
    stag.wilson_coeff = 0.0;
    sten[0] = new stencil_2d(lat[0], 1);
    get_square_staggered_u1_stencil(sten[0], &stag);
    for (int l = 1; l < L; l++) sten[l] = new stencil_2d(lat[l], 1);
    long off = 0;
    for (int l = 0; l < n_refine; l++) {
        const long fs = lat[l]->get_lattice_size();
        vecs[l] = new cd *[nvec[l]];
        for (int c = 0; c < nvec[l]; c++) vecs[l][c] = (cd *)nv + off + (long)c * fs;
        off += (long)nvec[l] * fs;
    }
    mg_operator_struct_complex mg;
    mg.x_fine = lx;
    mg.y_fine = ly;
    mg.n_refine = n_refine;
    mg.blocksize_x = bx.data();
    mg.blocksize_y = by.data();
    mg.Nc = nc;
    mg.latt = lat.data();
    mg.stencils = sten.data();
    mg.have_dagger_stencil = false;
    mg.dagger_stencils = nullptr;
    mg.n_vectors = nvs.data();
    mg.null_vectors = vecs.data();
    mg.matrix_vector = square_staggered_u1;
    mg.matrix_vector_dagger = square_staggered_dagger_u1;
    mg.matrix_extra_data = &stag;
    mg.curr_level = 0;
    mg.curr_dof_fine = 1;
    mg.curr_x_fine = lx;
    mg.curr_y_fine = ly;
    mg.curr_fine_size = lx * ly;
    mg.curr_dof_coarse = nvec[0];
    mg.curr_x_coarse = lat[1]->get_lattice_dimension(0);
    mg.curr_y_coarse = lat[1]->get_lattice_dimension(1);
    mg.curr_coarse_size = lat[1]->get_lattice_size();
    mg.dslash_count = new dslash_tracker(n_refine);
    // null vectors, then the coarse stencils, level by level (going down and back up)
    for (int l = 0; l < n_refine; l++) {
        block_orthonormalize(&mg);
        generate_coarse_from_fine_stencil(sten[l + 1], sten[l], &mg);
        if (l + 1 < n_refine) level_down(&mg);
    }
    for (int l = 0; l + 1 < n_refine; l++) level_up(&mg);
    std::vector<int> pre(n_pre, n_pre + n_refine), post(n_post, n_post + n_refine);
    std::vector<double> rr(rel_res, rel_res + n_refine);
    mg_precond_struct_complex mgp;
    mgp.in_smooth_type = (minv_inverter)smoother;
    mgp.omega_smooth = 1.0;
    mgp.n_pre_smooth = pre.data();
    mgp.n_post_smooth = post.data();
    mgp.normal_eqn_mg = false;
    mgp.normal_eqn_smooth = false;
    mgp.mlevel_type = (mg_multilevel_type)mlevel;
    mgp.in_solve_type = (inner_solver)inner;
    mgp.n_max = n_max;
    mgp.n_restart = n_restart;
    mgp.rel_res = rr.data();
    mgp.mgstruct = &mg;
    mgp.fine_matrix_vector = fine_square_staggered;
    mgp.coarse_matrix_vector = coarse_square_staggered;
    mgp.fine_matrix_vector_dagger = fine_square_staggered_dagger;
    mgp.coarse_matrix_vector_dagger = coarse_square_staggered_dagger;
    mgp.fine_matrix_vector_normal = fine_square_staggered_normal;
    mgp.coarse_matrix_vector_normal = coarse_square_staggered_normal;
    mgp.matrix_extra_data = &mg;
    std::vector<cd> b((const cd *)phi0, (const cd *)phi0 + (long)lx * ly);
    inversion_verbose_struct verb = make_verb(1, "[MGSOLVE] ");
    inversion_info inv;
    with_log(log, log_cap, [&]() {
        if (outer == 0)
            inv = minv_vector_cg_flex_precond((cd *)phi, b.data(), lx * ly, max_iter, eps, fine_square_staggered, &mg,
                                              mg_preconditioner, &mgp, &verb);
        else
            inv = minv_vector_gcr_var_precond((cd *)phi, b.data(), lx * ly, max_iter, eps, fine_square_staggered, &mg,
                                              mg_preconditioner, &mgp, &verb);
    });
    fill_info(inv, info4, nullptr, 0);
    delete mg.dslash_count;
    for (int l = 0; l < n_refine; l++) delete[] vecs[l];
    for (int l = 0; l < L; l++) {
        delete sten[l];
        delete lat[l];
    }
}

}  // extern "C"
