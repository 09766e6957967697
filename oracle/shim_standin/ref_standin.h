// ref_standin.h -- the part of the reference's C++ interface that the drop-in shim
// (generic-linalg_gb300/shim/glinalg_shim.cpp) compiles against, declared here so that the
// shim can be built and run where the reference checkout is absent (the GPU machine).  TEST
// INFRASTRUCTURE ONLY: oracle/shim_gpu_check.cpp links the shim with these declarations and the
// library, and tests/test_shim_gpu.py runs it.  A reference program builds the shim against the
// reference's own headers instead (oracle/Makefile, target shim).
//
// The names, fields and signatures follow the reference's, because the shim and its callers
// use them: inversion_info (inverter_struct.h:14-89), inversion_verbose_struct
// (verbosity.h:18-24), staggered_u1_op (operators.h:7-15), stencil_2d and its direction enum
// (coarse_stencil.h:33-155), the lattice accessors the shim reads (lattice/lattice.h), the
// operator callbacks (operators.h, operators_stencil.h, coarse_stencil.h, mg_complex.h) and the
// preconditioner callbacks with their structs (generic_precond.h).  Only what the shim and the
// test caller use is declared; the callbacks here are recognised by the shim by address and
// never run.
#pragma once

#include <complex>
#include <cstring>
#include <string>

using namespace std;

struct inversion_verbose_struct {
    int verbosity = 0;
    string verb_prefix;
    int precond_verbosity = 0;
    string precond_verb_prefix;
};

// Result of a solve; a multishift solve owns n_rhs per-shift squared residuals.
class inversion_info {
  public:
    double resSq = 0.0;
    int iter = 0;
    bool success = false;
    string name;
    int ops_count = 0;
    double *resSqmrhs = nullptr;
    int n_rhs = -1;

    inversion_info() {}
    explicit inversion_info(int n) : n_rhs(n) { resSqmrhs = n > 0 ? new double[n]() : nullptr; }
    inversion_info(const inversion_info &o) { copy_from(o); }
    inversion_info &operator=(const inversion_info &o)
    {
        if (this != &o) {
            delete[] resSqmrhs;
            copy_from(o);
        }
        return *this;
    }
    ~inversion_info() { delete[] resSqmrhs; }

  private:
    void copy_from(const inversion_info &o)
    {
        resSq = o.resSq;
        iter = o.iter;
        success = o.success;
        name = o.name;
        ops_count = o.ops_count;
        n_rhs = o.n_rhs;
        resSqmrhs = nullptr;
        if (o.resSqmrhs && o.n_rhs > 0) {
            resSqmrhs = new double[o.n_rhs];
            memcpy(resSqmrhs, o.resSqmrhs, sizeof(double) * o.n_rhs);
        }
    }
};

// Extra data of the U(1) operator callbacks: links U[2*i + mu], i = y*x_fine + x.
struct staggered_u1_op {
    complex<double> *lattice = nullptr;
    double mass = 0.0;
    int x_fine = 0, y_fine = 0;
    int Nc = 1;
    double wilson_coeff = 0.0;
};

// A 2D lattice with nc degrees of freedom per site.
class Lattice {
  public:
    Lattice(int lx, int ly, int nc) : lx_(lx), ly_(ly), nc_(nc) {}
    int get_lattice_dimension(int mu) const { return mu == 0 ? lx_ : ly_; }
    int get_nc() const { return nc_; }

  private:
    int lx_, ly_, nc_;
};

// Which terms apply_stencil_2d applies: all of them, or one hopping direction.
enum stencil_dir { DIR_ALL = 0, DIR_XP1 = 1, DIR_YP1 = 2, DIR_XM1 = 3, DIR_YM1 = 4 };

// Operator as data: clover[c + nc*i], hopping[c + nc*i + dir*nc*V*nc], two_link likewise.
struct stencil_2d {
    Lattice *lat = nullptr;
    complex<double> *clover = nullptr, *hopping = nullptr, *two_link = nullptr;
    bool has_two = false;
    complex<double> shift = 0.0, eo_shift = 0.0, dof_shift = 0.0;
    stencil_dir sdir = DIR_ALL;
};

// Operator callbacks: lhs = A rhs.
void square_staggered_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void square_staggered_dagger_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void square_staggered_normal_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void square_laplace_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void square_staggered_deo_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void square_staggered_doe_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void square_staggered_m2mdeodoe_u1(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_stencil_2d(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_stencil_2d_eo(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_stencil_2d_oe(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_stencil_2d_tb(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_stencil_2d_bt(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_square_staggered_m2mdeodoe_stencil(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_square_staggered_m2mdtbdbt_stencil(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_square_staggered_normal_eo_stencil(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_square_staggered_normal_tb_stencil(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_square_staggered_dagger_eo_stencil(complex<double> *lhs, complex<double> *rhs, void *extra);
void apply_square_staggered_dagger_tb_stencil(complex<double> *lhs, complex<double> *rhs, void *extra);

// Preconditioner callbacks and the structs their extra data points at.
void identity_preconditioner(complex<double> *lhs, complex<double> *rhs, int size, void *extra,
                             inversion_verbose_struct *verb);
void minres_preconditioner(complex<double> *lhs, complex<double> *rhs, int size, void *extra,
                           inversion_verbose_struct *verb);
void gcr_preconditioner(complex<double> *lhs, complex<double> *rhs, int size, void *extra,
                        inversion_verbose_struct *verb);
struct minres_precond_struct_complex {
    int n_step = 0;
    double rel_res = 0.0;
    void (*matrix_vector)(complex<double> *, complex<double> *, void *) = nullptr;
    void *matrix_extra_data = nullptr;
};
struct gcr_precond_struct_complex {
    int n_step = 0;
    double rel_res = 0.0;
    void (*matrix_vector)(complex<double> *, complex<double> *, void *) = nullptr;
    void *matrix_extra_data = nullptr;
};

// The complex solver entry points the test caller uses (the shim defines them).
inversion_info minv_vector_cg(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                              void (*matrix_vector)(complex<double> *, complex<double> *, void *), void *extra_info,
                              inversion_verbose_struct *verbosity = 0);
inversion_info minv_vector_bicgstab(complex<double> *phi, complex<double> *phi0, int size, int max_iter, double eps,
                                    void (*matrix_vector)(complex<double> *, complex<double> *, void *),
                                    void *extra_info, inversion_verbose_struct *verbosity = 0);
inversion_info minv_vector_cg_m(complex<double> **phi, complex<double> *phi0, int n_shift, int size,
                                int resid_freq_check, int max_iter, double eps, double *shifts,
                                void (*matrix_vector)(complex<double> *, complex<double> *, void *),
                                void *extra_info, bool worst_first = false, inversion_verbose_struct *verbosity = 0);
