// shim_gpu_check.cpp -- a C++ caller that reaches the library through the drop-in shim the way a
// reference program does (test infrastructure; tests/test_shim_gpu.py builds and runs it).  It
// is compiled against oracle/shim_standin/, the reference interface the shim needs, so that it
// builds where the reference checkout is absent.
//
//   shim_gpu_check <links.bin> <src.bin> <out_dir>
// links.bin: 2*32*32 complex<double>, src.bin: 32*32 complex<double> (the reference's 32x32
// test system).  One line per case on stdout, "case <name> key=value ...", and each solution
// written to <out_dir>/<name>.bin:
//   cg        minv_vector_cg on square_staggered_normal_u1, m = 0.1
//   bicgstab  minv_vector_bicgstab on square_staggered_u1, m = 0.1
//   cgm       minv_vector_cg_m on square_laplace_u1, mass 0.001, 7 shifts, resid_freq_check 1
//   foreign   a callback the library does not drive (refused: success = false, no CPU fallback)
//   onedir    apply_stencil_2d with a single hopping direction (refused)
#include <cstdio>
#include <string>
#include <vector>

#include "generic_cg.h"

typedef complex<double> cd;

static bool read_bin(const char *path, std::vector<cd> &v)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    const size_t got = fread(v.data(), sizeof(cd), v.size(), f);
    fclose(f);
    return got == v.size();
}

static void write_bin(const std::string &path, const cd *v, size_t n)
{
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return;
    fwrite(v, sizeof(cd), n, f);
    fclose(f);
}

static void report(const char *name, const inversion_info &r)
{
    printf("case %s success=%d iter=%d ops=%d resSq=%.17g name=%s", name, r.success ? 1 : 0, r.iter, r.ops_count,
           r.resSq, r.name.c_str());
    for (int i = 0; r.resSqmrhs && i < r.n_rhs; i++) printf(" res%d=%.17g", i, r.resSqmrhs[i]);
    printf("\n");
}

static void foreign_op(cd *lhs, cd *rhs, void *) { lhs[0] = rhs[0]; }

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: shim_gpu_check <links.bin> <src.bin> <out_dir>\n");
        return 2;
    }
    const int L = 32, V = L * L;
    std::vector<cd> U(2 * V), b(V);
    if (!read_bin(argv[1], U) || !read_bin(argv[2], b)) {
        fprintf(stderr, "cannot read the inputs\n");
        return 2;
    }
    const std::string out = argv[3];
    staggered_u1_op op;
    op.lattice = U.data();
    op.mass = 0.1;
    op.x_fine = L;
    op.y_fine = L;

    std::vector<cd> x(V, 0.0);
    inversion_info r = minv_vector_cg(x.data(), b.data(), V, 10000, 1e-10, square_staggered_normal_u1, &op);
    report("cg", r);
    write_bin(out + "/cg.bin", x.data(), V);

    std::fill(x.begin(), x.end(), cd(0.0));
    r = minv_vector_bicgstab(x.data(), b.data(), V, 10000, 1e-10, square_staggered_u1, &op);
    report("bicgstab", r);
    write_bin(out + "/bicgstab.bin", x.data(), V);

    staggered_u1_op lap = op;
    lap.mass = 0.001;
    double shifts[7] = {0.0, 0.004, 0.009, 0.049, 0.099, 0.499, 0.999};
    std::vector<cd> xs(7 * V, 0.0);
    cd *phis[7];
    for (int s = 0; s < 7; s++) phis[s] = xs.data() + (size_t)s * V;
    r = minv_vector_cg_m(phis, b.data(), 7, V, 1, 10000, 1e-10, shifts, square_laplace_u1, &lap);
    report("cgm", r);
    write_bin(out + "/cgm.bin", xs.data(), xs.size());

    r = minv_vector_cg(x.data(), b.data(), V, 100, 1e-10, foreign_op, &op);
    report("foreign", r);

    Lattice lat(L, L, 1);
    std::vector<cd> clover(V, 0.0), hopping(4 * V, 0.0);
    stencil_2d st;
    st.lat = &lat;
    st.clover = clover.data();
    st.hopping = hopping.data();
    st.shift = 0.1;
    st.sdir = DIR_XP1;
    r = minv_vector_cg(x.data(), b.data(), V, 100, 1e-10, apply_stencil_2d, &st);
    report("onedir", r);
    return 0;
}
