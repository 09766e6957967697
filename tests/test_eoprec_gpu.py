"""Even/odd preconditioning on the GPU against the reference's outputs (golden fixtures from
operators.cpp:455-620 and operators_stencil.cpp:179-236, compiled from the reference's
sources) and the reference's even/odd solve (tests/staggered_pieces/staggered_pieces.cpp:331-346).

Bars: operators and the prepare / reconstruct steps 1e-14 relative per site (the denominator
max(|ref_i|, s_i), s_i the summed magnitude of the terms at site i); the FP64 CG on
m^2 - D_eo D_oe takes the reference's iterations and operator applications, and its solution
is within 1e-11 of the reference's (the reconstructed full solution within 1e-11 (1 + 1/m):
the odd half is divided by the mass); the mixed-precision
even/odd solve reaches the FP64-true residual of its tolerance.

Where lx is a multiple of 256 and ly is even, the FP32 even/odd solve runs checkerboarded (the
even fields packed to half the lattice, the inner iterations in the rectangle-resident kernel
k_resident_eo); its bars, against the oracle's FP64 even/odd solve on the same inputs
(prepare, CG on m^2 - D_eo D_oe, reconstruct; tests/staggered_pieces/staggered_pieces.cpp:331-346):
the FP64-true relative residual of the even system below 1e-10, recomputed by the oracle's
operator; the even solution within 1e-9 of the oracle's (two solutions with relative residual
below 1e-10 differ by at most 2 kappa 1e-10; the measured distance is printed); odd sites of
the guess untouched; and the reconstructed full solution's residual |b - M x| equal to
|r_e| / m (the even rows of M x - b are r_e / m after reconstruct, the odd rows vanish), so
below 1.01e-10 |rhs_e| / m."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel, site_rel_err, staggered_scale

pytestmark = pytest.mark.gpu

LATS = {"l32": (32, 32), "l8": (8, 8), "l12x6": (12, 6)}
KIND = {"staggered_deo": 7, "staggered_doe": 8, "staggered_m2mdeodoe": 9}


def even_mask(lx, ly):
    y, x = np.divmod(np.arange(lx * ly), lx)
    return (x + y) % 2 == 0


@pytest.mark.parametrize("key", list(LATS))
@pytest.mark.parametrize("kind", list(KIND))
def test_eo_operators_match_reference(gl, gpu, golden, key, kind):
    vec, _ = golden
    lx, ly = LATS[key]
    U, b = vec[f"{key}_links"], vec[f"{key}_src"]
    out = np.full_like(b, complex("nan"))
    gl.Operator(KIND[kind], lx, ly, 0.1, U).apply(out, b)
    ref = vec[f"{key}_{kind}"]
    if kind == "staggered_m2mdeodoe":
        # the magnitude of D_oe b, then of D_eo applied to it, plus m^2 |b|
        doe = vec[f"{key}_staggered_doe"]
        scale = staggered_scale(U, doe, 0.0, lx, ly) + 0.01 * np.abs(b)
    else:
        scale = staggered_scale(U, b, 0.0, lx, ly)
    assert site_rel_err(out, ref, scale) < 1e-14
    assert np.all(out[~even_mask(lx, ly) if kind != "staggered_doe" else even_mask(lx, ly)] == 0)


@pytest.mark.parametrize("key", list(LATS))
def test_eo_prepare_reconstruct_match_reference(gl, gpu, golden, key):
    vec, _ = golden
    lx, ly = LATS[key]
    U, b, b2 = vec[f"{key}_links"], vec[f"{key}_src"], vec[f"{key}_src2"]
    extra = gl.StaggeredU1Op(U, 0.1, lx, ly)
    rhs_e = np.full_like(b, complex("nan"))
    gl.square_staggered_eoprec_prepare(rhs_e, b, extra)
    assert site_rel_err(rhs_e, vec[f"{key}_eo_prepare"], staggered_scale(U, b, 0.1, lx, ly)) < 1e-14
    full = np.full_like(b, complex("nan"))
    gl.square_staggered_eoprec_reconstruct(full, b2, b, extra)
    # odd sites: (b - D_oe b2) / m
    scale = (staggered_scale(U, b2, 0.0, lx, ly) + np.abs(b)) / 0.1
    assert site_rel_err(full, vec[f"{key}_eo_reconstruct"], scale) < 1e-14


def test_eo_stencil_form_matches_reference(gl, gpu, golden):
    vec, _ = golden
    lx = ly = 8
    U, b, b2 = vec["l8_links"], vec["l8_src"], vec["l8_src2"]
    st = gl.Stencil2D(lx, ly, 1)
    gl.get_square_staggered_u1_stencil(st, gl.StaggeredU1Op(U, 0.1, lx, ly))
    out = np.zeros_like(b)
    gl.apply_square_staggered_m2mdeodoe_stencil(out, b, st)
    scale = staggered_scale(U, vec["l8_staggered_doe"], 0.0, lx, ly) + 0.01 * np.abs(b)
    assert site_rel_err(out, vec["l8_stencil_m2mdeodoe"], scale) < 1e-14
    pe = np.zeros_like(b)
    gl.apply_square_staggered_eoprec_prepare_stencil(pe, b, st)
    assert site_rel_err(pe, vec["l8_stencil_eo_prepare"], staggered_scale(U, b, 0.1, lx, ly)) < 1e-14
    rc = np.zeros_like(b)
    gl.apply_square_staggered_eoprec_reconstruct_stencil(rc, b2, b, st)
    scale = (staggered_scale(U, b2, 0.0, lx, ly) + np.abs(b)) / 0.1
    assert site_rel_err(rc, vec["l8_stencil_eo_reconstruct"], scale) < 1e-14


def test_eo_solve_matches_reference(gl, gpu, golden):
    """prepare, FP64 CG on m^2 - D_eo D_oe, reconstruct: the reference's 183 iterations and
    185 operator applications, its solution within 1e-11."""
    vec, cases = golden
    c = cases["l32_eo_cg"]
    U, b = vec["l32_links"], vec["l32_src"]
    extra = gl.StaggeredU1Op(U, 0.1, 32, 32)
    rhs_e = np.zeros_like(b)
    gl.square_staggered_eoprec_prepare(rhs_e, b, extra)
    xe = np.zeros_like(b)
    info = gl.minv_vector_cg(xe, rhs_e, b.size, c["max_iter"], c["eps"], gl.square_staggered_m2mdeodoe_u1, extra)
    assert info.success and info.iter == c["iter"] and info.ops_count == c["ops_count"]
    assert rel(xe, vec["l32_eo_cg_even"]) < 1e-11
    full = np.zeros_like(b)
    gl.square_staggered_eoprec_reconstruct(full, xe, b, extra)
    # x_o = (b_o - D_oe x_e) / m: a difference in x_e reaches x_o amplified by up to 1/m
    assert rel(full, vec["l32_eo_solution"]) < 1e-11 * (1 + 1 / 0.1)


@pytest.mark.parametrize("prec", [1, 2])
def test_eo_mixed_solve(gl, gpu, golden, prec):
    """The mixed-precision CG on the even system (FP32 or FP16 inner iterations, FP64 reliable
    updates) reaches the FP64-true residual 1e-10 of the even system, writes only even sites,
    and its reconstructed solution agrees with the reference's to kappa * 1e-10."""
    vec, _ = golden
    U, b = vec["l32_links"], vec["l32_src"]
    extra = gl.StaggeredU1Op(U, 0.1, 32, 32)
    rhs_e = np.zeros_like(b)
    gl.square_staggered_eoprec_prepare(rhs_e, b, extra)
    odd = ~even_mask(32, 32)
    xe = np.zeros_like(b)
    xe[odd] = 7.0  # odd sites of the guess must come back untouched
    info = gl.minv_vector_cg(xe, rhs_e, b.size, 20000, 1e-10, gl.square_staggered_m2mdeodoe_u1, extra,
                             precision=prec)
    assert info.success
    assert np.all(xe[odd] == 7.0)
    xe[odd] = 0.0
    A = gl.Operator(9, 32, 32, 0.1, U)
    r = np.zeros_like(b)
    A.apply(r, xe)
    assert np.linalg.norm(rhs_e - r) / np.linalg.norm(rhs_e) < 1e-10
    full = np.zeros_like(b)
    gl.square_staggered_eoprec_reconstruct(full, xe, b, extra)
    assert rel(full, vec["l32_eo_solution"]) < 1e-7


def test_eo_solve_1024(gl, gpu):
    """M x = b on the 1024x1024, m = 0.01 system by even/odd preconditioning with the FP32
    mixed solver, checked with the FP64 operator M itself."""
    import torch
    lx = ly = 1024
    g = gl.Generator(1337)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    dev = torch.device("cuda:0")
    Ud, bd = torch.from_numpy(U).to(dev), torch.from_numpy(b).to(dev)
    eo = gl.Operator(9, lx, ly, 0.01, Ud)
    rhs_e = torch.zeros_like(bd)
    gl.square_staggered_eoprec_prepare(rhs_e, bd, eo)
    xe = torch.zeros_like(bd)
    info = gl.minv_vector_cg(xe, rhs_e, b.size, 100000, 1e-12, gl.square_staggered_m2mdeodoe_u1, eo, precision=1)
    assert info.success
    x = torch.zeros_like(bd)
    gl.square_staggered_eoprec_reconstruct(x, xe, bd, eo)
    Mx = torch.zeros_like(bd)
    gl.Operator(0, lx, ly, 0.01, Ud).apply(Mx, x)
    rr = (torch.linalg.vector_norm(Mx - bd) / torch.linalg.vector_norm(bd)).item()
    assert rr < 1e-9, rr


def oracle_eo(lx, ly, m, seed=1337):
    import pyoracle
    O = pyoracle.Oracle()
    O.set_threads(None)
    g = pyoracle.Generator(seed)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    eo = pyoracle.Operator("staggered_m2mdeodoe", lx, ly, m, U)
    rhs_e = O.eoprec_prepare(eo, b)
    xe, info, _ = O.solve("cg", eo, rhs_e, max_iter=100000, eps=1e-10)
    assert info["success"], info
    return U, b, rhs_e, xe, info, O, eo


@pytest.mark.parametrize("lx,ly,m", [(1024, 1024, 0.01), (256, 310, 0.05), (512, 76, 0.1)])
def test_eo_checkerboarded_solve_matches_oracle(gl, gpu, lx, ly, m):
    """The checkerboarded FP32 even/odd solve against the oracle's FP64 one.  1024^2 is the
    benchmark's system (4 x 38 rectangles of 128 packed columns by 27 rows); 256 x 310 has one
    rectangle across and a last row of rectangles one row high (3 rows elsewhere); 512 x 76 has
    rectangles one row high."""
    import pyoracle
    U, b, rhs_e, xo, io, O, eo = oracle_eo(lx, ly, m)
    n = lx * ly
    odd = ~even_mask(lx, ly)
    xe = np.zeros_like(b)
    xe[odd] = 7.0  # odd sites of the guess must come back untouched
    extra = gl.StaggeredU1Op(U, m, lx, ly)
    info = gl.minv_vector_cg(xe, rhs_e, n, 100000, 1e-10, gl.square_staggered_m2mdeodoe_u1, extra, precision=1)
    assert info.success, info
    assert info.name == "CG-FP32-EO" and info.kernel_launches >= 1, info
    assert np.all(xe[odd] == 7.0)
    xe[odd] = 0.0
    rr = float(np.linalg.norm(rhs_e - O.apply(eo, xe)) / np.linalg.norm(rhs_e))
    err = rel(xe, xo)
    full = np.zeros_like(b)
    gl.square_staggered_eoprec_reconstruct(full, xe, b, extra)
    M = pyoracle.Operator("staggered", lx, ly, m, U)
    res_full = float(np.linalg.norm(b - O.apply(M, full)))
    print(f"checkerboarded FP32 even/odd {lx}x{ly} m={m}: {info.iter} inner iterations "
          f"(oracle FP64 {io['iter']}), {info.reliable_updates} reliable updates, even relres {rr:.3e}, "
          f"err vs oracle {err:.3e}, full |b - Mx| / |b| {res_full / np.linalg.norm(b):.3e}")
    assert rr < 1e-10
    assert err < 1e-9
    assert res_full < 1.01e-10 * np.linalg.norm(rhs_e) / m
