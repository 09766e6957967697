"""Multigrid pieces on the GPU against the reference's outputs (golden fixtures from
multigrid/aa_mg/mg_complex.cpp and stencil_2d/coarse_stencil.cpp): block normalize /
orthonormalize, prolong / restrict, the Galerkin coarse stencil over two levels, the
top/bottom stencil kinds and the coarse-level operators of the multigrid code.

Bars: 1e-14 absolute on unit-normalised null vectors and on transferred fields of unit-size
entries; 1e-13 absolute on coarse stencil coefficients (sums of O(16) products of O(1) terms in
another order); operator outputs 1e-13 relative to the largest entry."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PIECES = {"stencil_tb": 11, "stencil_bt": 12, "stencil_m2mdtbdbt": 13, "stencil_normal_eo": 14,
          "stencil_normal_tb": 15, "stencil_dagger_eo": 16, "stencil_dagger_tb": 17}


def _maxrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _fine_op(gl, vec, c):
    return gl.Operator(4, 16, 16, nc=1, clover=np.zeros(256, np.complex128), hopping=vec["mg16_hop"],
                       shift=complex(*c["shift"]), eo_shift=complex(*c["eo_shift"]))


def test_block_orthonormalize_matches_reference(gl, gpu, golden):
    vec, _ = golden
    lv = gl.MgLevel(16, 16, 1, 4, 4, 4, vec["mg16_nv_in"])
    gl.block_normalize(lv)
    assert np.max(np.abs(lv.null_vectors().reshape(-1) - vec["mg16_nv_norm"])) < 1e-14
    lv = gl.MgLevel(16, 16, 1, 4, 4, 4, vec["mg16_nv_in"])
    gl.block_orthonormalize(lv)
    assert np.max(np.abs(lv.null_vectors().reshape(-1) - vec["mg16_nv_orth"])) < 1e-14
    lv2 = gl.MgLevel(4, 4, 4, 2, 2, 4, vec["mg4_nv_in"])
    gl.block_orthonormalize(lv2)
    assert np.max(np.abs(lv2.null_vectors().reshape(-1) - vec["mg4_nv_orth"])) < 1e-14


def test_prolong_restrict_match_reference(gl, gpu, golden):
    vec, _ = golden
    lv = gl.MgLevel(16, 16, 1, 4, 4, 4, vec["mg16_nv_orth"])
    f = np.zeros(256, np.complex128)
    gl.prolong(f, vec["mg16_coarse_in"], lv)
    assert np.max(np.abs(f - vec["mg16_prolong"])) < 1e-14
    c = np.zeros(64, np.complex128)
    gl.restrict(c, vec["mg16_src"], lv)
    assert np.max(np.abs(c - vec["mg16_restrict"])) < 1e-13
    lv2 = gl.MgLevel(4, 4, 4, 2, 2, 4, vec["mg4_nv_orth"])
    f2 = np.zeros(64, np.complex128)
    gl.prolong(f2, vec["mg4_coarse_in"], lv2)
    assert np.max(np.abs(f2 - vec["mg4_prolong"])) < 1e-14
    c2 = np.zeros(16, np.complex128)
    gl.restrict(c2, vec["mg16_coarse_in"], lv2)
    assert np.max(np.abs(c2 - vec["mg4_restrict"])) < 1e-13


@pytest.mark.parametrize("ig", [0, 1])
def test_coarse_stencil_matches_reference(gl, gpu, golden, ig):
    vec, cases = golden
    lv = gl.MgLevel(16, 16, 1, 4, 4, 4, vec["mg16_nv_orth"])
    st = gl.Stencil2D(4, 4, 4)
    coarse = gl.generate_coarse_from_fine_stencil(st, _fine_op(gl, vec, cases["mg16"]), lv, bool(ig))
    assert np.max(np.abs(st.clover - vec[f"mg16_coarse_clover_ig{ig}"])) < 1e-13
    assert np.max(np.abs(st.hopping - vec[f"mg16_coarse_hop_ig{ig}"])) < 1e-13
    # the device operator applies the same coefficients
    out = np.zeros(64, np.complex128)
    coarse.apply(out, vec["mg16_coarse_in"])
    ref = gl.Operator(4, 4, 4, nc=4, clover=vec[f"mg16_coarse_clover_ig{ig}"], hopping=vec[f"mg16_coarse_hop_ig{ig}"])
    out2 = np.zeros(64, np.complex128)
    ref.apply(out2, vec["mg16_coarse_in"])
    assert _maxrel(out, out2) < 1e-13


def test_second_level_coarse_stencil(gl, gpu, golden):
    vec, _ = golden
    lev2 = gl.Operator(4, 4, 4, nc=4, clover=vec["mg16_coarse_clover_ig0"], hopping=vec["mg16_coarse_hop_ig0"])
    lv2 = gl.MgLevel(4, 4, 4, 2, 2, 4, vec["mg4_nv_orth"])
    st = gl.Stencil2D(2, 2, 4)
    gl.generate_coarse_from_fine_stencil(st, lev2, lv2)
    assert np.max(np.abs(st.clover - vec["mg4_coarse_clover"])) < 1e-13
    assert np.max(np.abs(st.hopping - vec["mg4_coarse_hop"])) < 1e-13


@pytest.mark.parametrize("kind", list(PIECES))
def test_coarse_pieces_match_reference(gl, gpu, golden, kind):
    vec, _ = golden
    op = gl.Operator(PIECES[kind], 4, 4, nc=4, clover=vec["mg16_coarse_clover_ig0"],
                     hopping=vec["mg16_coarse_hop_ig0"], shift=0.1 + 0.02j)
    out = np.full(64, complex("nan"))
    op.apply(out, vec["mg16_piece_in"])
    assert _maxrel(out, vec[f"mg16_{kind}"]) < 1e-13


def test_tbprec_steps_match_reference(gl, gpu, golden):
    vec, _ = golden
    st = gl.Stencil2D(4, 4, 4, shift=0.1)
    st.clover[:], st.hopping[:] = vec["mg16_coarse_clover_ig0"], vec["mg16_coarse_hop_ig0"]
    out = np.zeros(64, np.complex128)
    gl.apply_square_staggered_tbprec_prepare_stencil(out, vec["mg16_piece_in"], st)
    assert _maxrel(out, vec["mg16_tb_prepare"]) < 1e-13
    gl.apply_square_staggered_tbprec_reconstruct_stencil(out, vec["mg16_coarse_in"], vec["mg16_piece_in"], st)
    assert _maxrel(out, vec["mg16_tb_reconstruct"]) < 1e-13


def test_galerkin_identity_256(gl, gpu, oracle):
    """At 256^2 with 4x4 blocks and 8 orthonormalised null vectors (device-resident): the coarse
    stencil applied to v equals R A P v, and the transfers are adjoint, <P c, f> = <c, R f>."""
    import torch
    lx = ly = 256
    g = gl.Generator(7)
    U = g.rand_gauge_u1(lx, ly)
    st = gl.Stencil2D(lx, ly, 1, shift=0.05)
    gl.get_square_staggered_u1_stencil(st, gl.StaggeredU1Op(U, 0.05, lx, ly))
    fine = gl.Operator(4, lx, ly, nc=1, clover=st.clover, hopping=st.hopping, shift=st.shift)
    nv = torch.from_numpy(np.stack([g.gaussian(lx * ly) for _ in range(8)])).to(gpu)
    lv = gl.MgLevel(lx, ly, 1, 4, 4, 8, nv)
    gl.block_orthonormalize(lv)
    coarse = gl.generate_coarse_from_fine_stencil(None, fine, lv)
    nc_size = 64 * 64 * 8
    v = torch.from_numpy(g.gaussian(nc_size)).to(gpu)
    a = torch.zeros_like(v)
    coarse.apply(a, v)
    pv = torch.zeros(lx * ly, dtype=torch.complex128, device=gpu)
    gl.prolong(pv, v, lv)
    apv = torch.zeros_like(pv)
    fine.apply(apv, pv)
    b = torch.zeros_like(v)
    gl.restrict(b, apv, lv)
    assert (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item() < 1e-13
    f = torch.from_numpy(g.gaussian(lx * ly)).to(gpu)
    rf = torch.zeros_like(v)
    gl.restrict(rf, f, lv)
    lhs, rhs = torch.vdot(pv, f).item(), torch.vdot(v, rf).item()
    assert abs(lhs - rhs) < 1e-12 * abs(rhs)


def _mg_hierarchy(gl, vec, case):
    """The reference driver's hierarchy rebuilt through the library: the 32x32 staggered stencil
    (m = 0.1), per level the given null vectors block-orthonormalised and the Galerkin coarse
    stencil, and the preconditioner's parameters."""
    U = vec["l32_links"]
    st = gl.Stencil2D(32, 32, 1)
    gl.get_square_staggered_u1_stencil(st, gl.StaggeredU1Op(U, case["mass"], 32, 32))
    st.shift = case["mass"]
    ops = [gl.Operator(4, 32, 32, nc=1, clover=st.clover, hopping=st.hopping, shift=st.shift)]
    levels = []
    nvs = [vec["mgs_nv1"], vec["mgs_nv2"]]
    lx, nc = 32, 1
    for l, (bs, nvec) in enumerate(zip(case["blocks"], case["nvecs"])):
        lv = gl.MgLevel(lx, lx, nc, bs, bs, nvec, nvs[l])
        gl.block_orthonormalize(lv)
        ops.append(gl.generate_coarse_from_fine_stencil(None, ops[-1], lv))
        levels.append(lv)
        lx, nc = lx // bs, nvec
    nr = len(levels)
    mgp = gl.MgPrecondStruct(ops, levels, in_smooth_type=case["smoother"], n_pre_smooth=[case["n_pre"]] * nr,
                             n_post_smooth=[case["n_post"]] * nr, in_solve_type=case["coarse"], n_max=case["n_max"],
                             n_restart=case["n_restart"], rel_res=[case["rel_res"]] * nr,
                             mlevel_type=case.get("mlevel", 0))
    return st, ops, mgp


@pytest.mark.parametrize("key", ["mgs2f", "mgs3f", "mgs3r", "mgs3v", "mgs2"])
def test_mg_preconditioned_vpgcr_matches_reference(gl, gpu, golden, capfd, key):
    """The variably preconditioned GCR with the multigrid preconditioner follows the reference's
    solve: the same iteration and operator counts, the printed relative residual, and the
    solution.  With fixed coarse work the preconditioner is a smooth function of its input and
    the solutions agree to 1e-9: two levels (mgs2f), three levels with the V cycle and a coarse
    GCR (mgs3f), the recursive form whose middle level runs a restarted variably preconditioned
    GCR preconditioned by the level below (mgs3r), and the V cycle with no coarse solver
    (mgs3v).  With the coarse GCR stopped at 1e-2 (mgs2) the stopping iteration of each coarse
    solve can move by one under rounding, and the bar is the residual within 10% and the
    solution within 1e-2."""
    vec, cases = golden
    c = cases[key]
    st, ops, mgp = _mg_hierarchy(gl, vec, c)
    b = vec["l32_src"]
    x = np.zeros_like(b)
    capfd.readouterr()
    info = gl.minv_vector_gcr_var_precond(x, b, b.size, c["max_iter"], 1e-10, gl.apply_stencil_2d, ops[0],
                                          gl.mg_preconditioner, mgp,
                                          gl.InversionVerboseStruct(gl.VERB_SUMMARY, "[MGSOLVE] "))
    out = capfd.readouterr().out.strip().splitlines()
    assert (info.iter, info.ops_count, info.success) == (c["iter"], c["ops_count"], c["success"])
    got = float(out[-1].rsplit(" ", 1)[1])
    want = float(c["summary"].rsplit(" ", 1)[1])
    assert out[-1].rsplit(" ", 1)[0] == c["summary"].rsplit(" ", 1)[0]
    ref = vec[f"{key}_solution"]
    if key.endswith("f"):
        assert abs(got - want) <= 1e-5 * want
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9
    else:
        assert abs(got - want) <= 0.1 * want
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-2


def test_mg_apply_reduces_error(gl, gpu, golden):
    """One V-cycle application: M^-1 applied to A e recovers e better than the identity does
    on the smooth null-space vectors the coarse space was built from."""
    vec, cases = golden
    st, ops, mgp = _mg_hierarchy(gl, vec, cases["mgs2f"])
    e = vec["mgs_nv1"][:1024] + vec["mgs_nv1"][4096:5120]  # a smooth vector (even + odd parts)
    Ae = np.zeros_like(e)
    ops[0].apply(Ae, e)
    z = np.zeros_like(e)
    mgp.apply(z, Ae)
    assert np.linalg.norm(z - e) < 0.5 * np.linalg.norm(e)
