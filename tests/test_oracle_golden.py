"""The CPU oracle (oracle/oracle.c) against the reference's own outputs (tests/golden/,
written by make_golden.py from the reference compiled from its sources).  Bit-exact: the
oracle keeps the reference's operation order and complex arithmetic."""
from __future__ import annotations

import numpy as np
import pytest

from pyoracle import Operator

LATS = {"l32": (32, 32), "l8": (8, 8), "l12x6": (12, 6)}


@pytest.mark.parametrize("key", list(LATS))
@pytest.mark.parametrize("kind", ["staggered", "staggered_dagger", "staggered_normal", "laplace"])
def test_operators_bit_exact(oracle, golden, key, kind):
    vec, _ = golden
    lx, ly = LATS[key]
    mass = 0.01 if kind == "laplace" else 0.1
    out = oracle.apply(Operator(kind, lx, ly, mass, vec[f"{key}_links"]), vec[f"{key}_src"])
    assert np.array_equal(out, vec[f"{key}_{kind}"])


@pytest.mark.parametrize("key", list(LATS))
@pytest.mark.parametrize("dagger", [0, 1])
def test_stencil_builder_bit_exact(oracle, golden, key, dagger):
    vec, _ = golden
    lx, ly = LATS[key]
    hop = oracle.staggered_stencil(vec[f"{key}_links"], lx, ly, dagger=bool(dagger))
    assert np.array_equal(hop, vec[f"{key}_stencil_hop{dagger}"])
    op = Operator("stencil", lx, ly, nc=1, clover=np.zeros(lx * ly, np.complex128), hopping=hop, shift=0.1)
    assert np.array_equal(oracle.apply(op, vec[f"{key}_src"]), vec[f"{key}_stencil_apply{dagger}"])


def test_stencil_equals_function(golden):
    """tests/staggered_stencil/staggered_stencil.cpp:212-251: stencil form == function form."""
    vec, _ = golden
    for key in LATS:
        assert np.abs(vec[f"{key}_stencil_apply0"] - vec[f"{key}_staggered"]).max() < 1e-15
        assert np.abs(vec[f"{key}_stencil_apply1"] - vec[f"{key}_staggered_dagger"]).max() < 1e-15


@pytest.mark.parametrize("kind", ["stencil", "stencil_eo", "stencil_oe"])
@pytest.mark.parametrize("two", [0, 1])
def test_generic_stencil_bit_exact(oracle, golden, kind, two):
    vec, cases = golden
    c = cases["st3"]
    op = Operator(kind, c["lx"], c["ly"], nc=c["nc"], clover=vec["st3_clover"], hopping=vec["st3_hopping"],
                  two_link=vec["st3_two"] if two else None, shift=complex(*c["shift"]),
                  eo_shift=complex(*c["eo_shift"]), dof_shift=complex(*c["dof_shift"]))
    assert np.array_equal(oracle.apply(op, vec["st3_x"]), vec[f"st3_{kind}_two{two}"])


SOLVES = [("cg", 0), ("cg", 17), ("bicgstab", 0), ("bicgstab", 17), ("gcr", 0), ("gcr", 17)]


@pytest.mark.parametrize("solver,rf", SOLVES)
def test_solvers_bit_exact(oracle, golden, solver, rf):
    vec, cases = golden
    key = f"l32_{solver}" + (f"_r{rf}" if rf else "")
    c = cases[key]
    op = Operator(c["op"], 32, 32, 0.1, vec["l32_links"])
    x, info, _ = oracle.solve(solver, op, vec["l32_src"], max_iter=c["max_iter"], eps=c["eps"], restart_freq=rf)
    for f in ("iter", "ops_count", "success", "name"):
        assert info[f] == c[f], f
    assert info["resSq"] == c["resSq"]
    assert np.array_equal(x, vec[key])


def test_cg_initial_guess(oracle, golden):
    vec, cases = golden
    op = Operator("staggered_normal", 32, 32, 0.1, vec["l32_links"])
    x, info, _ = oracle.solve("cg", op, vec["l32_src"], phi=vec["l32_src2"])
    assert info["iter"] == cases["l32_cg_guess"]["iter"]
    assert np.array_equal(x, vec["l32_cg_guess"])


@pytest.mark.parametrize("key,max_iter", [("l32_cg_maxiter7", 7), ("l32_bicgstab_maxiter5", 5), ("l32_gcr_maxiter5", 5)])
def test_max_iter_failure_path(oracle, golden, key, max_iter):
    """success == false when the loop reaches max_iter - 1 (generic_cg.cpp:356-363)."""
    vec, cases = golden
    solver = key.split("_")[1]
    kind = "staggered_normal" if solver == "cg" else "staggered"
    op = Operator(kind, 32, 32, 0.1, vec["l32_links"])
    _, info, hist = oracle.solve(solver, op, vec["l32_src"], max_iter=max_iter, hist_cap=max_iter)
    c = cases[key]
    assert (info["iter"], info["ops_count"], info["success"]) == (c["iter"], c["ops_count"], c["success"])
    assert info["resSq"] == c["resSq"]
    # the DETAIL log prints the same relative residuals, %g-formatted
    logged = [float(l.split("RelRes ")[1]) for l in c["log"].splitlines() if " Iter " in l and "Success" not in l]
    assert np.allclose(hist[: len(logged)], logged, rtol=1e-5)


@pytest.mark.parametrize("rfc,wf", [(1, 0), (3, 0), (1, 1)])
def test_cg_m_bit_exact(oracle, golden, rfc, wf):
    vec, cases = golden
    key = f"l32_cgm_rfc{rfc}_wf{wf}"
    c = cases[key]
    op = Operator("laplace", 32, 32, c["mass"], vec["l32_links"])
    x, info, res = oracle.cg_m(op, vec["l32_src"], c["shifts"], resid_freq_check=rfc, worst_first=bool(wf))
    assert (info["iter"], info["ops_count"], info["success"]) == (c["iter"], c["ops_count"], c["success"])
    assert np.array_equal(res, np.array(c["resSqmrhs"]))
    assert np.array_equal(x.reshape(-1), vec[key])


# ---- even/odd preconditioning (operators.cpp:455-620, operators_stencil.cpp:179-236)

@pytest.mark.parametrize("key", list(LATS))
@pytest.mark.parametrize("kind", ["staggered_deo", "staggered_doe", "staggered_m2mdeodoe"])
def test_eo_operators_bit_exact(oracle, golden, key, kind):
    vec, _ = golden
    lx, ly = LATS[key]
    out = oracle.apply(Operator(kind, lx, ly, 0.1, vec[f"{key}_links"]), vec[f"{key}_src"])
    assert np.array_equal(out, vec[f"{key}_{kind}"])


@pytest.mark.parametrize("key", list(LATS))
def test_eo_prepare_reconstruct_bit_exact(oracle, golden, key):
    vec, _ = golden
    lx, ly = LATS[key]
    eo = Operator("staggered_m2mdeodoe", lx, ly, 0.1, vec[f"{key}_links"])
    assert np.array_equal(oracle.eoprec_prepare(eo, vec[f"{key}_src"]), vec[f"{key}_eo_prepare"])
    rc = oracle.eoprec_reconstruct(eo, vec[f"{key}_src2"], vec[f"{key}_src"])
    assert np.array_equal(rc, vec[f"{key}_eo_reconstruct"])


def test_eo_stencil_form_bit_exact(oracle, golden):
    vec, _ = golden
    hop = oracle.staggered_stencil(vec["l8_links"], 8, 8)
    op = Operator("stencil_m2mdeodoe", 8, 8, nc=1, clover=np.zeros(64, np.complex128), hopping=hop, shift=0.1)
    assert np.array_equal(oracle.apply(op, vec["l8_src"]), vec["l8_stencil_m2mdeodoe"])
    assert np.array_equal(oracle.eoprec_prepare(op, vec["l8_src"]), vec["l8_stencil_eo_prepare"])
    assert np.array_equal(oracle.eoprec_reconstruct(op, vec["l8_src2"], vec["l8_src"]),
                          vec["l8_stencil_eo_reconstruct"])


def test_eo_identities(golden):
    """tests/staggered_pieces/staggered_pieces.cpp:297-332: D_eo + D_oe + m = D and
    m^2 - D_eo D_oe - D_oe D_eo = D^dagger D (on the even part of an even-only vector, the
    normal operator is m^2 - D_eo D_oe)."""
    vec, _ = golden
    for key in LATS:
        full = vec[f"{key}_staggered_deo"] + vec[f"{key}_staggered_doe"] + 0.1 * vec[f"{key}_src"]
        assert np.abs(full - vec[f"{key}_staggered"]).max() < 1e-14


def test_eo_solve_matches_reference(oracle, golden):
    """prepare, CG on m^2 - D_eo D_oe, reconstruct (staggered_pieces.cpp:331-346): the oracle's
    CG takes the reference's iterations and returns its solution bit for bit."""
    vec, cases = golden
    c = cases["l32_eo_cg"]
    eo = Operator("staggered_m2mdeodoe", 32, 32, 0.1, vec["l32_links"])
    rhs_e = oracle.eoprec_prepare(eo, vec["l32_src"])
    xe, info, _ = oracle.solve("cg", eo, rhs_e, max_iter=c["max_iter"], eps=c["eps"])
    assert info["iter"] == c["iter"] and info["ops_count"] == c["ops_count"]
    assert np.array_equal(xe, vec["l32_eo_cg_even"])
    assert np.array_equal(oracle.eoprec_reconstruct(eo, xe, vec["l32_src"]), vec["l32_eo_solution"])


def _gamma5(lx, ly):
    """gamma_5 (operator_utils/operators.cpp:242-259): (-1)^(x+y) at site i = y*lx + x."""
    i = np.arange(lx * ly)
    return 1.0 - 2.0 * ((i % lx + i // lx) % 2)


@pytest.mark.parametrize("key", list(LATS))
def test_gamma5_identity(oracle, golden, key):
    """tests/staggered_pieces/staggered_pieces.cpp:272-284: D^dagger = gamma_5 D gamma_5 (even
    periodic lattices): the oracle's D sandwiched by gamma_5 against the reference's D^dagger."""
    vec, _ = golden
    lx, ly = LATS[key]
    g5 = _gamma5(lx, ly)
    got = g5 * oracle.apply(Operator("staggered", lx, ly, 0.1, vec[f"{key}_links"]), g5 * vec[f"{key}_src"])
    want = vec[f"{key}_staggered_dagger"]
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()


@pytest.mark.parametrize("key", list(LATS))
def test_normal_operator_from_eo_pieces(oracle, golden, key):
    """tests/staggered_pieces/staggered_pieces.cpp:306-320: D^dagger D = m^2 - D_eo D_oe - D_oe D_eo
    (D_eo D_eo = 0): the oracle's pieces against the reference's D^dagger D vector."""
    vec, _ = golden
    lx, ly = LATS[key]
    U, b = vec[f"{key}_links"], vec[f"{key}_src"]
    deo, doe = Operator("staggered_deo", lx, ly, 0.1, U), Operator("staggered_doe", lx, ly, 0.1, U)
    got = 0.01 * b - oracle.apply(deo, oracle.apply(doe, b)) - oracle.apply(doe, oracle.apply(deo, b))
    want = vec[f"{key}_staggered_normal"]
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_cg_m_equals_sequential_cg(oracle, golden):
    """tests/multishift/multishift.cpp:424-494: each shift solution of the reference's CG-M on
    the gauge Laplacian (mass 0.001) against a CG on that shifted system, which for the
    Laplacian is the Laplacian of mass 0.001 + sigma.  Any two solutions with relative
    residuals r1, r2 differ by at most kappa (r1 + r2), kappa <= (m + sigma + 8) / (m + sigma)
    (the hopping part of -Delta_U lies in [0, 8]); measured, they agree within 7e-16, and the
    test holds them to 1e-12."""
    vec, cases = golden
    c = cases["l32_cgm_rfc1_wf0"]
    U, b = vec["l32_links"], vec["l32_src"]
    bn = np.linalg.norm(b)
    xs = vec["l32_cgm_rfc1_wf0"].reshape(len(c["shifts"]), -1)
    for j, s in enumerate(c["shifts"]):
        m = c["mass"] + s
        x, info, _ = oracle.solve("cg", Operator("laplace", 32, 32, m, U), b, eps=1e-10)
        r1, r2 = np.sqrt(info["resSq"]) / bn, np.sqrt(c["resSqmrhs"][j]) / bn
        kappa = (m + 8.0) / m
        d = np.linalg.norm(x - xs[j]) / np.linalg.norm(xs[j])
        assert d <= 1.01 * kappa * (r1 + r2) and d <= 1e-12, (j, d)


# ---- the oracle's own input generator and its threaded site loops

@pytest.mark.parametrize("key,lx,ly,seed", [("l32", 32, 32, 1337), ("l8", 8, 8, 7), ("l12x6", 12, 6, 3)])
def test_oracle_generator_bit_exact(golden, key, lx, ly, seed):
    """oracle/inputs.cpp reproduces the reference's rand_gauge_u1 and gaussian streams
    (u1_utils.cpp:79-87, generic_vector.h:48-60) bit for bit: links, then two sources."""
    import pyoracle
    vec, _ = golden
    g = pyoracle.Generator(seed)
    assert np.array_equal(g.rand_gauge_u1(lx, ly), vec[f"{key}_links"])
    assert np.array_equal(g.gaussian(lx * ly), vec[f"{key}_src"])
    assert np.array_equal(g.gaussian(lx * ly), vec[f"{key}_src2"])


def test_oracle_threads_change_no_bit(oracle):
    """Site loops on several threads, sums serial in the reference's order: CG (with its sums
    fused into the passes that form their terms) and CG-M give the single-thread results bit for
    bit, on a lattice large enough to be split into many chunks."""
    import pyoracle
    g = pyoracle.Generator(21)
    lx, ly = 192, 96
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    out = {}
    try:
        for nth in (1, 3, 8):
            oracle.set_threads(nth)
            op = pyoracle.Operator("staggered_normal", lx, ly, 0.05, U)
            x, info, hist = oracle.solve("cg", op, b, hist_cap=4000)
            xm, im, rm = oracle.cg_m(op, b, np.logspace(-4, 0, 5))
            xl, il, _ = oracle.solve("cg", pyoracle.Operator("laplace", lx, ly, 0.3, U), b)
            out[nth] = (x, info, hist, xm, im, rm, xl, il)
    finally:
        oracle.set_threads(1)
    for nth in (3, 8):
        for a, c in zip(out[1], out[nth]):
            if isinstance(a, np.ndarray):
                assert np.array_equal(a, c), nth
            else:
                assert a == c, nth
