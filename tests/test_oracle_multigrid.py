"""The CPU oracle's multigrid pieces against the reference's own outputs (golden fixtures
from multigrid/aa_mg/mg_complex.cpp and stencil_2d/coarse_stencil.cpp compiled from the
reference's sources): block_normalize / block_orthonormalize, prolong / restrict,
generate_coarse_from_fine_stencil (with and without the fine shifts), a second level over
an Nc = 4 stencil, the top/bottom stencil pieces and the top/bottom prepare / reconstruct
steps.  Bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from pyoracle import Operator

PIECES = ["stencil_tb", "stencil_bt", "stencil_m2mdtbdbt", "stencil_normal_eo", "stencil_normal_tb",
          "stencil_dagger_eo", "stencil_dagger_tb"]


def _fine(vec, c):
    return Operator("stencil", 16, 16, nc=1, clover=np.zeros(256, np.complex128), hopping=vec["mg16_hop"],
                    shift=complex(*c["shift"]), eo_shift=complex(*c["eo_shift"]))


def test_block_normalize_and_orthonormalize(oracle, golden):
    vec, _ = golden
    nv = vec["mg16_nv_in"].reshape(4, -1)
    assert np.array_equal(oracle.mg_block("normalize", 16, 16, 1, 4, 4, 4, nv).reshape(-1), vec["mg16_nv_norm"])
    assert np.array_equal(oracle.mg_block("orthonormalize", 16, 16, 1, 4, 4, 4, nv).reshape(-1), vec["mg16_nv_orth"])
    nv2 = vec["mg4_nv_in"].reshape(4, -1)
    assert np.array_equal(oracle.mg_block("orthonormalize", 4, 4, 4, 2, 2, 4, nv2).reshape(-1), vec["mg4_nv_orth"])


def test_prolong_restrict(oracle, golden):
    vec, _ = golden
    P = vec["mg16_nv_orth"]
    assert np.array_equal(oracle.mg_prolong(16, 16, 1, 4, 4, 4, P, vec["mg16_coarse_in"]), vec["mg16_prolong"])
    assert np.array_equal(oracle.mg_restrict(16, 16, 1, 4, 4, 4, P, vec["mg16_src"]), vec["mg16_restrict"])
    P2 = vec["mg4_nv_orth"]
    assert np.array_equal(oracle.mg_prolong(4, 4, 4, 2, 2, 4, P2, vec["mg4_coarse_in"]), vec["mg4_prolong"])
    assert np.array_equal(oracle.mg_restrict(4, 4, 4, 2, 2, 4, P2, vec["mg16_coarse_in"]), vec["mg4_restrict"])


@pytest.mark.parametrize("ig", [0, 1])
def test_coarse_stencil(oracle, golden, ig):
    vec, cases = golden
    c = cases["mg16"]
    cl, hp = oracle.mg_coarse_stencil(16, 16, 1, 4, 4, 4, vec["mg16_nv_orth"], _fine(vec, c), bool(ig))
    assert np.array_equal(cl, vec[f"mg16_coarse_clover_ig{ig}"])
    assert np.array_equal(hp, vec[f"mg16_coarse_hop_ig{ig}"])


def test_coarse_stencil_second_level(oracle, golden):
    vec, _ = golden
    lev2 = Operator("stencil", 4, 4, nc=4, clover=vec["mg16_coarse_clover_ig0"], hopping=vec["mg16_coarse_hop_ig0"])
    cl, hp = oracle.mg_coarse_stencil(4, 4, 4, 2, 2, 4, vec["mg4_nv_orth"], lev2)
    assert np.array_equal(cl, vec["mg4_coarse_clover"])
    assert np.array_equal(hp, vec["mg4_coarse_hop"])


def test_coarse_stencil_is_galerkin(oracle, golden):
    """The coarse stencil applied to v equals P^dagger A P v (the definition of the probed
    operator), to rounding."""
    vec, cases = golden
    c = cases["mg16"]
    fine = _fine(vec, c)
    P = vec["mg16_nv_orth"]
    coarse = Operator("stencil", 4, 4, nc=4, clover=vec["mg16_coarse_clover_ig0"], hopping=vec["mg16_coarse_hop_ig0"])
    v = vec["mg16_coarse_in"]
    lhs = oracle.apply(coarse, v)
    rhs = oracle.mg_restrict(16, 16, 1, 4, 4, 4, P, oracle.apply(fine, oracle.mg_prolong(16, 16, 1, 4, 4, 4, P, v)))
    assert np.max(np.abs(lhs - rhs)) < 1e-14


@pytest.mark.parametrize("kind", PIECES)
def test_coarse_stencil_pieces(oracle, golden, kind):
    vec, _ = golden
    op = Operator(kind, 4, 4, nc=4, clover=vec["mg16_coarse_clover_ig0"], hopping=vec["mg16_coarse_hop_ig0"],
                  shift=0.1 + 0.02j)
    assert np.array_equal(oracle.apply(op, vec["mg16_piece_in"]), vec[f"mg16_{kind}"])


def test_tbprec_prepare_reconstruct(oracle, golden):
    vec, _ = golden
    op = Operator("stencil_m2mdtbdbt", 4, 4, nc=4, clover=vec["mg16_coarse_clover_ig0"],
                  hopping=vec["mg16_coarse_hop_ig0"], shift=0.1)
    assert np.array_equal(oracle.tbprec_prepare(op, vec["mg16_piece_in"]), vec["mg16_tb_prepare"])
    assert np.array_equal(oracle.tbprec_reconstruct(op, vec["mg16_coarse_in"], vec["mg16_piece_in"]),
                          vec["mg16_tb_reconstruct"])
