"""GPU operators against the reference's outputs (golden fixtures) and the oracle.

Tolerance: 1e-14 relative per site, with the denominator max(|ref_i|, s_i) where s_i is the
summed magnitude of the terms at site i (so cancellation does not inflate the ratio)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import site_rel_err, staggered_scale
from pyoracle import Operator as OrcOperator

pytestmark = pytest.mark.gpu

LATS = {"l32": (32, 32), "l8": (8, 8), "l12x6": (12, 6)}
KINDS = {"staggered": 0, "staggered_dagger": 1, "staggered_normal": 2, "laplace": 3}


@pytest.mark.parametrize("key", list(LATS))
@pytest.mark.parametrize("kind", list(KINDS))
def test_u1_operators_match_reference(gl, gpu, golden, key, kind):
    vec, _ = golden
    lx, ly = LATS[key]
    U, b = vec[f"{key}_links"], vec[f"{key}_src"]
    mass = 0.01 if kind == "laplace" else 0.1
    op = gl.Operator(KINDS[kind], lx, ly, mass, U)
    out = np.zeros_like(b)
    op.apply(out, b)
    ref = vec[f"{key}_{kind}"]
    if kind == "staggered_normal":
        scale = staggered_scale(U, vec[f"{key}_staggered"], mass, lx, ly)
    elif kind == "laplace":
        scale = 2 * staggered_scale(U, b, 0.0, lx, ly) + (4 + mass) * np.abs(b)
    else:
        scale = staggered_scale(U, b, mass, lx, ly)
    assert site_rel_err(out, ref, scale) < 1e-14


def test_device_pointers_match_host(gl, gpu, golden):
    import torch
    vec, _ = golden
    U, b = vec["l32_links"], vec["l32_src"]
    op = gl.Operator(2, 32, 32, 0.1, U)
    h = np.zeros_like(b)
    op.apply(h, b)
    d_in = torch.from_numpy(b).to(gpu)
    d_out = torch.zeros_like(d_in)
    op.apply(d_out, d_in)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), h)
    # operator built from device-resident links
    op2 = gl.Operator(2, 32, 32, 0.1, torch.from_numpy(U).to(gpu))
    d2 = torch.zeros_like(d_in)
    op2.apply(d2, d_in)
    assert np.array_equal(d2.cpu().numpy(), h)


@pytest.mark.parametrize("key", list(LATS))
def test_stencil_builders_match_reference(gl, gpu, golden, key):
    vec, _ = golden
    lx, ly = LATS[key]
    for dag, build in ((0, gl.get_square_staggered_u1_stencil), (1, gl.get_square_staggered_dagger_u1_stencil)):
        st = gl.Stencil2D(lx, ly, 1)
        build(st, gl.StaggeredU1Op(vec[f"{key}_links"], 0.1, lx, ly))
        assert np.array_equal(st.hopping, vec[f"{key}_stencil_hop{dag}"])
        assert st.shift == 0.1 and st.generated
        out = np.zeros(lx * ly, np.complex128)
        gl.apply_stencil_2d(out, vec[f"{key}_src"], st)
        scale = staggered_scale(vec[f"{key}_links"], vec[f"{key}_src"], 0.1, lx, ly)
        assert site_rel_err(out, vec[f"{key}_stencil_apply{dag}"], scale) < 1e-14


@pytest.mark.parametrize("kind,k", [("stencil", 4), ("stencil_eo", 5), ("stencil_oe", 6)])
@pytest.mark.parametrize("two", [0, 1])
def test_generic_stencil_matches_reference(gl, gpu, golden, oracle, kind, k, two):
    vec, cases = golden
    c = cases["st3"]
    args = dict(nc=c["nc"], clover=vec["st3_clover"], hopping=vec["st3_hopping"],
                two_link=vec["st3_two"] if two else None, shift=complex(*c["shift"]),
                eo_shift=complex(*c["eo_shift"]), dof_shift=complex(*c["dof_shift"]))
    op = gl.Operator(k, c["lx"], c["ly"], **args)
    out = np.zeros_like(vec["st3_x"])
    op.apply(out, vec["st3_x"])
    # magnitude of the summed terms: the same stencil applied to |coefficients| and |x|
    absargs = {kk: (np.abs(v) + 0j if isinstance(v, np.ndarray) else complex(abs(v)))
               for kk, v in args.items() if kk != "nc" and v is not None}
    scale = np.abs(oracle.apply(OrcOperator(kind, c["lx"], c["ly"], nc=c["nc"], **absargs), np.abs(vec["st3_x"]) + 0j))
    assert site_rel_err(out, vec[f"st3_{kind}_two{two}"], scale) < 1e-14


@pytest.mark.parametrize("nc", [1, 2, 4, 5, 8])
@pytest.mark.parametrize("kind,k", [("stencil", 4), ("stencil_eo", 5), ("stencil_oe", 6)])
def test_stencil_nc_sizes_vs_oracle(gl, gpu, oracle, nc, kind, k):
    rng = np.random.default_rng(nc * 10 + k)
    lx, ly = 10, 6
    v = lx * ly * nc * nc
    z = lambda n: rng.normal(size=n) + 1j * rng.normal(size=n)
    args = dict(nc=nc, clover=z(v), hopping=z(4 * v), two_link=z(8 * v), shift=0.2 - 0.1j, eo_shift=0.3j, dof_shift=0.7)
    x = z(lx * ly * nc)
    op = gl.Operator(k, lx, ly, **args)
    out = np.zeros_like(x)
    op.apply(out, x)
    ref = oracle.apply(OrcOperator(kind, lx, ly, **args), x)
    absargs = {kk: (np.abs(vv) + 0j if isinstance(vv, np.ndarray) else complex(abs(vv))) for kk, vv in args.items() if kk != "nc"}
    scale = np.abs(oracle.apply(OrcOperator(kind, lx, ly, nc=nc, **absargs), np.abs(x) + 0j))
    assert site_rel_err(out, ref, scale) < 1e-14


@pytest.mark.parametrize("lx,ly", [(1024, 1024), (257, 130), (3, 5)])
def test_staggered_large_and_odd_sizes_vs_oracle(gl, gpu, oracle, lx, ly):
    g = gl.Generator(99)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    for kind, k in (("staggered", 0), ("staggered_dagger", 1), ("staggered_normal", 2), ("laplace", 3)):
        op = gl.Operator(k, lx, ly, 0.05, U)
        out = np.zeros_like(b)
        op.apply(out, b)
        ref = oracle.apply(OrcOperator(kind, lx, ly, 0.05, U), b)
        assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 1e-14, kind


def test_blas_dot_norm(gl, gpu, golden):
    vec, _ = golden
    a, b = vec["l32_src"], vec["l32_src2"]
    assert abs(gl.dot(a, b) - np.vdot(a, b)) < 1e-12 * abs(np.vdot(a, b))
    assert abs(gl.norm2sq(a) - np.vdot(a, a).real) < 1e-12 * np.vdot(a, a).real
