"""GPU solvers (FP64, the reference's recurrences) against the reference's own runs
(golden fixtures: the 32x32 U(1) system with m = 0.1, tol 1e-10).

Bars: CG solution within 1e-11 relative of the reference's CG solution with the same
iteration and operator counts; GCR within 1e-9 and +-1 iteration; CG-M per-shift solutions
within 1e-10 and the same counts.

BiCGstab on this system is sensitive to rounding: re-evaluating the reference's own
recurrence with only the summation order of the dot products changed takes 341 iterations
instead of the reference's 330 (and a 1e-16 perturbation of alpha gives 346), and moves
|Ax-b|^2 after 5 iterations by 2e-5 relative.  Its bar is therefore: the same stopping
tolerance reached, the iteration count within 5% of the reference's, the solution within
1e-8 relative (kappa(M) ~ 10 times the tolerance, twice), and 1e-4 on |Ax-b|^2 after 5
iterations."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def ops(gl, vec):
    U = vec["l32_links"]
    return {"staggered_normal": gl.StaggeredU1Op(U, 0.1, 32, 32), "staggered": gl.StaggeredU1Op(U, 0.1, 32, 32)}


def callback(gl, name):
    return {"staggered_normal": gl.square_staggered_normal_u1, "staggered": gl.square_staggered_u1}[name]


FNS = {("cg", 0): "minv_vector_cg", ("cg", 17): "minv_vector_cg_restart", ("bicgstab", 0): "minv_vector_bicgstab",
       ("bicgstab", 17): "minv_vector_bicgstab_restart", ("gcr", 0): "minv_vector_gcr", ("gcr", 17): "minv_vector_gcr_restart"}


@pytest.mark.parametrize("solver,rf", list(FNS))
def test_solver_matches_reference(gl, gpu, golden, solver, rf):
    vec, cases = golden
    key = f"l32_{solver}" + (f"_r{rf}" if rf else "")
    c = cases[key]
    b = vec["l32_src"]
    x = np.zeros_like(b)
    fn = getattr(gl, FNS[(solver, rf)])
    extra = gl.StaggeredU1Op(vec["l32_links"], 0.1, 32, 32)
    args = (x, b, b.size, c["max_iter"]) + ((c["eps"], rf) if rf else (c["eps"],))
    info = fn(*args, callback(gl, c["op"]), extra)
    bnorm = np.linalg.norm(b)
    assert info.success and info.name == c["name"]
    assert np.sqrt(info.resSq) / bnorm < 1e-10
    if solver == "cg":
        assert (info.iter, info.ops_count) == (c["iter"], c["ops_count"])
        assert rel(x, vec[key]) < 1e-11
    elif solver == "gcr":
        assert abs(info.iter - c["iter"]) <= 1
        assert rel(x, vec[key]) < 1e-9
    else:
        assert abs(info.iter - c["iter"]) <= 0.05 * c["iter"]
        assert rel(x, vec[key]) < 1e-8


def test_cg_initial_guess(gl, gpu, golden):
    vec, cases = golden
    b = vec["l32_src"]
    x = vec["l32_src2"].copy()
    info = gl.minv_vector_cg(x, b, b.size, 10000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(vec["l32_links"], 0.1, 32, 32))
    assert info.iter == cases["l32_cg_guess"]["iter"]
    assert rel(x, vec["l32_cg_guess"]) < 1e-11


@pytest.mark.parametrize("key,max_iter", [("l32_cg_maxiter7", 7), ("l32_bicgstab_maxiter5", 5), ("l32_gcr_maxiter5", 5)])
def test_max_iter_and_verbosity_lines(gl, gpu, golden, capfd, key, max_iter):
    vec, cases = golden
    c = cases[key]
    solver = key.split("_")[1]
    b = vec["l32_src"]
    x = np.zeros_like(b)
    fn = {"cg": gl.minv_vector_cg, "bicgstab": gl.minv_vector_bicgstab, "gcr": gl.minv_vector_gcr}[solver]
    cb = gl.square_staggered_normal_u1 if solver == "cg" else gl.square_staggered_u1
    prefix = "[CG] " if solver == "cg" else ""
    capfd.readouterr()
    info = fn(x, b, b.size, max_iter, 1e-10, cb, gl.StaggeredU1Op(vec["l32_links"], 0.1, 32, 32),
              gl.InversionVerboseStruct(gl.VERB_DETAIL, prefix))
    out = capfd.readouterr().out
    assert (info.iter, info.ops_count, info.success) == (c["iter"], c["ops_count"], c["success"])
    tol = 1e-4 if solver == "bicgstab" else 1e-9
    assert abs(info.resSq - c["resSq"]) < tol * c["resSq"]
    got, want = out.strip().splitlines(), c["log"].strip().splitlines()
    assert len(got) == len(want)
    for g_, w_ in zip(got, want):
        gh, gv = g_.rsplit(" ", 1)
        wh, wv = w_.rsplit(" ", 1)
        assert gh == wh  # prefix, name, Iter, Ops, Success fields identical
        assert abs(float(gv) - float(wv)) <= 2e-5 * abs(float(wv))


@pytest.mark.parametrize("rfc,wf", [(1, 0), (3, 0), (1, 1)])
def test_cg_m_matches_reference(gl, gpu, golden, capfd, rfc, wf):
    vec, cases = golden
    key = f"l32_cgm_rfc{rfc}_wf{wf}"
    c = cases[key]
    b = vec["l32_src"]
    ns = len(c["shifts"])
    xs = [np.zeros_like(b) for _ in range(ns)]
    shifts = np.array(c["shifts"])
    capfd.readouterr()
    info = gl.minv_vector_cg_m(xs, b, ns, b.size, rfc, 10000, 1e-10, shifts, gl.square_laplace_u1,
                               gl.StaggeredU1Op(vec["l32_links"], c["mass"], 32, 32), bool(wf),
                               gl.InversionVerboseStruct(gl.VERB_SUMMARY, "[CGM] "))
    out = capfd.readouterr().out
    assert (info.iter, info.ops_count, info.success, info.name) == (c["iter"], c["ops_count"], c["success"], "CG-M")
    assert info.resSq == 0.0
    assert np.array_equal(shifts, np.array(c["shifts"]))  # shifts left in the caller's order
    ref = vec[key].reshape(ns, -1)
    for j in range(ns):
        assert rel(xs[j], ref[j]) < 1e-10
        assert abs(info.resSqmrhs[j] - c["resSqmrhs"][j]) < 0.05 * c["resSqmrhs"][j] + 1e-22
    assert out.startswith("[CGM] CG-M  Success Y Iter %d Ops %d RelRes " % (c["iter"], c["ops_count"]))


def test_device_pointer_solve(gl, gpu, golden):
    import torch
    vec, cases = golden
    b = torch.from_numpy(vec["l32_src"]).to(gpu)
    x = torch.zeros_like(b)
    info = gl.minv_vector_cg(x, b, b.numel(), 10000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(vec["l32_links"], 0.1, 32, 32))
    assert info.iter == cases["l32_cg"]["iter"]
    assert rel(x.cpu().numpy(), vec["l32_cg"]) < 1e-11


def test_laplace_cg_vs_oracle(gl, gpu, oracle):
    from pyoracle import Operator as OO
    g = gl.Generator(5)
    U = g.rand_gauge_u1(48, 40)
    b = g.gaussian(48 * 40)
    x = np.zeros_like(b)
    info = gl.minv_vector_cg(x, b, b.size, 10000, 1e-10, gl.square_laplace_u1, gl.StaggeredU1Op(U, 0.05, 48, 40))
    xr, ir, _ = oracle.solve("cg", OO("laplace", 48, 40, 0.05, U), b)
    assert (info.iter, info.ops_count) == (ir["iter"], ir["ops_count"])
    assert rel(x, xr) < 1e-11


def test_stencil_cg_m_vs_oracle(gl, gpu, oracle):
    """CG-M driven by a stencil operator (the MG coarse-operator path): Hermitian positive
    stencil built as the staggered normal operator is not a stencil, so use the Laplacian
    written as an Nc=1 stencil."""
    from pyoracle import Operator as OO
    lx, ly = 16, 12
    g = gl.Generator(8)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    V = lx * ly
    hop = np.zeros(4 * V, np.complex128)
    Ux, Uy = U[0::2], U[1::2]
    idx = np.arange(V).reshape(ly, lx)
    hop[0:V] = -Ux
    hop[V:2 * V] = -Uy
    hop[2 * V:3 * V] = -np.conj(Ux[np.roll(idx, 1, 1).reshape(-1)])
    hop[3 * V:4 * V] = -np.conj(Uy[np.roll(idx, 1, 0).reshape(-1)])
    clover = np.full(V, 4.05 + 0j)
    shifts = [0.0, 0.01, 0.1]
    st = gl.Stencil2D(lx, ly, 1)
    st.clover[:], st.hopping[:] = clover, hop
    xs = [np.zeros_like(b) for _ in shifts]
    info = gl.minv_vector_cg_m(xs, b, 3, V, 1, 10000, 1e-10, np.array(shifts), gl.apply_stencil_2d, st)
    xr, ir, res = oracle.cg_m(OO("stencil", lx, ly, nc=1, clover=clover, hopping=hop), b, shifts)
    assert (info.iter, info.ops_count) == (ir["iter"], ir["ops_count"])
    for j in range(3):
        assert rel(xs[j], xr[j]) < 1e-10
