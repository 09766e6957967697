"""The sibling Krylov solvers on the GPU (FP64, the reference's recurrences) against the
reference's own runs on the 32x32 U(1) system (golden fixtures from generic_cr.cpp,
generic_minres.cpp, generic_cr_m.cpp, generic_bicgstab_l.cpp, generic_bicgstab_m.cpp,
generic_cg_flex_precond.cpp and generic_gcr_var_precond.cpp).

Bars: the CG-like methods (CR, CR(n), MinRes, FPCG, VPGCR and their restarts, CR-M) take the
reference's iteration and operator counts, report its success flag and name, and return its
solution within 1e-10 relative (multishift: per shift).  BiCGstab-l and BiCGstab-M are
rounding-sensitive like BiCGstab (a reduction order that differs from the reference's serial
sum changes the iterates after a few steps): the same stopping tolerance is reached, the
iteration count is within 5% of the reference's, and the solution within 1e-8 relative.
Verbosity lines match the reference's text field for field, the relative residual to 2e-5."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

MASS = {"staggered_normal": 0.1, "staggered": 0.1, "laplace_m0.5": 0.5, "laplace_m0.001": 0.001}
FN = {"cr": "minv_vector_cr", "minres": "minv_vector_minres", "bicgstab_l": "minv_vector_bicgstab_l",
      "fpcg": "minv_vector_cg_flex_precond", "vpgcr": "minv_vector_gcr_var_precond"}
ROBUST = ("cr", "minres", "fpcg", "vpgcr")


def _cases():
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_info.json")
    return json.load(open(here))["cases"]


def _sib_keys():
    return sorted(k for k, c in _cases().items() if "solver" in c and "maxiter" not in k)


def _cb(gl, opname):
    kind = opname.split("_m0")[0]
    return {"staggered_normal": gl.square_staggered_normal_u1, "staggered": gl.square_staggered_u1,
            "laplace": gl.square_laplace_u1}[kind]


def _run(gl, c, links, x, b, max_iter, verb=None):
    cb = _cb(gl, c["op"])
    extra = gl.StaggeredU1Op(links, MASS[c["op"]], 32, 32)
    kw = dict(c["kw"])
    rf = kw.pop("restart_freq", 0)
    s = c["solver"]
    if s == "minres":
        return gl.minv_vector_minres(x, b, b.size, max_iter, 1e-10, kw.get("omega", 1.0), cb, extra, verb)
    if s == "bicgstab_l":
        if rf:
            return gl.minv_vector_bicgstab_l_restart(x, b, b.size, max_iter, 1e-10, rf, kw["l"], cb, extra, verb)
        return gl.minv_vector_bicgstab_l(x, b, b.size, max_iter, 1e-10, kw["l"], cb, extra, verb)
    if s in ("fpcg", "vpgcr"):
        pname = kw.get("precond", "identity")
        pfn = getattr(gl, f"{pname}_preconditioner")
        pinfo = None if pname == "identity" else (gl.MinresPrecondStruct if pname == "minres" else
                                                  gl.GcrPrecondStruct)(4, 1e-1, cb, extra)
        fn = getattr(gl, FN[s] + ("_restart" if rf else ""))
        args = (x, b, b.size, max_iter, 1e-10) + ((rf,) if rf else ())
        return fn(*args, cb, extra, pfn, pinfo, verb)
    if rf:
        return gl.minv_vector_cr_restart(x, b, b.size, max_iter, 1e-10, rf, cb, extra, verb)
    return gl.minv_vector_cr(x, b, b.size, max_iter, 1e-10, cb, extra, verb)


@pytest.mark.parametrize("key", _sib_keys())
def test_sibling_solver_matches_reference(gl, gpu, golden, key):
    vec, cases = golden
    c = cases[key]
    b = vec["l32_src"]
    x = np.zeros_like(b)
    info = _run(gl, c, vec["l32_links"], x, b, c["max_iter"])
    assert info.name == c["name"]
    assert info.success == c["success"]
    if c["solver"] in ROBUST:
        assert (info.iter, info.ops_count) == (c["iter"], c["ops_count"])
        assert rel(x, vec[key]) < 1e-10
        assert abs(info.resSq - c["resSq"]) <= 0.1 * c["resSq"] + 1e-30
    else:
        assert np.sqrt(info.resSq) / np.linalg.norm(b) < 1e-10
        assert abs(info.iter - c["iter"]) <= 0.05 * c["iter"]
        assert rel(x, vec[key]) < 1e-8


def _compare_lines(out, log):
    got, want = out.strip().splitlines(), log.strip().splitlines()
    assert len(got) == len(want), (got, want)
    for g_, w_ in zip(got, want):
        gh, gv = g_.rsplit(" ", 1)
        wh, wv = w_.rsplit(" ", 1)
        assert gh == wh
        assert abs(float(gv) - float(wv)) <= 2e-5 * abs(float(wv))


@pytest.mark.parametrize("key", ["l32_cr_maxiter6", "l32_minres_maxiter5", "l32_bicgstab_l_maxiter6",
                                 "l32_fpcg_maxiter4", "l32_vpgcr_maxiter4"])
def test_sibling_max_iter_and_verbosity(gl, gpu, golden, capfd, key):
    vec, cases = golden
    c = cases[key]
    b = vec["l32_src"]
    x = np.zeros_like(b)
    capfd.readouterr()
    info = _run(gl, c, vec["l32_links"], x, b, c["max_iter"], gl.InversionVerboseStruct(gl.VERB_DETAIL, ""))
    out = capfd.readouterr().out
    assert (info.iter, info.ops_count, info.success) == (c["iter"], c["ops_count"], c["success"])
    _compare_lines(out, c["log"])


def test_precond_verbosity_interleaves(gl, gpu, golden, capfd):
    """The flexible CG's DETAIL lines and its MinRes preconditioner's summaries, printed in the
    reference's order with their own prefixes (shuffle_verbosity_precond, verbosity.h:46)."""
    vec, cases = golden
    c = cases["l32_fpcg_precond_log"]
    b = vec["l32_src"]
    x = np.zeros_like(b)
    extra = gl.StaggeredU1Op(vec["l32_links"], 0.1, 32, 32)
    cb = gl.square_staggered_normal_u1
    capfd.readouterr()
    info = gl.minv_vector_cg_flex_precond(x, b, b.size, 3, 1e-10, cb, extra, gl.minres_preconditioner,
                                          gl.MinresPrecondStruct(4, 1e-1, cb, extra),
                                          gl.InversionVerboseStruct(gl.VERB_DETAIL, "[OUT] ", gl.VERB_SUMMARY,
                                                                    "  [MR] "))
    out = capfd.readouterr().out
    assert (info.iter, info.ops_count) == (c["iter"], c["ops_count"])
    _compare_lines(out, c["log"])


@pytest.mark.parametrize("solver", ["cr_m", "bicgstab_m"])
@pytest.mark.parametrize("rfc,wf", [(1, 0), (3, 0), (1, 1)])
def test_multishift_sibling_matches_reference(gl, gpu, golden, capfd, solver, rfc, wf):
    vec, cases = golden
    key = f"l32_{solver}_rfc{rfc}_wf{wf}"
    c = cases[key]
    b = vec["l32_src"]
    ns = len(c["shifts"])
    xs = [np.zeros_like(b) for _ in range(ns)]
    shifts = np.array(c["shifts"])
    fn = gl.minv_vector_cr_m if solver == "cr_m" else gl.minv_vector_bicgstab_m
    capfd.readouterr()
    info = fn(xs, b, ns, b.size, rfc, 10000, 1e-10, shifts, _cb(gl, c["op"]),
              gl.StaggeredU1Op(vec["l32_links"], MASS[c["op"]], 32, 32), bool(wf),
              gl.InversionVerboseStruct(gl.VERB_SUMMARY, "[MS] "))
    out = capfd.readouterr().out
    assert info.name == c["name"] and info.resSq == 0.0
    assert info.success == c["success"]
    assert np.array_equal(shifts, np.array(c["shifts"]))
    ref = vec[key].reshape(ns, -1)
    bsq = float(np.vdot(b, b).real)
    if solver == "cr_m":
        assert (info.iter, info.ops_count) == (c["iter"], c["ops_count"])
        for j in range(ns):
            assert rel(xs[j], ref[j]) < 1e-10
    else:
        assert abs(info.iter - c["iter"]) <= 0.05 * c["iter"]
        assert info.ops_count - 2 * info.iter == c["ops_count"] - 2 * c["iter"]
        for j in range(ns):
            assert rel(xs[j], ref[j]) < 1e-8
    assert max(info.resSqmrhs) < (1e-9) ** 2 * bsq
    assert out.startswith("[MS] CG-M  Success %s Iter %d Ops %d RelRes " %
                          ("Y" if info.success else "N", info.iter, info.ops_count))


def test_siblings_on_device_pointers_256(gl, gpu):
    """CR on D^dagger D and BiCGstab-4 on D at 256^2, m = 0.05, from device-resident torch
    fields, checked through the FP64 operator itself: |b - A x| / |b| < 1e-9."""
    import torch
    lx = ly = 256
    g = gl.Generator(1337)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    Ud, bd = torch.from_numpy(U).to(gpu), torch.from_numpy(b).to(gpu)
    for kind, cb, fn in ((2, gl.square_staggered_normal_u1, "cr"), (0, gl.square_staggered_u1, "bicgstab_l")):
        op = gl.Operator(kind, lx, ly, 0.05, Ud)
        x = torch.zeros_like(bd)
        extra = gl.StaggeredU1Op(Ud, 0.05, lx, ly)
        if fn == "cr":
            info = gl.minv_vector_cr(x, bd, b.size, 20000, 1e-11, cb, extra)
        else:
            info = gl.minv_vector_bicgstab_l(x, bd, b.size, 20000, 1e-11, 4, cb, extra)
        assert info.status == 0, info
        Ax = torch.zeros_like(bd)
        op.apply(Ax, x)
        assert (torch.linalg.vector_norm(Ax - bd) / torch.linalg.vector_norm(bd)).item() < 1e-9
