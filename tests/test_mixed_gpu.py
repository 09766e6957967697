"""Mixed-precision CG (FP32 / FP16 / BF16 inner iterations, FP64 reliable updates).

Bar: every solve stops only at an FP64-true relative residual below eps (checked here again
with the FP64 operator), and its solution error against the FP64 reference solution is
stated; on the 32x32 system the error is at most 1e-8 relative (kappa(M^dagger M) ~ 200 at
m = 0.1 times 1e-10, with margin)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

PRECS = {"single": 1, "half": 2, "bfloat": 3}


def true_relres(gl, kind, lx, ly, mass, U, x, b):
    op = gl.Operator(kind, lx, ly, mass, U)
    Ax = np.zeros_like(b)
    op.apply(Ax, x)
    return np.linalg.norm(b - Ax) / np.linalg.norm(b)


@pytest.mark.parametrize("prec", list(PRECS))
def test_mixed_cg_32_vs_reference(gl, gpu, golden, prec):
    vec, cases = golden
    U, b = vec["l32_links"], vec["l32_src"]
    x = np.zeros_like(b)
    info = gl.minv_vector_cg(x, b, b.size, 20000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(U, 0.1, 32, 32), precision=PRECS[prec])
    assert info.success and info.status == 0
    assert np.sqrt(info.resSq) / np.linalg.norm(b) < 1e-10
    assert true_relres(gl, 2, 32, 32, 0.1, U, x, b) < 1e-10
    assert rel(x, vec["l32_cg"]) < 1e-8
    assert info.iter < 3 * cases["l32_cg"]["iter"]
    assert info.reliable_updates >= 2


@pytest.mark.parametrize("prec", list(PRECS))
def test_mixed_cg_laplace(gl, gpu, oracle, prec):
    from pyoracle import Operator as OO
    g = gl.Generator(21)
    U = g.rand_gauge_u1(64, 64)
    b = g.gaussian(64 * 64)
    x = np.zeros_like(b)
    info = gl.minv_vector_cg(x, b, b.size, 20000, 1e-10, gl.square_laplace_u1,
                             gl.StaggeredU1Op(U, 0.01, 64, 64), precision=PRECS[prec])
    assert info.success
    assert true_relres(gl, 3, 64, 64, 0.01, U, x, b) < 1e-10
    xr, _, _ = oracle.solve("cg", OO("laplace", 64, 64, 0.01, U), b)
    assert rel(x, xr) < 1e-7


def test_mixed_cg_initial_guess_and_device(gl, gpu, golden):
    import torch
    vec, _ = golden
    U, b = vec["l32_links"], vec["l32_src"]
    bt = torch.from_numpy(b).to(gpu)
    xt = torch.from_numpy(vec["l32_src2"]).to(gpu)
    info = gl.minv_vector_cg(xt, bt, b.size, 20000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(U, 0.1, 32, 32), precision=1)
    assert info.success
    assert rel(xt.cpu().numpy(), vec["l32_cg"]) < 1e-8


@pytest.mark.parametrize("prec", ["single", "half", "bfloat"])
def test_mixed_cg_1024_true_residual(gl, gpu, prec):
    """The large single-lattice system (1024x1024, m = 0.01): the mixed solve must reach
    an FP64-true relative residual of 1e-10, re-checked with the FP64 GPU operator, and agree
    with the FP64 GPU CG solution to kappa * 1e-10 (kappa ~ 2e4)."""
    import torch
    lx = ly = 1024
    g = gl.Generator(1337)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    op = gl.Operator(2, lx, ly, 0.01, torch.from_numpy(U).to(gpu))
    bt = torch.from_numpy(b).to(gpu)
    x = torch.zeros_like(bt)
    info = gl.minv_vector_cg(x, bt, b.size, 100000, 1e-10, gl.square_staggered_normal_u1, op, precision=PRECS[prec])
    assert info.success, info
    Ax = torch.zeros_like(bt)
    op.apply(Ax, x)
    rr = (torch.linalg.vector_norm(bt - Ax) / torch.linalg.vector_norm(bt)).item()
    assert rr < 1e-10
    x64 = torch.zeros_like(bt)
    i64 = gl.minv_vector_cg(x64, bt, b.size, 100000, 1e-10, gl.square_staggered_normal_u1, op)
    assert i64.success
    err = (torch.linalg.vector_norm(x - x64) / torch.linalg.vector_norm(x64)).item()
    assert err < 1e-5


def test_host_driven_loop_matches_graph(gl, gpu, golden, tmp_path):
    """GLINALG_SOLVER_GRAPHS=0 launches the same kernels from a host loop: the solutions of
    the FP64 CG, the mixed CG and CG-M are bit-identical to the graph-driven ones."""
    import subprocess
    import sys
    vec, _ = golden
    script = tmp_path / "run.py"
    script.write_text(f'''
import importlib, sys, numpy as np
sys.path.insert(0, {repr(str(gl.__path__[0]))}.rsplit("/", 1)[0])
gl = importlib.import_module("generic-linalg_gb300")
d = np.load({repr(str(tmp_path / "in.npz"))})
U, b = d["U"], d["b"]
out = {{}}
for prec in (0, 1, 2):
    x = np.zeros_like(b)
    inf = gl.minv_vector_cg(x, b, b.size, 20000, 1e-10, gl.square_staggered_normal_u1, gl.StaggeredU1Op(U, 0.1, 32, 32), precision=prec)
    out[f"cg{{prec}}"] = x
xs = [np.zeros_like(b) for _ in range(3)]
gl.minv_vector_cg_m(xs, b, 3, b.size, 1, 10000, 1e-10, np.array([0.0, 0.01, 0.1]), gl.square_laplace_u1, gl.StaggeredU1Op(U, 0.01, 32, 32))
out["cgm"] = np.stack(xs)
np.savez(sys.argv[1], **out)
''')
    np.savez(tmp_path / "in.npz", U=vec["l32_links"], b=vec["l32_src"])
    import os
    env = dict(os.environ)
    # the same tile shape in both processes (the autotuner's timing-based pick may differ)
    env["GLINALG_TILE"] = "1"
    env["GLINALG_PERSIST_SHAPE"] = "0"
    res = {}
    for mode in ("1", "0"):
        env["GLINALG_SOLVER_GRAPHS"] = mode
        subprocess.run([sys.executable, str(script), str(tmp_path / f"out{mode}.npz")], env=env, check=True)
        res[mode] = np.load(tmp_path / f"out{mode}.npz")
    for k in res["1"].files:
        assert np.array_equal(res["1"][k], res["0"][k]), k


def test_mixed_cg_default_delta(gl, gpu, golden):
    """An unset reliable-update trigger is the documented 0.01 for FP32 iterates: the same
    iterations and reliable updates as delta = 0.01, and fewer updates than delta = 0.1."""
    vec, _ = golden
    U, b = vec["l32_links"], vec["l32_src"]
    got = {}
    for d in (0.0, 0.01, 0.1):
        x = np.zeros_like(b)
        info = gl.minv_vector_cg(x, b, b.size, 20000, 1e-10, gl.square_staggered_normal_u1,
                                 gl.StaggeredU1Op(U, 0.1, 32, 32), precision=PRECS["single"], delta=d)
        assert info.success
        got[d] = (info.iter, info.reliable_updates)
    assert got[0.0] == got[0.01], got
    assert got[0.1][1] > got[0.01][1], got


def test_release_memory_between_solves(gl, gpu):
    """The library keeps the work vectors of finished calls in its memory pool; handing that
    memory back (glinalg_release_memory) between two identical solves changes nothing in the
    second solve's result."""
    import torch
    lx = ly = 256
    g = gl.Generator(31)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    op = gl.Operator(2, lx, ly, 0.05, torch.from_numpy(U).to(gpu))
    bd = torch.from_numpy(b).to(gpu)
    xs = []
    for k in range(2):
        x = torch.zeros_like(bd)
        info = gl.minv_vector_cg(x, bd, b.size, 10000, 1e-10, gl.square_staggered_normal_u1, op, precision=1)
        assert info.success, info
        xs.append(x)
        gl.release_memory()
    assert torch.equal(xs[0], xs[1])
