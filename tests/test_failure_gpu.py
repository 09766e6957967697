"""Failure paths of the solvers, every one made on the host: NaN / Inf planted in the source or
in the links, an all-zero source, a BiCGstab breakdown, and a bounded device-side wait that is
told to give up.  Nothing here faults, traps or hangs the GPU: the kernels check their own
conditions and return a status, and each test ends with an ordinary solve on the same device to
show the context is still usable.

Where the reference has no failure handling (generic_cg.cpp and generic_bicgstab.cpp divide by
the zero denominators and carry NaN to max_iter, generic_bicgstab.cpp:261,296), the library
stops at the first such denominator with GLINALG_SOLVE_BREAKDOWN and leaves x finite, and stops
at the first non-finite residual norm with GLINALG_SOLVE_NONFINITE."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
L = 64
MASS = 0.1


def system(gl, seed=1337, lx=L, ly=L):
    g = gl.Generator(seed)
    return g.rand_gauge_u1(lx, ly), g.gaussian(lx * ly)


def solve(gl, U, b, precision, lx=L, ly=L, x0=None, **kw):
    x = np.zeros_like(b) if x0 is None else x0.copy()
    info = gl.minv_vector_cg(x, b, b.size, 5000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(U, MASS, lx, ly), precision=precision, **kw)
    return x, info


def healthy(gl, precision=0):
    """An ordinary solve converges on the same device afterwards."""
    U, b = system(gl, seed=5)
    x, info = solve(gl, U, b, precision)
    assert info.success and info.status == gl.GLINALG_SOLVE_CONVERGED, info
    assert np.all(np.isfinite(x))


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
@pytest.mark.parametrize("where", ["source_nan", "source_inf", "link_nan", "link_inf"])
def test_nonfinite_input_stops_with_nonfinite(gl, gpu, precision, where):
    U, b = system(gl)
    bad = float("nan") if where.endswith("nan") else float("inf")
    if where.startswith("source"):
        b[L * L // 3] = complex(bad, 0.0)
    else:
        U[2 * 77 + 1] = complex(0.0, bad)
    _, info = solve(gl, U, b, precision)
    assert not info.success
    assert info.status == gl.GLINALG_SOLVE_NONFINITE, info
    healthy(gl, precision)


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_zero_source_stops_with_breakdown_and_finite_x(gl, gpu, precision):
    """b = 0 with x0 = 0: the first denominator (<p, Ap> in FP64, the residual rescale in the
    mixed solver) is exactly zero.  x is the exact solution 0 and stays so."""
    U, _ = system(gl)
    b = np.zeros(L * L, np.complex128)
    x, info = solve(gl, U, b, precision)
    assert not info.success
    assert info.status == gl.GLINALG_SOLVE_BREAKDOWN, info
    assert np.all(x == 0)


def test_bicgstab_breakdown_on_an_eigenvector(gl, gpu):
    """Gauge Laplacian with unit links and mass 1/2 on a constant source: A b = b / 2 exactly,
    so alpha = 2 and s = r - alpha A p = 0 exactly; <As, As> = 0 is the breakdown the reference
    turns into NaN (omega = 0/0, generic_bicgstab.cpp:261)."""
    U = np.ones(2 * L * L, np.complex128)
    b = np.ones(L * L, np.complex128)
    x = np.zeros_like(b)
    info = gl.minv_vector_bicgstab(x, b, b.size, 100, 1e-10, gl.square_laplace_u1,
                                   gl.StaggeredU1Op(U, 0.5, L, L))
    assert not info.success
    assert info.status == gl.GLINALG_SOLVE_BREAKDOWN, info
    assert info.iter == 1
    assert np.all(np.isfinite(x))
    healthy(gl)


TIMEOUT_SCRIPT = r'''
import importlib, json, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
gl = importlib.import_module("generic-linalg_gb300")
lx = ly = int(sys.argv[2])
prec = int(sys.argv[3])
g = gl.Generator(1337)
U = g.rand_gauge_u1(lx, ly)
b = g.gaussian(lx * ly)
dev = torch.device("cuda:0")
op = gl.Operator(2, lx, ly, 0.01, torch.from_numpy(U).to(dev))
bt = torch.from_numpy(b).to(dev)
out = {}
x = torch.zeros_like(bt)
first = gl.minv_vector_cg(x, bt, b.size, 100000, 1e-10, gl.square_staggered_normal_u1, op, precision=prec)
out["first"] = [bool(first.success), first.status, first.kernel_launches]
out["tuned"] = gl.lib().glinalg_tuned_persist(op.handle, prec)
x.zero_()
try:
    gl.minv_vector_cg(x, bt, b.size, 100000, 1e-10, gl.square_staggered_normal_u1, op, precision=prec,
                      wait_limit_us=-1)
    out["timeout"] = None
except gl.SolveTimeout as e:
    out["timeout"] = [e.info.status, bool(e.info.success), str(e)]
x.zero_()
after = gl.minv_vector_cg(x, bt, b.size, 100000, 1e-10, gl.square_staggered_normal_u1, op, precision=prec)
Ax = torch.zeros_like(bt)
op.apply(Ax, x)
out["after"] = [bool(after.success), after.status,
                (torch.linalg.vector_norm(bt - Ax) / torch.linalg.vector_norm(bt)).item()]
print(json.dumps(out))
'''


@pytest.mark.parametrize("shape,prec", [(13, 1), (11, 1), (8, 1), (0, 1), (15, 2), (15, 3)])
def test_persistent_wait_limit_runs_out_cleanly(gl, gpu, tmp_path, shape, prec):
    """glinalg_solver_params.wait_limit_us < 0 makes every wait of the persistent inner loop on
    other blocks give up at its first miss.  The kernel raises its error word, every block leaves
    its loop (tensor memory written back and freed), and the call reports
    GLINALG_SOLVE_TIMEOUT; a normal solve on the same device then converges.  Shapes: the
    resident kernel with x_lo and links in tensor memory (13), with x_lo in tensor memory (11),
    with x_lo in L2 (8), the register-tiled kernel with grid barriers (0), and the resident
    kernel of the FP16 and BF16 variants (15)."""
    script = tmp_path / "timeout_case.py"
    script.write_text(TIMEOUT_SCRIPT)
    env = dict(os.environ)
    env["GLINALG_PERSIST_SHAPE"] = str(shape)
    p = subprocess.run([sys.executable, str(script), ROOT, "1024", str(prec)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-3000:]
    res = json.loads(p.stdout.strip().splitlines()[-1])
    assert res["tuned"] == shape, res
    assert res["first"][0] and res["first"][2] >= 1, res
    assert res["timeout"] is not None, res
    status, success, msg = res["timeout"]
    assert status == gl.GLINALG_SOLVE_TIMEOUT and not success, res
    assert "bounded wait" in msg, res
    ok, st, relres = res["after"]
    assert ok and st == gl.GLINALG_SOLVE_CONVERGED and relres < 1e-10, res


def test_checkerboarded_wait_limit_runs_out_cleanly(gl, gpu):
    """The same bounded-wait exit in the checkerboarded even/odd kernel (k_resident_eo): a solve
    told to give up every wait at its first miss reports GLINALG_SOLVE_TIMEOUT, and a normal
    solve on the same device then converges."""
    import torch
    lx = ly = 1024
    U, b = system(gl, lx=lx, ly=ly)
    dev = torch.device("cuda:0")
    Ud, bd = torch.from_numpy(U).to(dev), torch.from_numpy(b).to(dev)
    eo = gl.Operator(9, lx, ly, 0.01, Ud)
    rhs_e = torch.zeros_like(bd)
    gl.square_staggered_eoprec_prepare(rhs_e, bd, eo)
    x = torch.zeros_like(bd)
    with pytest.raises(gl.SolveTimeout) as ei:
        gl.minv_vector_cg(x, rhs_e, b.size, 100000, 1e-10, gl.square_staggered_m2mdeodoe_u1, eo, precision=1,
                          wait_limit_us=-1)
    assert ei.value.info.status == gl.GLINALG_SOLVE_TIMEOUT and not ei.value.info.success
    assert "bounded wait" in str(ei.value)
    x.zero_()
    info = gl.minv_vector_cg(x, rhs_e, b.size, 100000, 1e-10, gl.square_staggered_m2mdeodoe_u1, eo, precision=1)
    assert info.success and info.status == gl.GLINALG_SOLVE_CONVERGED and info.name == "CG-FP32-EO", info
    Ax = torch.zeros_like(bd)
    eo.apply(Ax, x)
    rr = (torch.linalg.vector_norm(rhs_e - Ax) / torch.linalg.vector_norm(rhs_e)).item()
    assert rr < 1e-10, rr


@pytest.mark.parametrize("case", ["source_nan", "link_inf", "zero_source"])
def test_checkerboarded_failure_statuses(gl, gpu, case):
    """The checkerboarded even/odd solve (256 x 256, where lx allows the packed layout) stops
    with GLINALG_SOLVE_NONFINITE on a NaN in the prepared source or an Inf in the links, and
    with GLINALG_SOLVE_BREAKDOWN and x = 0 on an all-zero source; an ordinary solve converges
    on the same device afterwards."""
    lx = ly = 256
    U, b = system(gl, lx=lx, ly=ly)
    if case == "link_inf":
        U[2 * 1000 + 1] = complex(float("inf"), 0.0)
    extra = gl.StaggeredU1Op(U, 0.05, lx, ly)
    rhs_e = np.zeros_like(b)
    if case != "zero_source":
        gl.square_staggered_eoprec_prepare(rhs_e, b, extra)
    if case == "source_nan":
        rhs_e[2 * 777] = complex(float("nan"), 0.0)  # an even site (row 6, x = 18)
    x = np.zeros_like(b)
    info = gl.minv_vector_cg(x, rhs_e, b.size, 20000, 1e-10, gl.square_staggered_m2mdeodoe_u1, extra, precision=1)
    assert not info.success
    if case == "zero_source":
        assert info.status == gl.GLINALG_SOLVE_BREAKDOWN, info
        assert np.all(x == 0)
    else:
        assert info.status == gl.GLINALG_SOLVE_NONFINITE, info
    U2, b2 = system(gl, seed=9, lx=lx, ly=ly)
    ok = gl.StaggeredU1Op(U2, 0.05, lx, ly)
    r2 = np.zeros_like(b2)
    gl.square_staggered_eoprec_prepare(r2, b2, ok)
    x2 = np.zeros_like(b2)
    info2 = gl.minv_vector_cg(x2, r2, b2.size, 20000, 1e-10, gl.square_staggered_m2mdeodoe_u1, ok, precision=1)
    assert info2.success and info2.name == "CG-FP32-EO", info2
