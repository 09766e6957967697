"""The reference-side binding (generic-linalg_gb300/shim/glinalg_shim.cpp) built the way a
reference program adopts the library: the reference's unmodified sources, with the four files
that define the complex minv_vector_* overloads compiled under ref_* names, linked with the
shim and libglinalg_gb300 (``make -C oracle shim``), then driven through the reference's own
interface by oracle/shim_check.cpp.  Needs the reference checkout, so it runs where the golden
fixtures are made and is skipped elsewhere.

Checks: every reference callback the library drives is recognised by function-pointer
identity (without a device the call reaches the library and fails with "no CUDA device"; with
one, the Hermitian ones match the reference's CG within 1e-11); a foreign callback and a
single-direction stencil apply are refused as unsupported; CG-M's result owns n_shift per-shift
residuals as the reference's does (generic_cg_m.cpp:330), +infinity when the solve could not
run, so the reference's multishift test (tests/multishift/multishift.cpp:281) reads a failure
rather than a null pointer; the real-valued overloads still run the reference's own CG."""
from __future__ import annotations

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RECOGNISED = [
    "square_staggered_u1", "square_staggered_dagger_u1", "square_staggered_normal_u1", "square_laplace_u1",
    "square_staggered_deo_u1", "square_staggered_doe_u1", "square_staggered_m2mdeodoe_u1",
    "apply_stencil_2d", "apply_stencil_2d_eo", "apply_stencil_2d_oe", "apply_square_staggered_m2mdeodoe_stencil",
    "apply_stencil_2d_tb", "apply_stencil_2d_bt", "apply_square_staggered_m2mdtbdbt_stencil",
    "apply_square_staggered_normal_eo_stencil", "apply_square_staggered_normal_tb_stencil",
    "apply_square_staggered_dagger_eo_stencil", "apply_square_staggered_dagger_tb_stencil",
]
ENTRY_POINTS = ["cg_m", "cg_restart", "bicgstab", "bicgstab_restart", "gcr", "gcr_restart", "cr", "cr_restart",
                "minres", "minres_omega", "bicgstab_l", "bicgstab_l_restart", "cr_m", "bicgstab_m",
                "cg_flex_identity"]
PRECONDITIONED = ["cg_flex_minres", "cg_flex_restart_minres", "gcr_var_gcr", "gcr_var_restart_gcr"]


def parse(out):
    cases, extra = {}, {}
    for line in out.splitlines():
        head, _, rest = line.partition(" ")
        if head == "case":
            name, _, kv = rest.partition(" ")
            fields, _, label = kv.partition(" name=")
            d = dict(f.split("=") for f in fields.split())
            cases[name] = {"success": int(d["success"]), "iter": int(d["iter"]), "diff": float(d["diff"]),
                           "name": label}
        else:
            extra[head] = rest.split()
    return cases, extra


@pytest.fixture(scope="module")
def shim_run(gl):
    import pyoracle
    ref = pyoracle.reference_dir()
    if not ref:
        pytest.skip("the reference checkout is not present")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "shim", f"REF={ref}"],
                          stdout=subprocess.DEVNULL)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "shim_check")], capture_output=True, text=True,
                         timeout=300, check=True).stdout
    return parse(out)


def test_callbacks_recognised_by_identity(shim_run):
    cases, extra = shim_run
    device = extra["device"] == ["1"]
    for name in RECOGNISED:
        c = cases[name]
        if device:
            assert not c["name"].startswith("glinalg:"), (name, c)
        else:
            assert c["name"] == "glinalg: no CUDA device" and c["success"] == 0, (name, c)
    if device:
        for name in ("square_staggered_normal_u1", "square_laplace_u1"):
            assert cases[name]["success"] == 1 and cases[name]["diff"] < 1e-11, cases[name]


def test_foreign_callbacks_are_refused(shim_run):
    cases, _ = shim_run
    for name in ("unknown_callback", "single_direction_stencil"):
        assert cases[name]["name"] == "glinalg: unsupported operator" and cases[name]["success"] == 0


def test_every_complex_entry_point_reaches_the_library(shim_run):
    cases, extra = shim_run
    device = extra["device"] == ["1"]
    for name in ENTRY_POINTS:
        c = cases[name]
        assert (c["success"] == 1) if device else (c["name"] == "glinalg: no CUDA device"), (name, c)


@pytest.mark.parametrize("solver", ["cg_m", "cr_m"])
def test_multishift_result_owns_per_shift_residuals(shim_run, solver):
    cases, extra = shim_run
    words = extra[f"{solver}_resSqmrhs"]
    assert words[0] == "n_rhs=3" and len(words) == 4
    res = [float(w) for w in words[1:]]
    if extra["device"] == ["1"]:
        # |b|^2 ~ 2V = 128 on the 8x8 source: (1e-10)^2 |b|^2 ~ 1.3e-18, with room for the
        # explicit residual's rounding
        assert all(0.0 <= r < 1e-16 for r in res)
    else:
        assert all(r == float("inf") for r in res)


def test_preconditioners_recognised_by_identity(shim_run):
    """identity_preconditioner, and minres_ / gcr_preconditioner with a library operator inside,
    reach the library; a foreign inner operator or preconditioner callback is refused (never
    replaced by the identity)."""
    cases, extra = shim_run
    device = extra["device"] == ["1"]
    for name in PRECONDITIONED:
        c = cases[name]
        assert (c["success"] == 1) if device else c["name"].startswith("glinalg: no CUDA device"), (name, c)
    for name in ("precond_foreign_operator", "precond_foreign_callback"):
        assert cases[name]["name"] == "glinalg: unsupported operator (preconditioner)", cases[name]


def test_real_overloads_run_the_reference(shim_run):
    cases, _ = shim_run
    for name, label in (("real_cg", "CG"), ("real_cr", "CR")):
        c = cases[name]
        assert c["success"] == 1 and c["name"] == label and c["iter"] == 7 and c["diff"] <= 1e-12, c


def test_reference_multishift_program_runs_through_the_shim(shim_run):
    """The reference's own tests/multishift/multishift.cpp, unmodified, linked with the shim:
    it runs to the end.  Its real-valued solves keep the reference's code and converge; its
    complex CG, CG-M, CR and CR-M calls on square_laplace_u1 go to the library (without a device
    they do no work, "0 matrix ops"), and the per-shift checks after the multishift solves
    (multishift.cpp:482, 543, 601) read the residual arrays the shim returns.  Its complex
    BiCGstab-M on the real-field callback square_staggered is refused as unsupported."""
    import pyoracle
    _, extra = shim_run
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "shim_multishift",
                           f"REF={pyoracle.reference_dir()}"], stdout=subprocess.DEVNULL)
    run = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "multishift_shim")], capture_output=True,
                         text=True, timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]
    out = run.stdout
    assert "[BICGSTAB-REAL_mass=1]: BiCGStab Success Y" in out
    assert "[CR-REAL_mass=1]: CR Success Y" in out
    for solver in ("CG", "CR"):
        line = [l for l in out.splitlines() if l.startswith(f"[TEST]: {solver}-CPLX Multirhs took")]
        assert len(line) == 1
        if extra["device"] == ["0"]:
            assert line[0].startswith(f"[TEST]: {solver}-CPLX Multirhs took 0 matrix ops"), line
