"""The drop-in shim's success path on a GPU: a C++ program calls the reference's complex
minv_vector_* entry points with the reference's callbacks and extra-info structs, exactly as a
reference program does, and the shim routes them to the library (callbacks recognised by
address).  The reference checkout is absent on the GPU machine, so the program is built against
oracle/shim_standin/, a declaration of the reference interface the shim uses
(`make -C oracle shim_standin`); tests/test_shim.py builds the same shim against the
reference's own headers and sources where they exist.

Bars, against the reference's own runs on the same 32x32 system (tests/golden/):
  - CG on square_staggered_normal_u1: the reference's iterations and operator count (199, 201),
    solution within 1e-11;
  - BiCGstab on square_staggered_u1: iterations within 5% of 330, solution within 1e-8 (the
    BiCGstab bar of the solver tests: its iterates are rounding-sensitive);
  - CG-M on square_laplace_u1 with 7 shifts: 41 iterations, 48 operator applications, every
    shift within 1e-11, the per-shift residuals the shim returns below 1e-9 relative;
  - a callback the library does not drive, and a single-direction stencil apply: refused,
    success = false with the reason in the name (no CPU fallback)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from helpers import rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
L = 32


def run_check(gl, golden, tmp_path):
    vec, _ = golden
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "shim_standin"],
                          stdout=subprocess.DEVNULL)
    vec["l32_links"].astype(np.complex128).tofile(tmp_path / "links.bin")
    vec["l32_src"].astype(np.complex128).tofile(tmp_path / "src.bin")
    out = subprocess.run([os.path.join(ROOT, "oracle", "_build", "shim_gpu_check"), str(tmp_path / "links.bin"),
                          str(tmp_path / "src.bin"), str(tmp_path)], capture_output=True, text=True, timeout=300,
                         check=True).stdout
    cases = {}
    for line in out.splitlines():
        if not line.startswith("case "):
            continue
        parts = line.split()
        d = {}
        for kv in parts[2:]:
            if "=" in kv:
                k, v = kv.split("=", 1)
                d[k] = v
        # the name may hold spaces: everything between "name=" and the first residual
        d["name"] = line.split("name=", 1)[1].split(" res")[0]
        cases[parts[1]] = d
    return cases


def test_shim_refuses_what_the_library_does_not_drive(gl, golden, tmp_path):
    cases = run_check(gl, golden, tmp_path)
    for name in ("foreign", "onedir"):
        assert cases[name]["success"] == "0"
        assert cases[name]["name"].startswith("glinalg: ")


@pytest.mark.gpu
def test_shim_success_path_matches_reference(gl, gpu, golden, tmp_path):
    vec, info = golden
    cases = run_check(gl, golden, tmp_path)
    cg = cases["cg"]
    assert cg["success"] == "1" and cg["name"] == "CG", cg
    assert (int(cg["iter"]), int(cg["ops"])) == (info["l32_cg"]["iter"], info["l32_cg"]["ops_count"])
    x = np.fromfile(tmp_path / "cg.bin", dtype=np.complex128)
    assert rel(x, vec["l32_cg"]) < 1e-11

    bi = cases["bicgstab"]
    assert bi["success"] == "1", bi
    assert abs(int(bi["iter"]) - info["l32_bicgstab"]["iter"]) <= 0.05 * info["l32_bicgstab"]["iter"]
    x = np.fromfile(tmp_path / "bicgstab.bin", dtype=np.complex128)
    assert rel(x, vec["l32_bicgstab"]) < 1e-8

    cm = cases["cgm"]
    ref = info["l32_cgm_rfc1_wf0"]
    assert cm["success"] == "1", cm
    assert (int(cm["iter"]), int(cm["ops"])) == (ref["iter"], ref["ops_count"])
    xs = np.fromfile(tmp_path / "cgm.bin", dtype=np.complex128).reshape(7, L * L)
    xr = vec["l32_cgm_rfc1_wf0"].reshape(7, L * L)
    bn = np.linalg.norm(vec["l32_src"])
    for s in range(7):
        assert rel(xs[s], xr[s]) < 1e-11, s
        assert np.sqrt(float(cm[f"res{s}"])) / bn < 1e-9, s
