"""Host-side check of the rectangle plans of the resident kernels (stag_resident.cuh,
stag_resident_eo.cuh, stag_resident_s.cuh), compiled with nvcc and run on the host: no device
code runs.  Over lattices up to 4096 x 4096 every plan that reports ok fits GB300's per-block
shared memory, keeps one ring site per thread, uses at most one rectangle per SM and covers the
lattice; the 1024^2 plans are the ones the benchmark runs (FP32: 8 x 19 rectangles of 128 x 54,
14 rows a thread; checkerboarded: 4 x 38 of 128 packed columns x 27 rows; 16-bit: as FP32)."""
from __future__ import annotations

import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def plans(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("plans") / "plan_check"
    subprocess.check_call([nvcc, "-std=c++17", "-O1", "--expt-relaxed-constexpr", "-gencode",
                           "arch=compute_103a,code=sm_103a", f"-I{ROOT}/include",
                           f"-I{ROOT}/generic-linalg_gb300/csrc", os.path.join(ROOT, "tests", "host", "plan_check.cu"),
                           "-o", str(exe)], timeout=600)
    p = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    return p.returncode, [json.loads(line) for line in p.stdout.splitlines() if line.startswith("{")]


def test_no_plan_violates_the_limits(plans):
    rc, lines = plans
    assert [x for x in lines if "violation" in x] == []
    assert rc == 0 and lines[-1] == {"violations": 0}


def test_benchmark_plans(plans):
    _, lines = plans
    got = {(x["plan"], x["lx"], x["ly"]): x for x in lines if "plan" in x}
    fp32 = got[("fp32", 1024, 1024)]
    assert fp32["ok"] and (fp32["gx"], fp32["gy"], fp32["ty"], fp32["ny"]) == (8, 19, 54, 14)
    eo = got[("eo", 1024, 1024)]
    assert eo["ok"] and (eo["gx"], eo["gy"], eo["ty"], eo["ny"]) == (4, 38, 27, 8)
    for v in ("fp16", "bf16"):
        s = got[(v, 1024, 1024)]
        assert s["ok"] and (s["gx"], s["gy"], s["ty"], s["ny"]) == (8, 19, 54, 14)
    # FP16 and BF16 both store 16-bit fields and FP32 links
    assert got[("fp16", 1024, 1024)]["smem"] == got[("bf16", 1024, 1024)]["smem"] < fp32["smem"]
    # a lattice too large for one rectangle per SM
    assert not got[("fp32", 2048, 2048)]["ok"]
