"""Host-side checks that need no GPU: the C-ABI library builds, loads and exports every
function include/glinalg.h declares; compute entry points fail loudly (no CPU fallback)
when no device is present; the input generators reproduce the reference's streams."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(glinalg_\w+)\s*\(", txt, re.M))
    return sorted(names)


def test_header_declares_the_abi():
    names = header_functions()
    for must in ("glinalg_cg", "glinalg_cg_m", "glinalg_bicgstab", "glinalg_gcr", "glinalg_operator_apply",
                 "glinalg_staggered_force", "glinalg_cg_batch"):
        assert must in names


def test_library_exports_every_declared_symbol(gl):
    L = C.CDLL(gl._capi.LIB_PATH)
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert set(header_functions()) <= set(gl._capi.PROTOTYPES), "python prototypes incomplete"


def test_abi_version_and_strings(gl):
    L = gl.lib()
    assert L.glinalg_abi_version() == 2
    assert L.glinalg_status_string(0) == b"success"
    assert L.glinalg_status_string(4) == b"no CUDA device"


def test_no_cpu_fallback(gl):
    """Without a device every compute call reports GLINALG_ERROR_NO_DEVICE."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    U = np.ones(2 * 16, np.complex128)
    with pytest.raises(gl.GlinalgError, match="no CUDA device"):
        gl.Operator(2, 4, 4, 0.1, U)
    b = np.ones(16, np.complex128)
    with pytest.raises(gl.GlinalgError):
        gl.minv_vector_cg(np.zeros(16, np.complex128), b, 16, 10, 1e-10, gl.square_staggered_normal_u1,
                          gl.StaggeredU1Op(U, 0.1, 4, 4))


def test_unknown_callback_is_rejected(gl):
    def my_op(lhs, rhs, extra):
        lhs[:] = rhs
    with pytest.raises(gl.UnsupportedOperator):
        gl.minv_vector_cg(np.zeros(4, np.complex128), np.ones(4, np.complex128), 4, 10, 1e-10, my_op, None)


@pytest.mark.parametrize("key", ["l32", "l8", "l12x6"])
def test_generators_match_reference(gl, golden, key):
    vec, cases = golden
    c = cases[key]
    g = gl.Generator(c["seed"])
    U = g.rand_gauge_u1(c["lx"], c["ly"])
    s1 = g.gaussian(c["lx"] * c["ly"])
    s2 = g.gaussian(c["lx"] * c["ly"])
    assert np.array_equal(U, vec[f"{key}_links"])
    assert np.array_equal(s1, vec[f"{key}_src"])
    assert np.array_equal(s2, vec[f"{key}_src2"])


def test_gauss_gauge_matches_reference(gl, golden):
    vec, cases = golden
    c = cases["g16"]
    U = gl.Generator(c["seed"]).gauss_gauge_u1(c["lx"], c["ly"], c["beta"])
    assert np.array_equal(U, vec["g16_links"])


def test_product_never_touches_the_oracle():
    """The package and its CUDA sources name no oracle module, library or path: the oracle is
    test infrastructure only."""
    pkg = os.path.join(ROOT, "generic-linalg_gb300")
    offenders = []
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dirpath, fn)).read()
                if re.search(r"pyoracle|liboracle|oracle/|import\s+oracle|orc_", txt):
                    offenders.append(fn)
    assert not offenders, offenders


def test_rejected_arguments_name_the_check(gl):
    """A rejected argument sets the message glinalg_last_error() returns, so a caller never
    reads an empty or stale message after GLINALG_ERROR_INVALID_VALUE."""
    L = gl.lib()
    U = np.ones(2 * 16, np.complex128)
    ptr = U.ctypes.data_as(C.POINTER(C.c_double))
    assert L.glinalg_read_gauge_u1(ptr, 4, 4, b"/nonexistent/dir/f.dat") == 1
    assert b"cannot open" in L.glinalg_last_error()
    assert L.glinalg_read_gauge_u1(ptr, 4, 4, None) == 1
    assert L.glinalg_last_error() == b"invalid argument: !path"
    assert L.glinalg_write_gauge_u1(ptr, 4, 4, None) == 1
    assert L.glinalg_last_error() == b"invalid argument: !path"


def test_operator_arrays_shorter_than_the_lattice_are_refused(gl):
    """glinalg_operator_create reads 2*lx*ly links (or lx*ly*nc^2 clover, 4x that hopping, 8x
    two-link terms) through plain pointers; the Python layer refuses shorter arrays before
    the call instead of letting the library read past them."""
    with pytest.raises(ValueError, match="links holds 31 complex values"):
        gl.Operator(2, 4, 4, 0.1, np.ones(31, np.complex128))
    v, nc = 16, 2
    cl, hp = np.zeros(v * nc * nc, np.complex128), np.zeros(4 * v * nc * nc, np.complex128)
    with pytest.raises(ValueError, match="hopping"):
        gl.Operator(4, 4, 4, nc=nc, clover=cl, hopping=hp[:-1])
    with pytest.raises(ValueError, match="two_link"):
        gl.Operator(4, 4, 4, nc=nc, clover=cl, hopping=hp, two_link=np.zeros(8 * v * nc * nc - 1, np.complex128))


def test_operator_descriptor_checks_run_before_the_device(gl):
    """An empty lattice or missing links are rejected by the library with a message, before it
    looks for a device; arrays of the right length in another dtype are converted (and kept
    alive) and reach the device check."""
    import torch
    with pytest.raises(gl.GlinalgError, match=r"invalid argument: d->lx <= 0 \|\| d->ly <= 0"):
        gl.Operator(2, 0, 4, 0.1, np.ones(2, np.complex128))
    with pytest.raises(gl.GlinalgError, match=r"invalid argument: !sten && !d->links"):
        gl.Operator(2, 4, 4, 0.1, None)
    if not torch.cuda.is_available():
        with pytest.raises(gl.GlinalgError, match="no CUDA device"):
            gl.Operator(2, 4, 4, 0.1, np.ones(32, np.complex64))


def test_wrappers_refuse_short_or_mismatched_arrays(gl):
    """The Python layer checks what the C ABI cannot (plain pointers): array lengths against
    what the call reads or writes, dtypes of raw outputs, and arrays of one call on one side.
    Every refusal happens before the library is called (an operator stand-in with only a
    size is enough here)."""
    import types
    z = lambda n: np.zeros(n, np.complex128)
    with pytest.raises(ValueError, match="b holds 15 values"):
        gl.dot(z(16), z(15))
    with pytest.raises(ValueError, match="gauge_field holds 31"):
        gl.get_plaquette_u1(z(31), 4, 4)
    with pytest.raises(ValueError, match="gauge_field holds 31"):
        gl.unit_gauge_u1(z(31), 4, 4)
    with pytest.raises(ValueError, match="gauge_trans holds 15"):
        gl.apply_gauge_trans_u1(z(32), z(15), 4, 4)
    with pytest.raises(ValueError, match="smeared_field holds 31"):
        gl.apply_ape_smear_u1(z(31), z(32), 4, 4, 0.5, 1)
    op = types.SimpleNamespace(size=16, handle=C.c_void_p())
    with pytest.raises(TypeError, match="float64"):
        gl.staggered_force(op, z(16), z(16), np.zeros(32, np.float32))
    with pytest.raises(ValueError, match="grad holds 31 values"):
        gl.staggered_force(op, z(16), z(16), np.zeros(31))
    with pytest.raises(ValueError, match="phi0 holds 31 values"):
        gl.cg_m_multi(op, np.zeros((2, 3, 16), np.complex128), z(31), np.ones(3))
    with pytest.raises(ValueError, match="shifts holds 2 values"):
        gl.cg_m_multi(op, np.zeros((2, 3, 16), np.complex128), z(32), np.ones(2))
    with pytest.raises(ValueError, match="one solution and one source field per operator"):
        gl.cg_batch([op, op], [z(16)], [z(16), z(16)])
    with pytest.raises(ValueError, match=r"phis\[1\] holds 15 values"):
        gl.cg_batch([op, op], [z(16), z(15)], [z(16), z(16)])


def test_bench_capture_stamps_match_kernel_sources():
    """The ncu figures bench.py reports with the headline kernel (DRAM bytes and shared-memory
    wavefronts per launch) were captured from a kernel source whose SHA-256 they carry; a
    changed kernel must be re-captured (or its stamp cleared, which reports the figures as
    stale) before this passes.  The headline kernel's capture must be stamped."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.CAPTURES["resident"]["sha256"] is not None
    for key, cap in bench.CAPTURES.items():
        if cap["sha256"] is not None:
            assert bench.source_sha256(cap["source"]) == cap["sha256"], (key, cap["source"])
            assert os.path.exists(os.path.join(ROOT, cap["profile"])), key
