"""The allocation-free entry point glinalg_staggered_normal_apply_noalloc.

It exists for callers that must not allocate device memory while they run (an application
that has reserved HBM for its own pools, code under another framework's allocator or memory
budget, latency-critical loops).  Its D^dagger D result is compared, through the C-ABI, with
the operator entry point glinalg_operator_apply (which allocates its intermediate field per
call) at the same 1e-14 per-site tolerance as the other operator tests, on two calls in a row
with different inputs, so a stale intermediate left in the shared scratch array would show.
This file is collected last on purpose; it also passes run alone in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import site_rel_err, staggered_scale

pytestmark = pytest.mark.gpu


def _dp(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def test_noalloc_matches_operator_apply_twice(gl, gpu):
    import torch
    L = gl.lib()
    lx, ly, mass = 256, 128, 0.05
    g = gl.Generator(2718)
    U = g.rand_gauge_u1(lx, ly)
    Ud = torch.from_numpy(U).to(gpu)
    op = gl.Operator(2, lx, ly, mass, Ud)
    stream = torch.cuda.current_stream(gpu).cuda_stream
    for call in range(2):
        b = g.gaussian(lx * ly)
        bd = torch.from_numpy(b).to(gpu)
        ref = torch.zeros_like(bd)
        op.apply(ref, bd)
        out = torch.full_like(bd, complex("nan"))
        st = L.glinalg_staggered_normal_apply_noalloc(_dp(Ud), mass, lx, ly, _dp(out), _dp(bd),
                                                      C.c_void_p(stream))
        assert st == 0, L.glinalg_last_error().decode()
        torch.cuda.synchronize()
        o, r = out.cpu().numpy(), ref.cpu().numpy()
        Db = np.zeros_like(b)
        gl.Operator(0, lx, ly, mass, U).apply(Db, b)
        scale = staggered_scale(U, Db, mass, lx, ly)
        assert site_rel_err(o, r, scale) < 1e-14, call


def test_noalloc_rejects_lattices_beyond_the_scratch(gl, gpu):
    import torch
    L = gl.lib()
    lx = ly = 1024  # 2^20 sites > GLINALG_NOALLOC_MAX_SITES (2^18)
    z = torch.zeros(1, dtype=torch.complex128, device=gpu)
    st = L.glinalg_staggered_normal_apply_noalloc(_dp(z), 0.1, lx, ly, _dp(z), _dp(z), None)
    assert st == 1
    assert "exceeds the no-allocation scratch" in L.glinalg_last_error().decode()
