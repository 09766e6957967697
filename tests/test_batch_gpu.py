"""Batched entry points: many independent systems per call must give the same results as
one call per system."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def _true_relres(oracle, kind, L, mass, U, x, b):
    """FP64 true relative residual |b - A x| / |b| with the oracle's operator."""
    import pyoracle
    op = pyoracle.Operator(kind, L, L, mass, U)  # the C-ABI's operator kind numbers
    return np.linalg.norm(b - oracle.apply(op, x)) / np.linalg.norm(b)


def _uneven_batch(gl, n, sides, seed):
    """n systems with sides drawn from `sides`, masses log-uniform in [0.01, 0.5]; even systems
    are staggered D^dagger D (mass m), odd ones the gauge Laplacian -Delta_U + m^2."""
    g = gl.Generator(seed)
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        L = int(rng.choice(sides))
        m = float(np.exp(rng.uniform(np.log(0.01), np.log(0.5))))
        kind = 2 if q % 2 == 0 else 3
        U = g.rand_gauge_u1(L, L)
        b = g.gaussian(L * L)
        out.append((kind, L, m if kind == 2 else m * m, U, b))
    return out


@pytest.mark.parametrize("precision", [1, 2, 3])
def test_cg_batch_uneven(gl, gpu, oracle, precision):
    """Eight systems of sides 8..64 (sides that are not multiples of 32 take the general tile
    path) in one batch: every system reaches the FP64-true relative residual 1e-10 (checked with
    the oracle's operator) and agrees with its own single-system mixed solve."""
    systems = _uneven_batch(gl, 8, [8, 16, 32, 48, 64], 77)
    ops = [gl.Operator(k, L, L, mass, U) for k, L, mass, U, b in systems]
    xs = [np.zeros_like(b) for *_, b in systems]
    infos = gl.cg_batch(ops, xs, [b for *_, b in systems], 100000, 1e-10, precision=precision)
    for q, (kind, L, mass, U, b) in enumerate(systems):
        assert infos[q].success, (q, infos[q])
        assert np.sqrt(infos[q].resSq) / np.linalg.norm(b) < 1e-10
        assert _true_relres(oracle, kind, L, mass, U, xs[q], b) < 1e-10
        x1 = np.zeros_like(b)
        cb = gl.square_staggered_normal_u1 if kind == 2 else gl.square_laplace_u1
        gl.minv_vector_cg(x1, b, b.size, 100000, 1e-10, cb, ops[q], precision=precision)
        assert rel(xs[q], x1) < 1e-7


@pytest.mark.parametrize("precision", [1, 2])
def test_cg_batch_systems_that_stop_at_setup(gl, gpu, oracle, precision):
    """Systems that stop at the first reliable update never enter the list of iterating tiles,
    and the others iterate as if alone: a zero source stops with GLINALG_SOLVE_BREAKDOWN and
    x = 0, a NaN in a source with GLINALG_SOLVE_NONFINITE; the rest (sides 16..48, both
    kinds) reach the FP64-true relative residual 1e-10 and agree with their single-system
    solves."""
    systems = _uneven_batch(gl, 7, [16, 32, 48], 91)
    zero, bad = 1, 4
    systems[zero] = systems[zero][:4] + (np.zeros_like(systems[zero][4]),)
    b_bad = systems[bad][4].copy()
    b_bad[5] = complex(float("nan"), 0.0)
    systems[bad] = systems[bad][:4] + (b_bad,)
    ops = [gl.Operator(k, L, L, mass, U) for k, L, mass, U, b in systems]
    xs = [np.zeros_like(b) for *_, b in systems]
    infos = gl.cg_batch(ops, xs, [b for *_, b in systems], 100000, 1e-10, precision=precision)
    assert infos[zero].status == gl.GLINALG_SOLVE_BREAKDOWN and not infos[zero].success, infos[zero]
    assert np.all(xs[zero] == 0)
    assert infos[bad].status == gl.GLINALG_SOLVE_NONFINITE and not infos[bad].success, infos[bad]
    for q, (kind, L, mass, U, b) in enumerate(systems):
        if q in (zero, bad):
            continue
        assert infos[q].success and infos[q].status == gl.GLINALG_SOLVE_CONVERGED, (q, infos[q])
        assert _true_relres(oracle, kind, L, mass, U, xs[q], b) < 1e-10, q
        x1 = np.zeros_like(b)
        cb = gl.square_staggered_normal_u1 if kind == 2 else gl.square_laplace_u1
        gl.minv_vector_cg(x1, b, b.size, 100000, 1e-10, cb, ops[q], precision=precision)
        assert rel(xs[q], x1) < 1e-7, q


def test_cg_batch_more_systems_than_one_list_chunk(gl, gpu, oracle):
    """1100 small systems (sides 8 and 16, both kinds): the list kernel forms its prefix sum
    1024 systems at a time, so the tiles and vector blocks of systems 1024.. follow a carried
    offset.  Every system reaches the FP64-true relative residual 1e-10."""
    systems = _uneven_batch(gl, 1100, [8, 16], 4242)
    ops = [gl.Operator(k, L, L, mass, U) for k, L, mass, U, b in systems]
    xs = [np.zeros_like(b) for *_, b in systems]
    infos = gl.cg_batch(ops, xs, [b for *_, b in systems], 100000, 1e-10, precision=1)
    for q, (kind, L, mass, U, b) in enumerate(systems):
        assert infos[q].success, (q, infos[q])
        assert _true_relres(oracle, kind, L, mass, U, xs[q], b) < 1e-10, q


def test_cg_batch_256_uneven_systems(gl, gpu, oracle):
    """The uneven-batch workload: 256 systems with sides from {32, 64, 128, 256}, half staggered
    normal equations and half gauge Laplacians, FP32 inner iterations with FP64 reliable
    updates, all in one batch; every system reaches the FP64-true relative residual 1e-10."""
    systems = _uneven_batch(gl, 256, [32, 64, 128, 256], 2024)
    ops = [gl.Operator(k, L, L, mass, U) for k, L, mass, U, b in systems]
    xs = [np.zeros_like(b) for *_, b in systems]
    infos = gl.cg_batch(ops, xs, [b for *_, b in systems], 100000, 1e-10, precision=1)
    iters = [inf.iter for inf in infos]
    assert max(iters) > 2 * min(iters)  # systems stop at very different iterations
    for q, (kind, L, mass, U, b) in enumerate(systems):
        assert infos[q].success, (q, infos[q])
        assert _true_relres(oracle, kind, L, mass, U, xs[q], b) < 1e-10, q


@pytest.mark.parametrize("kind,rfc,max_iter", [(2, 1, 10000), (3, 3, 10000), (2, 2, 40)])
def test_cg_m_multi_equals_single_source_solves(gl, gpu, kind, rfc, max_iter):
    """All sources advanced together give, per source, the single-source CG-M: the same status,
    the iteration and op counts within one, and solutions within 5e-11 where the counts agree
    (the batched kernels reduce in the same order as the single-source ones, but the compiler
    may contract a multiply-add differently; the shifted systems' condition numbers, up to
    ~1.6e3, amplify those last-bit differences to ~1e-11, and now and then move the stop by
    one iteration).  A source that stops one iteration apart is held to 2 kappa 1e-10 per
    shift, the bound any two solutions with relative residual below 1e-10 meet (kappa of
    A + sigma from the operator's spectral bounds).  The explicit residuals are dominated by
    rounding at 1e-10, so they are checked against the tolerance, not bitwise.
    Twelve shifts log-spaced over [1e-4, 1] as in the 512^2 multishift workload, on 64x48;
    max_iter = 40 stops every source early."""
    lx, ly = 64, 48
    g = gl.Generator(12)
    U = g.rand_gauge_u1(lx, ly)
    n_rhs, shifts = 5, np.logspace(-4, 0, 12)
    B = np.stack([g.gaussian(lx * ly) for _ in range(n_rhs)])
    B[3] *= 1e-3  # a source of another scale
    mass = 0.05 if kind == 2 else 0.05 ** 2
    op = gl.Operator(kind, lx, ly, mass, U)
    X = np.zeros((n_rhs, len(shifts), lx * ly), np.complex128)
    infos = gl.cg_m_multi(op, X, B, shifts, rfc, max_iter, 1e-10)
    cb = gl.square_staggered_normal_u1 if kind == 2 else gl.square_laplace_u1
    iters = set()
    for q in range(n_rhs):
        xs = [np.zeros(lx * ly, np.complex128) for _ in shifts]
        inf = gl.minv_vector_cg_m(xs, B[q], len(shifts), lx * ly, rfc, max_iter, 1e-10, shifts.copy(), cb, op)
        assert abs(infos[q].iter - inf.iter) <= 1 and abs(infos[q].ops_count - inf.ops_count) <= 1
        assert infos[q].success == inf.success
        assert infos[q].success == (max_iter == 10000)
        iters.add(inf.iter)
        for j in range(len(shifts)):
            if infos[q].iter == inf.iter:
                assert rel(X[q, j], xs[j]) < 5e-11, (q, j)
            else:
                lo, hi = (mass * mass, mass * mass + 4) if kind == 2 else (mass, mass + 8)
                kappa = (hi + shifts[j]) / (lo + shifts[j])
                assert rel(X[q, j], xs[j]) < 2 * kappa * 1e-10, (q, j)
        bn = np.linalg.norm(B[q])
        rb, rs = np.sqrt(infos[q].resSqmrhs) / bn, np.sqrt(inf.resSqmrhs) / bn
        if max_iter == 10000:
            assert np.all(rb < 1e-9) and np.all(rs < 1e-9), (rb, rs)
        else:
            assert np.allclose(rb, rs, rtol=1e-6), (rb, rs)
    if kind == 2 and rfc == 1 and max_iter == 10000:
        assert len(iters) > 1, "sources should stop at different iterations"


def test_cg_m_multi_device_buffers(gl, gpu):
    """Device-resident sources and solutions (GLINALG_PTR_DEVICE) give the host-buffer result."""
    import torch
    lx = ly = 32
    g = gl.Generator(5)
    U = g.rand_gauge_u1(lx, ly)
    shifts = np.logspace(-4, 0, 12)
    B = np.stack([g.gaussian(lx * ly) for _ in range(4)])
    op = gl.Operator(2, lx, ly, 0.05, U)
    Xh = np.zeros((4, 12, lx * ly), np.complex128)
    gl.cg_m_multi(op, Xh, B, shifts, 1, 10000, 1e-10)
    Xd = torch.zeros((4, 12, lx * ly), dtype=torch.complex128, device=gpu)
    gl.cg_m_multi(op, Xd, torch.from_numpy(B).to(gpu), shifts, 1, 10000, 1e-10)
    assert np.array_equal(Xd.cpu().numpy(), Xh)  # the same kernels on the same inputs
