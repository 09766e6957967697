"""Batched entry points: many independent systems per call must give the same results as
one call per system."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def test_cg_batch_uneven(gl, gpu):
    g = gl.Generator(77)
    rng = np.random.default_rng(3)
    ops, bs, xs, singles = [], [], [], []
    for q in range(8):
        L = int(rng.choice([8, 16, 32, 64]))
        m = float(np.exp(rng.uniform(np.log(0.01), np.log(0.5))))
        kind = 2 if q % 2 == 0 else 3
        U = g.rand_gauge_u1(L, L)
        b = g.gaussian(L * L)
        mass = m if kind == 2 else m * m
        ops.append(gl.Operator(kind, L, L, mass, U))
        bs.append(b)
        xs.append(np.zeros_like(b))
        x1 = np.zeros_like(b)
        cb = gl.square_staggered_normal_u1 if kind == 2 else gl.square_laplace_u1
        singles.append((x1, gl.minv_vector_cg(x1, b, b.size, 100000, 1e-10, cb, ops[-1], precision=1)))
    infos = gl.cg_batch(ops, xs, bs, 100000, 1e-10, precision=1)
    for q in range(8):
        assert infos[q].success
        assert np.sqrt(infos[q].resSq) / np.linalg.norm(bs[q]) < 1e-10
        assert rel(xs[q], singles[q][0]) < 1e-7


def test_cg_m_multi_vs_single(gl, gpu):
    lx = ly = 32
    g = gl.Generator(12)
    U = g.rand_gauge_u1(lx, ly)
    n_rhs, shifts = 3, np.array([1e-4, 1e-2, 1.0])
    B = np.stack([g.gaussian(lx * ly) for _ in range(n_rhs)])
    op = gl.Operator(2, lx, ly, 0.05, U)
    X = np.zeros((n_rhs, 3, lx * ly), np.complex128)
    infos = gl.cg_m_multi(op, X, B, shifts, 1, 10000, 1e-10)
    for q in range(n_rhs):
        xs = [np.zeros(lx * ly, np.complex128) for _ in range(3)]
        inf = gl.minv_vector_cg_m(xs, B[q], 3, lx * ly, 1, 10000, 1e-10, shifts.copy(), gl.square_staggered_normal_u1, op)
        assert infos[q].iter == inf.iter and infos[q].success
        for j in range(3):
            assert rel(X[q, j], xs[j]) < 1e-12
