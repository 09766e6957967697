"""Parity at the sizes the benchmark and the multishift workload are quoted on, against the CPU
oracle (the reference's CG and CG-M restated, generic_cg.cpp:278-382 and
generic_cg_m.cpp:312-600, run with its site loops on every host core; its sums stay serial in
the reference's order, so it iterates exactly as the single-threaded reference does: 2093
iterations and 2095 operator applications on the 1024^2 system, as the reference itself).

Inputs come from the oracle's own restatement of the reference tests' generators
(std::mt19937(1337): rand_gauge_u1, then gaussian sources), handed to the library.

Bars (each measured figure is printed by the test):
  - FP64 GPU CG, 1024^2, m = 0.01: iterations within one of the oracle's; solution within 1e-11
    relative of the oracle's.  A CG whose sums only run in another order lands 6.6e-13 from
    it (2093 iterations): the difference is rounding, and 1e-11 leaves a margin of 15.
  - Mixed CG (FP32 / FP16 / BF16 inner iterations, FP64 reliable updates): FP64-true relative
    residual below 1e-10, recomputed here by the oracle's operator; solution within 1e-9
    relative of the oracle's.  Measured on GB300: 1.4e-13 (FP32), 5.7e-13 (FP16, FP32 links),
    1.4e-11 (BF16); 6.1e-11 for FP16 when it kept FP16 links.  Nothing tighter holds by
    construction (their Krylov paths differ from the FP64 one; any two solutions with relative
    residual below 1e-10 differ by at most 2 kappa 1e-10 = 8e-6, kappa(M^dagger M) <=
    (4 + m^2) / m^2 = 40001), so the bar is the worst case measured over both link formats
    with a margin of 16.
  - Multishift, 512^2, m = 0.05, 12 shifts log-spaced over [1e-4, 1], 2 sources: per source the
    oracle's CG-M iteration count; every shift's solution within 1e-10 relative of the oracle's.
    CG-M retires a shift on its iterated residual |zeta_s| |r| < 1e-10 |b|
    (generic_cg_m.cpp:440); the explicit residual drifts from it by rounding, so it is held
    to 1e-9, as in the batched multishift tests.
  - Mixed multishift (FP32 multishift with FP64 scalar recurrences, then every shift refined by
    the mixed CG), same system: every shift's FP64-true relative residual below 1e-10 (what the
    refinement stops on), and its solution within 1e-9 of the oracle's CG-M solution, the bar of
    the mixed CG above.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1, M1 = 1024, 0.01
L3, M3 = 512, 0.05
SHIFTS = np.logspace(-4, 0, 12)


def oracle_lib():
    import pyoracle
    O = pyoracle.Oracle()
    O.set_threads(None)
    return pyoracle, O


@pytest.fixture(scope="module")
def system1024():
    pyoracle, O = oracle_lib()
    g = pyoracle.Generator(1337)
    U = g.rand_gauge_u1(L1, L1)
    b = g.gaussian(L1 * L1)
    op = pyoracle.Operator("staggered_normal", L1, L1, M1, U)
    x, info, _ = O.solve("cg", op, b, max_iter=100000, eps=1e-10)
    assert info["success"] and info["iter"] == 2093 and info["ops_count"] == 2095, info
    return U, b, x, info, O, op


def true_relres(O, op, x, b):
    return float(np.linalg.norm(b - O.apply(op, x)) / np.linalg.norm(b))


def test_fp64_cg_1024_matches_oracle(gl, gpu, system1024):
    U, b, xo, io, O, op = system1024
    x = np.zeros_like(b)
    info = gl.minv_vector_cg(x, b, b.size, 100000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(U, M1, L1, L1))
    err = float(np.linalg.norm(x - xo) / np.linalg.norm(xo))
    rr = true_relres(O, op, x, b)
    print(f"fp64 GPU CG 1024^2: {info.iter} iterations (oracle {io['iter']}), relres {rr:.3e}, "
          f"err vs oracle {err:.3e}")
    assert info.success
    assert abs(info.iter - io["iter"]) <= 1
    assert rr < 1e-10
    assert err < 1e-11


@pytest.mark.parametrize("precision,name", [(1, "fp32"), (2, "fp16"), (3, "bf16")])
def test_mixed_cg_1024_matches_oracle(gl, gpu, system1024, precision, name):
    U, b, xo, io, O, op = system1024
    x = np.zeros_like(b)
    info = gl.minv_vector_cg(x, b, b.size, 100000, 1e-10, gl.square_staggered_normal_u1,
                             gl.StaggeredU1Op(U, M1, L1, L1), precision=precision)
    err = float(np.linalg.norm(x - xo) / np.linalg.norm(xo))
    rr = true_relres(O, op, x, b)
    print(f"{name} mixed CG 1024^2: {info.iter} inner iterations, {info.reliable_updates} reliable updates, "
          f"relres {rr:.3e}, err vs oracle {err:.3e}")
    assert info.success
    assert rr < 1e-10
    assert err < 1e-9


@pytest.fixture(scope="module")
def system512():
    pyoracle, O = oracle_lib()
    g = pyoracle.Generator(1337)
    U = g.rand_gauge_u1(L3, L3)
    B = np.stack([g.gaussian(L3 * L3) for _ in range(2)])
    op = pyoracle.Operator("staggered_normal", L3, L3, M3, U)
    ref = [O.cg_m(op, B[q], SHIFTS, resid_freq_check=1, max_iter=100000, eps=1e-10) for q in range(2)]
    return U, B, ref, O, op


def test_multishift_512_two_sources_match_oracle(gl, gpu, system512):
    import torch
    U, B, ref, O, op = system512
    dev = gpu
    gop = gl.Operator(2, L3, L3, M3, torch.from_numpy(U).to(dev))
    Bd = torch.from_numpy(B).to(dev)
    X = torch.zeros((2, len(SHIFTS), L3 * L3), dtype=torch.complex128, device=dev)
    infos = gl.cg_m_multi(gop, X, Bd, SHIFTS, 1, 100000, 1e-10)
    Xh = X.cpu().numpy()
    for q in range(2):
        xo, io, _ = ref[q]
        assert infos[q].success
        assert infos[q].iter == io["iter"], (q, infos[q], io)
        worst_err = worst_rr = 0.0
        for k, sg in enumerate(SHIFTS):
            err = float(np.linalg.norm(Xh[q, k] - xo[k]) / np.linalg.norm(xo[k]))
            r = B[q] - O.apply(op, Xh[q, k]) - sg * Xh[q, k]
            rr = float(np.linalg.norm(r) / np.linalg.norm(B[q]))
            worst_err, worst_rr = max(worst_err, err), max(worst_rr, rr)
            assert err < 1e-10, (q, k, err)
            assert rr < 1e-9, (q, k, rr)
        print(f"multishift 512^2 source {q}: {infos[q].iter} iterations (oracle {io['iter']}), "
              f"worst shift err vs oracle {worst_err:.3e}, worst relres {worst_rr:.3e}")


def test_mixed_multishift_512_two_sources_match_oracle(gl, gpu, system512):
    import torch
    U, B, ref, O, op = system512
    gop = gl.Operator(2, L3, L3, M3, torch.from_numpy(U).to(gpu))
    Bd = torch.from_numpy(B).to(gpu)
    X = torch.zeros((2, len(SHIFTS), L3 * L3), dtype=torch.complex128, device=gpu)
    infos = gl.cg_m_multi(gop, X, Bd, SHIFTS, 1, 100000, 1e-10, precision=gl.PREC_SINGLE)
    Xh = X.cpu().numpy()
    for q in range(2):
        xo, io, _ = ref[q]
        assert infos[q].success, (q, infos[q])
        worst_err = worst_rr = 0.0
        for k, sg in enumerate(SHIFTS):
            err = float(np.linalg.norm(Xh[q, k] - xo[k]) / np.linalg.norm(xo[k]))
            r = B[q] - O.apply(op, Xh[q, k]) - sg * Xh[q, k]
            rr = float(np.linalg.norm(r) / np.linalg.norm(B[q]))
            worst_err, worst_rr = max(worst_err, err), max(worst_rr, rr)
            assert rr < 1e-10, (q, k, rr)
            assert err < 1e-9, (q, k, err)
            assert np.sqrt(infos[q].resSqmrhs[k]) / np.linalg.norm(B[q]) < 1e-10, (q, k)
        print(f"mixed multishift 512^2 source {q}: {infos[q].iter} FP32 multishift iterations, "
              f"{infos[q].ops_count} operator applications in all, worst shift err vs oracle {worst_err:.3e}, "
              f"worst relres {worst_rr:.3e}")
