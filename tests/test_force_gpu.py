"""Adjoint force dS/dtheta for S = phi^dagger (D^dagger D + sigma)^-1 phi.

Bars: the GPU force kernel equals the FP64 CPU force built from the reference's operator and
CG (oracle) to 1e-12 relative; the gradient from the GPU forward solve agrees with central
finite differences (h = 1e-5, FP64) on randomly chosen links to 1e-6 relative.

StaggeredAction is the thin torch.autograd.Function over the C ABI that exists only here, in
the test harness: torch.autograd through it must give the same gradient against the CPU
gradient and against central differences, with the chain rule applied on top."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from pyoracle import Operator as OO

pytestmark = pytest.mark.gpu


class StaggeredAction(torch.autograd.Function):
    """S(theta) = phi^dagger (D^dagger D + sigma)^-1 phi as a function of the link angles theta
    (float64, 2*lx*ly, U = exp(i theta) in the U[2i+mu] layout).  Forward and backward come from
    one C-ABI call, glinalg_staggered_action_grad (forward CG, then the adjoint force kernel);
    backward scales the saved dS/dtheta by the incoming gradient."""

    @staticmethod
    def forward(ctx, theta, gl, phi, lx, ly, mass, sigma, eps, precision):
        U = np.exp(1j * theta.detach().cpu().numpy())
        S, grad, info = gl.staggered_action_grad(gl.Operator(2, lx, ly, mass, U), phi, sigma, eps=eps,
                                                 precision=precision)
        if not info.success:
            raise RuntimeError(f"forward solve did not converge: {info}")
        ctx.save_for_backward(torch.from_numpy(np.asarray(grad)).to(theta.device))
        return theta.new_tensor(S)

    @staticmethod
    def backward(ctx, grad_S):
        (dS,) = ctx.saved_tensors
        return (grad_S * dS,) + (None,) * 8


def action(gl, theta, phi, lx, ly, mass, sigma=0.0, eps=1e-12, precision=0):
    return StaggeredAction.apply(theta, gl, phi, lx, ly, mass, sigma, eps, precision)


def test_force_kernel_vs_oracle(gl, gpu, oracle):
    lx, ly, m = 32, 32, 0.05
    g = gl.Generator(4)
    U = g.rand_gauge_u1(lx, ly)
    phi = g.gaussian(lx * ly)
    X, _, _ = oracle.solve("cg", OO("staggered_normal", lx, ly, m, U), phi, eps=1e-13)
    Y = oracle.apply(OO("staggered", lx, ly, m, U), X)
    ref = oracle.staggered_force(U, m, lx, ly, X, Y)
    op = gl.Operator(0, lx, ly, m, U)
    out = np.zeros(2 * lx * ly)
    gl.staggered_force(op, X, Y, out)
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("prec", [0, 1])
def test_action_grad_vs_cpu_gradient(gl, gpu, oracle, prec):
    lx, ly, m = 64, 64, 0.05
    g = gl.Generator(6)
    U = g.rand_gauge_u1(lx, ly)
    phi = g.gaussian(lx * ly)
    op = gl.Operator(2, lx, ly, m, U)
    S, grad, info = gl.staggered_action_grad(op, phi, 0.0, eps=1e-12, precision=prec)
    assert info.success
    X, _, _ = oracle.solve("cg", OO("staggered_normal", lx, ly, m, U), phi, eps=1e-13)
    Y = oracle.apply(OO("staggered", lx, ly, m, U), X)
    ref = oracle.staggered_force(U, m, lx, ly, X, Y)
    assert np.max(np.abs(grad - ref)) <= 1e-6 * np.max(np.abs(ref))
    assert abs(S - np.vdot(phi, X).real) < 1e-10 * abs(S)


def test_gradient_vs_finite_differences_small(gl, gpu):
    """Plain central differences (h = 1e-5) of S on an 8x8 lattice, solves to 1e-14: small
    enough that S(theta+h) - S(theta-h) keeps its digits in FP64."""
    lx, ly, m, h = 8, 8, 0.05, 1e-5
    g = gl.Generator(31)
    U = g.rand_gauge_u1(lx, ly)
    phi = g.gaussian(lx * ly)
    theta = np.angle(U)
    S0, grad, info = gl.staggered_action_grad(gl.Operator(2, lx, ly, m, U), phi, 0.0, eps=1e-14)

    def action(th):
        x = np.zeros_like(phi)
        inf = gl.minv_vector_cg(x, phi, phi.size, 100000, 1e-14, gl.square_staggered_normal_u1,
                                gl.Operator(2, lx, ly, m, np.exp(1j * th)))
        return np.vdot(phi, x).real

    for j in range(2 * lx * ly):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        fd = (action(tp) - action(tm)) / (2 * h)
        assert abs(fd - grad[j]) <= 1e-6 * max(abs(grad[j]), 1e-3 * np.max(np.abs(grad))), j


def test_gradient_vs_finite_differences_256(gl, gpu):
    """The adjoint-gradient workload: 256x256, m = 0.05, sigma = 0, forward mixed-precision CG to
    1e-12; 64 seeded random links; central differences with h = 1e-5 in FP64.

    At this volume S is ~1e6 times a single link derivative, so S(theta+h) - S(theta-h)
    formed from two separately rounded totals cannot hold 1e-6 relative accuracy in FP64.  The
    same difference is therefore evaluated through the exact identity
      S(+h) - S(-h) = X+^dagger (A(-h) - A(+h)) X-,   X+- = A(+-h)^-1 phi,
    where A(-h) X- and A(+h) X- differ only at the sites within two hops of the link, so the
    sum carries no cancellation.  X+- come from FP64 GPU CG solves to 1e-13."""
    import torch
    lx, ly, m, h = 256, 256, 0.05, 1e-5
    g = gl.Generator(1337)
    U = g.rand_gauge_u1(lx, ly)
    phi = g.gaussian(lx * ly)
    theta = np.angle(U)
    phit = torch.from_numpy(phi).to(gpu)
    S0, grad, info = gl.staggered_action_grad(gl.Operator(2, lx, ly, m, U), phit, 0.0, eps=1e-12,
                                              precision=1)
    assert info.success
    grad = grad.cpu().numpy()
    rng = np.random.default_rng(7)
    picks = rng.choice(2 * lx * ly, size=64, replace=False)

    def solve(op):
        x = torch.zeros_like(phit)
        inf = gl.minv_vector_cg(x, phit, phit.numel(), 100000, 1e-13, gl.square_staggered_normal_u1, op)
        assert inf.success
        return x

    worst = 0.0
    for j in picks:
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        op_p = gl.Operator(2, lx, ly, m, torch.from_numpy(np.exp(1j * tp)).to(gpu))
        op_m = gl.Operator(2, lx, ly, m, torch.from_numpy(np.exp(1j * tm)).to(gpu))
        xp, xm = solve(op_p), solve(op_m)
        am, ap = torch.zeros_like(xm), torch.zeros_like(xm)
        op_m.apply(am, xm)
        op_p.apply(ap, xm)
        dS = torch.vdot(xp, am - ap).real.item()
        fd = dS / (2 * h)
        worst = max(worst, abs(fd - grad[j]) / abs(grad[j]))
    assert worst < 1e-6, worst


def test_autograd_wrapper_vs_cpu_gradient_and_chain_rule(gl, gpu, oracle):
    """torch.autograd through StaggeredAction gives the CPU gradient built from the reference's
    operator and CG (the oracle's CG and force), within 1e-6 relative, on the 64x64 system of
    test_action_grad_vs_cpu_gradient; a loss f(S) = 3 S + S^2 gets f'(S) dS/dtheta."""
    lx, ly, m = 64, 64, 0.05
    g = gl.Generator(6)
    U0 = g.rand_gauge_u1(lx, ly)
    phi = g.gaussian(lx * ly)
    theta = torch.tensor(np.angle(U0), dtype=torch.float64, requires_grad=True)
    U = np.exp(1j * theta.detach().numpy())
    S = action(gl, theta, phi, lx, ly, m)
    (dS,) = torch.autograd.grad(S, theta)
    X, _, _ = oracle.solve("cg", OO("staggered_normal", lx, ly, m, U), phi, eps=1e-13)
    Y = oracle.apply(OO("staggered", lx, ly, m, U), X)
    ref = oracle.staggered_force(U, m, lx, ly, X, Y)
    assert np.max(np.abs(dS.numpy() - ref)) <= 1e-6 * np.max(np.abs(ref))
    assert abs(S.item() - np.vdot(phi, X).real) < 1e-10 * abs(S.item())

    theta2 = theta.detach().clone().requires_grad_(True)
    S2 = action(gl, theta2, phi, lx, ly, m)
    (3.0 * S2 + S2 * S2).backward()
    want = (3.0 + 2.0 * S2.item()) * dS
    assert torch.max(torch.abs(theta2.grad - want)).item() <= 1e-10 * torch.max(torch.abs(want)).item()


def test_autograd_wrapper_vs_finite_differences(gl, gpu):
    """Central differences (h = 1e-5, FP64) of the wrapper's own forward against its autograd
    gradient on 16 seeded links of the 8x8 system of test_gradient_vs_finite_differences_small
    (solves to 1e-14), with that test's bar."""
    lx, ly, m, h = 8, 8, 0.05, 1e-5
    g = gl.Generator(31)
    U = g.rand_gauge_u1(lx, ly)
    phi = g.gaussian(lx * ly)
    theta = torch.tensor(np.angle(U), dtype=torch.float64, requires_grad=True)
    S = action(gl, theta, phi, lx, ly, m, eps=1e-14)
    S.backward()
    grad = theta.grad.numpy()
    picks = np.random.default_rng(3).choice(2 * lx * ly, size=16, replace=False)
    with torch.no_grad():
        for j in picks:
            tp, tm = theta.detach().clone(), theta.detach().clone()
            tp[j] += h
            tm[j] -= h
            Sp = action(gl, tp, phi, lx, ly, m, eps=1e-14).item()
            Sm = action(gl, tm, phi, lx, ly, m, eps=1e-14).item()
            fd = (Sp - Sm) / (2 * h)
            assert abs(fd - grad[j]) <= 1e-6 * max(abs(grad[j]), 1e-3 * np.max(np.abs(grad))), j
