"""The adjoint's C-ABI backward entry behind a torch.autograd.Function --
a test harness only (the product boundary is scafes_adj_backward): torch
drives the reverse pass of u_T = S(u0, k), and torch.autograd.gradcheck
compares the analytic vector-Jacobian products with central differences of
the GPU forward solve on a small grid (FP64; gradcheck's default tolerances,
atol 1e-5 and rtol 1e-3, on a map that is linear in u0 and smooth in k)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class HeatSolve(torch.autograd.Function):
    """u_T = forward solve over n_steps from u0 with conductivity k."""

    @staticmethod
    def forward(ctx, u0, k, solver, n_steps):
        solver.set_conductivity(k.detach().cpu().numpy())
        uT = solver.forward(u0.detach().cpu().numpy(), n_steps)
        ctx.save_for_backward(u0, k)
        ctx.solver, ctx.n_steps = solver, n_steps
        return torch.from_numpy(uT)

    @staticmethod
    def backward(ctx, grad_uT):
        u0, k = ctx.saved_tensors
        s = ctx.solver
        s.set_conductivity(k.detach().cpu().numpy())
        gk, gu = s.backward(u0.detach().cpu().numpy(), grad_uT.detach().cpu().numpy(), ctx.n_steps)
        return torch.from_numpy(gu), torch.from_numpy(gk), None, None


def problem(n, seed):
    rng = np.random.default_rng(seed)
    shape = (n[2], n[1], n[0])
    k = np.exp(0.3 * rng.standard_normal(shape))
    tau = 0.5 / (2.0 * k.max() * sum((m - 1) ** 2 for m in n))
    return rng.uniform(-1.0, 1.0, shape), k, tau


def test_autograd_backward_matches_c_abi(gpu):
    M = gpu
    n, T = (9, 8, 7), 12
    u0, k, tau = problem(n, 31)
    w = np.random.default_rng(32).uniform(-1.0, 1.0, u0.shape)
    with M.Adjoint(n, tau, 4) as a:
        tu0 = torch.tensor(u0, requires_grad=True)
        tk = torch.tensor(k, requires_grad=True)
        loss = (torch.from_numpy(w) * HeatSolve.apply(tu0, tk, a, T)).sum()
        loss.backward()
        gk, gu = a.backward(u0, w, T)
    assert np.array_equal(tu0.grad.numpy(), gu)
    assert np.array_equal(tk.grad.numpy(), gk)


def test_autograd_gradcheck(gpu):
    M = gpu
    n, T = (5, 5, 4), 6
    u0, k, tau = problem(n, 33)
    with M.Adjoint(n, tau, 3) as a:
        tu0 = torch.tensor(u0, requires_grad=True)
        tk = torch.tensor(k, requires_grad=True)
        assert torch.autograd.gradcheck(lambda x, y: HeatSolve.apply(x, y, a, T), (tu0, tk), eps=1e-6)
