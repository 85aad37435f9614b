"""Hand-written adjoint of the FP64 step (mbg_adj_*, GPU).

Gradient of L = 1/2 ||T_final - T_target||^2 with respect to the initial
temperature field, checked against central finite differences of the same
forward along seeded random directions, for checkpoint intervals that split
the run unevenly, and through the torch.autograd.Function wrapper.  The
base temperature is 0.1 (the reference scheme diverges near R T = 1/3 at low
viscosity), the other parameters as in the adjoint workload."""
import math

import numpy as np
import pytest

import inputs

pytestmark = pytest.mark.gpu


def _params(n, nu=0.05):
    import marbles_gb300 as M
    p = M.default_params()
    p.n_cell[:] = n
    p.prob_lo[:] = [0.0] * 3
    p.prob_hi[:] = [float(v) for v in n]
    p.is_periodic[:] = [1, 1, 1]
    p.nu, p.alpha = nu, nu
    return p


def _fields(n, seed=3, corr=2.0):
    T0 = 0.1 + 0.005 * inputs.gaussian_field(n, seed, corr)
    Tt = 0.1 + 0.005 * inputs.gaussian_field(n, seed + 1, corr)
    return T0, Tt


def test_adjoint_matches_finite_differences():
    import marbles_gb300 as M
    n = [8, 10, 12]
    adj = M.Adjoint(_params(n))
    T0, Tt = _fields(n)
    nsteps, K = 12, 5

    def loss(T):
        Tf = adj.forward(T, nsteps, K)
        return 0.5 * float(np.sum((Tf - Tt) ** 2)), Tf

    L0, Tf = loss(T0)
    grad = adj.backward(Tf - Tt)
    assert np.isfinite(grad).all() and np.abs(grad).max() > 0
    # Errors are relative to the directional derivative, floored at 1e-3 of
    # |grad| (a random direction can be nearly orthogonal to the gradient,
    # where the difference quotient's round-off, ~1e-11 here, would dominate).
    rng = np.random.default_rng(5)
    gnorm = float(np.linalg.norm(grad))
    worst = {1e-6: 0.0, 1e-5: 0.0}
    for _ in range(16):
        d = rng.standard_normal(T0.size)
        d /= np.linalg.norm(d)
        ad = float(grad @ d)
        for eps in worst:
            fd = (loss(T0 + eps * d)[0] - loss(T0 - eps * d)[0]) / (2 * eps)
            worst[eps] = max(worst[eps], abs(fd - ad) / max(abs(fd), 1e-3 * gnorm))
    print("adjoint vs central differences: worst relative error", worst)
    assert worst[1e-6] < 1e-6
    assert worst[1e-5] < 1e-7


def test_checkpoint_interval_does_not_change_the_gradient():
    import marbles_gb300 as M
    n = [6, 6, 8]
    adj = M.Adjoint(_params(n))
    T0, Tt = _fields(n, seed=9)
    grads = []
    for K in (1, 4, 10):
        Tf = adj.forward(T0, 10, K)
        grads.append(adj.backward(Tf - Tt))
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


def test_autograd_function():
    torch = pytest.importorskip("torch")
    import marbles_gb300 as M
    n = [6, 8, 6]
    adj = M.Adjoint(_params(n))
    T0, Tt = _fields(n, seed=13)
    evolve = M.temperature_evolution(adj, 6, 3)
    t0 = torch.tensor(T0, dtype=torch.float64, requires_grad=True)
    loss = 0.5 * ((evolve(t0) - torch.tensor(Tt)) ** 2).sum()
    loss.backward()
    Tf = adj.forward(T0, 6, 3)
    ref = adj.backward(Tf - Tt)
    assert np.array_equal(t0.grad.numpy(), ref)


def test_adjoint_matches_torch_tape():
    """Reference gradient: autograd over an FP64 PyTorch restatement of the
    same forward (tests/torch_tape.py).  The forward fields agree to
    round-off and the gradients to 1e-9 of their largest entry."""
    torch = pytest.importorskip("torch")
    import marbles_gb300 as M
    import torch_tape as TT
    n = [6, 6, 8]
    nsteps = 6
    adj = M.Adjoint(_params(n))
    T0, Tt = _fields(n, seed=21)
    Tf = adj.forward(T0, nsteps, 4)
    grad = adj.backward(Tf - Tt)
    shape = (n[2], n[1], n[0])
    t0 = torch.tensor(T0.reshape(shape), dtype=torch.float64, requires_grad=True)
    tf = TT.final_temperature(t0, nsteps, TT.Params(nu=0.05, alpha=0.05))
    loss = 0.5 * ((tf - torch.tensor(Tt.reshape(shape), dtype=torch.float64)) ** 2).sum()
    loss.backward()
    assert np.max(np.abs(tf.detach().numpy().reshape(-1) - Tf)) <= 1e-12 * np.max(np.abs(Tf))
    gt = t0.grad.numpy().reshape(-1)
    rel = float(np.max(np.abs(gt - grad)) / np.max(np.abs(gt)))
    print("adjoint vs FP64 autograd tape: max relative difference", rel)
    assert rel < 1e-9
