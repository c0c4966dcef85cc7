"""The NumPy oracle of the learned preconditioner (CPU only): its hand-derived gradient against central finite
differences, its factor algebra (L = D^1/2 L^ reproduces the scaled loss), its initial state (M = diag(A), the
Jacobi preconditioner) and one Adam step against the published update rule.  The CUDA kernels are checked against
this oracle in test_gpu_learned.py."""
import numpy as np
import scipy.sparse as sp

import oracle
from navier_stokes_fem_gb300 import mesh as M
from oracle import learned_oracle as LO


def _graph(n=6):
    o = oracle.Oracle(M.cavity(n), 0.01, 0.01)
    A = o.scipy_matrix("pressure_stiffness").tocsr()
    o.close()
    F = oracle.McFactor(A)
    return A, LO.Graph(A, F.colour, F.lrp, F.lci)


def test_gradient_matches_central_differences():
    A, g = _graph(6)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(A.shape[0])
    b = A @ x
    theta = LO.init_params(5).astype(np.float64)
    theta += 0.05 * rng.standard_normal(theta.size)      # away from the ReLU kinks of the initial state
    _, grad = LO.loss_and_grad(theta, g, x, b)
    idx = rng.choice(theta.size, 60, replace=False)
    h = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (LO.loss_and_grad(tp, g, x, b)[0] - LO.loss_and_grad(tm, g, x, b)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_scaled_loss_equals_the_factor_residual_of_A():
    A, g = _graph(5)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(A.shape[0])
    b = A @ x
    theta = LO.init_params(2)
    lower, diag = LO.forward(theta, g)
    lo, dg = LO.factor_values(g, lower, diag)
    n = A.shape[0]
    L = sp.csr_matrix((lo, (g.c, g.p)), shape=(n, n)) + sp.diags(dg)
    # M = D^1/2 L^ L^T D^1/2; the scaled residual is D^-1/2 (M x - b)
    res = (L @ (L.T @ x) - b) / g.sqrt_d
    bh = b / g.sqrt_d
    loss, _ = LO.loss_and_grad(theta, g, x, b)
    assert np.isclose(loss, res @ res / (bh @ bh), rtol=1e-10)


def test_initial_factor_is_jacobi():
    A, g = _graph(5)
    lower, diag = LO.forward(LO.init_params(0), g)
    # the decoder starts at L^_ii = 1; the off-diagonal output is the decoder bias (0) plus e . wde with wde = 0
    assert np.allclose(diag, 1.0)
    assert np.allclose(lower, 0.0)
    _, dg = LO.factor_values(g, lower, diag)
    assert np.allclose(dg * dg, A.diagonal())


def test_adam_step_follows_the_update_rule():
    rng = np.random.default_rng(0)
    theta = rng.standard_normal(10).astype(np.float32)
    grad = rng.standard_normal(10).astype(np.float32)
    m = np.zeros(10, np.float32)
    v = np.zeros(10, np.float32)
    t0 = theta.copy()
    LO.adam(theta, grad, m, v, 1, lr=1e-2)
    # the first bias-corrected step moves every parameter by lr * sign(grad) (up to eps)
    assert np.allclose(t0 - theta, 1e-2 * np.sign(grad), atol=1e-6)
