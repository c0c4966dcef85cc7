"""The learned preconditioner on the GPU: the tcgen05 dense layer against a BF16-rounded NumPy product, the
network's forward pass and gradients against the NumPy oracle (itself checked by finite differences on the CPU),
training that lowers the loss, and the installed factor driving PCG to the FP64 residual."""
import numpy as np
import pytest

import navier_stokes_fem_gb300 as nsf
import oracle
from navier_stokes_fem_gb300 import mesh as M
from oracle import learned_oracle as LO

pytestmark = pytest.mark.gpu


def _bf(x):
    return LO._bf(np.asarray(x, np.float32), True)


@pytest.mark.parametrize("rows,K,N", [(128, 32, 32), (300, 96, 32), (257, 32, 96), (1000, 64, 64)])
def test_tensor_core_dense_layer(rows, K, N):
    d = nsf.GPUSimulationDevice(0)
    rng = np.random.default_rng(rows + K + N)
    X = rng.standard_normal((rows, K)).astype(np.float32)
    W = rng.standard_normal((K, N)).astype(np.float32)
    b = rng.standard_normal(N).astype(np.float32)
    ref = _bf(X) @ _bf(W) + b
    Y = nsf.tc_dense(d, X, W, b)
    assert np.abs(Y - ref).max() <= 1e-4 * np.abs(ref).max()
    Yr = nsf.tc_dense(d, X, W, b, relu=True)
    assert np.abs(Yr - np.maximum(ref, 0)).max() <= 1e-4 * np.abs(ref).max()
    d.close()


@pytest.mark.parametrize("rows,K", [(128, 32), (1000, 96), (4099, 64), (50000, 32), (77, 4)])
def test_tensor_core_weight_gradient(rows, K):
    """X^T G and colsum G on the tensor cores against the BF16-rounded product in FP64 (FP32 accumulation over up
    to 50 000 rows: 1e-4 of the largest entry)."""
    d = nsf.GPUSimulationDevice(0)
    rng = np.random.default_rng(rows + K)
    X = rng.standard_normal((rows, K)).astype(np.float32)
    G = rng.standard_normal((rows, 32)).astype(np.float32)
    dW, db = nsf.tc_weight_gradient(d, X, G)
    d.close()
    ref = _bf(X).T @ _bf(G)
    rb = _bf(G).sum(axis=0)
    assert np.abs(dW - ref).max() <= 1e-4 * np.abs(ref).max() + 1e-3
    assert np.abs(db - rb).max() <= 1e-4 * np.abs(rb).max() + 1e-3


def _system(n, seed=0):
    o = oracle.Oracle(M.cavity(n), 0.01, 0.01)
    rp, col, val, shape = o.matrix("pressure_stiffness")
    A = o.scipy_matrix("pressure_stiffness").tocsr()
    o.close()
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(A.shape[0])
    return (rp.astype(np.int32), col, val, shape), A, x, A @ x


def _oracle_graph(A):
    F = oracle.McFactor(A)
    return LO.Graph(A, F.colour, F.lrp, F.lci)


@pytest.fixture(scope="module")
def learner():
    d = nsf.GPUSimulationDevice(0)
    L = nsf.Learner(d, seed=7)
    yield d, L
    L.close()
    d.close()


def test_network_forward_matches_oracle(learner):
    d, L = learner
    mat, A, x, b = _system(16)
    d.upload_matrix("pressure_stiffness", *mat)
    idx = L.add_system("pressure_stiffness", x, b)
    rng = np.random.default_rng(1)
    theta = (L.params() + 0.05 * rng.standard_normal(L.param_count)).astype(np.float32)
    L.set_params(theta)
    lower, diag = L.forward(idx)
    g = _oracle_graph(A)
    rl, rd = LO.forward(theta, g, bf16=True)
    assert lower.shape == rl.shape and diag.shape == rd.shape
    assert np.abs(lower - rl).max() <= 2e-3 * max(1.0, np.abs(rl).max())
    assert np.abs(diag - rd).max() <= 2e-3 * max(1.0, np.abs(rd).max())


def test_network_gradient_matches_oracle(learner):
    d, L = learner
    mat, A, x, b = _system(12, seed=3)
    d.upload_matrix("pressure_stiffness", *mat)
    idx = L.add_system("pressure_stiffness", x, b)
    rng = np.random.default_rng(2)
    theta = (L.params() + 0.05 * rng.standard_normal(L.param_count)).astype(np.float32)
    L.set_params(theta)
    loss, grad = L.loss_grad(idx)
    g = _oracle_graph(A)
    rloss, rgrad = LO.loss_and_grad(theta, g, x, b, bf16=True)
    assert abs(loss - rloss) <= 2e-3 * abs(rloss)
    assert np.linalg.norm(grad - rgrad) <= 2e-2 * np.linalg.norm(rgrad)
    # tensor by tensor, so that no small block hides behind the big ones
    k = 0
    for name, shape in LO.SHAPES:
        sz = int(np.prod(shape))
        a, r = grad[k:k + sz], rgrad[k:k + sz]
        assert np.linalg.norm(a - r) <= 5e-2 * np.linalg.norm(r) + 1e-6 * np.linalg.norm(rgrad), name
        k += sz


def test_training_lowers_the_loss_and_the_factor_helps_pcg():
    """Trained on the pressure matrices of three cavities assembled by the plain method, the network's factor must
    beat the method without it: PCG with the learned L needs fewer iterations than plain CG on a held-out cavity's
    pressure solve, at the same FP64 residual.  The training pairs are random probes (z, A z): pairs made of
    smooth solutions alone fit M to A on the smooth modes only and give no preconditioner at all."""
    d = nsf.GPUSimulationDevice(0)
    L = nsf.Learner(d, seed=11)
    rng = np.random.default_rng(4)
    for n in (12, 16, 20):
        sim = nsf.NavierStokesAssembly(M.cavity(n), 0.01, 0.01)
        mat = sim.download_matrix("pressure_stiffness")
        A = sim.scipy_matrix("pressure_stiffness")
        sim.close()
        d.upload_matrix("pressure_stiffness", mat[0], mat[1], mat[2], mat[3])
        for _ in range(4):
            z = rng.standard_normal(A.shape[0])
            L.add_system("pressure_stiffness", z, A @ z)
    losses = L.train(400, batch=2, lr=3e-3, seed=5)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.5 * losses[:5].mean()
    # held-out cavity
    sim = nsf.NavierStokesAssembly(M.cavity(24), 0.01, 0.01)
    sim.step(2)
    A = sim.scipy_matrix("pressure_stiffness")
    b = A @ sim.fields()[1]
    mat = sim.download_matrix("pressure_stiffness")
    sim.close()
    d.upload_matrix("pressure_stiffness", mat[0], mat[1], mat[2], mat[3])
    n = A.shape[0]
    _, it_plain, _ = d.conjugate_gradient("pressure_stiffness", b, np.zeros(n), eps=1e-8, solver="fp64")
    L.apply("pressure_stiffness")
    assert d.precond_kind("pressure_stiffness") == "learned"
    x, it_learned, rr = d.conjugate_gradient("pressure_stiffness", b, np.zeros(n), eps=1e-8, solver="pcg_fp64")
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1.5e-8
    assert it_learned < it_plain
    L.close()
    d.close()
