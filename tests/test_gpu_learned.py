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
