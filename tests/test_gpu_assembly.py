"""GPU assembly (colour-ordered scatter) against the oracle's element-order triplet assembly: identical
sparsity patterns and values within 1e-12 relative (only the summation order differs); plus size-independent
properties at a larger size where the oracle is not run."""
import numpy as np
import pytest

import navier_stokes_fem_gb300 as nsf
import oracle
from navier_stokes_fem_gb300 import mesh as M
from tests._meshes import golden_mesh

pytestmark = pytest.mark.gpu

PAIRS = [("pressure_stiffness", "pressure_stiffness", False), ("velocity_mass", "velocity_mass", False),
         ("diffusion", "diffusion", False), ("velocity_divergence", "velocity_divergence", False),
         ("pressure_divergence", "pressure_divergence", False),
         ("velocity_lift", "velocity_dirichlet_weights", True), ("pressure_lift", "pressure_dirichlet_weights", True)]


def _meshes(golden):
    return [("cavity32", M.cavity(32), 0.01, 0.01), ("mesh_small", golden_mesh(golden, "mesh_small"), 0.001, 0.01),
            ("channel", M.channel_with_obstacle(128, 32), 1e-3, 2e-3)]


@pytest.mark.parametrize("k", range(3))
def test_matrices_match_oracle(golden, k):
    tag, m, nu, dt = _meshes(golden)[k]
    sim = nsf.NavierStokesAssembly(m, nu, dt)
    o = oracle.Oracle(m, nu, dt)
    for gname, oname, transposed in PAIRS:
        G = sim.scipy_matrix(gname)
        R = o.scipy_matrix(oname)
        if transposed:
            R = R.T.tocsr()
        R.sort_indices()
        G.sort_indices()
        assert G.shape == R.shape, gname
        assert np.array_equal(G.indptr, R.indptr) and np.array_equal(G.indices, R.indices), gname
        scale = np.abs(R.data).max()
        assert np.abs(G.data - R.data).max() <= 1e-12 * scale, gname
    sim.close()


def test_assembly_properties_large():
    m = M.cavity(512)
    sim = nsf.NavierStokesAssembly(m, 1e-3, 1e-3)
    Mm = sim.scipy_matrix("velocity_mass")
    D = sim.scipy_matrix("diffusion")
    K = sim.scipy_matrix("pressure_stiffness")
    assert abs(Mm.sum() - 1.0) < 1e-11
    assert abs(Mm - Mm.T).max() < 1e-17 and abs(D - D.T).max() < 1e-15 and abs(K - K.T).max() < 1e-12
    # pressure stiffness rows of free nodes sum to zero except next to the pinned node
    pinned = 0
    rows = np.asarray(K.sum(axis=1)).ravel()
    W = sim.scipy_matrix("pressure_lift")
    rows_full = rows + np.asarray(W.sum(axis=1)).ravel()
    free = np.ones(m.n_pressure, bool)
    free[pinned] = False
    assert np.abs(rows_full[free]).max() < 1e-9
    assert K.nnz == 7 * 512 ** 2 + 6 * 512 + 1 - 2 * (np.diff(W.indptr) > 0).sum()
    sim.close()


def test_assembly_is_deterministic():
    m = M.channel_with_obstacle(64, 16)
    a = nsf.NavierStokesAssembly(m, 1e-3, 2e-3)
    b = nsf.NavierStokesAssembly(m, 1e-3, 2e-3)
    for name in ("diffusion", "velocity_divergence"):
        assert np.array_equal(a.download_matrix(name)[2], b.download_matrix(name)[2])
    a.close()
    b.close()
