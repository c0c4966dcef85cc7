"""The multicolour IC(0) oracle (test infrastructure): a valid colouring, a factor that is exactly Cholesky where
no fill is dropped, and PCG that reaches the plain CG solution in far fewer iterations."""
import numpy as np
import scipy.sparse as sp

import oracle
from navier_stokes_fem_gb300 import mesh as M


def _system(n=24, name="pressure_stiffness"):
    o = oracle.Oracle(M.cavity(n), 0.01, 0.01)
    A = o.scipy_matrix(name).tocsr()
    o.close()
    return A


def test_colouring_is_proper_and_pattern_is_lower():
    A = _system()
    F = oracle.McFactor(A)
    rows, cols = A.nonzero()                                           # (the non-zero entries only)
    off = rows != cols
    assert (F.colour[rows[off]] != F.colour[cols[off]]).all()          # coupled rows never share a colour
    assert F.colours <= 3                                              # P1 triangulated grid: small palette
    for i in range(A.shape[0]):
        js = F.lci[F.lrp[i]:F.lrp[i + 1]]
        assert (F.colour[js] < F.colour[i]).all()
        key = F.colour[js].astype(np.int64) * A.shape[0] + js
        assert (np.diff(key) > 0).all()                                # ordered by (colour, column)


def test_ic0_reproduces_the_matrix_on_its_pattern():
    # the defining property of IC(0): (L L^T)_ij = a_ij wherever L has an entry (and on the diagonal)
    A = _system(16)
    n = A.shape[0]
    F = oracle.McFactor(A)
    assert F.ic0() == 0.0
    perm = np.lexsort((np.arange(n), F.colour))      # colour-major order: L is lower triangular there
    pos = np.empty(n, int)
    pos[perm] = np.arange(n)
    rows = np.repeat(np.arange(n), np.diff(F.lrp))
    L = sp.csr_matrix((np.r_[F.lval[:F.nnz_lower], F.diag],
                       (np.r_[pos[rows], pos], np.r_[pos[F.lci[:F.nnz_lower]], pos])), shape=(n, n))
    LLt = (L @ L.T).tocsr()
    Ap = A[perm][:, perm].tocsr()
    pr, pc = L.nonzero()
    assert np.abs(np.asarray(LLt[pr, pc]) - np.asarray(Ap[pr, pc])).max() < 1e-12


def test_pcg_matches_cg_in_fewer_iterations():
    A = _system(32)
    F = oracle.McFactor(A)
    F.ic0()
    rng = np.random.default_rng(3)
    b = A @ rng.standard_normal(A.shape[0])
    x, it, rel, st = F.pcg(b, np.zeros_like(b), tol=1e-10)
    assert st == 0 and rel <= 1e-10
    xs = sp.linalg.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-7
    Fi = oracle.McFactor(A)          # identity factor: PCG degenerates to plain CG
    Fi.set(np.zeros(Fi.nnz_lower), np.ones(A.shape[0]))
    _, it_plain, _, _ = Fi.pcg(b, np.zeros_like(b), tol=1e-10)
    assert it < 0.6 * it_plain
