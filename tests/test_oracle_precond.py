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


def test_two_colour_pattern_caps_the_black_diagonal():
    """On the two-colour pattern of a uniform cavity's pressure system, a factor that reproduces the red block and
    the red-black couplings is a diagonal preconditioner of the black Schur complement S, and IC(0)'s choice
    (diag S) is matched by every other diagonal the pattern allows: relaxed modified IC, which subtracts up to 98 %
    of the dropped fill's row sums from D_b^2 (shrinking it up to 50x), takes IC(0)'s iteration count to within 2 %
    (the boundary rows, where the rescaling is not uniform, weigh more on this small mesh).  This is the cap the
    learned factor meets on this pattern."""
    import scipy.sparse as sp

    from navier_stokes_fem_gb300 import mesh as M

    o = oracle.Oracle(M.cavity(64), 1e-4, 1e-4)
    A = o.scipy_matrix("pressure_stiffness").tocsr()
    o.close()
    F = oracle.McFactor(A)
    assert F.colours == 2
    F.ic0()
    lo0, d0 = F.lval[: F.nnz_lower].copy(), F.diag.copy()
    b = A @ np.random.default_rng(1).standard_normal(A.shape[0])
    _, it0, _, st = F.pcg(b, np.zeros_like(b))
    assert st == 0
    rows = np.repeat(np.arange(F.n), np.diff(F.lrp))
    L = sp.csr_matrix((lo0, (rows, F.lci[: F.nnz_lower])), shape=A.shape)
    black = F.colour == 1
    Bm = sp.diags(black.astype(float))
    fill = (Bm @ (L @ L.T) @ Bm).tocsr()
    rowsum = np.asarray(fill.sum(axis=1)).ravel() - fill.diagonal()
    for omega in (0.5, 0.9, 0.98):
        d = d0.copy()
        d[black] = np.sqrt(d0[black] ** 2 - omega * rowsum[black])
        F.set(lo0, d)
        _, it, _, st = F.pcg(b, np.zeros_like(b))
        assert st == 0 and abs(it - it0) <= max(2, it0 // 50), (omega, it, it0)


def test_two_colour_ic0_pcg_is_jacobi_pcg_on_the_schur_complement():
    """The reduced iteration's premise, in FP64: on two colours (the colour-0 block A_00 diagonal), IC(0)-PCG on A from
    an initial guess whose colour-0 rows are projected (x_0 = A_00^-1 (b_0 - A_01 x_1), so r_0 = 0) runs the iterates of
    PCG on the Schur complement S = A_11 - A_10 A_00^-1 A_01 with the factor's colour-1 diagonal L_11^2 = diag S as
    preconditioner: the same iteration count, and the same solution after the colour-0 unknowns are recovered."""
    A = _system(32)
    F = oracle.McFactor(A)
    assert F.colours == 2
    F.ic0()
    c0, c1 = np.flatnonzero(F.colour == 0), np.flatnonzero(F.colour == 1)
    A00, A01 = A[c0][:, c0].tocsr(), A[c0][:, c1].tocsr()
    A10, A11 = A[c1][:, c0].tocsr(), A[c1][:, c1].tocsr()
    assert (A00 - sp.diags(A00.diagonal())).nnz == 0                    # the colour-0 block is diagonal
    d0 = A00.diagonal()
    S = (A11 - A10 @ sp.diags(1.0 / d0) @ A01).tocsr()
    assert np.allclose(F.diag[c1] ** 2, S.diagonal(), rtol=1e-12)       # IC(0)'s colour-1 diagonal is diag S
    b = A @ np.random.default_rng(9).standard_normal(A.shape[0])
    tol = 1e-10
    x0 = np.zeros(A.shape[0])
    x0[c0] = b[c0] / d0                                                 # projected start: r_0 = 0
    x, it_full, _, st = F.pcg(b, x0, tol=tol)
    assert st == 0
    # PCG on S with diag S, stopping on the full residual's norm (equal to the Schur residual's when r_0 = 0)
    bS = b[c1] - A10 @ (b[c0] / d0)
    y = np.zeros(len(c1))
    r = bS.copy()
    z = r / S.diagonal()
    p = z.copy()
    rz = r @ z
    it_schur = 0
    while np.linalg.norm(r) > tol * np.linalg.norm(b):
        q = S @ p
        alpha = rz / (p @ q)
        y += alpha * p
        r -= alpha * q
        z = r / S.diagonal()
        rz, rz_old = r @ z, rz
        p = z + (rz / rz_old) * p
        it_schur += 1
    assert it_schur == it_full, (it_schur, it_full)
    xs = np.zeros_like(x)
    xs[c1] = y
    xs[c0] = (b[c0] - A01 @ y) / d0
    assert np.linalg.norm(xs - x) <= 1e-8 * np.linalg.norm(x)
