"""Preconditioned CG on the GPU: the multicolour pattern and IC(0) factor against the oracle's, FP64 PCG
against the oracle's PCG, mixed-precision PCG to the FP64 residual, installed (learned-path) factors, the
fallback to plain CG over the iteration cap, and whole steps with the pressure solve preconditioned."""
import numpy as np
import pytest

import navier_stokes_fem_gb300 as nsf
import oracle
from navier_stokes_fem_gb300 import mesh as M
from tests._meshes import rel

pytestmark = pytest.mark.gpu
TOL = 1e-8
NAMES = ["pressure_stiffness", "diffusion"]


@pytest.fixture(scope="module")
def system():
    m = M.cavity(32)
    o = oracle.Oracle(m, 0.01, 0.01)
    d = nsf.GPUSimulationDevice(0)
    for name in ("pressure_stiffness", "diffusion", "velocity_mass"):
        rp, col, val, shape = o.matrix(name)
        d.upload_matrix(name, rp.astype(np.int32), col, val, shape)
    yield d, o
    d.close()


def _relres(o, name, x, b):
    A = o.scipy_matrix(name)
    return np.linalg.norm(b - A @ x) / np.linalg.norm(b)


@pytest.mark.parametrize("name", NAMES)
def test_pattern_and_ic0_match_oracle(system, name):
    d, o = system
    rp, col, colour = d.precond_pattern(name)
    F = oracle.McFactor(o.scipy_matrix(name))
    assert np.array_equal(colour, F.colour)
    assert np.array_equal(rp, F.lrp) and np.array_equal(col, F.lci[:F.nnz_lower])
    assert d.precond_ic0(name) == F.ic0()
    lower, diag = d.precond_get(name)
    assert np.abs(lower - F.lval[:F.nnz_lower]).max() <= 1e-12 * np.abs(F.lval).max()
    assert np.abs(diag - F.diag).max() <= 1e-12 * np.abs(F.diag).max()
    assert d.precond_kind(name) == "ic0"


@pytest.mark.parametrize("name", NAMES)
def test_fp64_pcg_matches_oracle_pcg(system, name):
    d, o = system
    d.precond_ic0(name)
    n = d.matrix_shape(name)[0]
    rng = np.random.default_rng(5)
    b = rng.standard_normal(n)
    x0 = 0.1 * rng.standard_normal(n)
    x, it, rr = d.conjugate_gradient(name, b, x0, eps=TOL, solver="pcg_fp64")
    F = oracle.McFactor(o.scipy_matrix(name))
    F.ic0()
    xr, itr, _, st = F.pcg(b, x0, tol=TOL)
    assert st == 0
    assert abs(it - itr) <= max(2, itr // 50)
    assert _relres(o, name, x, b) < 1.5 * TOL
    assert rel(x, xr) < 1e-6
    _, it_plain, _ = d.conjugate_gradient(name, b, x0, eps=TOL, solver="fp64")
    assert it < it_plain


@pytest.mark.parametrize("name", NAMES)
def test_mixed_pcg_reaches_fp64_residual(system, name):
    d, o = system
    d.precond_ic0(name)
    n = d.matrix_shape(name)[0]
    b = np.random.default_rng(6).standard_normal(n)
    x, it, rr = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="pcg_mixed")
    xr, st, itr, _ = o.cg(name, b, np.zeros(n), tol=TOL)
    assert _relres(o, name, x, b) < 1.5 * TOL           # the FP64 true residual drives the refinement loop
    assert rel(x, xr) < 1e-6
    assert it < itr


def test_installed_factor_is_used_as_given(system):
    """nsf_precond_set is the learned preconditioner's entry point: IC(0) values installed through it must give
    the IC(0) solve, and the identity factor must give plain CG."""
    d, o = system
    name = "pressure_stiffness"
    n = d.matrix_shape(name)[0]
    b = np.random.default_rng(7).standard_normal(n)
    d.precond_ic0(name)
    _, it_ic0, _ = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="pcg_fp64")
    lower, diag = d.precond_get(name)
    d.precond_clear(name)
    assert d.precond_kind(name) == "none"
    d.precond_set(name, lower, diag)
    assert d.precond_kind(name) == "learned"
    _, it_set, _ = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="pcg_fp64")
    assert it_set == it_ic0
    d.precond_set(name, np.zeros_like(lower), np.ones(n))
    _, it_id, _ = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="pcg_fp64")
    _, it_plain, _ = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="fp64")
    assert abs(it_id - it_plain) <= 1
    with pytest.raises(nsf.NSFemError):
        d.precond_set(name, lower, -diag)
    d.precond_ic0(name)


@pytest.mark.parametrize("solver", ["pcg_fp64", "pcg_mixed"])
def test_over_the_cap_falls_back_to_plain_cg(system, solver):
    d, o = system
    name = "pressure_stiffness"
    n = d.matrix_shape(name)[0]
    b = np.random.default_rng(8).standard_normal(n)
    d.precond_ic0(name)
    d.precond_cap(name, 3)
    d.profile(True)
    x, it, rr = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver=solver)
    prof = d.profile_read()
    d.profile(False)
    d.precond_cap(name, 0)
    assert prof["fallback"][-1] == 1
    assert _relres(o, name, x, b) < 1.5 * TOL


@pytest.mark.parametrize("solver", ["pcg_fp64", "pcg_mixed"])
def test_steps_with_preconditioned_pressure_match_oracle(solver):
    """Solvers that stop at the same 1e-8 relative residual differ by ~cond(A) * 1e-8 in the solution, so the
    preconditioned runs are held against the discrete solution (the oracle driven to 1e-13): within 1e-3, and of
    the same size as the plain FP64 path's own error."""
    m = M.cavity(24)
    o = oracle.Oracle(m, 0.01, 0.01)
    o.set_tolerance(1e-13)
    st, rit = o.step(10)
    assert st == 0
    ruv, rp = o.fields()

    def run(solver, precondition):
        sim = nsf.NavierStokesAssembly(m, 0.01, 0.01, solver=solver)
        if precondition:
            sim.precond_ic0("pressure_stiffness")
        it = sim.step(10)
        uv, p = sim.fields()
        sim.close()
        return max(rel(uv, ruv), rel(p, rp)), it

    err, it = run(solver, True)
    err_plain, it_plain = run("fp64", False)
    assert err < 1e-3 and err < 10 * err_plain + 1e-7
    # the pressure solves need fewer iterations; the mixed form restarts its FP32 recurrence at every FP64 refresh
    # (robust on the ill-conditioned large systems), which costs it some of the gain on small ones
    assert it[:, 2].sum() < (0.7 if solver == "pcg_fp64" else 0.9) * it_plain[:, 2].sum()


@pytest.mark.parametrize("n", [32, 96])
def test_reduced_pcg_matches_full_pcg(n):
    """The reduced (Schur complement) iteration of the mixed PCG on a two-colour pressure system: with IC(0) it runs
    the full PCG's iterates in exact arithmetic (an FP64 NumPy model of both takes 100 and 299 iterations on these
    two systems).  In FP32 the Schur complement's near-constant mode (Jacobi-scaled condition number 7e4 at n = 96)
    is resolved less well than by the full form's difference-form product, which costs the reduced form 25-35 %
    more iterations on these small systems (5-6 % on the 2048 cavity).  The FP64 true residual meets the tolerance
    and the solution is the oracle CG's; it reads the factor's colour-1 diagonal only, so a factor whose other
    entries are scaled gives the same solve, bit for bit."""
    m = M.cavity(n)
    o = oracle.Oracle(m, 0.01, 0.01)
    d = nsf.GPUSimulationDevice(0)
    name = "pressure_stiffness"
    rp, col, val, shape = o.matrix(name)
    d.upload_matrix(name, rp.astype(np.int32), col, val, shape)
    colour = d.precond_pattern(name)[2]
    assert colour.max() == 1                                          # two colours
    d.precond_ic0(name)
    b = np.random.default_rng(31).standard_normal(shape[0])
    x0 = 0.01 * np.random.default_rng(32).standard_normal(shape[0])
    out = {}
    for form in ("full", "reduced", "schur"):
        d.set_pcg_form(form)
        out[form] = d.conjugate_gradient(name, b, x0, eps=TOL, solver="pcg_mixed")
        assert d.precond_inner_form(name).startswith(form) or form == "full" and \
            d.precond_inner_form(name) in ("resident", "cta1024")
    xf, itf, _ = out["full"]
    xo, st, ito, _ = o.cg(name, b, x0, tol=TOL)
    assert st == 0
    for form in ("reduced", "schur"):
        xr_, itr_, _ = out[form]
        assert _relres(o, name, xr_, b) < 1.5 * TOL, form
        assert itr_ <= 1.4 * itf + 5, (form, itr_, itf)
        assert rel(xr_, xo) < 1e-6, form
    xr_, itr_, _ = out["reduced"]
    # only L_11 enters: scaling the factor's off-diagonal entries and its colour-0 diagonal changes nothing
    lower, diag = d.precond_get(name)
    diag2 = diag.copy()
    diag2[colour == 0] *= 1.3
    d.precond_set(name, 1.7 * lower, diag2)
    d.set_pcg_form("reduced")
    x2, it2, _ = d.conjugate_gradient(name, b, x0, eps=TOL, solver="pcg_mixed")
    assert it2 == itr_ and np.array_equal(x2, xr_)
    d.set_pcg_form("full")
    d.close()
    o.close()


def test_reduced_pcg_steps_match_discrete_solution():
    """Whole steps with the reduced mixed PCG on the pressure (IC(0)): within 1e-3 of the discrete solution, as the
    full form, with at most 40 % more pressure iterations on this small cavity."""
    m = M.cavity(24)
    o = oracle.Oracle(m, 0.01, 0.01)
    o.set_tolerance(1e-13)
    assert o.step(10)[0] == 0
    ruv, rp = o.fields()
    its = {}
    for form in ("full", "reduced", "schur"):
        sim = nsf.NavierStokesAssembly(m, 0.01, 0.01, solver="pcg_mixed")
        sim.set_pcg_form(form)
        sim.precond_ic0("pressure_stiffness")
        its[form] = sim.step(10)
        uv, p = sim.fields()
        assert sim.precond_inner_form("pressure_stiffness").startswith(form) or form == "full"
        sim.close()
        assert max(rel(uv, ruv), rel(p, rp)) < 1e-3, form
    f = its["full"][:, 2].sum()
    for form in ("reduced", "schur"):
        r = its[form][:, 2].sum()
        assert r <= 1.4 * f + 10, (form, r, f)


def _perturbed_cavity(n, seed=11, amp=0.3):
    """A cavity whose interior vertices are moved randomly (no edge axis-aligned): its pressure matrix has no
    exact zeros off the diagonal, three colours and at most 7 entries per row (the narrow, split solver)."""
    m = M.cavity(n)
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    xy = m.nodes.astype(np.float64)
    P = m.n_pressure
    interior = (xy[:P, 0] > 0) & (xy[:P, 0] < 1) & (xy[:P, 1] > 0) & (xy[:P, 1] < 1)
    xy[:P][interior] += rng.uniform(-amp * h, amp * h, size=(int(interior.sum()), 2))
    for e in m.elements:
        for k, (a, b) in zip((3, 4, 5), ((1, 2), (0, 2), (0, 1))):
            xy[e[k]] = 0.5 * (xy[e[a]] + xy[e[b]])
    m.nodes = xy.astype(np.float32)
    return m


def _golden_small():
    import os
    from tests._meshes import golden_mesh
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_kdtree_lookup.npz"))
    return golden_mesh(g, "mesh_small")


@pytest.mark.parametrize("which", ["perturbed64", "mesh_small"])
def test_multicolour_pcg_on_unstructured_pressure(which):
    """Three colours on a narrow system (the split mixed solver, colours >= 2 after the fused first colour) and
    five on the reference's own unstructured mesh (the one-launch solver): FP64 PCG against the oracle's PCG with
    the same factor, and mixed PCG to the FP64 residual."""
    m = _perturbed_cavity(64) if which == "perturbed64" else _golden_small()
    o = oracle.Oracle(m, 0.01, 0.01)
    name = "pressure_stiffness"
    rp, col, val, shape = o.matrix(name)
    d = nsf.GPUSimulationDevice(0)
    d.upload_matrix(name, rp.astype(np.int32), col, val, shape)
    colours = int(d.precond_pattern(name)[2].max()) + 1
    assert colours == (3 if which == "perturbed64" else 5)
    d.precond_ic0(name)
    n = shape[0]
    rng = np.random.default_rng(12)
    b = rng.standard_normal(n)
    x0 = 0.1 * rng.standard_normal(n)
    x, it, _ = d.conjugate_gradient(name, b, x0, eps=TOL, solver="pcg_fp64")
    F = oracle.McFactor(o.scipy_matrix(name))
    F.ic0()
    xr, itr, _, st = F.pcg(b, x0, tol=TOL)
    assert st == 0
    assert abs(it - itr) <= max(2, itr // 50)
    assert _relres(o, name, x, b) < 1.5 * TOL
    xm, itm, _ = d.conjugate_gradient(name, b, x0, eps=TOL, solver="pcg_mixed")
    assert _relres(o, name, xm, b) < 1.5 * TOL           # the contract: the FP64 residual
    assert d.precond_index_bytes(name) == 2              # small systems: the 16-bit column copies
    xt, st, _, _ = o.cg(name, b, x0, max_iter=20 * n, tol=1e-13)
    assert st == 0 and rel(xm, xt) < 1e-5 and rel(x, xt) < 1e-5
    _, it_plain, _ = d.conjugate_gradient(name, b, x0, eps=TOL, solver="fp64")
    assert itm < it_plain
    d.close()
    o.close()


def test_mixed_pcg_when_slice_columns_span_beyond_16_bits():
    """A periodic chain of 140000 rows: after the two-colour permutation the wrap-around couples permuted rows
    70000 apart, so neither the matrix nor the factor gets a 16-bit column copy and the inner iterations read the
    32-bit columns; the solve still reaches the FP64 residual and matches FP64 PCG."""
    import scipy.sparse as sp
    n = 140000
    A = sp.diags([np.full(n - 1, -1.0), np.full(n, 2.001), np.full(n - 1, -1.0)], [-1, 0, 1], format="lil")
    A[0, n - 1] = A[n - 1, 0] = -1.0
    A = A.tocsr()
    A.sort_indices()
    name = "pressure_stiffness"
    d = nsf.GPUSimulationDevice(0)
    d.upload_matrix(name, A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data, A.shape)
    assert int(d.precond_pattern(name)[2].max()) + 1 == 2
    d.precond_ic0(name)
    b = np.random.default_rng(13).standard_normal(n)
    xm, itm, _ = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="pcg_mixed")
    assert np.linalg.norm(b - A @ xm) / np.linalg.norm(b) < 1.5 * TOL
    assert d.precond_index_bytes(name) == 4
    x, it, _ = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="pcg_fp64")
    assert rel(xm, x) < 1e-6 and itm <= 2 * it + 10
    d.close()


def test_fp16_factor_copies_only_within_range():
    """The mixed PCG reads FP16 factor values where every value fits FP16's normal range (the cavity's pressure
    factor); a system scaled by 1e-12 puts the factor's values (about its square root) below it, so the factor keeps
    FP32 values only, and
    the mixed PCG still reaches the FP64 residual either way."""
    m = M.cavity(24)
    o = oracle.Oracle(m, 0.01, 0.01)
    A = o.scipy_matrix("pressure_stiffness").tocsr()
    o.close()
    b = np.random.default_rng(12).standard_normal(A.shape[0])
    for scale, want in ((1.0, 2), (1e-12, 4)):
        d = nsf.GPUSimulationDevice(0)
        As = (A * scale).tocsr()
        d.upload_matrix("pressure_stiffness", As.indptr.astype(np.int32), As.indices, As.data, As.shape)
        d.precond_ic0("pressure_stiffness")
        assert d.precond_value_bytes("pressure_stiffness") == want
        x, it, _ = d.conjugate_gradient("pressure_stiffness", b * scale, np.zeros_like(b), eps=TOL,
                                        solver="pcg_mixed")
        assert np.linalg.norm(b * scale - As @ x) <= 1.5 * TOL * np.linalg.norm(b * scale)
        _, it_plain, _ = d.conjugate_gradient("pressure_stiffness", b * scale, np.zeros_like(b), eps=TOL,
                                              solver="mixed")
        assert it < it_plain, (scale, it, it_plain)
        d.close()


@pytest.mark.parametrize("name,solver", [("pressure_stiffness", "mixed"), ("pressure_stiffness", "pcg_mixed"),
                                         ("diffusion", "mixed")])
def test_mixed_solves_do_not_depend_on_the_scale(name, solver):
    """The mixed solvers rescale their FP32 vectors by powers of two at the true-residual refreshes, so a right-hand
    side 2^-60 times another (unscaled, p.q would fall below FP32's range) takes the same iterations and gives
    exactly 2^-60 times the same solution; the plain mixed CG on the whole system times 2^-40 (its FP32 matrix
    copy times 2^-40) gives exactly the same solution.  (The PCG's factor of 2^-40 A has values below FP16's
    range and is read as FP32 instead, so that case would run other arithmetic.)"""
    m = M.cavity(64)
    o = oracle.Oracle(m, 0.01, 0.01)
    A = o.scipy_matrix(name).tocsr()
    o.close()
    b = np.random.default_rng(5).standard_normal(A.shape[0])
    s = 2.0 ** -60
    d = nsf.GPUSimulationDevice(0)
    d.upload_matrix(name, A.indptr.astype(np.int32), A.indices, A.data, A.shape)
    if solver == "pcg_mixed":
        d.precond_ic0(name)
    x, it, _ = d.conjugate_gradient(name, b, np.zeros_like(b), eps=TOL, solver=solver)
    xs, its, _ = d.conjugate_gradient(name, b * s, np.zeros_like(b), eps=TOL, solver=solver)
    d.close()
    assert its == it and np.array_equal(xs, x * s), (it, its, rel(xs / s, x))
    if solver == "mixed":
        g = 2.0 ** -40
        As = (A * g).tocsr()
        d = nsf.GPUSimulationDevice(0)
        d.upload_matrix(name, As.indptr.astype(np.int32), As.indices, As.data, As.shape)
        xg, itg, _ = d.conjugate_gradient(name, b * g, np.zeros_like(b), eps=TOL, solver=solver)
        d.close()
        assert itg == it and np.array_equal(xg, x), (it, itg, rel(xg, x))
