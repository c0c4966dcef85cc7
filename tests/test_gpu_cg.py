"""The persistent CG megakernels (FP64 and mixed precision) through the C ABI, against the oracle CG and an
FP64 residual recomputed on the host; plus the error paths (iteration cap, breakdown, barrier time limit)."""
import numpy as np
import pytest
import scipy.sparse as sp

import navier_stokes_fem_gb300 as nsf
import oracle
from navier_stokes_fem_gb300 import mesh as M

pytestmark = pytest.mark.gpu
TOL = 1e-8


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


@pytest.mark.parametrize("form", ["three_sync", "pipelined", "multi_kernel"])
@pytest.mark.parametrize("name", ["pressure_stiffness", "diffusion", "velocity_mass"])
def test_fp64_cg_matches_oracle(system, name, form):
    """Every iteration form of the FP64 CG: the megakernel with three grid barriers, or one with the pipelined
    recurrences, and the multi-kernel form (one launch per phase, the reference's conjugateGradientMultiKernel)."""
    d, o = system
    n = d.matrix_shape(name)[0]
    rng = np.random.default_rng(1)
    b = rng.standard_normal(n)
    x0 = 0.1 * rng.standard_normal(n)
    d.set_cg_form(form)
    try:
        x, it, rr = d.conjugate_gradient(name, b, x0, eps=TOL)
    finally:
        d.set_cg_form("auto")
    xr, st, itr, _ = o.cg(name, b, x0, tol=TOL)
    assert st == 0
    assert _relres(o, name, x, b) < 1.5 * TOL
    assert abs(it - itr) <= max(2, itr // 50)
    assert rr <= TOL
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-6


@pytest.mark.parametrize("form", ["three_sync", "pipelined", "multi_kernel"])
def test_fp64_cg_forms_on_a_larger_pressure_system(form):
    """The 256 x 256 cavity's pressure system (66 k rows, about 700 iterations from zero): the true residual meets
    the tolerance and the iteration count stays within 2 % of the oracle CG's, for both forms."""
    m = M.cavity(256)
    o = oracle.Oracle(m, 0.01, 0.01)
    d = nsf.GPUSimulationDevice(0)
    rp, col, val, shape = o.matrix("pressure_stiffness")
    d.upload_matrix("pressure_stiffness", rp.astype(np.int32), col, val, shape)
    b = np.random.default_rng(3).standard_normal(shape[0])
    d.set_cg_form(form)
    x, it, rr = d.conjugate_gradient("pressure_stiffness", b, np.zeros_like(b), eps=TOL)
    d.close()
    xr, st, itr, _ = o.cg("pressure_stiffness", b, np.zeros_like(b), tol=TOL)
    res = _relres(o, "pressure_stiffness", x, b)
    o.close()
    assert st == 0
    assert res < 1.5 * TOL
    assert abs(it - itr) <= max(2, itr // 50), (it, itr)


@pytest.mark.parametrize("name", ["pressure_stiffness", "diffusion"])
def test_mixed_cg_reaches_fp64_residual(system, name):
    d, o = system
    n = d.matrix_shape(name)[0]
    b = np.random.default_rng(2).standard_normal(n)
    x, it, rr = d.conjugate_gradient(name, b, np.zeros(n), eps=TOL, solver="mixed")
    xr, st, itr, _ = o.cg(name, b, np.zeros(n), tol=TOL)
    assert _relres(o, name, x, b) < 1.5 * TOL          # FP64 true residual drives the refinement loop
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-6


@pytest.mark.parametrize("form", ["three_sync", "multi_kernel"])
def test_cg_edge_cases(system, form):
    d, o = system
    d.set_cg_form(form)
    try:
        _edge_cases(d)
    finally:
        d.set_cg_form("auto")


def _edge_cases(d):
    name = "pressure_stiffness"
    n = d.matrix_shape(name)[0]
    z = np.zeros(n)
    x, it, rr = d.conjugate_gradient(name, z, z)                   # b = 0, x0 = 0: converged, x = 0
    assert it == 0 and not x.any()
    b = np.random.default_rng(3).standard_normal(n)
    xs, _, _ = d.conjugate_gradient(name, b, z)
    x2, it2, _ = d.conjugate_gradient(name, b, xs)                 # initial guess already converged
    assert it2 == 0 and np.array_equal(x2, xs)
    x3, it3, rr3, st = d.conjugate_gradient(name, b, z, max_iterations=3, raise_on_error=False)
    assert st == 2 and it3 == 3 and np.abs(x3).sum() > 0          # NOT_CONVERGED, last iterate written
    with pytest.raises(nsf.NSFemError) as e:
        d.conjugate_gradient(name, b, z, max_iterations=3)
    assert e.value.status == 2 and "Max iterations reached!" in e.value.message
    bn = b.copy()
    bn[5] = np.nan
    with pytest.raises(nsf.NSFemError) as e:
        d.conjugate_gradient(name, bn, z)
    assert e.value.status == 3


@pytest.mark.parametrize("form", ["three_sync", "multi_kernel"])
def test_cg_breakdown_on_indefinite_matrix(form):
    d = nsf.GPUSimulationDevice(0)
    d.set_cg_form(form)
    n = 64
    A = sp.diags([np.r_[np.ones(n // 2), -np.ones(n // 2)]], [0]).tocsr()
    d.upload_matrix("velocity_mass", A.indptr, A.indices, A.data, A.shape)
    with pytest.raises(nsf.NSFemError) as e:
        d.conjugate_gradient("velocity_mass", np.ones(n), np.zeros(n))
    assert e.value.status == 3
    d.close()


def test_multi_kernel_form_repeats_the_megakernel(system):
    """The multi-kernel form runs the three-barrier megakernel's products, row partition and fixed-order
    reductions, with alpha and beta formed on the device: the same iteration count and, up to the last bits, the same
    iterate, on solves that stop at the tolerance and at an iteration cap (which spans several graph replays and
    stops inside one)."""
    d, o = system
    for name in ("pressure_stiffness", "diffusion"):
        n = d.matrix_shape(name)[0]
        rng = np.random.default_rng(11)
        b = rng.standard_normal(n)
        x0 = 0.05 * rng.standard_normal(n)
        for max_it in (-1, 21):
            out = {}
            for form in ("three_sync", "multi_kernel"):
                d.set_cg_form(form)
                out[form] = d.conjugate_gradient(name, b, x0, eps=TOL, max_iterations=max_it, raise_on_error=False)
            d.set_cg_form("auto")
            x3, it3, _, st3 = out["three_sync"]
            xm, itm, _, stm = out["multi_kernel"]
            assert (itm, stm) == (it3, st3), (name, max_it, itm, it3, stm, st3)
            assert np.linalg.norm(xm - x3) <= 1e-12 * np.linalg.norm(x3), (name, max_it)
            if max_it == 21:
                assert stm == 2 and itm == 21


def test_barrier_time_limit_returns_status_and_handle_survives(system):
    d, o = system
    name = "pressure_stiffness"
    n = d.matrix_shape(name)[0]
    b = np.random.default_rng(4).standard_normal(n)
    d.set_barrier_timeout(0.0)                                    # every grid-wide wait expires at once
    with pytest.raises(nsf.NSFemError) as e:
        d.conjugate_gradient(name, b, np.zeros(n))
    assert e.value.status == 4
    d.set_barrier_timeout(2.0)
    x, it, _ = d.conjugate_gradient(name, b, np.zeros(n))        # the context is still healthy
    assert _relres(o, name, x, b) < 1.5 * TOL


def test_triplet_upload_sums_duplicates_and_f32_signature():
    d = nsf.GPUSimulationDevice(0)
    rng = np.random.default_rng(8)
    n = 200
    R = sp.random(n, n, density=0.03, random_state=8)
    A = (R @ R.T + sp.eye(n) * n * 0.1).tocoo()
    rows = np.r_[A.row, A.row]
    cols = np.r_[A.col, A.col]
    vals = np.r_[A.data * 0.25, A.data * 0.75]
    perm = rng.permutation(len(rows))
    d.upload_matrix_triplets("pressure_stiffness", rows[perm], cols[perm], vals[perm], A.shape)
    G = d.scipy_matrix("pressure_stiffness")
    assert abs(G - A.tocsr()).max() < 1e-14
    b = rng.standard_normal(n).astype(np.float32)
    x = d.conjugate_gradient_f32("pressure_stiffness", b, np.zeros(n, np.float32), eps=1e-6)
    assert np.linalg.norm(A @ x.astype(np.float64) - b) / np.linalg.norm(b) < 1e-5
    y = d.sp_r_mult("pressure_stiffness", np.ones(n))
    assert np.allclose(y, A.tocsr() @ np.ones(n), rtol=1e-13)
    d.close()


def test_bad_arguments_are_statuses():
    d = nsf.GPUSimulationDevice(0)
    with pytest.raises(nsf.NSFemError) as e:
        d.conjugate_gradient("diffusion", np.ones(4), np.zeros(4))            # empty slot
    assert e.value.status == 6
    with pytest.raises(nsf.NSFemError) as e:
        d.upload_matrix("velocity_mass", np.array([0, 1, 1]), np.array([5]), np.array([1.0]), (2, 2))
    assert e.value.status == 5
    with pytest.raises(nsf.NSFemError):
        d.locate(np.zeros((3, 2), np.float32))                               # no mesh yet
    d.close()


@pytest.mark.parametrize("name,solver", [("pressure_stiffness", "mixed"), ("diffusion", "mixed"),
                                         ("pressure_stiffness", "pcg_mixed"), ("diffusion", "pcg_mixed")])
def test_barrier_time_limit_in_every_mixed_form(system, name, solver):
    """The one-launch and the split (refresh + inner-iteration launches) mixed solvers, narrow and wide systems:
    with a zero wait limit every grid-wide wait expires, the solve returns the time-out status without hanging
    the host loop, and the next solve on the same handle converges."""
    d, o = system
    n = d.matrix_shape(name)[0]
    b = np.random.default_rng(9).standard_normal(n)
    if solver == "pcg_mixed":
        d.precond_ic0(name)
    d.set_barrier_timeout(0.0)
    with pytest.raises(nsf.NSFemError) as e:
        d.conjugate_gradient(name, b, np.zeros(n), solver=solver)
    assert e.value.status == 4
    d.set_barrier_timeout(2.0)
    x, it, _ = d.conjugate_gradient(name, b, np.zeros(n), solver=solver)
    assert _relres(o, name, x, b) < 1.5 * TOL
    d.precond_clear(name)
