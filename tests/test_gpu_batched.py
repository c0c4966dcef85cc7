"""The batched form: many cavities of uneven size in one persistent launch per step (CUDA-graph replay), each
instance checked against its own FP64 oracle run; plus the autotuned plan's invariants."""
import numpy as np
import pytest

import navier_stokes_fem_gb300 as nsf
import oracle
from navier_stokes_fem_gb300 import mesh as M
from tests._meshes import rel

pytestmark = pytest.mark.gpu
FIELD_TOL = 1e-6


def _problems(count, seed, n_lo, n_hi):
    out = []
    for prm in M.batched_cavity_params(count, seed=seed, n_lo=n_lo, n_hi=n_hi):
        out.append((M.cavity(prm["n"], lid_u=repr(prm["lid"])), prm["nu"], prm["dt"]))
    return out


def test_batched_instances_match_oracle():
    probs = _problems(6, seed=5, n_lo=6, n_hi=40)
    b = nsf.BatchedNavierStokes(probs, autotune_rounds=2)
    it = b.step(5)
    assert it.shape == (5, 6, 5) and (it[:, :, 2] > 0).all()
    for i, (m, nu, dt) in enumerate(probs):
        o = oracle.Oracle(m, nu, dt)
        assert o.step(5)[0] == 0
        ruv, rp = o.fields()
        uv, p = b.fields(i)
        assert rel(uv, ruv) < FIELD_TOL and rel(p, rp) < FIELD_TOL, i
    plan = b.plan()
    assert (plan["blocks"] >= 1).all() and plan["blocks"].sum() == plan["grid_blocks"]
    assert len(plan["trial_ms"]) == 3
    b.close()


def test_batched_matches_single_instance_path_and_mixed_mode():
    probs = _problems(3, seed=9, n_lo=10, n_hi=24)
    b64 = nsf.BatchedNavierStokes(probs, autotune_rounds=1)
    bmx = nsf.BatchedNavierStokes(probs, autotune_rounds=1, solver="mixed")
    b64.step(4)
    bmx.step(4)
    for i, (m, nu, dt) in enumerate(probs):
        s = nsf.NavierStokesAssembly(m, nu, dt)
        s.step(4)
        suv, sp = s.fields()
        uv, p = b64.fields(i)
        assert rel(uv, suv) < 1e-9 and rel(p, sp) < 1e-8
        xuv, xp = bmx.fields(i)
        assert rel(xuv, suv) < 1e-3 and rel(xp, sp) < 1e-3
        s.close()
    b64.close()
    bmx.close()


def test_batched_set_fields_roundtrip():
    probs = _problems(2, seed=3, n_lo=8, n_hi=12)
    b = nsf.BatchedNavierStokes(probs, autotune_rounds=0)
    uv, p = b.fields(1)
    uv2 = uv + 0.0
    uv2[: len(uv2) // 2] += 1e-3
    b.set_fields(1, uv2, p)
    assert np.array_equal(b.fields(1)[0], uv2)
    with pytest.raises(nsf.NSFemError):
        b.fields(5)
    b.close()
