"""bench.py's CPU side: the timed whole oracle steps (count, budget rule, the step-1 fields handed to the GPU FP64
comparison) and the field differences the field and oracle checks report."""
import numpy as np

import bench
import oracle
from navier_stokes_fem_gb300 import mesh as M

W = dict(kind="cavity", n=8, nu=0.01, dt=0.01)


def test_cpu_oracle_steps_counts_and_budget():
    m = M.cavity(8)
    full = bench.cpu_oracle_steps(m, W, 4)
    assert len(full["times_s"]) == 4 and len(full["iterations"]) == 4 and full["status"] == 0
    assert full["ms_per_step"] > 0 and full["cores"] >= 1
    one = bench.cpu_oracle_steps(m, W, 4, budget_s=0.0)      # the budget runs out after the first step
    assert len(one["times_s"]) == 1
    o = oracle.Oracle(m, W["nu"], W["dt"])
    o.step(1)
    uv, p = o.fields()
    o.close()
    # the oracle's OpenMP reductions add in thread-arrival order, so a CG solve may stop an iteration earlier or
    # later from one run to the next: runs agree to about the 1e-8 solver tolerance, not bit for bit
    assert bench.rel_l2(full["fields_1"][0], uv) < 1e-8 and bench.rel_l2(full["fields_1"][1], p) < 1e-8
    assert np.abs(np.asarray(one["iterations"][0]) - np.asarray(full["iterations"][0])).max() <= 1


def test_field_diff():
    nv = 3
    a = (np.array([1.0, 2.0, 2.0, 0.0, 1.0, 0.0]), np.array([1.0, 1.0]))
    b = (np.array([1.0, 2.0, 2.0, 0.0, 2.0, 0.0]), np.array([1.0, 2.0]))
    d = bench.field_diff(a, b, nv)
    assert d["rel_l2_u"] == 0.0
    assert abs(d["rel_l2_v"] - 0.5) < 1e-15
    assert abs(d["rel_l2_p"] - 1.0 / np.sqrt(5.0)) < 1e-15


def test_field_diff_pressure_gradient_and_offset():
    """The pressure is checked through its gradient: a uniform offset of p changes rel_l2_p but neither the
    gradient nor the mean-free difference."""
    nv = 2
    uv = np.array([1.0, 2.0, 3.0, 4.0])
    p = np.array([0.0, 1.0, 3.0])
    grad = lambda q: np.diff(q)   # noqa: E731  (a stand-in for the pressure divergence product)
    d = bench.field_diff((uv, p + 0.5), (uv, p), nv, grad)
    assert d["rel_l2_p"] > 0.1
    assert d["rel_l2_grad_p"] == 0.0 and d["rel_l2_p_mean_free"] < 1e-15
    assert set(bench.FIELD_CHECK_TOL) == {"u", "v", "grad_p"}
