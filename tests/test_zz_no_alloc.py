"""The allocation-free CG entry point (nsf_conjugate_gradient_noalloc), for callers that cannot call cudaMalloc
(an application whose device memory all belongs to its own pool, or a loop where an allocation's implicit
device synchronisation is not acceptable).  The caller owns every buffer it passes; the solver's work vectors
live in a fixed array inside the library.

Checked through the C ABI against the regular entry point (nsf_conjugate_gradient) on the same system, on two
calls in a row with different right-hand sides (the shared array keeps the previous call's contents, which must
not leak into the next result).  This file is collected last so that a stop at its first failure has already
run every other test.  Device buffers come from torch: the test owns them, the library allocates nothing."""
import ctypes

import numpy as np
import pytest

import navier_stokes_fem_gb300 as nsf
import oracle
from navier_stokes_fem_gb300 import mesh as M

pytestmark = pytest.mark.gpu
REL_TOL = 1e-12     # same algorithm, grid and iteration count as the regular solver: agreement to rounding
REL_TOL_OFF_BY_ONE = 1e-6   # the regular solver's SELL product sums in another order; one iteration more or
                            # less moves x by about the 1e-8 residual times the system's condition number


def _solve_noalloc(torch, A, b, x0, max_iter=-1, eps=1e-8):
    dev = torch.device("cuda:0")
    rp = torch.tensor(A.indptr.astype(np.int32), device=dev)
    col = torch.tensor(A.indices.astype(np.int32), device=dev)
    val = torch.tensor(A.data, dtype=torch.float64, device=dev)
    tb = torch.tensor(b, dtype=torch.float64, device=dev)
    tx0 = torch.tensor(x0, dtype=torch.float64, device=dev)
    tx = torch.zeros_like(tb)
    torch.cuda.synchronize()
    it, rr = ctypes.c_int(), ctypes.c_double()
    st = nsf.library().nsf_conjugate_gradient_noalloc(
        A.shape[0], rp.data_ptr(), col.data_ptr(), val.data_ptr(), tb.data_ptr(), tx0.data_ptr(), tx.data_ptr(),
        int(max_iter), float(eps), None, ctypes.byref(it), ctypes.byref(rr))
    return st, tx.cpu().numpy(), it.value, rr.value


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    m = M.cavity(48)
    o = oracle.Oracle(m, 0.01, 0.01)
    A = o.scipy_matrix("pressure_stiffness")
    d = nsf.GPUSimulationDevice(0)
    d.set_cg_form("three_sync")       # the regular entry point's form of the same FP64 CG the allocation-free one runs
    d.upload_matrix("pressure_stiffness", A.indptr.astype(np.int32), A.indices, A.data, A.shape)
    rng = np.random.default_rng(21)
    for call in range(2):
        b = rng.standard_normal(A.shape[0])
        x0 = np.zeros_like(b) if call == 0 else 0.01 * rng.standard_normal(A.shape[0])
        x_ref, it_ref, rr_ref = d.conjugate_gradient("pressure_stiffness", b, x0)
        st, x, it, rr = _solve_noalloc(torch, A, b, x0)
        assert st == 0, f"call {call}: status {st}"
        assert np.linalg.norm(b - A @ x) <= 1.5e-8 * np.linalg.norm(b), f"call {call}"
        assert abs(it - it_ref) <= 1, (call, it, it_ref)
        tol = REL_TOL if it == it_ref else REL_TOL_OFF_BY_ONE
        assert np.linalg.norm(x - x_ref) <= tol * np.linalg.norm(x_ref), f"call {call}"
    d.close()


def test_noalloc_rejects_oversized_systems():
    torch = pytest.importorskip("torch")
    with open(nsf.header_path) as f:
        limit = int([ln for ln in f if "#define NSF_NOALLOC_MAX_ROWS" in ln][0].split()[-1])
    dev = torch.device("cuda:0")
    one = torch.zeros(1, dtype=torch.float64, device=dev)
    onei = torch.zeros(1, dtype=torch.int32, device=dev)
    st = nsf.library().nsf_conjugate_gradient_noalloc(
        limit + 1, onei.data_ptr(), onei.data_ptr(), one.data_ptr(), one.data_ptr(), one.data_ptr(), one.data_ptr(),
        -1, 1e-8, None, None, None)
    assert st == 5                                                   # NSF_ERR_BAD_ARG, nothing launched
