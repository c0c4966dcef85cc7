"""The roofline arithmetic of bench.py on the CPU: algorithmic bytes per solve from each solve's record, the
dominant kernel by summed time, the index width the mixed PCG reports, and the traffic scaled from the measured
DRAM bytes per row-iteration.  A stand-in simulation object supplies the matrices and profile records."""
import types

import numpy as np
import pytest

import bench


def _csr(n, per_row):
    rp = np.arange(0, n * per_row + 1, per_row, dtype=np.int32)
    col = np.tile(np.arange(per_row, dtype=np.int32), n)
    val = np.ones(n * per_row)
    val[::per_row] = 0.0   # one exact zero per row: not counted
    return rp, col, val, (n, n)


class FakeSim:
    def __init__(self, idx, form="cta1024", fvb=4):
        self.mats = {0: _csr(1000, 7), 1: _csr(4000, 12), 2: _csr(4000, 12)}
        self.idx = idx
        self.form = form
        self.fvb = fvb

    def precond_inner_form(self, slot):
        return self.form

    def precond_value_bytes(self, slot):
        return self.fvb

    def download_matrix(self, slot):
        return self.mats[slot]

    def precond_kind(self, slot):
        return "learned" if slot == 0 else "none"

    def precond_pattern(self, slot):
        return np.zeros(1001, np.int32), np.zeros(2000, np.int32), np.zeros(1000, np.uint8)

    def precond_index_bytes(self, slot):
        return self.idx


@pytest.mark.parametrize("idx,form,fvb", [(2, "cta1024", 4), (4, "cta1024", 4), (2, "resident", 4), (2, "resident", 2)])
def test_roofline_accounts_the_mixed_pcg_under_its_inner_kernel(idx, form, fvb):
    sim = FakeSim(idx, form, fvb)
    prof = {"slot": np.array([0, 0, 1, 2]), "mode": np.array([2, 2, 1, 1]),
            "rows": np.array([1000, 1000, 4000, 4000]), "iterations": np.array([300, 320, 30, 14]),
            "outer": np.array([6, 7, 4, 4]), "ms": np.array([5.0, 6.0, 1.0, 0.5], np.float32)}
    r = bench.roofline(sim, {"prof": prof}, types.SimpleNamespace(steps=2))
    resident = form == "resident"
    kernel = "pcg_mixed_inner_kernel_resident" if resident else "pcg_mixed_inner_kernel_cta1024"
    assert r["kernel"] == kernel and r["launches"] == 2
    nz, nzl = 1000 * 6, 2000
    want = bench.pcg_bytes(True, 1000, nz, nzl, 300, 6, idx, resident, fvb) + \
        bench.pcg_bytes(True, 1000, nz, nzl, 320, 7, idx, resident, fvb)
    assert r["algorithmic_bytes_per_launch"] == round(want / 2)
    # the resident form keeps 16 of the 60 vector bytes per row on the chip; FP16 factor values save 2 per entry
    per_it = (4 + idx) * nz + (fvb + idx) * 2 * nzl + 4 * 1001 + (44 if resident else 60) * 1000 + 16 * 1000 / 16
    assert bench.pcg_bytes(True, 1000, nz, nzl, 1, 0, idx, resident, fvb) - \
        bench.pcg_bytes(True, 1000, nz, nzl, 0, 0, idx, resident, fvb) == per_it
    assert r["achieved"] == pytest.approx(want / 11e-3 / 1e9, abs=0.05)   # GB/s, rounded to 0.1
    peak, _ = bench.peaks()
    assert r["frac"] == pytest.approx(r["achieved"] / peak, abs=1e-4)
    rate = bench.DRAM_BYTES_PER_ROW_ITERATION.get(kernel)
    assert r["traffic"] == (round(rate * 1000 * 620 / 2) if rate else None)
    assert r["kernel_ms_per_step"] == pytest.approx(5.5, abs=1e-3)
    assert r["kernel_share_of_solver_time"] == pytest.approx(11.0 / 12.5, abs=1e-3)


def test_plain_cg_bytes_match_the_per_unit_figures():
    n, nnz = 4_198_401, 20_975_000
    fp64 = bench.algorithmic_bytes(0, n, nnz, 1, 0) - bench.algorithmic_bytes(0, n, nnz, 0, 0)
    assert fp64 == 12 * nnz + 4 * (n + 1) + 88 * n          # one FP64 CG iteration (about 638 MB here)
    assert 630e6 < fp64 < 645e6
    mixed = bench.algorithmic_bytes(1, n, nnz, 1, 0) - bench.algorithmic_bytes(1, n, nnz, 0, 0)
    assert mixed == 8 * nnz + 4 * (n + 1) + 44 * n + n   # (+ the correction fold: x read and written every 16)
    pipe = bench.algorithmic_bytes(0, n, nnz, 1, 1, True) - bench.algorithmic_bytes(0, n, nnz, 0, 1, True)
    assert pipe == 12 * nnz + 4 * (n + 1) + 104 * n        # the pipelined form: 13 vector passes
    assert bench.header_constant("NSF_CG_PIPELINED_MAX_ROWS") > 0


def test_schur_form_bytes_per_iteration():
    """The explicit Schur complement form reads S once (FP32 values, 16-bit columns) and 18 vector bytes per row with
    its row state resident (16 bytes: 1/L_ii kept there too; 30 without), plus the correction fold's FP64 x every FOLD_EVERY iterations."""
    n, nzs = 1000, 4500
    for resident, vec in ((True, 16), (False, 30)):
        per_it = bench.pcg_schur_bytes(n, nzs, 1, 0, 2, resident) - bench.pcg_schur_bytes(n, nzs, 0, 0, 2, resident)
        assert per_it == 6 * nzs + 4 * (n + 1) + vec * n + 16 * n / bench.FOLD_EVERY
