#!/usr/bin/env python
"""Benchmark of the per-time-step hot path: ms per operator-split time step and CG iterations per solve at a
1e-8 relative residual, on one GB300 (N GPUs run N independent replicas; the path does not shard).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--solver S] [--precond P] [--impl reference]

The default line is the metric's method on the 2048 x 2048 cavity: mixed-precision PCG with the learned
preconditioner (trained on the GPU during set-up, untimed); in the same run, over the same steps, the same method
with IC(0) in place of the learned factor ("ic0_pcg_mixed") and the plain FP64 CG megakernel ("plain_fp64_cg").

A step is one pass of the hot path over the resident fields: advection, two diffusion solves, the pressure solve,
the gradient product and two mass solves (NavierStokesAssembly::semiLagrangianSolve's loop body,
include/assembly.h:1516-1556).  Every arm times steps 1..K of the run from its initial state (u = 0 with the
Dirichlet values, p = 0), after W warm-up steps whose fields are dropped.  `value` is device time per step (CUDA
events on the library's stream) with the fields resident in HBM; `e2e` is the same steps through the C ABI with host
fields copied in and out every step.  `field_check` compares the fields the fast arms end with against the plain
FP64 arm's; `oracle_check` compares the GPU FP64 step 1 with the FP64 oracle's step 1, which is also the timed CPU
baseline.  `--impl reference` times whole steps of the CPU oracle (the restated reference path; the reference's own
CPU CG lives in an absent submodule) on the same workload with every host thread.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/time-step & CG iters at 1e-8 resid: learned-PCG mixed vs plain FP64 CG, GB300"

WORKLOADS = {
    # the lid-driven cavity the reference can run on a CPU: 32x32, nu=0.01, dt=0.01
    "cavity32": dict(kind="cavity", n=32, nu=0.01, dt=0.01),
    # channel 4x1 on 1024x256 cells, [0.9,1.1]x[0.4,0.6] removed, nu=1e-3, dt=2e-3
    "channel1024x256": dict(kind="channel", nx=1024, ny=256, nu=1e-3, dt=2e-3),
    # the large combined form: 2048x2048 cavity, nu=1e-4, dt=1e-4
    "cavity2048": dict(kind="cavity", n=2048, nu=1e-4, dt=1e-4),
    "cavity512": dict(kind="cavity", n=512, nu=1e-3, dt=1e-3),
    "cavity1024": dict(kind="cavity", n=1024, nu=1e-4, dt=1e-4),
    # the batched form: 64 cavities, n ~ U{16..256}, nu log-U[1e-3,1e-1], lid U[0.5,2], dt = 0.25 h / lid
    "batched64": dict(kind="batched", count=64, seed=20261203, n_lo=16, n_hi=256, nu=None, dt=None),
}
DEFAULT_WORKLOAD = "cavity2048"
L2_BYTES = 129 << 20


def make_mesh(w):
    from navier_stokes_fem_gb300 import mesh as M

    if w["kind"] == "cavity":
        return M.cavity(w["n"])
    return M.channel_with_obstacle(w["nx"], w["ny"])


def header_constant(name):
    """An integer #define of the library's C header."""
    with open(os.path.join(ROOT, "include", "nsfem_gb300.h")) as f:
        for line in f:
            if line.startswith("#define " + name + " "):
                return int(line.split()[2])
    raise KeyError(name)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        idxs = sorted({r[0] for r in rows})
        want = vis.split(",")[0] if vis.split(",")[0] in idxs else idxs[0]
        rows = [r for r in rows if r[0] == want]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        loaded = [s for s in sm if s >= 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows)}


# the mixed solvers fold their FP32 correction into the FP64 iterate every FOLD_EVERY iterations of a cycle
FOLD_EVERY = 16


def algorithmic_bytes(mode, n, nnz, its, outer, pipelined=False):
    """Minimal DRAM bytes of one persistent CG launch (int32 indices).

    FP64 iteration: nnz*(8+4) + 4(n+1) + 11 vector passes of 8n (SpMV gathers p and writes q, dot fused; x and r
    read+write with p and q reads; p update reads r, p and writes p).  Prologue: one SpMV with x0 plus b, r, p, x.
    The pipelined FP64 form moves 13 passes (its product gathers w; z, s, p, x, r and w read and written), and
    every replacement (outer - 1 of them) four products.
    Mixed: inner FP32 iterations nnz*(4+4) + 4(n+1) + 11*4n, plus the FP64 x read and written every
    FOLD_EVERY iterations when the correction is folded into it (16n / FOLD_EVERY); every refinement sweep one FP64
    residual nnz*(8+4) + 4(n+1) + 28n and an x += d pass of 20n.
    """
    if mode == 0:
        passes = 13 if pipelined else 11
        it_bytes = 12 * nnz + 4 * (n + 1) + 8 * passes * n
        prologue = 12 * nnz + 4 * (n + 1) + 40 * n
        extra = max(outer - 1, 0) * 4 * (12 * nnz + 4 * (n + 1) + 24 * n) if pipelined else 0
        return prologue + extra + its * it_bytes
    inner = 8 * nnz + 4 * (n + 1) + 44 * n + 16 * n / FOLD_EVERY
    sweep = 12 * nnz + 4 * (n + 1) + 28 * n
    return (outer + 1) * sweep + outer * 20 * n + its * inner


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_oracle_steps(mesh, w, timed_steps, budget_s=None, threads=None):
    """The FP64 oracle (the restated reference path) on the host cores: whole operator-split steps 1, 2, ... of the
    run from its initial state, each timed - up to `timed_steps` of them, fewer when the next step would take the
    timed steps past `budget_s` seconds, but at least one.  Returns the per-step times and iteration counts, the
    set-up time, and the fields after step 1 (for the GPU FP64 comparison)."""
    import oracle

    oracle.build(ref=False)
    if threads:
        oracle.set_threads(threads)
    cores = oracle.max_threads()
    t0 = time.perf_counter()
    o = oracle.Oracle(mesh, w["nu"], w["dt"])
    setup = time.perf_counter() - t0
    times, its, f1, status = [], [], None, 0
    while len(times) < max(1, timed_steps):
        t0 = time.perf_counter()
        st, it = o.step(1)
        times.append(time.perf_counter() - t0)
        its.append(it[0].tolist())
        status = status or int(st)
        if f1 is None:
            f1 = o.fields()
        if budget_s is not None and sum(times) + times[-1] > budget_s:
            break
    o.close()
    return {"times_s": times, "ms_per_step": 1e3 * sum(times) / len(times), "iterations": its, "setup_s": setup,
            "cores": cores, "status": status, "fields_1": f1}


def run_reference(args):
    world, rank, local, pg = dist_setup()
    w = WORKLOADS[args.workload]
    if rank != 0:
        barrier(pg)
        return
    import oracle

    oracle.build(ref=False)
    cores = oracle.max_threads()
    if w["kind"] == "batched":
        # every instance's whole step on the host (one oracle per instance, instances one after another, each
        # using every host thread): one untimed step, then timed steps within the time budget
        probs = batched_problems(w)
        oracles = [oracle.Oracle(m, nu, dt) for m, nu, dt in probs]
        times, its = [], []
        while len(times) < max(1, args.steps):
            t0 = time.perf_counter()
            per = [o.step(1)[1][0] for o in oracles]
            times.append(time.perf_counter() - t0)
            its.append(np.sum(per, axis=0))
            if sum(times) + times[-1] > args.ref_budget_s:
                break
        for o in oracles:
            o.close()
        k = len(times)
        sample_txt = (f"all {len(probs)} instances stepped whole on the host; steps 1..{k} from the initial state "
                      f"timed ({args.steps} requested, time budget {args.ref_budget_s:.0f} s)")
        ms = 1e3 * sum(times) / k
        line = {
            "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms/step", "n_gpus": world,
            "steps": k, "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "instances": len(probs), "solver": "fp64 CG (CPU oracle)"},
            "cg_iterations_per_step": np.mean(its, axis=0).round(1).tolist(),
            "cpu_baseline": {"value": round(ms, 3), "unit": "ms/step", "cores": cores, "kind": "port",
                             "sample": sample_txt},
            "e2e": {"value": round(ms, 3), "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        barrier(pg)
        return
    mesh = make_mesh(w)
    # whole steps from rest: one untimed step, then timed whole steps - all args.steps of them when they fit the
    # arm's time budget, else as many as fit (at least one); `steps` reports the number actually timed
    cpu = cpu_oracle_steps(mesh, w, args.steps, budget_s=args.ref_budget_s)
    k = len(cpu["times_s"])
    ms = cpu["ms_per_step"]
    sample_txt = (f"whole FP64 oracle steps 1..{k} of the run from its initial state, each timed ({args.steps} "
                  f"requested, time budget {args.ref_budget_s:.0f} s; no warm-up is needed on the host); set-up "
                  f"{cpu['setup_s']:.1f} s excluded; all {cpu['cores']} host threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms/step", "n_gpus": world,
        "steps": k, "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_block(args, w, mesh, solver="fp64 CG (CPU oracle)"),
        "cg_iterations_per_step": np.mean(cpu["iterations"], axis=0).round(1).tolist(),
        "cg_iterations_each_step": cpu["iterations"],
        "step_times_s": [round(t, 3) for t in cpu["times_s"]],
        "oracle_status": cpu["status"],
        "cpu_baseline": {"value": round(ms, 3), "unit": "ms/step", "cores": cpu["cores"], "kind": "port",
                         "sample": sample_txt},
        "e2e": {"value": round(ms, 3), "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(pg)


def config_block(args, w, mesh, solver):
    cfg = {"workload": args.workload, "triangles": mesh.n_elements, "velocity_nodes": mesh.n_nodes,
           "pressure_nodes": mesh.n_pressure, "nu": w["nu"], "dt": w["dt"], "tol": 1e-8, "solver": solver,
           "parallelism": "replicas" if args.gpus > 1 else "single GPU"}
    return cfg


def pcg_reduced_bytes(n, nz, its, outer, idx=4, resident=False):
    """Minimal DRAM bytes of one reduced (Schur complement) mixed PCG solve of a two-colour system (half the rows
    in each colour): per iteration every matrix row once (FP32 values + idx-byte columns; the colour-0 rows for u_0,
    the colour-1 rows for q_1) and FP32 vector traffic of 42 bytes per row: colour-0 rows gather z and p, read
    1/a_ii and write u (8n); colour-1 rows read the row sums and their own z and p, gather u, write p and q (12n);
    the update reads u and d and writes d on colour-0 rows (6n), reads p, q, d, r and 1/L_ii^2 and writes d, r and
    z on colour-1 rows (16n).  With the CTA-private state resident in shared memory (q, d and r of the colour-1
    rows, d of the colour-0 rows) 26 bytes per row.  Plus the FP64 x read and written every FOLD_EVERY iterations.
    Per refresh an FP64 projection of the colour-0 unknowns (the colour-0 rows of the matrix) and an FP64
    residual."""
    it_bytes = (4 + idx) * nz + 4 * (n + 1) + (26 if resident else 42) * n + 16 * n / FOLD_EVERY
    refresh = 12 * nz + 12 * nz / 2 + 8 * (n + 1) + 36 * n
    return (outer + 1) * refresh + its * it_bytes


def pcg_schur_bytes(n, nzs, its, outer, idx=2, resident=False):
    """Minimal DRAM bytes of one reduced mixed PCG solve with the Schur complement S formed explicitly (nzs entries
    over the colour-1 rows, half of the n rows): per iteration S once (FP32 values + idx-byte columns) and FP32
    vector traffic per row of 16 bytes with the CTA-private state resident (colour-1 rows: S's row sums, own z and p,
    z and p gathered, p written; the update reads p and writes z; q, d, r and 1/L_ii in shared memory), 30 without
    it (q written and read, d and r read and written, 1/L_ii read); plus the FP64 x read and written every FOLD_EVERY iterations.  Per refresh the
    projection of the colour-0 unknowns and an FP64 residual with the permuted matrix (nz is not needed: its rows
    are counted as 1.5 products of S's size)."""
    it_bytes = (4 + idx) * nzs + 4 * (n + 1) + (16 if resident else 30) * n + 16 * n / FOLD_EVERY
    refresh = 12 * 1.5 * nzs + 8 * (n + 1) + 36 * n
    return (outer + 1) * refresh + its * it_bytes


def pcg_bytes(mixed, n, nz, nzl, its, outer, idx=4, resident=False, fvb=None, reduced=False):
    """Minimal DRAM bytes of one preconditioned solve: per iteration the product with the non-zeros of A and both
    triangular sweeps over the factor's nzl strictly lower entries (values + idx-byte column indices: 2 where the
    mixed iterations read 16-bit column copies), plus about 15 vector passes (product gathers and outputs, the x/r
    update, the sweeps' right-hand sides, inverse diagonals and in-place results), 11 when the inner kernel keeps
    the correction (read and written every iteration) and the colour-1 rows' r and q (half the rows) in shared
    memory.  The mixed form moves FP32 values and vectors - the factor's values in FP16 where the factor keeps FP16
    copies (fvb = 2 bytes per factor value), reads and writes the FP64 x every FOLD_EVERY iterations (the correction
    fold) - and adds an FP64 residual (int32 indices) per refresh."""
    if reduced:
        return pcg_reduced_bytes(n, nz, its, outer, idx, resident)
    v = 4 if mixed else 8
    fv = v if fvb is None or not mixed else fvb
    passes = 11 if resident else 15
    it_bytes = (v + idx) * nz + (fv + idx) * 2 * nzl + 4 * (n + 1) + passes * v * n + (16 * n / FOLD_EVERY if mixed else 0)
    refresh = 12 * nz + 4 * (n + 1) + 28 * n
    return (outer + 1) * refresh + its * it_bytes


def time_arm(sim, args, pg, start=None):
    """Warm-up steps, then args.steps timed steps (CUDA events on the library's stream, L2 flushed in between)
    with every persistent solve recorded; returns the measurements, the fields the timed steps started from and
    the fields they ended with.  With `start` (uv, p) the timed steps start from those fields instead of the
    warm-up's, so that several arms time the same steps."""
    for _ in range(args.warmup):
        sim.flush_l2(256 << 20)
        sim.step(1)
    sim.synchronize()
    if start is not None:
        sim.set_fields(*start)
    start_fields = sim.fields()
    clocks = ClockSampler()
    clocks.start()
    sim.profile(True)
    launches0 = sim.launch_count()
    barrier(pg)
    sim.synchronize()
    sim.timer_start()
    its = []
    for _ in range(args.steps):
        sim.flush_l2(256 << 20)       # L2 evicted between steps (the step's matrices exceed L2 anyway)
        its.append(sim.step(1)[0])
    ms_total = sim.timer_stop()
    sim.synchronize()
    barrier(pg)
    launches = sim.launch_count() - launches0
    clk = clocks.stop()
    prof = sim.profile_read()
    sim.profile(False)
    return {"ms": max_over_ranks(pg, ms_total / args.steps), "its": np.asarray(its), "prof": prof,
            "launches": launches, "clocks": clk, "start_fields": start_fields, "end_fields": sim.fields()}


# Field agreement after the timed steps between the fast method and the plain FP64 CG (both stop every solve at a
# 1e-8 relative residual, so their solutions may differ by up to about cond(A) * 1e-8 per solve; the pressure
# system's condition number grows as h^-2), and between the GPU FP64 step and the FP64 oracle's step (the same
# algorithm, summation order aside).  The pressure is checked through what the step uses of it, its gradient
# (-dt grad p, the pressure divergence product that corrects the velocity): the lowest mode of the cavity's
# pressure system (one pinned node; nearly constant elsewhere, Jacobi-scaled eigenvalue about 1e-8 of the largest
# at 2048) is left loose by any solve that stops at a 1e-8 residual, and two solvers' pressures differ mostly by
# that near-constant offset, which accumulates over steps through the warm start.  rel_l2_p and the same without
# the mean are reported beside it.
FIELD_CHECK_TOL = {"u": 1e-5, "v": 1e-5, "grad_p": 1e-5}
ORACLE_FIELD_TOL = 1e-6


def rel_l2(a, b):
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b))) / (nb if nb > 0 else 1.0)


def field_diff(fa, fb, nv, grad=None):
    """Relative L2 differences of u, v and p between two (uv, p) field sets; with grad (p -> -dt grad p) also of the
    pressure gradient, and of p without the mean of the difference."""
    (uva, pa), (uvb, pb) = fa, fb
    d = {"rel_l2_u": rel_l2(uva[:nv], uvb[:nv]), "rel_l2_v": rel_l2(uva[nv:], uvb[nv:]), "rel_l2_p": rel_l2(pa, pb)}
    if grad is not None:
        diff = np.asarray(pa) - np.asarray(pb)
        nb = float(np.linalg.norm(pb))
        d["rel_l2_p_mean_free"] = float(np.linalg.norm(diff - diff.mean())) / (nb if nb > 0 else 1.0)
        d["rel_l2_grad_p"] = rel_l2(grad(pa), grad(pb))
    return d


def nonzeros(sim, slot):
    rp, col, val, shape = sim.download_matrix(slot)
    return int(np.count_nonzero(val))


# DRAM traffic per row and iteration of the solver kernels, each from one ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum of a launch that ran a known number of iterations on the 2048 cavity's pressure system,
# 4,198,401 rows, whose vectors exceed L2): the reduced inner kernel with the Schur complement formed explicitly and
# its row state (and 1 / L_11) in shared memory 4.57 GB over 40 iterations; the reduced inner kernel forming u_0 (row state in
# shared memory) 5.53 GB over 40 iterations; the full-form resident inner kernel (row state in shared memory,
# 16-bit column copies, FP16 factor values) 11.01 GB over 40 iterations; the 1024-thread inner kernel without the
# resident state (16-bit column copies, FP32 factor values) 17.49 GB over 40 iterations; cg_fp64_kernel 30.67 GB
# over 60 iterations (its prologue included).
DRAM_BYTES_PER_ROW_ITERATION = {"pcg_mixed_inner_kernel_schur_resident": 27.2,
                                "pcg_mixed_inner_kernel_reduced_resident": 32.9,
                                "pcg_mixed_inner_kernel_resident": 65.5, "pcg_mixed_inner_kernel_cta1024": 104.1,
                                "cg_fp64_kernel": 121.7}


def roofline(sim, arm, args):
    """Algorithmic bytes over every persistent solve of the timed steps / their summed kernel time.  A mixed PCG
    solve of a narrow system runs as a refresh kernel and inner-iteration kernels; the inner kernel (one
    1024-thread CTA per SM on two or more colours) takes over 99% of its time, and the solve is reported under
    that kernel's name."""
    prof = arm["prof"]
    nz = {slot: nonzeros(sim, slot) for slot in (0, 1, 2)}
    nzl, idx, res, red, fvb, nzs = {}, {}, {}, {}, {}, {}
    for slot in (0, 1, 2):
        if sim.precond_kind(slot) != "none":
            nzl[slot] = int(sim.precond_pattern(slot)[1].size)
            idx[slot] = sim.precond_index_bytes(slot)
            form_ = sim.precond_inner_form(slot)
            res[slot] = form_.endswith("resident")
            red[slot] = form_.startswith(("reduced", "schur"))
            nzs[slot] = sim.precond_schur_nnz(slot) if form_.startswith("schur") else 0
            fvb[slot] = sim.precond_value_bytes(slot)
    resident, reduced, schur = any(res.values()), any(red.values()), any(nzs.values())
    base = "pcg_mixed_inner_kernel_schur" if schur else "pcg_mixed_inner_kernel_reduced"
    names = {0: "cg_fp64_kernel", 1: "cg_mixed_kernel",
             2: (base + "_resident" if resident else base) if reduced else
                "pcg_mixed_inner_kernel_resident" if resident else "pcg_mixed_inner_kernel_cta1024",
             3: "pcg_fp64_kernel"}
    form = getattr(args, "cg_form", "auto")
    pipe_max = header_constant("NSF_CG_PIPELINED_MAX_ROWS")
    bytes_by, ms_by, rowit_by = {}, {}, {}
    for sl, m_, n_, i_, o_, t_ in zip(prof["slot"], prof["mode"], prof["rows"], prof["iterations"], prof["outer"],
                                      prof["ms"]):
        m_, sl = int(m_), int(sl)
        pipe = m_ == 0 and (form == "pipelined" or (form == "auto" and int(n_) < pipe_max))
        if m_ == 2 and nzs.get(sl, 0):
            b = pcg_schur_bytes(int(n_), nzs[sl], int(i_), int(o_), idx.get(sl, 2), res.get(sl, False))
        elif m_ in (2, 3):
            b = pcg_bytes(m_ == 2, int(n_), nz[sl], nzl.get(sl, 0), int(i_), int(o_), idx.get(sl, 4) if m_ == 2 else 4,
                          res.get(sl, False) and m_ == 2, fvb.get(sl), red.get(sl, False) and m_ == 2)
        else:
            b = algorithmic_bytes(1 if m_ == 1 else 0, int(n_), nz[sl], int(i_), int(o_), pipe)
        name = "cg_fp64_pipe_kernel" if pipe else names[m_]
        bytes_by[name] = bytes_by.get(name, 0.0) + b
        ms_by[name] = ms_by.get(name, 0.0) + float(t_)
        rowit_by[name] = rowit_by.get(name, 0.0) + float(n_) * float(i_)
    top = max(ms_by, key=ms_by.get)
    peak, peak_kind = peaks()
    achieved = bytes_by[top] / (ms_by[top] * 1e-3) / 1e9 if ms_by[top] > 0 else 0.0
    launches = int(sum(1 for m_, n_ in zip(prof["mode"], prof["rows"])
                       if ("cg_fp64_pipe_kernel" if int(m_) == 0 and (form == "pipelined" or (
                           form == "auto" and int(n_) < pipe_max)) else names[int(m_)]) == top))
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs", "kernel": top,
            "launches": launches, "kernel_ms_per_step": round(ms_by[top] / args.steps, 3),
            "kernel_share_of_solver_time": round(ms_by[top] / max(sum(ms_by.values()), 1e-9), 3),
            "algorithmic_bytes_per_launch": round(bytes_by[top] / max(launches, 1)),
            "traffic": (round(DRAM_BYTES_PER_ROW_ITERATION[top] * rowit_by[top] / max(launches, 1))
                        if top in DRAM_BYTES_PER_ROW_ITERATION else None),
            "traffic_source": "ncu dram bytes per row-iteration x rows x iterations of each launch"}


def run_gpu(args):
    world, rank, local, pg = dist_setup()
    import navier_stokes_fem_gb300 as nsf

    w = WORKLOADS[args.workload]
    mesh = make_mesh(w)
    t0 = time.perf_counter()
    sim = nsf.NavierStokesAssembly(mesh, w["nu"], w["dt"], device=local, solver=args.solver,
                                   inner_tolerance=args.inner_tol)
    sim.set_cg_form(args.cg_form)
    sim.set_pcg_form(args.pcg_form)
    setup_s = time.perf_counter() - t0
    init = sim.fields()        # the run's initial state: u = 0 with the Dirichlet values imposed, p = 0
    learned = None
    t0 = time.perf_counter()
    if args.precond == "ic0":
        sim.precond_ic0("pressure_stiffness")
    elif args.precond == "learned":
        from navier_stokes_fem_gb300 import learn

        trainer = nsf.GPUSimulationDevice(local)
        learner, learned = learn.train(trainer, seed=args.seed, steps=args.train_steps)
        t1 = time.perf_counter()
        learner.apply("pressure_stiffness", sim)
        learned["apply_s"] = round(time.perf_counter() - t1, 3)
        learner.close()
        trainer.close()
    precond_s = time.perf_counter() - t0
    # every arm times steps 1..K of the run from the initial state, after warm-up steps whose fields are dropped
    arm = time_arm(sim, args, pg, start=init)
    ms, its, clk, launches = arm["ms"], arm["its"], arm["clocks"], arm["launches"]
    roof = roofline(sim, arm, args)
    prof = arm["prof"]
    mixed = (prof["mode"] == 1) | (prof["mode"] == 2)
    mixed_stats = {"mixed_solves": int(mixed.sum()), "finished_in_fp64": int((prof["fallback"] == 1).sum()),
                   "mean_fp64_refreshes": round(float(prof["outer"][mixed].mean()), 2) if mixed.any() else 0}
    start = arm["start_fields"]
    nv = mesh.n_nodes

    # end to end through the C ABI: host fields copied in and out around every step (pinned buffers), over the
    # same steps as the timed region (from the fields it started with)
    uv, p = start
    uv_in, p_in = sim.pinned(uv.shape), sim.pinned(p.shape)
    uv_out, p_out = sim.pinned(uv.shape), sim.pinned(p.shape)
    uv_in[:] = uv
    p_in[:] = p
    e2e_steps = args.steps
    sim.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.step_host(uv_in, p_in, 1, uv_out, p_out)
        uv_in, uv_out = uv_out, uv_in
        p_in, p_out = p_out, p_in
    e2e_ms = max_over_ranks(pg, 1e3 * (time.perf_counter() - t0) / e2e_steps)
    field_bytes = int(uv.nbytes + p.nbytes)
    e2e_same = bool(np.array_equal(uv_in, arm["end_fields"][0]) and np.array_equal(p_in, arm["end_fields"][1]))

    # the classical preconditioner on the same handle, solver and steps: IC(0) in place of the learned factor
    ic0 = None
    if args.precond == "learned" and args.ic0_arm:
        sim.precond_ic0("pressure_stiffness")
        iarm = time_arm(sim, args, pg, start=start)
        ic0 = {"ms_per_step": round(iarm["ms"], 3), "cg_iterations_per_step": iarm["its"].mean(axis=0).round(1).tolist(),
               "learned_speedup_over_ic0": round(iarm["ms"] / ms, 3), "clocks": iarm["clocks"],
               "end_fields": iarm["end_fields"]}
    sim.close()

    # the plain FP64 CG megakernel on the same workload, from the same start fields, over the same steps (the
    # comparison the metric names); its own warm-up steps are not timed
    plain, plain_sim, field_check = None, None, None
    if args.compare and not (args.solver == "fp64" and args.precond == "none"):
        plain_sim = nsf.NavierStokesAssembly(mesh, w["nu"], w["dt"], device=local, solver="fp64")
        plain_sim.set_cg_form(args.cg_form)
        parm = time_arm(plain_sim, args, pg, start=start)
        plain = {"ms_per_step": round(parm["ms"], 3), "cg_iterations_per_step": parm["its"].mean(axis=0).round(1).tolist(),
                 "speedup": round(parm["ms"] / ms, 3), "clocks": parm["clocks"]}
        # both arms ran the same steps from the same fields: how far apart are the fields they ended with
        tol = FIELD_CHECK_TOL
        grad = lambda p: plain_sim.sp_r_mult("pressure_divergence", p)   # noqa: E731
        res = {"learned_pcg_mixed" if args.precond == "learned" else args.solver:
               field_diff(arm["end_fields"], parm["end_fields"], nv, grad)}
        if ic0 is not None:
            res["ic0_pcg_mixed"] = field_diff(ic0["end_fields"], parm["end_fields"], nv, grad)
        ok = all(d["rel_l2_u"] <= tol["u"] and d["rel_l2_v"] <= tol["v"] and d["rel_l2_grad_p"] <= tol["grad_p"]
                 for d in res.values())
        field_check = {"against": "plain FP64 CG, the same steps 1..K from the initial state", "steps": args.steps,
                       "tol": tol, "pass": ok, **res}
    if ic0 is not None:
        ic0.pop("end_fields")

    base, oracle_check = None, None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_oracle_steps(mesh, w, args.cpu_steps)
        k = len(cpu["times_s"])
        base = {"value": round(cpu["ms_per_step"], 3), "unit": "ms/step", "cores": cpu["cores"], "kind": "port",
                "sample": (f"whole FP64 oracle step(s) 1..{k} of the run from its initial state (the GPU arms time "
                           f"steps 1..{args.steps} of the same run); set-up {cpu['setup_s']:.1f} s excluded; "
                           f"iterations {cpu['iterations']}"),
                "status": cpu["status"]}
        # the GPU FP64 path's step 1 from the initial state against the oracle's
        if plain_sim is None:
            plain_sim = nsf.NavierStokesAssembly(mesh, w["nu"], w["dt"], device=local, solver="fp64")
        plain_sim.set_fields(*init)
        git = plain_sim.step(1)[0]
        d = field_diff(plain_sim.fields(), cpu["fields_1"], nv)
        oracle_check = {"against": "FP64 oracle, step 1 from the initial state", "tol": ORACLE_FIELD_TOL, **d,
                        "pass": max(d.values()) <= ORACLE_FIELD_TOL,
                        "gpu_iterations": git.tolist(), "oracle_iterations": cpu["iterations"][0]}
    if plain_sim is not None:
        plain_sim.close()
    if rank != 0:
        return
    solver = args.solver + ("" if args.precond == "none" else f" + {args.precond} preconditioner")
    line = {
        "metric": METRIC, "value": round(ms, 3), "unit": "ms/step", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.solver in ("fp64", "pcg_fp64") else "f32+f64",
        "data": "synthetic (seeded structured mesh; inputs resident in HBM, L2 flushed between steps)",
        "config": config_block(args, w, mesh, solver),
        "cg_iterations_per_step": its.mean(axis=0).round(1).tolist(),
        "cg_solves": ["diffusion u", "diffusion v", "pressure", "mass u", "mass v"],
        "plain_fp64_cg": plain,
        "plain_cg_form": args.cg_form,
        "ic0_pcg_mixed": ic0,
        "field_check": field_check,
        "oracle_check": oracle_check,
        "mixed_precision": mixed_stats if args.solver in ("mixed", "pcg_mixed") else None,
        "learned_preconditioner": learned,
        "setup_s": round(setup_s, 3),
        "preconditioner_setup_s": round(precond_s, 3),
        "roofline": roof,
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms/step", "h2d_bytes_per_step": field_bytes,
                "d2h_bytes_per_step": field_bytes, "steps": e2e_steps, "same_fields_as_timed_steps": e2e_same},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if base is not None:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)


def batched_problems(w):
    from navier_stokes_fem_gb300 import mesh as M

    return [(M.cavity(p["n"], lid_u=repr(p["lid"])), p["nu"], p["dt"])
            for p in M.batched_cavity_params(w["count"], seed=w["seed"], n_lo=w["n_lo"], n_hi=w["n_hi"])]


def run_batched(args):
    """The batched form: every instance advances one step per graph replay of the persistent step kernel."""
    world, rank, local, pg = dist_setup()
    import navier_stokes_fem_gb300 as nsf

    w = WORKLOADS[args.workload]
    probs = batched_problems(w)
    t0 = time.perf_counter()
    b = nsf.BatchedNavierStokes(probs, device=local, solver=args.solver, inner_tolerance=args.inner_tol,
                                autotune_rounds=3)
    setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.flush_l2(256 << 20)
        b.step(1)
    b.synchronize()
    clocks = ClockSampler()
    clocks.start()
    launches0 = b.launch_count()
    barrier(pg)
    b.synchronize()
    b.timer_start()
    its = []
    for _ in range(args.steps):
        b.flush_l2(256 << 20)
        its.append(b.step(1)[0])
    ms_total = b.timer_stop()
    b.synchronize()
    barrier(pg)
    launches = b.launch_count() - launches0
    clk = clocks.stop()
    ms = max_over_ranks(pg, ms_total / args.steps)
    its = np.asarray(its)                       # [steps, count, 5]
    # algorithmic bytes of the CG work per step (FP64 model), over every instance and solve
    nnz = {}
    bytes_step = 0.0
    for i, (m, nu, dt) in enumerate(probs):
        nv, npr = m.n_nodes, m.n_pressure
        # nnz of the diagonal-split cavity patterns: 46n^2+16n+1 (P2) and 7n^2+6n+1 (P1)
        n = int(round(np.sqrt(m.n_elements / 2)))
        nz_v, nz_p = 46 * n * n + 16 * n + 1, 7 * n * n + 6 * n + 1
        for j, (rows, nz) in enumerate(((nv, nz_v), (nv, nz_v), (npr, nz_p), (nv, nz_v), (nv, nz_v))):
            bytes_step += algorithmic_bytes(0, rows, nz, float(its[:, i, j].mean()), 1)
    peak, peak_kind = peaks()
    achieved = bytes_step / (ms * 1e-3) / 1e9
    # end to end through the public API: every instance's fields in and out around each step
    fields = [b.fields(i) for i in range(b.count)]
    field_bytes = int(sum(uv.nbytes + p.nbytes for uv, p in fields))
    e2e_steps = max(1, min(args.steps, 3))
    b.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for i, (uv, p) in enumerate(fields):
            b.set_fields(i, uv, p)
        b.step(1)
        fields = [b.fields(i) for i in range(b.count)]
    e2e_ms = max_over_ranks(pg, 1e3 * (time.perf_counter() - t0) / e2e_steps)
    plan = b.plan()
    base = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle

        oracle.build(ref=False)
        t_cpu = 0.0
        for m, nu, dt in probs:
            o = oracle.Oracle(m, nu, dt)
            tt = time.perf_counter()
            o.step(1)
            t_cpu += time.perf_counter() - tt
            o.close()
        base = {"value": round(1e3 * t_cpu, 3), "unit": "ms/step", "cores": oracle.max_threads(), "kind": "port",
                "sample": f"FP64 oracle, step 1 from the initial state of all {len(probs)} instances"}
    b.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(ms, 3), "unit": "ms/step", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.solver == "fp64" else "f32+f64",
        "data": "synthetic (seeded cavities; inputs resident in HBM, L2 flushed between steps)",
        "config": {"workload": args.workload, "instances": len(probs),
                   "n_range": [int(min(round(np.sqrt(m.n_elements / 2)) for m, _, _ in probs)),
                               int(max(round(np.sqrt(m.n_elements / 2)) for m, _, _ in probs))],
                   "velocity_nodes_total": int(sum(m.n_nodes for m, _, _ in probs)), "tol": 1e-8,
                   "solver": args.solver, "launch": "one persistent step kernel per step, CUDA-graph replay",
                   "parallelism": "replicas" if args.gpus > 1 else "single GPU"},
        "cg_iterations_per_step": its.sum(axis=1).mean(axis=0).round(1).tolist(),
        "cg_solves": ["diffusion u", "diffusion v", "pressure", "mass u", "mass v"],
        "setup_s": round(setup_s, 3),
        "plan": {"grid_blocks": plan["grid_blocks"], "blocks_min": int(plan["blocks"].min()),
                 "blocks_max": int(plan["blocks"].max()), "autotune_trial_ms": [round(x, 3) for x in plan["trial_ms"]]},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                     "kernel": "step_kernel", "algorithmic_bytes_per_launch": round(bytes_step), "traffic": None},
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms/step", "h2d_bytes_per_step": field_bytes,
                "d2h_bytes_per_step": field_bytes, "steps": e2e_steps},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if base is not None:
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)


def run_cg_probe(args):
    """Two pressure-matrix solves with a fixed iteration count, on a handle that holds the pressure system alone
    (the simulation that assembled it is freed first, so a profiler capture sees a few GB of device memory)."""
    import navier_stokes_fem_gb300 as nsf

    w = WORKLOADS[args.workload]
    mesh = make_mesh(w)
    sim = nsf.NavierStokesAssembly(mesh, w["nu"], w["dt"])
    mat = sim.download_matrix("pressure_stiffness")
    sim.close()
    dev = nsf.GPUSimulationDevice(0)
    dev.set_cg_form(args.cg_form)
    dev.set_pcg_form(args.pcg_form)
    if args.inner_tol > 0:   # e.g. 1e-6: the mixed solvers' first inner launch then runs the whole probe budget
        dev.set_solver(args.solver, args.inner_tol)
    dev.upload_matrix("pressure_stiffness", *mat)
    if args.precond == "ic0":
        dev.precond_ic0("pressure_stiffness")
    elif args.precond == "learned":
        from navier_stokes_fem_gb300 import learn

        trainer = nsf.GPUSimulationDevice(0)
        learner, _ = learn.train(trainer, seed=args.seed, steps=args.train_steps)
        learner.apply("pressure_stiffness", dev)
        learner.close()
        trainer.close()
    b = np.random.default_rng(0).standard_normal(mesh.n_pressure)
    for _ in range(2):
        x, it, rr, st = dev.conjugate_gradient("pressure_stiffness", b, np.zeros_like(b), max_iterations=args.cg_probe,
                                               solver=args.solver, raise_on_error=False)
        print(json.dumps({"probe": "pressure CG", "rows": mesh.n_pressure, "iterations": it, "status": st}))
    dev.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--solver", default=None, choices=["fp64", "mixed", "pcg_mixed", "pcg_fp64"],
                    help="default: pcg_mixed with the learned preconditioner (the metric's method)")
    ap.add_argument("--precond", default=None, choices=["none", "ic0", "learned"])
    ap.add_argument("--train-steps", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="skip the plain FP64 CG run on the same workload")
    ap.add_argument("--inner-tol", type=float, default=-1.0)
    ap.add_argument("--cpu-steps", type=int, default=1, help="whole oracle steps timed for cpu_baseline")
    ap.add_argument("--ref-budget-s", type=float, default=150.0,
                    help="--impl reference: time budget of the timed whole CPU steps")
    ap.add_argument("--cg-form", default="auto", choices=["auto", "three_sync", "pipelined"],
                    help="iteration form of the plain FP64 CG (auto: by system size)")
    ap.add_argument("--pcg-form", default="auto", choices=["auto", "full", "reduced", "schur"],
                    help="iteration of the mixed PCG on two-colour systems (nsf_set_pcg_form)")
    ap.add_argument("--no-ic0-arm", dest="ic0_arm", action="store_false",
                    help="skip the IC(0) run beside the learned preconditioner")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cg-probe", type=int, default=0, help="profiling aid: 2 pressure solves of this many iterations")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.solver is None:
        if WORKLOADS[args.workload]["kind"] == "batched":
            args.solver = "mixed"        # (the batched step kernel runs the unpreconditioned solvers)
        else:
            args.solver = "pcg_mixed" if args.precond in (None, "learned") else "fp64"
    if args.precond is None:
        args.precond = "learned" if args.solver in ("pcg_mixed", "pcg_fp64") else "none"
    if args.cg_probe:
        run_cg_probe(args)
    elif args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload]["kind"] == "batched":
        run_batched(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
