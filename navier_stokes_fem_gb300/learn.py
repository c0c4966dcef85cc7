"""Training and evaluation of the learned preconditioner (the network of csrc/nsf_learn.cu, driven through the C ABI).

The training systems are the matrices the plain method assembles for lid-driven cavities of several sizes and
viscosities (the pressure stiffness, and optionally the diffusion matrix M + dt nu K), each paired with random
probe vectors z and b = A z.  The loss ||L^ L^T z^ - b^||^2 / ||b^||^2 over probes fits M = L L^T to A on every
mode; pairs made of the plain method's smooth solutions alone fit M on the smooth modes only and did not
precondition at all (a held-out 24 x 24 cavity needed more iterations than plain CG with such a factor, and 70 with
the probe-trained one against 65 for incomplete Cholesky and 147 for Jacobi).

    python -m navier_stokes_fem_gb300.learn --steps 1000 --eval-n 512      (prints one JSON line)

The configured study - 4000 training systems (pressure and diffusion matrices of cavities with n uniform in
[64, 256] and viscosity log-uniform in [1e-3, 1e-1]), 20 000 Adam steps at lr 1e-3, evaluation on 200 held-out
cavities at n = 512 - is

    python -m navier_stokes_fem_gb300.learn --cavities 250 --probes 8 --slots pressure_stiffness,diffusion \
        --n-lo 64 --n-hi 256 --steps 20000 --lr 1e-3 --eval-n 512 --eval-seeds 200
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import GPUSimulationDevice, Learner, NavierStokesAssembly
from . import mesh as M


def training_cavities(count: int, seed: int, n_lo: int = 64, n_hi: int = 160):
    """Seeded cavity parameters: grid size uniform in [n_lo, n_hi], viscosity log-uniform in [1e-3, 1e-1],
    lid speed uniform in [0.5, 2], dt = 0.25 h / lid speed."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_lo, n_hi + 1))
        nu = float(10 ** rng.uniform(-3, -1))
        lid = float(rng.uniform(0.5, 2.0))
        out.append({"n": n, "nu": nu, "lid": lid, "dt": 0.25 / n / lid})
    return out


def collect_systems(learner: Learner, device: GPUSimulationDevice, cavities, probes: int = 4, seed: int = 0,
                    slots=("pressure_stiffness",)):
    """Adds `probes` random-probe pairs per cavity and slot; the matrices are assembled by the plain method."""
    rng = np.random.default_rng(seed + 7919)
    count = 0
    for c in cavities:
        sim = NavierStokesAssembly(M.cavity(c["n"], lid_u=repr(c["lid"])), c["nu"], c["dt"])
        mats = {s: sim.download_matrix(s) for s in slots}
        sim.close()
        for s in slots:
            rp, col, val, shape = mats[s]
            device.upload_matrix(s, rp, col, val, shape)
            A = device.scipy_matrix(s)
            for _ in range(probes):
                z = rng.standard_normal(shape[0])
                learner.add_system(s, z, A @ z)
                count += 1
    return count


def train(device: GPUSimulationDevice, seed: int = 0, cavities: int = 6, probes: int = 4, steps: int = 1000,
          batch: int = 2, lr: float = 3e-3, n_lo: int = 64, n_hi: int = 160, slots=("pressure_stiffness",)):
    """A learner trained on the GPU; returns (learner, stats)."""
    t0 = time.perf_counter()
    learner = Learner(device, seed=seed)
    systems = collect_systems(learner, device, training_cavities(cavities, seed, n_lo, n_hi), probes, seed, slots)
    t1 = time.perf_counter()
    losses = learner.train(steps, batch=batch, lr=lr, seed=seed)
    device.synchronize()
    t2 = time.perf_counter()
    k = max(1, steps // 20)
    stats = {"systems": systems, "steps": steps, "batch": batch, "lr": lr, "params": learner.param_count,
             "loss_first": float(losses[:k].mean()), "loss_last": float(losses[-k:].mean()),
             "collect_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2)}
    return learner, stats


def _timed_solve(device, slot, b, x0, tol, solver):
    """One solve with its CUDA-event time (the persistent solver launches only)."""
    device.profile(True)
    x, it, _ = device.conjugate_gradient(slot, b, x0, eps=tol, solver=solver)
    ms = float(device.profile_read()["ms"].sum())
    device.profile(False)
    return x, int(it), ms


def evaluate(device: GPUSimulationDevice, learner: Learner, n: int, seeds=(1001, 1002, 1003), steps: int = 2,
             tol: float = 1e-8, slots=("pressure_stiffness",), solver: str = "pcg_fp64"):
    """Solves of held-out cavities of size n, right-hand sides b = A u from the fields after `steps` steps of the
    plain method (u: the pressure for the pressure system, the x velocity for the diffusion system), from a zero
    initial guess: iterations and solve time of plain CG, incomplete-Cholesky PCG and learned PCG to the same
    relative residual (`solver`: the preconditioned solver's precision; plain CG matches it)."""
    plain = "fp64" if solver == "pcg_fp64" else "mixed"
    rows = []
    for s in seeds:
        c = training_cavities(1, s, n, n)[0]
        sim = NavierStokesAssembly(M.cavity(n, lid_u=repr(c["lid"])), c["nu"], c["dt"])
        sim.step(steps)
        uv, p = sim.fields()
        mats = {slot: sim.download_matrix(slot) for slot in slots}
        sim.close()
        for slot in slots:
            device.upload_matrix(slot, *mats[slot])
            A = device.scipy_matrix(slot)
            u = p if slot == "pressure_stiffness" else uv[:A.shape[0]]
            b = A @ u
            x0 = np.zeros_like(b)
            row = {"seed": s, "slot": slot}
            _, row["plain"], row["plain_ms"] = _timed_solve(device, slot, b, x0, tol, plain)
            device.precond_ic0(slot)
            _, row["ic0"], row["ic0_ms"] = _timed_solve(device, slot, b, x0, tol, solver)
            learner.apply(slot, device)
            x, row["learned"], row["learned_ms"] = _timed_solve(device, slot, b, x0, tol, solver)
            row["learned_relres"] = float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))
            device.precond_clear(slot)
            rows.append(row)
    return rows


def summarise(rows):
    """Per slot: mean iterations and ms of each method, learned over IC(0) and over plain, and the worst residual."""
    out = {}
    for slot in sorted({r["slot"] for r in rows}):
        rs = [r for r in rows if r["slot"] == slot]
        m = {k: float(np.mean([r[k] for r in rs])) for k in ("plain", "ic0", "learned", "plain_ms", "ic0_ms",
                                                                 "learned_ms")}
        m["systems"] = len(rs)
        m["learned_fewer_iterations_than_ic0"] = int(sum(r["learned"] < r["ic0"] for r in rs))
        m["learned_fewer_iterations_than_plain"] = int(sum(r["learned"] < r["plain"] for r in rs))
        m["learned_over_ic0_iterations"] = m["learned"] / m["ic0"]
        m["learned_over_plain_ms"] = m["learned_ms"] / m["plain_ms"]
        m["worst_learned_relres"] = float(max(r["learned_relres"] for r in rs))
        out[slot] = m
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cavities", type=int, default=6)
    ap.add_argument("--probes", type=int, default=4)
    ap.add_argument("--slots", default="pressure_stiffness", help="comma-separated: pressure_stiffness,diffusion")
    ap.add_argument("--n-lo", type=int, default=64)
    ap.add_argument("--n-hi", type=int, default=160)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--batch", type=int, default=2)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--eval-n", type=int, default=512)
    ap.add_argument("--eval-seeds", type=int, default=3)
    ap.add_argument("--eval-solver", default="pcg_fp64", choices=["pcg_fp64", "pcg_mixed"])
    ap.add_argument("--rows", action="store_true", help="also print every evaluated system")
    args = ap.parse_args()
    slots = tuple(s for s in args.slots.split(",") if s)
    d = GPUSimulationDevice(0)
    learner, stats = train(d, args.seed, args.cavities, args.probes, args.steps, args.batch, args.lr, args.n_lo,
                           args.n_hi, slots)
    t0 = time.perf_counter()
    rows = evaluate(d, learner, args.eval_n, seeds=tuple(1000 + k for k in range(args.eval_seeds)), slots=slots,
                    solver=args.eval_solver)
    out = {"train": stats, "training_slots": list(slots), "n_range": [args.n_lo, args.n_hi], "eval_n": args.eval_n,
           "eval_seeds": args.eval_seeds, "eval_solver": args.eval_solver, "eval_s": round(time.perf_counter() - t0, 1),
           "summary": summarise(rows)}
    if args.rows:
        out["eval"] = rows
    print(json.dumps(out))
    learner.close()
    d.close()


if __name__ == "__main__":
    main()
