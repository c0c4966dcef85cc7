"""Training and evaluation of the learned preconditioner (the network of csrc/nsf_learn.cu, driven through the C ABI).

The training systems are the matrices the plain method assembles for lid-driven cavities of several sizes and
viscosities (the pressure stiffness, and optionally the diffusion matrix M + dt nu K), each paired with random
probe vectors z and b = A z.  The loss ||L^ L^T z^ - b^||^2 / ||b^||^2 over probes fits M = L L^T to A on every
mode; pairs made of the plain method's smooth solutions alone fit M on the smooth modes only and did not
precondition at all (a held-out 24 x 24 cavity needed more iterations than plain CG with such a factor, and 70 with
the probe-trained one against 65 for incomplete Cholesky and 147 for Jacobi).

    python -m navier_stokes_fem_gb300.learn --steps 1000 --eval-n 512      (prints one JSON line)
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


def evaluate(device: GPUSimulationDevice, learner: Learner, n: int, seeds=(1001, 1002, 1003), steps: int = 2,
             tol: float = 1e-8):
    """Pressure solves of held-out cavities of size n (right-hand sides from steps of the plain method): CG
    iterations of plain CG, incomplete-Cholesky PCG and learned PCG, FP64, to the same relative residual."""
    rows = []
    for s in seeds:
        c = training_cavities(1, s, n, n)[0]
        sim = NavierStokesAssembly(M.cavity(n, lid_u=repr(c["lid"])), c["nu"], c["dt"])
        sim.step(steps)
        _, p = sim.fields()
        mat = sim.download_matrix("pressure_stiffness")
        sim.close()
        device.upload_matrix("pressure_stiffness", *mat)
        A = device.scipy_matrix("pressure_stiffness")
        b = A @ p
        x0 = np.zeros_like(b)
        row = {"seed": s}
        _, row["plain"], _ = device.conjugate_gradient("pressure_stiffness", b, x0, eps=tol, solver="fp64")
        device.precond_ic0("pressure_stiffness")
        _, row["ic0"], _ = device.conjugate_gradient("pressure_stiffness", b, x0, eps=tol, solver="pcg_fp64")
        learner.apply("pressure_stiffness", device)
        x, row["learned"], _ = device.conjugate_gradient("pressure_stiffness", b, x0, eps=tol, solver="pcg_fp64")
        row["learned_relres"] = float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))
        rows.append(row)
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cavities", type=int, default=6)
    ap.add_argument("--probes", type=int, default=4)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--batch", type=int, default=2)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--eval-n", type=int, default=512)
    ap.add_argument("--eval-seeds", type=int, default=3)
    args = ap.parse_args()
    d = GPUSimulationDevice(0)
    learner, stats = train(d, args.seed, args.cavities, args.probes, args.steps, args.batch, args.lr)
    rows = evaluate(d, learner, args.eval_n, seeds=tuple(1000 + k for k in range(args.eval_seeds)))
    mean = {k: float(np.mean([r[k] for r in rows])) for k in ("plain", "ic0", "learned")}
    print(json.dumps({"train": stats, "eval_n": args.eval_n, "eval": rows, "mean_iterations": mean}))
    learner.close()
    d.close()


if __name__ == "__main__":
    main()
