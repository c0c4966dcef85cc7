"""Writes the golden point-location fixtures from the reference's OWN KD tree.

The reference's KDTreeBuilder + KDTree<FemGrid2D>::findElement (cpp/kd_tree_builder.cpp,
gpu_cpu_shared/kd_tree.cuh) are compiled unchanged by `make -C oracle ref` into oracle/_ref/libref_kdtree.so.
This script runs them on seeded point sets over three meshes and stores, per point, the containing element,
the float barycentrics (xi, eta) and the nearest-node fallback, so that the oracle port and the GPU path can be
checked against the reference where the reference checkout does not exist.

    NSFEM_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
    (needs the reference sources: oracle/_ref is built from them first)

Meshes: the reference's assets/mesh_small.json (stored here as arrays), the 32x32 lid-driven cavity, and a 12x12
cavity whose interior vertices are randomly perturbed (seed 11) so that no edge is axis-aligned.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from navier_stokes_fem_gb300 import mesh as M  # noqa: E402

REF_DIR = os.environ.get("NSFEM_REFERENCE_DIR", "")
REF_MESH = os.path.join(REF_DIR, "assets", "mesh_small.json")


def perturbed_cavity(n: int = 12, seed: int = 11, amp: float = 0.3) -> M.Mesh:
    m = M.cavity(n)
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    xy = m.nodes.astype(np.float64)
    P = m.n_pressure
    interior = (xy[:P, 0] > 0) & (xy[:P, 0] < 1) & (xy[:P, 1] > 0) & (xy[:P, 1] < 1)
    xy[:P][interior] += rng.uniform(-amp * h, amp * h, size=(int(interior.sum()), 2))
    # midside nodes back on the (straight) edges
    for e in m.elements:
        for k, (a, b) in zip((3, 4, 5), ((1, 2), (0, 2), (0, 1))):
            xy[e[k]] = 0.5 * (xy[e[a]] + xy[e[b]])
    m.nodes = xy.astype(np.float32)
    m.name = f"perturbed{n}"
    return m


def point_set(m: M.Mesh, seed: int, n_random: int = 4000) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lo = m.nodes.min(0) - 0.03
    hi = m.nodes.max(0) + 0.03
    pts = [rng.uniform(size=(n_random, 2)) * (hi - lo) + lo]
    pts.append(m.nodes[rng.choice(m.n_nodes, size=min(1500, m.n_nodes), replace=False)])   # on nodes/edges
    sel = rng.choice(m.n_nodes, size=min(1500, m.n_nodes), replace=False)
    pts.append(m.nodes[sel] + rng.normal(scale=1e-6, size=(len(sel), 2)))                   # next to them
    # back-traced departure points of a swirling field with a big step (many land outside the mesh)
    c = m.nodes.mean(0)
    d = m.nodes - c
    vel = np.stack([-d[:, 1], d[:, 0]], 1) * 3.0 + 0.5
    pts.append((m.nodes - vel.astype(np.float32) * np.float32(0.05)))
    return np.concatenate(pts).astype(np.float32)


def main():
    if not REF_DIR:
        raise SystemExit("set NSFEM_REFERENCE_DIR to the reference checkout")
    oracle.build(ref=True)
    meshes = [M.read_mesh_json(REF_MESH), M.cavity(32), perturbed_cavity()]
    out = {}
    for k, m in enumerate(meshes):
        pts = point_set(m, seed=100 + k)
        tree = oracle.ReferenceTree(m)
        e, xi, eta, nn = tree.locate(pts)
        tag = m.name
        out[f"{tag}/nodes"] = m.nodes
        out[f"{tag}/elements"] = m.elements
        out[f"{tag}/n_pressure"] = np.array([m.n_pressure])
        out[f"{tag}/points"] = pts
        out[f"{tag}/elem"] = e
        out[f"{tag}/xi"] = xi
        out[f"{tag}/eta"] = eta
        out[f"{tag}/nearest"] = nn
        out[f"{tag}/bbox"] = tree.bbox()
        if tag == "mesh_small":
            for g, (nodes, ue, ve) in enumerate(m.u_dirichlet):
                out[f"{tag}/u_dirichlet/{g}/nodes"] = nodes
                out[f"{tag}/u_dirichlet/{g}/expr"] = np.array([ue, ve])
            for g, (nodes, pe) in enumerate(m.p_dirichlet):
                out[f"{tag}/p_dirichlet/{g}/nodes"] = nodes
                out[f"{tag}/p_dirichlet/{g}/expr"] = np.array([pe])
        print(tag, len(pts), "points,", int((e < 0).sum()), "outside")
    np.savez_compressed(os.path.join(HERE, "ref_kdtree_lookup.npz"), **out)


if __name__ == "__main__":
    main()
