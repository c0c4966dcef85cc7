"""Writes the element-matrix fixture from the reference's OWN element code.

`make -C oracle ref-assembly` compiles the reference's shape functions, quadrature, Jacobian and local mass /
stiffness / divergence functors (include/assembly.h:98-304 and 725-882) and the convection functor of
assembleConvectionMatrix (include/assembly.h:1584-1622) from its own lines into
oracle/_ref/libref_assembly.so.  This script evaluates them, in the reference's float arithmetic, on the triangles of
the reference's assets/mesh_small.json, a perturbed 12 x 12 cavity, the 8 x 8 cavity and 256 seeded random
counter-clockwise triangles, and stores vertices and matrices so that the oracle's restatement can be checked where
the reference checkout does not exist.

    NSFEM_REFERENCE_DIR=<reference checkout> python tests/golden/make_assembly_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from navier_stokes_fem_gb300 import mesh as M  # noqa: E402

OUT = os.path.join(HERE, "ref_local_matrices.npz")


def random_triangles(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.uniform(-1.0, 1.0, size=(n, 6)).astype(np.float32)
    cross = (v[:, 2] - v[:, 0]) * (v[:, 5] - v[:, 1]) - (v[:, 3] - v[:, 1]) * (v[:, 4] - v[:, 0])
    v[cross < 0] = v[cross < 0][:, [0, 1, 4, 5, 2, 3]]      # counter-clockwise, as the meshes are
    return v


def main():
    ref_dir = os.environ.get("NSFEM_REFERENCE_DIR", "")
    if not ref_dir:
        raise SystemExit("set NSFEM_REFERENCE_DIR to the reference checkout")
    oracle.build(ref=True)
    from make_golden import perturbed_cavity

    meshes = [M.read_mesh_json(os.path.join(ref_dir, "assets", "mesh_small.json")), perturbed_cavity(), M.cavity(8)]
    verts = [m.nodes[m.elements[:, :3]].reshape(-1, 6) for m in meshes] + [random_triangles(256, 5)]
    v = np.concatenate(verts).astype(np.float32)
    ref = oracle.ref_local_matrices(v)
    out = {"vertices": v, "sources": np.array([len(x) for x in verts])}
    out.update({k: a for k, a in ref.items()})
    # the convection functor of assembleConvectionMatrix, with seeded nodal velocities per triangle
    vel = np.random.default_rng(11).standard_normal((len(v), 12)).astype(np.float32)
    out["velocities"] = vel
    out["convection"] = oracle.ref_local_convection(v, vel)
    np.savez_compressed(OUT, **out)
    print(len(v), "triangles")


if __name__ == "__main__":
    main()
