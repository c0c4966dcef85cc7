"""Writes the large-mesh point-location fixture from the reference's OWN KD tree.

For the 256 x 256, 1024 x 1024 and 2048 x 2048 lid-driven cavities (0.26 M, 4.2 M and 16.8 M velocity nodes), the
departure points of every velocity node under the cavity-like field of tests/_meshes.departure_points are located
by three trees:

* the reference's KDTreeBuilder + KDTree<FemGrid2D>::findElement with its leaf offsets read as integers
  (`make -C oracle ref-int`: KDNode::getTriangleOffset's return type changed from float to unsigned int,
  gpu_cpu_shared/kd_tree_common.cuh:91,148-150, nothing else) - the answers the fixture stores;
* the same reference build unchanged (`make -C oracle ref`), whose float offsets are exact only below 2^24 leaf
  entries: the number of points it answers differently is recorded;
* the oracle's restatement of the tree (oracle.PortTree), which must match the int-offset reference bit for bit.

The fixture keeps, per mesh, SHA-256 digests of (element, xi, eta) over 64 slices of the points, every outside
point's nearest-node answer, a seeded sample of 4096 explicit answers, and the counts above, so that the GPU test can
check every point without the reference being present.

    NSFEM_REFERENCE_DIR=<reference checkout> python tests/golden/make_lookup_golden.py [n ...]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from navier_stokes_fem_gb300 import mesh as M  # noqa: E402
from tests._meshes import departure_points, lookup_digests, nearest_ties_ok  # noqa: E402

OUT = os.path.join(HERE, "ref_kdtree_lookup_large.npz")
SIZES = (256, 1024, 2048)
SAMPLE = 4096


def _same(a, b):
    e0, x0, y0, _ = a
    e1, x1, y1, _ = b
    return (e0 == e1) & (x0.view(np.uint32) == x1.view(np.uint32)) & (y0.view(np.uint32) == y1.view(np.uint32))


def one_mesh(n: int) -> dict:
    t0 = time.perf_counter()
    m = M.cavity(n)
    pts = departure_points(m)
    ref = oracle.ReferenceTree(m, int_offsets=True)
    t1 = time.perf_counter()
    want = ref.locate(pts)
    ref.close()
    t2 = time.perf_counter()
    port = oracle.PortTree(m)
    got = port.locate(pts)
    stats = port.stats()
    port.close()
    same = _same(got, want)
    if not same.all():
        raise SystemExit(f"n={n}: the oracle port differs from the int-offset reference at {int((~same).sum())} points")
    outside = np.nonzero(want[0] < 0)[0]
    ties_port = nearest_ties_ok(m, pts[outside], got[3][outside], want[3][outside])
    flt = oracle.ReferenceTree(m, int_offsets=False)
    fl = flt.locate(pts)
    flt.close()
    fsame = _same(fl, want)
    f_out = (fl[0] < 0) & (want[0] < 0)
    rng = np.random.default_rng(n)
    sample = np.sort(rng.choice(len(pts), size=min(SAMPLE, len(pts)), replace=False)).astype(np.int64)
    rec = {
        "n": n, "points": int(len(pts)), "outside": int(len(outside)),
        "leaf_entries": stats["leaf_entries"], "tree_nodes": stats["nodes"], "max_depth": stats["max_depth"],
        "float_offset_differences": int((~fsame).sum()),
        "float_offset_nearest_differences": int((fl[3][f_out] != want[3][f_out]).sum()),
        "port_nearest_ties": int(ties_port),
        "reference_build_and_locate_s": round(t2 - t0, 1),
    }
    arrays = {
        f"n{n}/digests": np.array(lookup_digests(*want[:3])),
        f"n{n}/outside": outside.astype(np.int64),
        f"n{n}/outside_nearest": want[3][outside],
        f"n{n}/sample": sample,
        f"n{n}/sample_elem": want[0][sample],
        f"n{n}/sample_xi": want[1][sample],
        f"n{n}/sample_eta": want[2][sample],
        f"n{n}/record": np.array([json.dumps(rec)]),
    }
    print(json.dumps(rec), flush=True)
    return arrays


def main():
    if not os.environ.get("NSFEM_REFERENCE_DIR"):
        raise SystemExit("set NSFEM_REFERENCE_DIR to the reference checkout")
    oracle.build(ref=True)
    sizes = [int(a) for a in sys.argv[1:]] or list(SIZES)
    out = dict(np.load(OUT)) if os.path.exists(OUT) else {}
    for n in sizes:
        out.update(one_mesh(n))
    np.savez_compressed(OUT, **out)


if __name__ == "__main__":
    main()
