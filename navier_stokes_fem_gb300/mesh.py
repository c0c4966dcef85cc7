"""Seeded, deterministic P2-P1 triangle meshes in the reference's mesh/scene JSON format.

The reference reads meshes with ``FemGrid2D::loadJSON`` (cpp/grid.cpp:9-78): keys ``elements``
(6 node indices per triangle), ``nodes`` ([x, y] pairs, read as float), ``elementsCount``,
``velocityNodesCount``, ``pressureNodesCount``, ``elementSize`` (6), ``uDirichlet`` (list of
``{"nodes", "u", "v"}``) and ``pDirichlet`` (list of ``{"nodes", "p"}``).  Conventions this module
keeps, all checked on the reference's own ``assets/mesh_small.json``:

* pressure (P1) nodes are the triangle vertices and are numbered first, ``0 .. P-1``; the P2
  midside nodes follow, so pressure node ``i`` is velocity node ``i`` (include/assembly.h:577-581
  reads pressure node coordinates from the velocity node buffer);
* an element is ``[v0, v1, v2, m12, m02, m01]`` with the vertices counter-clockwise
  (the P2 shape-function order of include/assembly.h:210-224; ``isPointInTriagle`` assumes CCW,
  gpu_cpu_shared/kd_tree_common.cuh:38-47);
* every boundary node belongs to exactly one velocity Dirichlet group (a node listed twice has its
  lift subtracted twice, include/assembly.h:505-523), and an enclosed cavity pins one pressure node.

Structured grids are split along each cell's SW-NE diagonal.  Within the fine (2nx+1) x (2ny+1)
lattice of P2 positions, vertices are numbered row-major (y outer, x inner) and midside nodes
likewise, which keeps CSR bands narrow for the SpMV x-gather.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Mesh", "structured_mesh", "cavity", "channel_with_obstacle", "batched_cavity_params",
    "write_mesh_json", "read_mesh_json", "write_scene_json", "read_scene_json",
]


@dataclass
class Mesh:
    """A P2-P1 mesh plus its Dirichlet groups, in the reference's index conventions."""

    nodes: np.ndarray            # float32 [Nv, 2]
    elements: np.ndarray         # int32 [T, 6]
    n_pressure: int              # P: the first P nodes are the P1 vertices
    u_dirichlet: list = field(default_factory=list)   # [(int32 nodes, u_expr, v_expr)]
    p_dirichlet: list = field(default_factory=list)   # [(int32 nodes, p_expr)]
    name: str = "mesh"

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])


def structured_mesh(nx: int, ny: int, lx: float, ly: float, keep: np.ndarray | None = None):
    """Diagonally split nx x ny grid on [0,lx] x [0,ly]; ``keep[j, i]`` False removes cell (i, j).

    Returns (nodes float32 [Nv,2], elements int32 [T,6], P, fine_id int64 [(2ny+1),(2nx+1)] giving the
    node index of each lattice point or -1, boundary bool [(2ny+1),(2nx+1)]).
    """
    if keep is None:
        keep = np.ones((ny, nx), dtype=bool)
    keep = np.asarray(keep, dtype=bool)
    FX, FY = 2 * nx + 1, 2 * ny + 1
    exists = np.zeros((FY, FX), dtype=bool)
    cj, ci = np.nonzero(keep)
    for dj in range(3):
        for di in range(3):
            exists[2 * cj + dj, 2 * ci + di] = True
    J, I = np.nonzero(exists)            # row-major order (J outer, I inner)
    is_vertex = (J % 2 == 0) & (I % 2 == 0)
    fine_id = np.full((FY, FX), -1, dtype=np.int64)
    nv = int(is_vertex.sum())
    fine_id[J[is_vertex], I[is_vertex]] = np.arange(nv)
    fine_id[J[~is_vertex], I[~is_vertex]] = nv + np.arange(int((~is_vertex).sum()))
    order = np.argsort(fine_id[J, I])
    xs = (I[order].astype(np.float64) / (2 * nx)) * lx
    ys = (J[order].astype(np.float64) / (2 * ny)) * ly
    nodes = np.stack([xs, ys], axis=1).astype(np.float32)

    # two triangles per kept cell, cell-major (row j outer, column i inner)
    a, b = 2 * cj, 2 * ci   # lattice row / column of the SW corner
    sw, se = fine_id[a, b], fine_id[a, b + 2]
    ne, nw = fine_id[a + 2, b + 2], fine_id[a + 2, b]
    low = np.stack([sw, se, ne, fine_id[a + 1, b + 2], fine_id[a + 1, b + 1], fine_id[a, b + 1]], axis=1)
    up = np.stack([sw, ne, nw, fine_id[a + 2, b + 1], fine_id[a + 1, b], fine_id[a + 1, b + 1]], axis=1)
    elements = np.empty((2 * len(cj), 6), dtype=np.int32)
    elements[0::2] = low
    elements[1::2] = up

    # boundary lattice points: the three points along every cell side that faces a removed/outside cell
    padded = np.zeros((ny + 2, nx + 2), dtype=bool)
    padded[1:-1, 1:-1] = keep
    boundary = np.zeros((FY, FX), dtype=bool)
    for (dj, di, side) in ((-1, 0, "S"), (1, 0, "N"), (0, -1, "W"), (0, 1, "E")):
        facing = keep & ~padded[1 + dj:1 + dj + ny, 1 + di:1 + di + nx]
        fj, fi = np.nonzero(facing)
        for t in range(3):
            if side == "S":
                boundary[2 * fj, 2 * fi + t] = True
            elif side == "N":
                boundary[2 * fj + 2, 2 * fi + t] = True
            elif side == "W":
                boundary[2 * fj + t, 2 * fi] = True
            else:
                boundary[2 * fj + t, 2 * fi + 2] = True
    return nodes, elements, nv, fine_id, boundary


def _ids(fine_id: np.ndarray, mask: np.ndarray) -> np.ndarray:
    ids = fine_id[mask]
    ids = ids[ids >= 0]
    return np.sort(ids).astype(np.int32)


def cavity(n: int, lid_u: str = "1") -> Mesh:
    """Lid-driven cavity on the unit square: n x n cells, 2n^2 triangles.

    Lid (y=1, corners excluded) has u=(lid_u, 0); the other walls, corners included, have u=0.
    Pressure node 0 (the vertex at (0,0)) is pinned to p=0 so the pressure matrix is regular.
    """
    nodes, elements, P, fine_id, boundary = structured_mesh(n, n, 1.0, 1.0)
    FY, FX = fine_id.shape
    jj, ii = np.meshgrid(np.arange(FY), np.arange(FX), indexing="ij")
    lid = boundary & (jj == FY - 1) & (ii > 0) & (ii < FX - 1)
    walls = boundary & ~lid
    return Mesh(nodes, elements, P,
                u_dirichlet=[(_ids(fine_id, lid), str(lid_u), "0"), (_ids(fine_id, walls), "0", "0")],
                p_dirichlet=[(np.array([0], dtype=np.int32), "0")],
                name=f"cavity{n}")


def channel_with_obstacle(nx: int = 1024, ny: int = 256, lx: float = 4.0, ly: float = 1.0,
                          hole=(0.9, 1.1, 0.4, 0.6)) -> Mesh:
    """Channel [0,lx] x [0,ly] with the cells lying inside ``hole`` = (x0, x1, y0, y1) removed.

    Inflow u = (4y(1-y), 0) at x=0 (corners excluded), no-slip on y=0, y=ly and the obstacle,
    do-nothing outflow at x=lx with p=0 on its pressure (vertex) nodes.
    """
    hx, hy = lx / nx, ly / ny
    i = np.arange(nx)
    j = np.arange(ny)
    in_x = (i * hx >= hole[0] - 1e-12) & ((i + 1) * hx <= hole[1] + 1e-12)
    in_y = (j * hy >= hole[2] - 1e-12) & ((j + 1) * hy <= hole[3] + 1e-12)
    keep = ~(in_y[:, None] & in_x[None, :])
    nodes, elements, P, fine_id, boundary = structured_mesh(nx, ny, lx, ly, keep)
    FY, FX = fine_id.shape
    jj, ii = np.meshgrid(np.arange(FY), np.arange(FX), indexing="ij")
    inflow = boundary & (ii == 0) & (jj > 0) & (jj < FY - 1)
    outflow_open = boundary & (ii == FX - 1) & (jj > 0) & (jj < FY - 1)
    walls = boundary & ~inflow & ~outflow_open
    out_vertices = (ii == FX - 1) & (jj % 2 == 0)
    return Mesh(nodes, elements, P,
                u_dirichlet=[(_ids(fine_id, inflow), "4*y*(1-y)", "0"), (_ids(fine_id, walls), "0", "0")],
                p_dirichlet=[(_ids(fine_id, out_vertices), "0")],
                name=f"channel{nx}x{ny}")


def batched_cavity_params(count: int = 64, seed: int = 20261203, n_lo: int = 16, n_hi: int = 256):
    """Per-instance (n, nu, lid speed, dt) for the batched cavity workload.

    n uniform over integers in [n_lo, n_hi], nu log-uniform in [1e-3, 1e-1], lid speed uniform in
    [0.5, 2], dt = 0.25 * h / lid speed.  numpy's PCG64 stands in for the seeded generator.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = rng.integers(n_lo, n_hi + 1, size=count)
    nus = np.exp(rng.uniform(math.log(1e-3), math.log(1e-1), size=count))
    lids = rng.uniform(0.5, 2.0, size=count)
    dts = 0.25 * (1.0 / ns) / lids
    return [dict(n=int(n), nu=float(nu), lid=float(l), dt=float(dt)) for n, nu, l, dt in zip(ns, nus, lids, dts)]


def _fmt_float(v: float) -> str:
    r = repr(float(v))
    return r[:-2] if r.endswith(".0") else r


def write_mesh_json(mesh: Mesh, path: str) -> None:
    """Write ``mesh`` in the reference's mesh JSON layout (cpp/grid.cpp:19-77 reads it)."""
    parts = ['{\n"elements":[']
    parts.append(",".join("[" + ",".join(str(int(v)) for v in e) + "]" for e in mesh.elements))
    parts.append('],\n"nodes":[')
    parts.append(",".join("[" + _fmt_float(x) + "," + _fmt_float(y) + "]" for x, y in mesh.nodes.astype(np.float64)))
    parts.append('],\n"elementsCount":%d,\n"velocityNodesCount":%d,\n"pressureNodesCount":%d,\n"elementSize":6,\n'
                 % (mesh.n_elements, mesh.n_nodes, mesh.n_pressure))
    ud = [{"nodes": [int(v) for v in g[0]], "u": g[1], "v": g[2]} for g in mesh.u_dirichlet]
    pd = [{"nodes": [int(v) for v in g[0]], "p": g[1]} for g in mesh.p_dirichlet]
    parts.append('"uDirichlet":' + json.dumps(ud) + ',\n"pDirichlet":' + json.dumps(pd) + "\n}\n")
    with open(path, "w") as f:
        f.write("".join(parts))


def read_mesh_json(path: str) -> Mesh:
    with open(path) as f:
        d = json.load(f)
    nodes = np.asarray(d["nodes"], dtype=np.float32).reshape(-1, 2)
    elements = np.asarray(d["elements"], dtype=np.int32).reshape(-1, int(d["elementSize"]))
    if nodes.shape[0] != int(d["velocityNodesCount"]) or elements.shape[0] != int(d["elementsCount"]):
        raise ValueError(f"{path}: node/element counts disagree with the declared counts")
    ud = [(np.asarray(g["nodes"], dtype=np.int32), str(g["u"]), str(g["v"])) for g in d.get("uDirichlet", [])]
    pd = [(np.asarray(g["nodes"], dtype=np.int32), str(g["p"])) for g in d.get("pDirichlet", [])]
    return Mesh(nodes, elements, int(d["pressureNodesCount"]), ud, pd,
                name=os.path.splitext(os.path.basename(path))[0])


def write_scene_json(path: str, mesh_path: str, total_time: float, viscosity: float, dt: float,
                     steps: int | None = None, **extra) -> None:
    """Scene file as read by NavierStokesAssembly::init (include/assembly.h:885-935).

    ``steps`` is an optional extension: when present it is the exact number of time steps; when
    absent the reference rule applies (int(total_time/dt) - 1 steps, include/assembly.h:1480,1516).
    """
    scene = {"mesh_path": mesh_path, "total_time": total_time, "viscosity": viscosity, "dt": dt}
    if steps is not None:
        scene["steps"] = int(steps)
    scene.update(extra)
    with open(path, "w") as f:
        json.dump(scene, f, indent=4)


def read_scene_json(path: str) -> dict:
    with open(path) as f:
        scene = json.load(f)
    for key in ("mesh_path", "dt", "viscosity", "total_time"):
        if key not in scene:
            raise ValueError(f"{path}: missing required param: {key}")
    mp = scene["mesh_path"]
    if not os.path.isabs(mp):
        scene["mesh_path"] = os.path.normpath(os.path.join(os.path.dirname(os.path.abspath(path)), mp))
    return scene
