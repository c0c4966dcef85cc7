"""Meshes shared by the tests: the generated cavities/channel and the reference's mesh_small (from the fixture)."""
import numpy as np

from navier_stokes_fem_gb300 import mesh as M


def golden_mesh(golden, tag):
    """Rebuild a fixture mesh (nodes, elements, and for mesh_small its Dirichlet groups)."""
    m = M.Mesh(golden[f"{tag}/nodes"], golden[f"{tag}/elements"], int(golden[f"{tag}/n_pressure"][0]), name=tag)
    g = 0
    while f"{tag}/u_dirichlet/{g}/nodes" in golden:
        ue, ve = (str(s) for s in golden[f"{tag}/u_dirichlet/{g}/expr"])
        m.u_dirichlet.append((golden[f"{tag}/u_dirichlet/{g}/nodes"], ue, ve))
        g += 1
    g = 0
    while f"{tag}/p_dirichlet/{g}/nodes" in golden:
        m.p_dirichlet.append((golden[f"{tag}/p_dirichlet/{g}/nodes"], str(golden[f"{tag}/p_dirichlet/{g}/expr"][0])))
        g += 1
    return m


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def departure_points(mesh, still_every: int = 7):
    """Seeded-free, platform-independent back-traced departure points x - dt*u of every velocity node of a
    structured cavity, in float32 exactly as the advection computes them (the float product rounded, then the
    float difference).  u is a lid-driven-cavity-like field: the vortex of the stream function
    (x(1-x) y(1-y))^2 scaled to a peak speed near 1, plus a lid shear y^8; every `still_every`-th node has u = 0 and
    stays on its node (exact vertex and edge-midpoint ties).  dt = 2.5/n moves points up to about 2.5 cells, and
    the lid carries the top-left points out of the domain (the nearest-node fallback).  Only IEEE +, -, * are
    used, so x86 and Arm produce the same bits."""
    n = int(round(np.sqrt(mesh.n_elements / 2)))
    x = mesh.nodes[:, 0].astype(np.float64)
    y = mesh.nodes[:, 1].astype(np.float64)
    a = x * (1.0 - x)
    b = y * (1.0 - y)
    y2 = y * y
    y4 = y2 * y2
    u = 160.0 * a * a * b * (1.0 - 2.0 * y) + y4 * y4
    v = -160.0 * a * b * b * (1.0 - 2.0 * x)
    u[::still_every] = 0.0
    v[::still_every] = 0.0
    dt = np.float32(2.5 / n)
    px = mesh.nodes[:, 0] - u.astype(np.float32) * dt
    py = mesh.nodes[:, 1] - v.astype(np.float32) * dt
    return np.stack([px, py], axis=1).astype(np.float32)


LOOKUP_CHUNKS = 64


def lookup_digests(elem, xi, eta, chunks: int = LOOKUP_CHUNKS):
    """SHA-256 of (element id, xi bits, eta bits) over `chunks` equal slices of the points: equal digests mean
    bit-identical answers, and a mismatch names the slice to look at."""
    import hashlib

    n = len(elem)
    out = []
    for c in range(chunks):
        lo, hi = n * c // chunks, n * (c + 1) // chunks
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(elem[lo:hi], np.int32).tobytes())
        h.update(np.ascontiguousarray(xi[lo:hi], np.float32).view(np.uint32).tobytes())
        h.update(np.ascontiguousarray(eta[lo:hi], np.float32).view(np.uint32).tobytes())
        out.append(h.hexdigest())
    return out


def nearest_ties_ok(mesh, pts, got, want):
    """Nearest-node answers may differ only where both nodes are at exactly the same float distance (the
    reference keeps the first its traversal meets, the GPU and the port the lowest index); returns the number of
    such ties and raises on a difference that is not a tie."""
    diff = np.nonzero(got != want)[0]
    for i in diff:
        p = pts[i].astype(np.float32)
        dg = np.float32(p[0] - mesh.nodes[got[i], 0]) ** 2 + np.float32(p[1] - mesh.nodes[got[i], 1]) ** 2
        dw = np.float32(p[0] - mesh.nodes[want[i], 0]) ** 2 + np.float32(p[1] - mesh.nodes[want[i], 1]) ** 2
        if dg != dw:
            raise AssertionError(f"point {i}: nearest {got[i]} vs {want[i]} is not a tie ({dg} vs {dw})")
    return len(diff)
