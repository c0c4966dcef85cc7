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
