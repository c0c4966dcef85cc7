"""ORACLE — test infrastructure, never part of the product.

CPU checker for the GB300 hot path.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg may import this package, and only as the thing results are compared against (or, for
the baseline, the thing timed beside the GPU).  Contents:

* ``liboracle.so`` (built from ``nsfem_oracle.cpp`` by ``make``): the C++ restatement of the reference's
  semi-Lagrangian path - assembly, Dirichlet elimination, CG, the reference's KD tree and advection, and
  the operator-split step - templated on the scalar type (FP64 oracle / the reference's FP32 arithmetic).
* ``_ref/libref_kdtree.so`` (built by ``make ref`` from the reference's own sources, only where the
  reference checkout exists): the reference's KDTreeBuilder + KDTree::findElement, used to pin the port.
* ``evaluate_expression``: a restatement of the reference's boundary-condition expression language
  (cpp/expression.cpp: ``+ - * / ^``, unary minus, ``sin``/``cos``, variables x y z t, constants E, Pi;
  precedence +,- < *,/ < unary minus < ^ (left associative) < function call).

Parity status: the element lookup is pinned against the reference's compiled tree.  The CG stopping
rule cannot be pinned (the reference's CPU CG is in the absent sparse_matrix_math submodule); it is
restated from the thesis algorithm (tex/Chapters/01_chapter_FEM.tex:644-661) with a relative residual.
"""
from __future__ import annotations

import ctypes
import math
import os
import re
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

SLOTS = {
    "pressure_stiffness": 0, "velocity_mass": 1, "diffusion": 2, "velocity_divergence": 3,
    "pressure_divergence": 4, "velocity_dirichlet_weights": 5, "pressure_dirichlet_weights": 6,
}

_p = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_fptr = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_dptr = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_iptr = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_lptr = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compile liboracle.so, and the reference tree when NSFEM_REFERENCE_DIR names a reference checkout."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    ref_dir = os.environ.get("NSFEM_REFERENCE_DIR", "")
    if ref is None:
        ref = bool(ref_dir) and os.path.isdir(os.path.join(ref_dir, "cpp"))
    if ref:
        if not ref_dir:
            raise RuntimeError("set NSFEM_REFERENCE_DIR to the reference checkout to build the reference tree")
        subprocess.run(["make", "-s", "-C", _HERE, "ref", "ref-int", "ref-assembly", f"REF={ref_dir}"], check=True)
        with open(os.path.join(_HERE, "_ref", "REFERENCE_DIR"), "w") as f:
            f.write(os.path.abspath(ref_dir))


def reference_dir() -> str | None:
    """The reference checkout: NSFEM_REFERENCE_DIR, else the one the reference builds in _ref/ were made from; None
    where neither exists (as on a machine without the checkout)."""
    cands = [os.environ.get("NSFEM_REFERENCE_DIR", "")]
    rec = os.path.join(_HERE, "_ref", "REFERENCE_DIR")
    if os.path.exists(rec):
        with open(rec) as f:
            cands.append(f.read().strip())
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    return None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref=False)
        L = ctypes.CDLL(path)
        L.orc_create.restype = _p
        L.orc_create.argtypes = [_i, _fptr, _i, _iptr, _i, _i, _iptr, _dptr, _dptr, _i, _iptr, _dptr, _d, _d, _i]
        L.orc_destroy.argtypes = [_p]
        L.orc_set_threads.argtypes = [_i]
        L.orc_max_threads.restype = _i
        L.orc_matrix_shape.argtypes = [_p, _i, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_int64)]
        L.orc_matrix_get.argtypes = [_p, _i, _lptr, _iptr, _dptr]
        L.orc_spmv.argtypes = [_p, _i, _dptr, _dptr]
        L.orc_cg.restype = _i
        L.orc_cg.argtypes = [_p, _i, _dptr, _dptr, _dptr, _i, _d, ctypes.POINTER(_i), ctypes.POINTER(_d)]
        L.orc_locate.argtypes = [_p, _i, _fptr, _iptr, _fptr, _fptr, _iptr]
        L.orc_tree_size.argtypes = [_p, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]
        L.orc_local_matrices.argtypes = [_i, _i, _fptr] + [_dptr] * 7
        L.orc_tree_create.restype = _p
        L.orc_tree_create.argtypes = [_i, _fptr, _i, _iptr]
        L.orc_tree_destroy.argtypes = [_p]
        L.orc_tree_locate.argtypes = [_p, _i, _fptr, _iptr, _fptr, _fptr, _iptr]
        L.orc_tree_stats.argtypes = [_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(_i)]
        L.orc_advect.argtypes = [_p, _dptr, _dptr, _dptr, _dptr]
        L.orc_step.restype = _i
        L.orc_step.argtypes = [_p, _i, _iptr]
        L.orc_set_fields.argtypes = [_p, _dptr, _dptr]
        L.orc_get_fields.argtypes = [_p, _dptr, _dptr]
        L.orc_set_tolerance.argtypes = [_p, _d]
        L.orc_set_bc.argtypes = [_p, _dptr, _dptr, _dptr]
        L.orc_set_scheme.argtypes = [_p, _i]
        L.orc_local_convection.argtypes = [_i, _i, _fptr, _dptr, _dptr]
        L.orc_point_in_triangle.restype = _i
        L.orc_point_in_triangle.argtypes = [_fptr, _fptr, _fptr]
        _u8ptr = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        L.orc_mc_colour.restype = _i
        L.orc_mc_colour.argtypes = [_i, _lptr, _iptr, _dptr, _u8ptr]
        L.orc_mc_lower.restype = ctypes.c_int64
        L.orc_mc_lower.argtypes = [_i, _lptr, _iptr, _dptr, _u8ptr, _p, _p, _p, _p]
        L.orc_ic0.restype = _i
        L.orc_ic0.argtypes = [_i, _i, _u8ptr, _lptr, _iptr, _lptr, _lptr, _dptr, _d, _dptr, _dptr]
        L.orc_pcg.restype = _i
        L.orc_pcg.argtypes = [_i, _lptr, _iptr, _dptr, _i, _u8ptr, _lptr, _iptr, _dptr, _dptr, _dptr, _dptr, _dptr,
                              _i, _d, ctypes.POINTER(_i), ctypes.POINTER(_d)]
        _LIB = L
    return _LIB


_REF_NAMES = {False: "libref_kdtree.so", True: "libref_kdtree_int.so"}


def ref_available(int_offsets: bool = False) -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", _REF_NAMES[bool(int_offsets)]))


def ref_lib(int_offsets: bool = False):
    """The reference's tree as compiled from its sources (`make ref`), or the copy whose leaf offsets are read as
    integers instead of float (`make ref-int`)."""
    global _REF
    if _REF is None:
        _REF = {}
    key = bool(int_offsets)
    if key not in _REF:
        L = ctypes.CDLL(os.path.join(_HERE, "_ref", _REF_NAMES[key]))
        L.ref_tree_create.restype = _p
        L.ref_tree_create.argtypes = [_i, _fptr, _i, _iptr, _i]
        L.ref_tree_destroy.argtypes = [_p]
        L.ref_tree_locate.argtypes = [_p, _i, _fptr, _iptr, _fptr, _fptr, _iptr]
        L.ref_grid_bbox.argtypes = [_p, _fptr]
        L.ref_expression_eval.restype = _i
        L.ref_expression_eval.argtypes = [ctypes.c_char_p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                          ctypes.POINTER(ctypes.c_float)]
        _REF[key] = L
    return _REF[key]


def ref_evaluate_expression(expr: str, x: float, y: float, t: float = 0.0) -> float:
    """The reference's own Expression::init + ::evaluate (cpp/expression.cpp), float variables x, y, t as
    cpp/grid.cpp:80-94 passes them; the float result.  Raises ValueError where the reference reports an error."""
    out = ctypes.c_float(0.0)
    st = ref_lib().ref_expression_eval(expr.encode(), x, y, t, ctypes.byref(out))
    if st != 0:
        raise ValueError(f"reference rejects {expr!r} ({'init' if st == 1 else 'evaluate'})")
    return out.value


# ---------------------------------------------------------------------------------------------------
# Boundary-condition expressions (restatement of cpp/expression.cpp semantics)
# ---------------------------------------------------------------------------------------------------
_TOKEN = re.compile(r"\s*(?:(sin|cos)|(Pi|E)|(\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)|([xyzt])|([-+*/^()]))")


def _tokenize(expr: str):
    pos, out = 0, []
    expr = expr.strip()
    while pos < len(expr):
        m = _TOKEN.match(expr, pos)
        if not m or m.end() == pos:
            raise ValueError(f"Error while parsing expression: {expr}. Unexpected symbol at {pos}")
        fn, const, num, var, op = m.groups()
        if fn:
            out.append(("fn", fn))
        elif const:
            out.append(("num", math.e if const == "E" else math.pi))
        elif num:
            out.append(("num", float(num)))
        elif var:
            out.append(("var", var))
        else:
            out.append(("op", op))
        pos = m.end()
    return out


def evaluate_expression(expr: str, variables: dict) -> float:
    """Evaluate a reference BC expression in double precision."""
    toks = _tokenize(expr)
    i = 0

    def peek():
        return toks[i] if i < len(toks) else (None, None)

    def take():
        nonlocal i
        t = toks[i]
        i += 1
        return t

    def atom():
        kind, val = peek()
        if kind == "num":
            take()
            return val
        if kind == "var":
            take()
            if val not in variables:
                raise ValueError(f"Missing variable: {val}")
            return float(variables[val])
        if kind == "fn":
            take()
            if peek() != ("op", "("):
                raise ValueError(f"Error parsing expression: {expr}. Functions must be surrounded by ()")
            return math.sin(atom()) if val == "sin" else math.cos(atom())
        if (kind, val) == ("op", "("):
            take()
            v = add()
            if peek() != ("op", ")"):
                raise ValueError(f"Error parsing expression: {expr}. Mismatched brackets.")
            take()
            return v
        raise ValueError(f"Wrong expression: {expr}")

    def power():
        v = atom()
        while peek() == ("op", "^"):
            take()
            if peek() == ("op", "-"):
                take()
                e = -power()
            else:
                e = atom()
            v = v ** e
        return v

    def unary():
        if peek() == ("op", "-"):
            take()
            return -unary()
        return power()

    def mul():
        v = unary()
        while peek() in (("op", "*"), ("op", "/")):
            op = take()[1]
            r = unary()
            v = v * r if op == "*" else v / r
        return v

    def add():
        v = mul()
        while peek() in (("op", "+"), ("op", "-")):
            op = take()[1]
            r = mul()
            v = v + r if op == "+" else v - r
        return v

    v = add()
    if i != len(toks):
        raise ValueError(f"Wrong expression: {expr}")
    return float(v)


def bc_occurrences(mesh, t=None):
    """Dirichlet data as the reference walks it: every (group, node) occurrence in file order.

    Returns (u_nodes int32, gu float64, gv float64, p_nodes int32, gp float64).  Values are the group's
    expressions evaluated in double at the node's (float) coordinates with variables x and y, and t when given
    (time-dependent data, which the reference's grammar accepts but its driver never passes).
    """
    un, gu, gv, pn, gp = [], [], [], [], []
    for nodes, ue, ve in mesh.u_dirichlet:
        for nd in nodes:
            x, y = float(mesh.nodes[nd, 0]), float(mesh.nodes[nd, 1])
            var = {"x": x, "y": y} if t is None else {"x": x, "y": y, "t": float(t)}
            un.append(int(nd))
            gu.append(evaluate_expression(ue, var))
            gv.append(evaluate_expression(ve, var))
    for nodes, pe in mesh.p_dirichlet:
        for nd in nodes:
            x, y = float(mesh.nodes[nd, 0]), float(mesh.nodes[nd, 1])
            var = {"x": x, "y": y} if t is None else {"x": x, "y": y, "t": float(t)}
            pn.append(int(nd))
            gp.append(evaluate_expression(pe, var))
    return (np.asarray(un, np.int32), np.asarray(gu, np.float64), np.asarray(gv, np.float64),
            np.asarray(pn, np.int32), np.asarray(gp, np.float64))


class Oracle:
    """The CPU restatement of one simulation (mesh + BCs + nu + dt), FP64 by default."""

    def __init__(self, mesh, viscosity: float, dt: float, real_bits: int = 64):
        L = lib()
        self.mesh = mesh
        self.nv, self.np_ = mesh.n_nodes, mesh.n_pressure
        exprs = [e for _, ue, ve in mesh.u_dirichlet for e in (ue, ve)] + [pe for _, pe in mesh.p_dirichlet]
        # time-dependent Dirichlet data: evaluated at t0 + k dt before step k (t0 = 0: the initial state)
        self.timed = any("t" in e.replace("Pi", "") for e in exprs)
        self.t0, self.steps = 0.0, 0
        un, gu, gv, pn, gp = bc_occurrences(mesh, 0.0 if self.timed else None)
        nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float32).reshape(-1)
        els = np.ascontiguousarray(mesh.elements, dtype=np.int32).reshape(-1)
        self._h = L.orc_create(mesh.n_nodes, nodes, mesh.n_elements, els, mesh.n_pressure, len(un), un, gu, gv,
                               len(pn), pn, gp, float(viscosity), float(dt), int(real_bits))
        self.dt = dt
        self.viscosity = viscosity

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    __del__ = close

    def matrix(self, name):
        """(rowptr int64, col int32, val float64, shape) of one assembled matrix."""
        L = lib()
        slot = SLOTS[name] if isinstance(name, str) else int(name)
        r, c, nnz = _i(), _i(), ctypes.c_int64()
        L.orc_matrix_shape(self._h, slot, ctypes.byref(r), ctypes.byref(c), ctypes.byref(nnz))
        rp = np.zeros(r.value + 1, np.int64)
        col = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value, np.float64)
        L.orc_matrix_get(self._h, slot, rp, col, val)
        return rp, col, val, (r.value, c.value)

    def scipy_matrix(self, name):
        import scipy.sparse as sp
        rp, col, val, shape = self.matrix(name)
        return sp.csr_matrix((val, col, rp), shape=shape)

    def spmv(self, name, x):
        rp, col, val, shape = self.matrix(name)
        y = np.zeros(shape[0])
        lib().orc_spmv(self._h, SLOTS[name], np.ascontiguousarray(x, np.float64), y)
        return y

    def cg(self, name, b, x0, max_iter=-1, tol=1e-8):
        n = len(b)
        x = np.zeros(n)
        it, rr = _i(), _d()
        st = lib().orc_cg(self._h, SLOTS[name], np.ascontiguousarray(b, np.float64),
                          np.ascontiguousarray(x0, np.float64), x, int(max_iter), float(tol),
                          ctypes.byref(it), ctypes.byref(rr))
        return x, st, it.value, rr.value

    def locate(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
        n = pts.shape[0]
        e = np.zeros(n, np.int32)
        xi = np.zeros(n, np.float32)
        eta = np.zeros(n, np.float32)
        nn = np.zeros(n, np.int32)
        lib().orc_locate(self._h, n, pts.reshape(-1), e, xi, eta, nn)
        return e, xi, eta, nn

    def tree_size(self):
        a, b, c = _i(), _i(), _i()
        lib().orc_tree_size(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def advect(self, u, v):
        uo, vo = np.zeros(self.nv), np.zeros(self.nv)
        lib().orc_advect(self._h, np.ascontiguousarray(u, np.float64), np.ascontiguousarray(v, np.float64), uo, vo)
        return uo, vo

    def set_tolerance(self, tol: float):
        """Relative residual of every CG solve of `step` (1e-8 by default)."""
        lib().orc_set_tolerance(self._h, float(tol))

    def set_scheme(self, scheme: str = "semi_lagrangian"):
        """"semi_lagrangian" (semiLagrangianSolve) or "explicit_convection" (NavierStokesAssembly::solve)."""
        lib().orc_set_scheme(self._h, {"semi_lagrangian": 0, "explicit_convection": 1}[scheme])

    def step(self, n=1):
        iters = np.zeros(5 * n, np.int32)
        if not self.timed:
            st = lib().orc_step(self._h, int(n), iters)
            return st, iters.reshape(n, 5)
        st = 0
        for k in range(n):
            self.steps += 1
            _, gu, gv, _, gp = bc_occurrences(self.mesh, self.t0 + self.steps * self.dt)
            lib().orc_set_bc(self._h, gu, gv, gp)
            st |= lib().orc_step(self._h, 1, iters[5 * k:5 * k + 5])
        return st, iters.reshape(n, 5)

    def set_fields(self, uv, p):
        lib().orc_set_fields(self._h, np.ascontiguousarray(uv, np.float64), np.ascontiguousarray(p, np.float64))

    def fields(self):
        uv, p = np.zeros(2 * self.nv), np.zeros(self.np_)
        lib().orc_get_fields(self._h, uv, p)
        return uv, p


LOCAL_MATRIX_SHAPES = {"mass": (6, 6), "stiffness_p2": (6, 6), "stiffness_p1": (3, 3), "divergence_x": (3, 6),
                       "divergence_y": (3, 6), "gradient_x": (6, 3), "gradient_y": (6, 3)}


def local_matrices(vertices, real_bits: int = 64):
    """The oracle's local element matrices of triangles given as [n, 6] float32 vertex coordinates (x0 y0 x1 y1 x2 y2),
    computed in float (real_bits 32) or double: a dict of [n, rows, cols] float64 arrays keyed as
    LOCAL_MATRIX_SHAPES."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 6)
    n = v.shape[0]
    out = {k: np.zeros((n,) + s) for k, s in LOCAL_MATRIX_SHAPES.items()}
    lib().orc_local_matrices(int(real_bits), n, v.reshape(-1), *[out[k].reshape(-1) for k in LOCAL_MATRIX_SHAPES])
    return out


def local_convection(vertices, velocities, real_bits: int = 64):
    """The oracle's local convection matrices [n, 6, 6] of triangles ([n, 6] float32 vertices) with nodal velocities
    [n, 12] (u0..u5, v0..v5), in float (real_bits 32) or double."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 6)
    u = np.ascontiguousarray(velocities, np.float64).reshape(-1, 12)
    out = np.zeros((v.shape[0], 6, 6))
    lib().orc_local_convection(int(real_bits), v.shape[0], v.reshape(-1), u.reshape(-1), out.reshape(-1))
    return out


def ref_local_convection(vertices, velocities):
    """The same from the reference's own convection functor (`make ref-assembly`), in float."""
    path = os.path.join(_HERE, "_ref", "libref_assembly.so")
    L = ctypes.CDLL(path)
    L.ref_local_convection.argtypes = [_i, _fptr, _fptr, _fptr]
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 6)
    u = np.ascontiguousarray(velocities, np.float32).reshape(-1, 12)
    out = np.zeros((v.shape[0], 6, 6), np.float32)
    L.ref_local_convection(v.shape[0], v.reshape(-1), u.reshape(-1), out.reshape(-1))
    return out


def ref_local_matrices(vertices):
    """The same matrices from the reference's own element code (`make ref-assembly`), in float."""
    path = os.path.join(_HERE, "_ref", "libref_assembly.so")
    L = ctypes.CDLL(path)
    L.ref_local_matrices.argtypes = [_i, _fptr] + [_fptr] * 7
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 6)
    n = v.shape[0]
    out = {k: np.zeros((n,) + s, np.float32) for k, s in LOCAL_MATRIX_SHAPES.items()}
    L.ref_local_matrices(n, v.reshape(-1), *[out[k].reshape(-1) for k in LOCAL_MATRIX_SHAPES])
    return out


def ref_assembly_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libref_assembly.so"))


class PortTree:
    """The oracle's restatement of the reference tree (int leaf offsets) without the rest of the oracle."""

    def __init__(self, mesh):
        nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float32).reshape(-1)
        els = np.ascontiguousarray(mesh.elements, dtype=np.int32).reshape(-1)
        self._h = lib().orc_tree_create(mesh.n_nodes, nodes, mesh.n_elements, els)

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_tree_destroy(self._h)
            self._h = None

    __del__ = close

    def locate(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
        n = pts.shape[0]
        e, xi, eta, nn = np.zeros(n, np.int32), np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.int32)
        lib().orc_tree_locate(self._h, n, pts.reshape(-1), e, xi, eta, nn)
        return e, xi, eta, nn

    def stats(self):
        a, b, d = ctypes.c_int64(), ctypes.c_int64(), _i()
        lib().orc_tree_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(d))
        return {"nodes": a.value, "leaf_entries": b.value, "max_depth": d.value}


class ReferenceTree:
    """The reference's own KD tree (oracle/_ref), built over a mesh; only where the reference compiled.
    ``int_offsets=True`` uses the build whose KDNode::getTriangleOffset returns the integer offset instead of
    float (gpu_cpu_shared/kd_tree_common.cuh:91,148-150); the two agree while every leaf offset is below 2^24."""

    def __init__(self, mesh, int_offsets: bool = False):
        self._lib = ref_lib(int_offsets)
        nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float32).reshape(-1)
        els = np.ascontiguousarray(mesh.elements, dtype=np.int32).reshape(-1)
        self._h = self._lib.ref_tree_create(mesh.n_nodes, nodes, mesh.n_elements, els, mesh.n_pressure)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ref_tree_destroy(self._h)
            self._h = None

    __del__ = close

    def locate(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
        n = pts.shape[0]
        e = np.zeros(n, np.int32)
        xi = np.zeros(n, np.float32)
        eta = np.zeros(n, np.float32)
        nn = np.zeros(n, np.int32)
        self._lib.ref_tree_locate(self._h, n, pts.reshape(-1), e, xi, eta, nn)
        return e, xi, eta, nn

    def bbox(self):
        out = np.zeros(4, np.float32)
        self._lib.ref_grid_bbox(self._h, out)
        return out


# ---------------------------------------------------------------------------------------------------
# Multicolour IC(0) preconditioner and PCG (precond_oracle.cpp)
# ---------------------------------------------------------------------------------------------------
class McFactor:
    """Multicolour pattern of a CSR matrix (scipy), its IC(0) values, and PCG with M = L L^T."""

    def __init__(self, A):
        A = A.tocsr()
        A.sort_indices()
        self.A = A
        self.n = A.shape[0]
        self.rp = np.ascontiguousarray(A.indptr, np.int64)
        self.ci = np.ascontiguousarray(A.indices, np.int32)
        self.av = np.ascontiguousarray(A.data, np.float64)
        L = lib()
        self.colour = np.zeros(self.n, np.uint8)
        self.colours = L.orc_mc_colour(self.n, self.rp, self.ci, self.av, self.colour)
        nnz = L.orc_mc_lower(self.n, self.rp, self.ci, self.av, self.colour, None, None, None, None)
        self.lrp = np.zeros(self.n + 1, np.int64)
        self.lci = np.zeros(max(nnz, 1), np.int32)
        self.aidx = np.zeros(max(nnz, 1), np.int64)
        self.adiag = np.full(self.n, -1, np.int64)
        L.orc_mc_lower(self.n, self.rp, self.ci, self.av, self.colour, self.lrp.ctypes.data, self.lci.ctypes.data,
                       self.aidx.ctypes.data, self.adiag.ctypes.data)
        self.nnz_lower = int(nnz)
        self.lval = np.zeros(max(nnz, 1))
        self.diag = np.ones(self.n)
        self.shift = 0.0

    def ic0(self):
        """IC(0) values; on breakdown retried with a diagonal shift of 1e-3, 1e-2, ... (as the GPU path does)."""
        shift = 0.0
        for _ in range(8):
            failed = lib().orc_ic0(self.n, self.colours, self.colour, self.lrp, self.lci, self.aidx, self.adiag,
                                   self.av, shift, self.lval, self.diag)
            if not failed:
                self.shift = shift
                return shift
            shift = 1e-3 if shift == 0.0 else shift * 10
        raise RuntimeError("IC(0) broke down")

    def set(self, lower, diag):
        self.lval[: self.nnz_lower] = lower
        self.diag[:] = diag

    def pcg(self, b, x0, max_iter=-1, tol=1e-8):
        x = np.zeros(self.n)
        it, rel = _i(), _d()
        st = lib().orc_pcg(self.n, self.rp, self.ci, self.av, self.colours, self.colour, self.lrp, self.lci,
                           self.lval, self.diag, np.ascontiguousarray(b, np.float64),
                           np.ascontiguousarray(x0, np.float64), x, int(max_iter), float(tol), ctypes.byref(it),
                           ctypes.byref(rel))
        return x, it.value, rel.value, st


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())
