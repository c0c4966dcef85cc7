"""GB300-native hot path of the P2-P1 Taylor-Hood Navier-Stokes solver (vasil-pashov/Navier_Stokes_FEM).

Python mirror of the reference's GPU device layer and assembly driver, over the C ABI of
``include/nsfem_gb300.h`` (``libnsfem_gb300.so``, built in-tree by ``_build.build()``):

* :class:`GPUSimulationDevice` - ``GPUSimulationDevice`` (include/gpu_simulation_device.h:13-206):
  ``upload_matrix``, ``sp_r_mult``, ``conjugate_gradient``, ``upload_kd_tree``, ``advect``, plus ``locate``.
* :class:`NavierStokesAssembly` - ``NavierStokesAssembly<P2, P1>`` (include/assembly.h:306-935) with the whole
  operator-split step resident on the GPU: ``init`` from a scene file or a mesh, ``semi_lagrangian_solve``,
  ``step``, ``fields``.

There is no CPU fallback: every call goes to the CUDA library, and a missing library raises.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from . import mesh as mesh_io

__all__ = [
    "NSFemError", "GPUSimulationDevice", "NavierStokesAssembly", "BatchedNavierStokes", "library", "library_path",
    "evaluate_expression",
    "bc_occurrences", "SLOT", "SOLVER", "STATUS", "declared_symbols",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
library_path = os.path.join(_PKG, "libnsfem_gb300.so")
header_path = os.path.join(_ROOT, "include", "nsfem_gb300.h")

STATUS = {0: "NSF_OK", 1: "NSF_ERR_CUDA", 2: "NSF_ERR_NOT_CONVERGED", 3: "NSF_ERR_BREAKDOWN",
          4: "NSF_ERR_BARRIER_TIMEOUT", 5: "NSF_ERR_BAD_ARG", 6: "NSF_ERR_STATE", 7: "NSF_ERR_NO_DEVICE"}
SLOT = {"pressure_stiffness": 0, "velocity_mass": 1, "diffusion": 2, "velocity_divergence": 3,
        "pressure_divergence": 4, "velocity_lift": 5, "pressure_lift": 6}
CG_FORM = {"auto": 0, "three_sync": 1, "pipelined": 2, "multi_kernel": 3}
PCG_FORM = {"auto": 0, "full": 1, "reduced": 2, "schur": 3}
SOLVER = {"fp64": 0, "mixed": 1, "pcg_mixed": 2, "pcg_fp64": 3}
PRECOND = {0: "none", 1: "ic0", 2: "learned"}


class NSFemError(RuntimeError):
    """A non-zero nsf_status, with the library's message (EC::ErrorCode, include/error_code.h:9-39)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


_LIB = None
_v, _i, _i64, _d, _f, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_float, ctypes.c_size_t
_P = ctypes.POINTER


def _arr(dtype):
    return np.ctypeslib.ndpointer(dtype, flags="C_CONTIGUOUS")


_SIGS = {
    "nsf_create": (_i, [_i, _P(_v)]),
    "nsf_destroy": (None, [_v]),
    "nsf_last_error": (ctypes.c_char_p, [_v]),
    "nsf_device_info": (_i, [_v, _P(_i), _P(_i), _P(_i)]),
    "nsf_synchronize": (_i, [_v]),
    "nsf_upload_matrix_csr": (_i, [_v, _i, _i, _i, _i64, _arr(np.int32), _arr(np.int32), _arr(np.float64)]),
    "nsf_upload_matrix_triplets": (_i, [_v, _i, _i, _i, _i64, _arr(np.int32), _arr(np.int32), _arr(np.float64)]),
    "nsf_matrix_shape": (_i, [_v, _i, _P(_i), _P(_i), _P(_i64)]),
    "nsf_download_matrix": (_i, [_v, _i, _arr(np.int32), _arr(np.int32), _arr(np.float64)]),
    "nsf_spmv": (_i, [_v, _i, _arr(np.float64), _arr(np.float64)]),
    "nsf_conjugate_gradient": (_i, [_v, _i, _arr(np.float64), _arr(np.float64), _arr(np.float64), _i, _d, _i,
                                    _P(_i), _P(_d)]),
    "nsf_conjugate_gradient_f32": (_i, [_v, _i, _arr(np.float32), _arr(np.float32), _arr(np.float32), _i, _f]),
    "nsf_conjugate_gradient_dev": (_i, [_v, _i, _v, _v, _v, _i, _d, _i, _P(_i), _P(_d)]),
    "nsf_upload_mesh": (_i, [_v, _i, _arr(np.float32), _i, _arr(np.int32), _i]),
    "nsf_locate": (_i, [_v, _i, _arr(np.float32), _arr(np.int32), _arr(np.float32), _arr(np.float32),
                        _arr(np.int32)]),
    "nsf_advect": (_i, [_v, _i, _arr(np.float32), _arr(np.float32), _f, _arr(np.float32), _arr(np.float32)]),
    "nsf_advect_f64": (_i, [_v, _i, _arr(np.float64), _arr(np.float64), _d, _arr(np.float64), _arr(np.float64)]),
    "nsf_sim_setup": (_i, [_v, _i, _arr(np.float32), _i, _arr(np.int32), _i, _i, _arr(np.int32), _arr(np.float64),
                           _arr(np.float64), _i, _arr(np.int32), _arr(np.float64), _d, _d]),
    "nsf_sim_set_fields": (_i, [_v, _v, _v]),
    "nsf_sim_get_fields": (_i, [_v, _v, _v]),
    "nsf_sim_step": (_i, [_v, _i, _v]),
    "nsf_sim_step_host": (_i, [_v, _v, _v, _i, _v, _v, _v]),
    "nsf_set_tolerance": (_i, [_v, _d]),
    "nsf_set_solver": (_i, [_v, _i, _d]),
    "nsf_set_cg_form": (_i, [_v, _i]),
    "nsf_set_pcg_form": (_i, [_v, _i]),
    "nsf_precond_schur_nnz": (_i, [_v, _i, _P(_i64)]),
    "nsf_set_barrier_timeout": (_i, [_v, _d]),
    "nsf_profile": (_i, [_v, _i]),
    "nsf_profile_read": (_i, [_v, _i, _arr(np.int32), _arr(np.int32), _arr(np.int32), _arr(np.int32),
                              _arr(np.int64), _arr(np.int32), _arr(np.int32), _arr(np.float32)]),
    "nsf_precond_pattern": (_i, [_v, _i, _P(_i), _P(_i64)]),
    "nsf_precond_get_pattern": (_i, [_v, _i, _arr(np.int32), _arr(np.int32), _arr(np.uint8)]),
    "nsf_precond_ic0": (_i, [_v, _i, _P(_d)]),
    "nsf_precond_set": (_i, [_v, _i, _arr(np.float64), _arr(np.float64)]),
    "nsf_precond_get": (_i, [_v, _i, _arr(np.float64), _arr(np.float64)]),
    "nsf_precond_kind": (_i, [_v, _i]),
    "nsf_precond_index_bytes": (_i, [_v, _i]),
    "nsf_precond_inner_form": (_i, [_v, _i, ctypes.POINTER(_i)]),
    "nsf_precond_value_bytes": (_i, [_v, _i]),
    "nsf_precond_clear": (_i, [_v, _i]),
    "nsf_precond_cap": (_i, [_v, _i, _i]),
    "nsf_tc_dense": (_i, [_v, _i, _i, _i, _arr(np.float32), _arr(np.float32), _v, _i, _arr(np.float32)]),
    "nsf_tc_weight_gradient": (_i, [_v, _i, _i, _i, _arr(np.float32), _arr(np.float32), _arr(np.float32),
                                    _arr(np.float32)]),
    "nsf_learn_create": (_i, [_v, ctypes.c_uint64, _P(_v)]),
    "nsf_learn_destroy": (None, [_v]),
    "nsf_learn_last_error": (ctypes.c_char_p, [_v]),
    "nsf_learn_param_count": (_i, [_v, _P(_i64)]),
    "nsf_learn_get_params": (_i, [_v, _arr(np.float32)]),
    "nsf_learn_set_params": (_i, [_v, _arr(np.float32)]),
    "nsf_learn_add_system": (_i, [_v, _i, _arr(np.float64), _arr(np.float64), _P(_i)]),
    "nsf_learn_clear_systems": (_i, [_v]),
    "nsf_learn_system_size": (_i, [_v, _i, _P(_i), _P(_i64)]),
    "nsf_learn_forward": (_i, [_v, _i, _arr(np.float32), _arr(np.float32)]),
    "nsf_learn_loss_grad": (_i, [_v, _i, _P(_d), _arr(np.float32)]),
    "nsf_learn_train": (_i, [_v, _i, _i, _d, ctypes.c_uint64, _v]),
    "nsf_learn_apply": (_i, [_v, _v, _i]),
    "nsf_timer": (_i, [_v, _i, _P(_f)]),
    "nsf_host_alloc": (_i, [_v, _sz, _P(_v)]),
    "nsf_host_free": (_i, [_v, _v]),
    "nsf_eval_expression": (_i, [ctypes.c_char_p, _d, _d, _P(_d), ctypes.c_char_p, _sz]),
    "nsf_eval_expression_t": (_i, [ctypes.c_char_p, _d, _d, _d, _P(_d), ctypes.c_char_p, _sz]),
    "nsf_sim_set_bc_expressions": (_i, [_v, _i, _v, _v, _v, _v, _d]),
    "nsf_sim_time": (_i, [_v, _P(_d)]),
    "nsf_sim_set_scheme": (_i, [_v, _i]),
    "nsf_launch_count": (_i, [_v, _P(_i64)]),
    "nsf_batch_clear": (_i, [_v]),
    "nsf_batch_add": (_i, [_v, _i, _arr(np.float32), _i, _arr(np.int32), _i, _i, _arr(np.int32), _arr(np.float64),
                           _arr(np.float64), _i, _arr(np.int32), _arr(np.float64), _d, _d, _P(_i)]),
    "nsf_batch_finalize": (_i, [_v, _i]),
    "nsf_batch_step": (_i, [_v, _i, _v]),
    "nsf_batch_get_fields": (_i, [_v, _i, _v, _v]),
    "nsf_batch_set_fields": (_i, [_v, _i, _v, _v]),
    "nsf_batch_plan": (_i, [_v, _v, _P(_i), _v, _i, _P(_i)]),
    "nsf_conjugate_gradient_noalloc": (_i, [_i, _v, _v, _v, _v, _v, _v, _i, _d, _v, _P(_i), _P(_d)]),
    "nsf_flush_l2": (_i, [_v, _sz]),
}


def library():
    """The loaded CUDA library.  Raises if it has not been built (there is no fallback path)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(library_path):
            raise RuntimeError(f"{library_path} is missing: build it with `python -m navier_stokes_fem_gb300._build` "
                               "or __graft_entry__.build()")
        L = ctypes.CDLL(library_path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def declared_symbols():
    """Function names declared in include/nsfem_gb300.h."""
    with open(header_path) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+\**(nsf_\w+)\s*\(", text, re.M)))


def evaluate_expression(expression: str, x: float, y: float, t: float | None = None) -> float:
    """A mesh-file boundary expression evaluated by the library's C++ evaluator (double precision); with t, the
    variable t as well."""
    out = _d()
    msg = ctypes.create_string_buffer(256)
    if t is None:
        st = library().nsf_eval_expression(expression.encode(), float(x), float(y), ctypes.byref(out), msg, 256)
    else:
        st = library().nsf_eval_expression_t(expression.encode(), float(x), float(y), float(t), ctypes.byref(out),
                                             msg, 256)
    if st != 0:
        raise NSFemError(st, msg.value.decode())
    return out.value


def uses_time(expression: str) -> bool:
    """True when a mesh-file expression contains the variable t (the grammar's only lower-case letters are the
    variables and the function names sin and cos)."""
    return "t" in expression.replace("Pi", "")


def bc_occurrences(mesh, t: float | None = None):
    """Dirichlet data per listed occurrence in the mesh's group order, values evaluated at each node (at time t
    when given)."""
    un, gu, gv, pn, gp = [], [], [], [], []
    for nodes, ue, ve in mesh.u_dirichlet:
        for nd in np.asarray(nodes):
            x, y = float(mesh.nodes[nd, 0]), float(mesh.nodes[nd, 1])
            un.append(int(nd))
            gu.append(evaluate_expression(ue, x, y, t))
            gv.append(evaluate_expression(ve, x, y, t))
    for nodes, pe in mesh.p_dirichlet:
        for nd in np.asarray(nodes):
            x, y = float(mesh.nodes[nd, 0]), float(mesh.nodes[nd, 1])
            pn.append(int(nd))
            gp.append(evaluate_expression(pe, x, y, t))
    return (np.asarray(un, np.int32), np.asarray(gu, np.float64), np.asarray(gv, np.float64),
            np.asarray(pn, np.int32), np.asarray(gp, np.float64))


def _bc_fast(mesh):
    """bc_occurrences for groups whose expressions are constants or simple polynomials, vectorised.

    Falls back to the per-node evaluator unless every expression is a plain number; used for large meshes.
    """
    def const(e):
        try:
            return float(e)
        except ValueError:
            return None
    un, gu, gv, pn, gp = [], [], [], [], []
    for nodes, ue, ve in mesh.u_dirichlet:
        cu, cv = const(ue), const(ve)
        nodes = np.asarray(nodes, np.int32)
        if cu is None or cv is None:
            xs, ys = mesh.nodes[nodes, 0].astype(np.float64), mesh.nodes[nodes, 1].astype(np.float64)
            vals_u = np.array([evaluate_expression(ue, a, b) for a, b in zip(xs, ys)]) if cu is None else np.full(len(nodes), cu)
            vals_v = np.array([evaluate_expression(ve, a, b) for a, b in zip(xs, ys)]) if cv is None else np.full(len(nodes), cv)
        else:
            vals_u, vals_v = np.full(len(nodes), cu), np.full(len(nodes), cv)
        un.append(nodes); gu.append(vals_u); gv.append(vals_v)
    for nodes, pe in mesh.p_dirichlet:
        cp = const(pe)
        nodes = np.asarray(nodes, np.int32)
        if cp is None:
            vals = np.array([evaluate_expression(pe, float(mesh.nodes[n, 0]), float(mesh.nodes[n, 1])) for n in nodes])
        else:
            vals = np.full(len(nodes), cp)
        pn.append(nodes); gp.append(vals)
    cat = lambda a, t: np.ascontiguousarray(np.concatenate(a).astype(t)) if a else np.zeros(0, t)
    return cat(un, np.int32), cat(gu, np.float64), cat(gv, np.float64), cat(pn, np.int32), cat(gp, np.float64)


def _slot(s):
    return SLOT[s] if isinstance(s, str) else int(s)


class GPUSimulationDevice:
    """One GPU, one stream: the reference's GPUSimulationDevice (include/gpu_simulation_device.h:13-206)."""

    def __init__(self, device: int = 0):
        L = library()
        h = _v()
        st = L.nsf_create(int(device), ctypes.byref(h))
        if st != 0:
            raise NSFemError(st, f"cannot create a handle on CUDA device {device}")
        self._h = h
        self.device = device

    # -- plumbing ------------------------------------------------------------------------------------
    def _check(self, st: int):
        if st != 0:
            raise NSFemError(st, library().nsf_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            library().nsf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def info(self):
        a, b, c = _i(), _i(), _i()
        self._check(library().nsf_device_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"sm_count": a.value, "cg_grid_blocks": b.value, "cg_block_threads": c.value}

    def synchronize(self):
        self._check(library().nsf_synchronize(self._h))

    # -- matrices (uploadMatrix) ---------------------------------------------------------------------
    def upload_matrix(self, slot, rowptr, col, val, shape):
        rp = np.ascontiguousarray(rowptr, np.int32)
        self._check(library().nsf_upload_matrix_csr(self._h, _slot(slot), int(shape[0]), int(shape[1]),
                                                    int(rp[-1]), rp, np.ascontiguousarray(col, np.int32),
                                                    np.ascontiguousarray(val, np.float64)))

    def upload_matrix_triplets(self, slot, rows, cols, vals, shape):
        r = np.ascontiguousarray(rows, np.int32)
        self._check(library().nsf_upload_matrix_triplets(self._h, _slot(slot), int(shape[0]), int(shape[1]), len(r), r,
                                                         np.ascontiguousarray(cols, np.int32),
                                                         np.ascontiguousarray(vals, np.float64)))

    def matrix_shape(self, slot):
        r, c, n = _i(), _i(), _i64()
        self._check(library().nsf_matrix_shape(self._h, _slot(slot), ctypes.byref(r), ctypes.byref(c), ctypes.byref(n)))
        return r.value, c.value, n.value

    def download_matrix(self, slot):
        rows, cols, nnz = self.matrix_shape(slot)
        rp = np.zeros(rows + 1, np.int32)
        col = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1), np.float64)
        self._check(library().nsf_download_matrix(self._h, _slot(slot), rp, col, val))
        return rp, col[:nnz], val[:nnz], (rows, cols)

    def scipy_matrix(self, slot):
        import scipy.sparse as sp
        rp, col, val, shape = self.download_matrix(slot)
        return sp.csr_matrix((val, col, rp), shape=shape)

    # -- algebra (spRMult, conjugateGradient) --------------------------------------------------------
    def sp_r_mult(self, slot, x):
        rows, cols, _ = self.matrix_shape(slot)
        y = np.zeros(rows)
        self._check(library().nsf_spmv(self._h, _slot(slot), np.ascontiguousarray(x, np.float64), y))
        return y

    def conjugate_gradient(self, slot, b, x0, max_iterations=-1, eps=1e-8, solver="fp64", raise_on_error=True):
        """Returns (x, iterations, relative residual).  Non-convergence raises NSFemError (x is still written)."""
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b)
        it, rr = _i(), _d()
        st = library().nsf_conjugate_gradient(self._h, _slot(slot), b, np.ascontiguousarray(x0, np.float64), x,
                                              int(max_iterations), float(eps), SOLVER[solver], ctypes.byref(it),
                                              ctypes.byref(rr))
        if raise_on_error:
            self._check(st)
            return x, it.value, rr.value
        return x, it.value, rr.value, st

    def conjugate_gradient_f32(self, slot, b, x0, max_iterations=-1, eps=1e-8):
        b = np.ascontiguousarray(b, np.float32)
        x = np.zeros_like(b)
        self._check(library().nsf_conjugate_gradient_f32(self._h, _slot(slot), b, np.ascontiguousarray(x0, np.float32),
                                                         x, int(max_iterations), float(eps)))
        return x

    # -- mesh, point location, advection (uploadKDTree, advect) --------------------------------------
    def upload_kd_tree(self, mesh):
        self._check(library().nsf_upload_mesh(self._h, mesh.n_nodes,
                                              np.ascontiguousarray(mesh.nodes, np.float32).reshape(-1),
                                              mesh.n_elements, np.ascontiguousarray(mesh.elements, np.int32).reshape(-1),
                                              mesh.n_pressure))

    upload_mesh = upload_kd_tree

    def locate(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
        n = pts.shape[0]
        e, nn = np.zeros(n, np.int32), np.zeros(n, np.int32)
        xi, eta = np.zeros(n, np.float32), np.zeros(n, np.float32)
        self._check(library().nsf_locate(self._h, n, pts.reshape(-1), e, xi, eta, nn))
        return e, xi, eta, nn

    def advect(self, u, v, dt):
        u = np.ascontiguousarray(u, np.float32)
        uo, vo = np.zeros_like(u), np.zeros_like(u)
        self._check(library().nsf_advect(self._h, len(u), u, np.ascontiguousarray(v, np.float32), float(dt), uo, vo))
        return uo, vo

    def advect_f64(self, u, v, dt):
        u = np.ascontiguousarray(u, np.float64)
        uo, vo = np.zeros_like(u), np.zeros_like(u)
        self._check(library().nsf_advect_f64(self._h, len(u), u, np.ascontiguousarray(v, np.float64), float(dt), uo, vo))
        return uo, vo

    # -- configuration and timing ---------------------------------------------------------------------
    def set_tolerance(self, eps):
        self._check(library().nsf_set_tolerance(self._h, float(eps)))

    def set_solver(self, solver="fp64", inner_tolerance=-1.0):
        self._check(library().nsf_set_solver(self._h, SOLVER[solver], float(inner_tolerance)))

    def set_pcg_form(self, form="auto"):
        """Iteration of the mixed PCG on two-colour systems: "auto" or "reduced" (PCG on the Schur complement of the
        colour-0 block) or "full" (product and both colour sweeps on the whole system)."""
        self._check(library().nsf_set_pcg_form(self._h, PCG_FORM[form]))

    def set_cg_form(self, form="auto"):
        """Iteration form of the plain FP64 CG: "auto", "three_sync", "pipelined" (one grid barrier) or
        "multi_kernel" (one launch per phase, the reference's conjugateGradientMultiKernel)."""
        self._check(library().nsf_set_cg_form(self._h, CG_FORM[form]))

    def set_barrier_timeout(self, seconds):
        self._check(library().nsf_set_barrier_timeout(self._h, float(seconds)))

    def profile(self, enable=True):
        self._check(library().nsf_profile(self._h, 1 if enable else 0))

    def profile_read(self, max_records=100000):
        n = max_records
        slot, mode, fb, rows, it, outer = (np.zeros(n, np.int32) for _ in range(6))
        nnz = np.zeros(n, np.int64)
        ms = np.zeros(n, np.float32)
        got = library().nsf_profile_read(self._h, n, slot, mode, fb, rows, nnz, it, outer, ms)
        if got < 0:
            self._check(-got)
        return {"slot": slot[:got], "mode": mode[:got], "fallback": fb[:got], "rows": rows[:got], "nnz": nnz[:got],
                "iterations": it[:got], "outer": outer[:got], "ms": ms[:got]}

    # ---- preconditioners (M = L L^T on the multicolour pattern of the slot's matrix) ----
    def precond_pattern(self, slot):
        """(rowptr, col, colour) of the factor's strictly lower part; row entries ordered by (colour, column)."""
        c, nnz = _i(), _i64()
        self._check(library().nsf_precond_pattern(self._h, _slot(slot), ctypes.byref(c), ctypes.byref(nnz)))
        rows, _, _ = self.matrix_shape(slot)
        rp = np.zeros(rows + 1, np.int32)
        col = np.zeros(max(nnz.value, 1), np.int32)
        colour = np.zeros(rows, np.uint8)
        self._check(library().nsf_precond_get_pattern(self._h, _slot(slot), rp, col, colour))
        return rp, col[:nnz.value], colour

    def precond_ic0(self, slot) -> float:
        """Incomplete Cholesky factor on the pattern; returns the diagonal shift it needed."""
        sh = _d()
        self._check(library().nsf_precond_ic0(self._h, _slot(slot), ctypes.byref(sh)))
        return sh.value

    def precond_set(self, slot, lower, diag):
        lower = np.ascontiguousarray(lower, np.float64)
        self._check(library().nsf_precond_set(self._h, _slot(slot), lower if lower.size else np.zeros(1),
                                              np.ascontiguousarray(diag, np.float64)))

    def precond_get(self, slot):
        rp, col, _ = self.precond_pattern(slot)
        lower = np.zeros(max(col.size, 1))
        diag = np.zeros(rp.size - 1)
        self._check(library().nsf_precond_get(self._h, _slot(slot), lower, diag))
        return lower[:col.size], diag

    def precond_kind(self, slot) -> str:
        k = library().nsf_precond_kind(self._h, _slot(slot))
        if k < 0:
            self._check(-k)
        return PRECOND[k]

    def precond_index_bytes(self, slot) -> int:
        """Bytes per column index the slot's mixed PCG iterations read (2: 16-bit column copies, else 4)."""
        k = library().nsf_precond_index_bytes(self._h, _slot(slot))
        if k < 0:
            self._check(-k)
        return k

    def precond_value_bytes(self, slot) -> int:
        """Bytes per factor value the slot's mixed PCG iterations read (2: FP16 copies, else 4)."""
        k = library().nsf_precond_value_bytes(self._h, _slot(slot))
        if k < 0:
            self._check(-k)
        return k

    def precond_schur_nnz(self, slot) -> int:
        """Entries of the slot's explicitly formed Schur complement (0 before its first reduced solve with it)."""
        k = _i64()
        self._check(library().nsf_precond_schur_nnz(self._h, _slot(slot), ctypes.byref(k)))
        return k.value

    def precond_inner_form(self, slot) -> str:
        """The inner-iteration kernel of the slot's last split mixed PCG solve: "cta256", "cta1024", "resident"
        (the full iteration), "reduced", "reduced_resident" (the reduced iteration forming u_0), "schur",
        "schur_resident" (the explicit Schur complement) or "none" (no such solve yet)."""
        k = _i()
        self._check(library().nsf_precond_inner_form(self._h, _slot(slot), ctypes.byref(k)))
        return {-1: "none", 0: "cta256", 1: "cta1024", 2: "resident", 3: "reduced", 4: "reduced_resident",
                5: "schur", 6: "schur_resident"}[k.value]

    def precond_clear(self, slot):
        self._check(library().nsf_precond_clear(self._h, _slot(slot)))

    def precond_cap(self, slot, max_iterations):
        self._check(library().nsf_precond_cap(self._h, _slot(slot), int(max_iterations)))

    def timer_start(self):
        self._check(library().nsf_timer(self._h, 0, None))

    def timer_stop(self) -> float:
        ms = _f()
        self._check(library().nsf_timer(self._h, 1, ctypes.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        n = _i64()
        self._check(library().nsf_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def flush_l2(self, nbytes: int = 512 << 20):
        self._check(library().nsf_flush_l2(self._h, int(nbytes)))

    def pinned(self, shape, dtype=np.float64):
        """A zeroed numpy array in page-locked host memory mapped for the device (freed with the handle's process);
        set_fields, fields and step_host move fields to and from such arrays with copy kernels."""
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = _v()
        self._check(library().nsf_host_alloc(self._h, max(nbytes, 1), ctypes.byref(p)))
        buf = (ctypes.c_byte * max(nbytes, 1)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
        return arr


class Learner:
    """The learned preconditioner (nsf_learn_*): a message-passing network that outputs the factor L of a slot's
    matrix, trained on the GPU on (matrix, solution, right-hand side) triples of the plain method."""

    def __init__(self, device: "GPUSimulationDevice", seed: int = 0):
        self.device = device
        h = _v()
        st = library().nsf_learn_create(device._h, ctypes.c_uint64(seed), ctypes.byref(h))
        if st != 0:
            raise NSFemError(st, library().nsf_last_error(device._h).decode())
        self._h = h

    def _check(self, st):
        if st != 0:
            raise NSFemError(st, library().nsf_learn_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            library().nsf_learn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def param_count(self) -> int:
        n = _i64()
        self._check(library().nsf_learn_param_count(self._h, ctypes.byref(n)))
        return n.value

    def params(self):
        th = np.zeros(self.param_count, np.float32)
        self._check(library().nsf_learn_get_params(self._h, th))
        return th

    def set_params(self, theta):
        self._check(library().nsf_learn_set_params(self._h, np.ascontiguousarray(theta, np.float32)))

    def add_system(self, slot, x, b) -> int:
        idx = _i()
        self._check(library().nsf_learn_add_system(self._h, _slot(slot), np.ascontiguousarray(x, np.float64),
                                                   np.ascontiguousarray(b, np.float64), ctypes.byref(idx)))
        return idx.value

    def clear_systems(self):
        self._check(library().nsf_learn_clear_systems(self._h))

    def system_size(self, index):
        n, m = _i(), _i64()
        self._check(library().nsf_learn_system_size(self._h, int(index), ctypes.byref(n), ctypes.byref(m)))
        return n.value, m.value

    def forward(self, index):
        """(L^ off-diagonal values in the factor pattern's order, L^ diagonal) of a stored system."""
        n, m = self.system_size(index)
        lower, diag = np.zeros(max(m, 1), np.float32), np.zeros(n, np.float32)
        self._check(library().nsf_learn_forward(self._h, int(index), lower, diag))
        return lower[:m], diag

    def loss_grad(self, index):
        loss = _d()
        g = np.zeros(self.param_count, np.float32)
        self._check(library().nsf_learn_loss_grad(self._h, int(index), ctypes.byref(loss), g))
        return loss.value, g

    def train(self, steps, batch=1, lr=1e-3, seed=0):
        losses = np.zeros(max(steps, 1), np.float32)
        self._check(library().nsf_learn_train(self._h, int(steps), int(batch), float(lr), ctypes.c_uint64(seed),
                                              losses.ctypes.data_as(_v)))
        return losses[:steps]

    def apply(self, slot, device: "GPUSimulationDevice" = None):
        """Installs the network's factor for the slot's current matrix (preconditioner kind "learned") on `device`
        (default: the learner's own device handle; it must be on the same GPU)."""
        self._check(library().nsf_learn_apply(self._h, device._h if device is not None else None, _slot(slot)))


def tc_dense(device, X, W, bias=None, relu=False):
    """One tensor-core dense layer (BF16 operands, FP32 accumulation): relu?(X W + bias)."""
    X = np.ascontiguousarray(X, np.float32)
    W = np.ascontiguousarray(W, np.float32)
    rows, K = X.shape
    N = W.shape[1]
    Y = np.zeros((rows, N), np.float32)
    b = None if bias is None else np.ascontiguousarray(bias, np.float32)
    st = library().nsf_tc_dense(device._h, rows, K, N, X.reshape(-1), W.reshape(-1),
                                b.ctypes.data_as(_v) if b is not None else None, 1 if relu else 0, Y.reshape(-1))
    device._check(st)
    return Y


def tc_weight_gradient(device, X, G):
    """A dense layer's weight gradients on the tensor cores (BF16 operands, FP32 accumulation): (X^T G, colsum G)."""
    X = np.ascontiguousarray(X, np.float32)
    G = np.ascontiguousarray(G, np.float32)
    rows, K = X.shape
    N = G.shape[1]
    dW = np.zeros((K, N), np.float32)
    db = np.zeros(N, np.float32)
    device._check(library().nsf_tc_weight_gradient(device._h, rows, K, N, X.reshape(-1), G.reshape(-1),
                                                   dW.reshape(-1), db))
    return dW, db


class NavierStokesAssembly(GPUSimulationDevice):
    """NavierStokesAssembly<P2, P1> (include/assembly.h:306-935) with the step loop resident on the GPU."""

    def __init__(self, mesh, viscosity: float, dt: float, device: int = 0, solver: str = "fp64",
                 tol: float = 1e-8, inner_tolerance: float = -1.0, total_time: float | None = None,
                 steps: int | None = None):
        super().__init__(device)
        self.mesh = mesh
        self.viscosity = float(viscosity)
        self.dt = float(dt)
        self.total_time = total_time
        self.steps = steps
        self.set_tolerance(tol)
        self.set_solver(solver, inner_tolerance)
        big = mesh.n_nodes > 200_000
        timed = any(uses_time(e) for _, ue, ve in mesh.u_dirichlet for e in (ue, ve)) or \
            any(uses_time(pe) for _, pe in mesh.p_dirichlet)
        un, gu, gv, pn, gp = bc_occurrences(mesh, 0.0) if timed else _bc_fast(mesh) if big else bc_occurrences(mesh)
        self._check(library().nsf_sim_setup(
            self._h, mesh.n_nodes, np.ascontiguousarray(mesh.nodes, np.float32).reshape(-1), mesh.n_elements,
            np.ascontiguousarray(mesh.elements, np.int32).reshape(-1), mesh.n_pressure, len(un), un, gu, gv,
            len(pn), pn, gp, self.viscosity, self.dt))
        self.nv, self.np_ = mesh.n_nodes, mesh.n_pressure
        if timed:
            self.set_bc_expressions(0.0)

    def set_bc_expressions(self, t0: float = 0.0):
        """Evaluate the mesh's Dirichlet expressions on the device at every step, at the time the step ends
        (t0 + k dt for step k), so that they may use the variable t; imposes the data at t0 on the resident velocity
        (nsf_sim_set_bc_expressions).  Called by the constructor when an expression uses t."""
        exprs, index = [], {}

        def idx(e):
            if e not in index:
                index[e] = len(exprs)
                exprs.append(e)
            return index[e]

        u, v, p = [], [], []
        for nodes, ue, ve in self.mesh.u_dirichlet:
            for _ in np.asarray(nodes):
                u.append(idx(ue))
                v.append(idx(ve))
        for nodes, pe in self.mesh.p_dirichlet:
            for _ in np.asarray(nodes):
                p.append(idx(pe))
        if not exprs:
            exprs.append("0")
        arr = (ctypes.c_char_p * len(exprs))(*[e.encode() for e in exprs])
        u, v, p = (np.ascontiguousarray(a, np.int32) for a in (u, v, p))
        self._check(library().nsf_sim_set_bc_expressions(self._h, len(exprs), ctypes.cast(arr, _v),
                                                         u.ctypes.data_as(_v), v.ctypes.data_as(_v),
                                                         p.ctypes.data_as(_v), float(t0)))

    def set_scheme(self, scheme: str = "semi_lagrangian"):
        """Operator-split scheme of step(): "semi_lagrangian" (semiLagrangianSolve) or "explicit_convection" (the
        reference's NavierStokesAssembly::solve: explicit convection and diffusion, then the projection)."""
        self._check(library().nsf_sim_set_scheme(self._h, {"semi_lagrangian": 0, "explicit_convection": 1}[scheme]))

    def time(self) -> float:
        """Simulated time of the resident fields (nsf_sim_time)."""
        t = _d()
        self._check(library().nsf_sim_time(self._h, ctypes.byref(t)))
        return t.value

    @classmethod
    def init(cls, scene_path: str, **kw):
        """From a scene JSON (include/assembly.h:885-935)."""
        scene = mesh_io.read_scene_json(scene_path)
        m = mesh_io.read_mesh_json(scene["mesh_path"])
        return cls(m, scene["viscosity"], scene["dt"], total_time=scene["total_time"], steps=scene.get("steps"),
                   solver=scene.get("solver", kw.pop("solver", "fp64")), **kw)

    def step_count(self) -> int:
        if self.steps is not None:
            return int(self.steps)
        s = int(np.float32(self.total_time) / np.float32(self.dt))
        return max(s - 1, 0)

    def step(self, n: int = 1):
        """Runs n operator-split steps; returns int32 [n, 5] CG iterations (diff u, diff v, pressure, mass u, v)."""
        it = np.zeros(5 * max(n, 1), np.int32)
        self._check(library().nsf_sim_step(self._h, int(n), it.ctypes.data_as(_v)))
        return it[:5 * n].reshape(n, 5)

    def semi_lagrangian_solve(self):
        return self.step(self.step_count())

    def fields(self):
        uv, p = np.zeros(2 * self.nv), np.zeros(self.np_)
        self._check(library().nsf_sim_get_fields(self._h, uv.ctypes.data_as(_v), p.ctypes.data_as(_v)))
        return uv, p

    def set_fields(self, uv, p):
        uv = np.ascontiguousarray(uv, np.float64)
        p = np.ascontiguousarray(p, np.float64)
        self._check(library().nsf_sim_set_fields(self._h, uv.ctypes.data_as(_v), p.ctypes.data_as(_v)))

    def step_host(self, uv_in, p_in, n, uv_out, p_out):
        """n steps from host fields to host fields (copies inside the call), returns iterations [n, 5]."""
        it = np.zeros(5 * max(n, 1), np.int32)
        self._check(library().nsf_sim_step_host(self._h, uv_in.ctypes.data_as(_v), p_in.ctypes.data_as(_v), int(n),
                                                uv_out.ctypes.data_as(_v), p_out.ctypes.data_as(_v),
                                                it.ctypes.data_as(_v)))
        return it[:5 * n].reshape(n, 5)


class BatchedNavierStokes(GPUSimulationDevice):
    """Many independent NavierStokesAssembly problems advanced together: one persistent launch per step in
    which every instance is served by its own team of CTAs, the step replayed from a CUDA graph.

    ``problems`` is a list of (mesh, viscosity, dt).  Team sizes are picked by the library's autotuner over
    ``autotune_rounds`` timed trial steps (the fields are restored afterwards)."""

    def __init__(self, problems, device: int = 0, solver: str = "fp64", tol: float = 1e-8,
                 inner_tolerance: float = -1.0, autotune_rounds: int = 3):
        super().__init__(device)
        self.set_tolerance(tol)
        self.set_solver(solver, inner_tolerance)
        self.sizes = []
        for mesh, nu, dt in problems:
            un, gu, gv, pn, gp = _bc_fast(mesh) if mesh.n_nodes > 200_000 else bc_occurrences(mesh)
            idx = _i()
            self._check(library().nsf_batch_add(
                self._h, mesh.n_nodes, np.ascontiguousarray(mesh.nodes, np.float32).reshape(-1), mesh.n_elements,
                np.ascontiguousarray(mesh.elements, np.int32).reshape(-1), mesh.n_pressure, len(un), un, gu, gv,
                len(pn), pn, gp, float(nu), float(dt), ctypes.byref(idx)))
            self.sizes.append((mesh.n_nodes, mesh.n_pressure))
        self._check(library().nsf_batch_finalize(self._h, int(autotune_rounds)))

    @property
    def count(self) -> int:
        return len(self.sizes)

    def step(self, n: int = 1):
        """n steps of every instance; returns int32 [n, count, 5] CG iterations."""
        it = np.zeros(max(n, 1) * self.count * 5, np.int32)
        self._check(library().nsf_batch_step(self._h, int(n), it.ctypes.data_as(_v)))
        return it[: n * self.count * 5].reshape(n, self.count, 5)

    def _index(self, index: int) -> int:
        if not 0 <= int(index) < self.count:
            raise NSFemError(5, f"instance index {index} out of range [0, {self.count})")
        return int(index)

    def fields(self, index: int):
        nv, npr = self.sizes[self._index(index)]
        uv, p = np.zeros(2 * nv), np.zeros(npr)
        self._check(library().nsf_batch_get_fields(self._h, int(index), uv.ctypes.data_as(_v), p.ctypes.data_as(_v)))
        return uv, p

    def set_fields(self, index: int, uv, p):
        nv, npr = self.sizes[self._index(index)]
        uv = np.ascontiguousarray(uv, np.float64)
        p = np.ascontiguousarray(p, np.float64)
        if uv.size != 2 * nv or p.size != npr:
            raise NSFemError(5, "field sizes do not match the instance")
        self._check(library().nsf_batch_set_fields(self._h, int(index), uv.ctypes.data_as(_v), p.ctypes.data_as(_v)))

    def plan(self):
        blocks = np.zeros(self.count, np.int32)
        grid, nt = _i(), _i()
        trials = np.zeros(64, np.float32)
        self._check(library().nsf_batch_plan(self._h, blocks.ctypes.data_as(_v), ctypes.byref(grid),
                                             trials.ctypes.data_as(_v), 64, ctypes.byref(nt)))
        return {"blocks": blocks, "grid_blocks": grid.value, "trial_ms": trials[: nt.value].tolist()}
