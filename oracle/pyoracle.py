"""ctypes binding of the CPU oracle (test infrastructure only).

Used by tests/ (as the checker), by __graft_entry__.smoke() and by the
CPU-baseline leg of bench.py. The product library never imports it.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")

FIELDS = [
    ("n_nodes", C.c_int64), ("n_panels", C.c_int64), ("n_links", C.c_int64), ("n_conductors", C.c_int32),
    ("node_type", C.c_void_p), ("node_left", C.c_void_p), ("node_right", C.c_void_p),
    ("node_leaf_first", C.c_void_p), ("node_leaf_count", C.c_void_p),
    ("node_vertices", C.c_void_p), ("node_centroid", C.c_void_p), ("node_normal", C.c_void_p),
    ("node_area", C.c_void_p), ("node_maxside", C.c_void_p),
    ("link_ptr", C.c_void_p), ("link_src", C.c_void_p), ("leaf_diel", C.c_void_p),
    ("cond_is_diel", C.c_void_p), ("cond_leaf_first", C.c_void_p), ("cond_leaf_count", C.c_void_p),
    ("cond_outperm", C.c_void_p), ("cond_inperm", C.c_void_p), ("cond_surf_ptr", C.c_void_p),
    ("cond_surf_outperm", C.c_void_p),
]

DTYPES = {
    "node_type": np.uint8, "node_left": np.int32, "node_right": np.int32, "node_leaf_first": np.int64,
    "node_leaf_count": np.int64, "node_vertices": np.float32, "node_centroid": np.float32, "node_normal": np.float32,
    "node_area": np.float64, "node_maxside": np.float64, "link_ptr": np.int64, "link_src": np.int32,
    "leaf_diel": np.uint8, "cond_is_diel": np.uint8, "cond_leaf_first": np.int64, "cond_leaf_count": np.int64,
    "cond_outperm": np.float64, "cond_inperm": np.float64, "cond_surf_ptr": np.int32, "cond_surf_outperm": np.float64,
}


class OrcModel(C.Structure):
    _fields_ = FIELDS


class OrcSuper(C.Structure):
    _fields_ = [("m", C.c_int32), ("elem_node", C.POINTER(C.c_int64)), ("sup_index", C.POINTER(C.c_int32)),
                ("area", C.POINTER(C.c_float)), ("dim", C.POINTER(C.c_double)), ("minv", C.POINTER(C.c_double))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("%s is missing: run fastercap_gb300.build.build() first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.orc_fill.argtypes = [C.POINTER(OrcModel), vp, vp, C.c_int]
        L.orc_fill.restype = None
        L.orc_matvec.argtypes = [C.POINTER(OrcModel), vp, vp, vp, vp, C.c_int]
        L.orc_matvec.restype = None
        L.orc_solve.argtypes = [C.POINTER(OrcModel), vp, vp, C.c_double, C.c_int, vp, vp, vp, C.c_int]
        L.orc_solve_ex.argtypes = [C.POINTER(OrcModel), vp, vp, C.c_double, C.c_int, C.c_uint, vp, vp, vp, C.c_int]
        L.orc_solve_rows.argtypes = [C.POINTER(OrcModel), vp, vp, C.c_double, C.c_int, C.c_uint, C.c_int, C.c_int, vp, vp,
                                     vp, C.c_int]
        L.orc_super_build.argtypes = [C.POINTER(OrcModel), C.c_uint, C.POINTER(OrcSuper)]
        L.orc_super_free.argtypes = [C.POINTER(OrcSuper)]
        L.orc_super_free.restype = None
        _lib = L
    return _lib


class Oracle:
    """CPU oracle over one model's arrays (a dict of numpy arrays)."""

    def __init__(self, arrays: dict, threads: int = 0):
        self.a = {k: np.ascontiguousarray(arrays[k], dtype=v) for k, v in DTYPES.items()}
        s = OrcModel()
        s.n_nodes = len(self.a["node_type"])
        s.n_panels = len(self.a["leaf_diel"])
        s.n_links = len(self.a["link_src"])
        s.n_conductors = len(self.a["cond_is_diel"])
        for k in DTYPES:
            setattr(s, k, self.a[k].ctypes.data)
        self.s = s
        self.threads = threads
        self.coef = None
        self.self_coef = None

    @property
    def n_panels(self):
        return int(self.s.n_panels)

    def fill(self):
        self.coef = np.empty(self.s.n_links, np.float64)
        self.self_coef = np.empty(self.s.n_panels, np.float64)
        lib().orc_fill(C.byref(self.s), self.coef.ctypes.data, self.self_coef.ctypes.data, self.threads)
        return self.coef, self.self_coef

    def matvec(self, q, coef=None, self_coef=None):
        coef = self.coef if coef is None else np.ascontiguousarray(coef, np.float64)
        sc = self.self_coef if self_coef is None else np.ascontiguousarray(self_coef, np.float64)
        q = np.ascontiguousarray(q, np.float64)
        v = np.empty_like(q)
        lib().orc_matvec(C.byref(self.s), coef.ctypes.data, sc.ctypes.data, q.ctypes.data, v.ctypes.data, self.threads)
        return v

    def super_build(self, dim):
        """The two-level preconditioner of dimension dim: (elements, leaf map, leaf areas, inverse matrix)."""
        sp = OrcSuper()
        m = lib().orc_super_build(C.byref(self.s), dim, C.byref(sp))
        out = None
        if m > 0:
            n = self.s.n_panels
            out = (np.ctypeslib.as_array(sp.elem_node, (m,)).copy(), np.ctypeslib.as_array(sp.sup_index, (n,)).copy(),
                   np.ctypeslib.as_array(sp.area, (n,)).copy(), np.ctypeslib.as_array(sp.minv, (m, m)).copy())
        lib().orc_super_free(C.byref(sp))
        return out

    def solve(self, tol=0.01, precond=1, coef=None, self_coef=None, super_dim=0):
        """precond: 0 none, 1 Jacobi, 2 two-level of dimension super_dim."""
        coef = self.coef if coef is None else np.ascontiguousarray(coef, np.float64)
        sc = self.self_coef if self_coef is None else np.ascontiguousarray(self_coef, np.float64)
        nc = int((self.a["cond_is_diel"] == 0).sum())
        cap = np.empty((nc, nc), np.float64)
        it = np.empty(nc, np.int32)
        ch = np.empty((nc, self.s.n_panels), np.float64)
        capped = lib().orc_solve_ex(C.byref(self.s), coef.ctypes.data, sc.ctypes.data, tol, precond, super_dim,
                                    cap.ctypes.data, it.ctypes.data, ch.ctypes.data, self.threads)
        return cap, it, ch, bool(capped)

    def solve_rows(self, row_first, row_count, tol=0.01, precond=1, coef=None, self_coef=None, super_dim=0):
        """Rows row_first .. row_first + row_count - 1 of the capacitance
        matrix (those conductors' solves only): (rows, iterations)."""
        coef = self.coef if coef is None else np.ascontiguousarray(coef, np.float64)
        sc = self.self_coef if self_coef is None else np.ascontiguousarray(self_coef, np.float64)
        nc = int((self.a["cond_is_diel"] == 0).sum())
        row_count = max(0, min(row_count, nc - row_first))
        cap = np.empty((row_count, nc), np.float64)
        it = np.empty(max(1, row_count), np.int32)
        lib().orc_solve_rows(C.byref(self.s), coef.ctypes.data, sc.ctypes.data, tol, precond, super_dim, row_first,
                             row_count, cap.ctypes.data, it.ctypes.data, None, self.threads)
        return cap, it[:row_count]
