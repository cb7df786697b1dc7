"""fastercap_gb300: GB300-native solve path for FasterCap input files.

Python binding over the C ABI of ``libfastercap_gb300.so``
(``include/fastercap_gb300.h``). The library is built in-tree by
``fastercap_gb300.build.build()``; importing this package never falls back to
another implementation: if the library is missing, :func:`lib` raises.

Typical use::

    import fastercap_gb300 as fc
    model = fc.Model.build("bus.txt", mesh_eps=0.01)
    with fc.Context() as ctx:
        prob = ctx.problem(model, precision=fc.PREC_MIXED)
        prob.fill()
        cap, iters = prob.solve(tol=1e-4)
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfastercap_gb300.so")

NORMAL_END = 0
GENERIC_ERROR = 1
COMMAND_LINE_ERROR = 64
CANNOT_OPEN_FILE = 66
OUT_OF_MEMORY = 71
FILE_ERROR = 74
USER_BREAK = 125
DEVICE_ERROR = 90
NOT_CONVERGED = 91

PRECOND_NONE = 0
PRECOND_JACOBI = 1
PRECOND_TWO_LEVEL = 2
PREC_FP64 = 0
PREC_MIXED = 1
# Krylov basis arithmetic of mixed-precision solves (FP64 problems: always FP64)
KRYLOV_PAIR, KRYLOV_FP64 = 0, 1

# element type bits
IS_LEAF, IS_DIEL, OUTPERM_NORMAL_DIR, IS_SUPER_NODE = 1, 2, 4, 128


class FCError(RuntimeError):
    """A C ABI call returned a non-zero FC_* status."""

    def __init__(self, code: int, msg: str):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


class BuildOptions(C.Structure):
    _fields_ = [("mesh_eps", C.c_double), ("eps_ratio", C.c_double), ("mesh_curv", C.c_double), ("verbose", C.c_int)]


class ModelArrays(C.Structure):
    _fields_ = [
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


class ModelInfo(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("n_panels", C.c_int64), ("n_links", C.c_int64), ("input_panels", C.c_int64),
                ("n_conductors", C.c_int32), ("n_dielectrics", C.c_int32), ("max_level", C.c_int32),
                ("max_mesh_eps", C.c_double), ("eps", C.c_double), ("mesh_eps", C.c_double)]


class ProblemStats(C.Structure):
    _fields_ = [("kernel_launches", C.c_int64), ("link_launches", C.c_int64), ("link_ms", C.c_double),
                ("link_bytes", C.c_int64), ("fill_ms", C.c_double), ("solve_ms", C.c_double),
                ("refine_checks", C.c_int64), ("refine_cycles", C.c_int64), ("fill_fp64", C.c_int64),
                ("rhs_width", C.c_int64)]


class SolveOptions(C.Structure):
    _fields_ = [("tol", C.c_double), ("precond", C.c_int), ("max_iter", C.c_int), ("rhs_width", C.c_int),
                ("precond_dim", C.c_int), ("refine", C.c_int), ("krylov", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("memory_budget", C.c_int64), ("iterations_hint", C.c_int)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("status", C.c_int), ("n_cond", C.c_int), ("iterations_max", C.c_int),
                ("slot", C.c_int), ("footprint_bytes", C.c_int64), ("device_bytes", C.c_int64),
                ("queue_ms", C.c_double), ("run_ms", C.c_double), ("fill_ms", C.c_double), ("solve_ms", C.c_double),
                ("kernel_launches", C.c_int64), ("build_ms", C.c_double), ("n_panels", C.c_int64),
                ("n_links", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [("slots", C.c_int), ("running", C.c_int), ("queued", C.c_int), ("max_running", C.c_int),
                ("budget", C.c_int64), ("in_use", C.c_int64), ("peak_in_use", C.c_int64),
                ("submitted", C.c_int64), ("completed", C.c_int64)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_CANCELLED = 0, 1, 2, 3


# (field, dtype, length key, columns)
ARRAY_FIELDS = [
    ("node_type", np.uint8, "n_nodes", 1), ("node_left", np.int32, "n_nodes", 1), ("node_right", np.int32, "n_nodes", 1),
    ("node_leaf_first", np.int64, "n_nodes", 1), ("node_leaf_count", np.int64, "n_nodes", 1),
    ("node_vertices", np.float32, "n_nodes", 9), ("node_centroid", np.float32, "n_nodes", 3),
    ("node_normal", np.float32, "n_nodes", 3), ("node_area", np.float64, "n_nodes", 1),
    ("node_maxside", np.float64, "n_nodes", 1), ("link_ptr", np.int64, "n_nodes+1", 1),
    ("link_src", np.int32, "n_links", 1), ("leaf_diel", np.uint8, "n_panels", 1),
    ("cond_is_diel", np.uint8, "n_conductors", 1), ("cond_leaf_first", np.int64, "n_conductors", 1),
    ("cond_leaf_count", np.int64, "n_conductors", 1), ("cond_outperm", np.float64, "n_conductors", 1),
    ("cond_inperm", np.float64, "n_conductors", 1), ("cond_surf_ptr", np.int32, "n_conductors+1", 1),
]

_lib = None


def lib() -> C.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("%s is missing: run fastercap_gb300.build.build() first" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dp, ip = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.fcg_model_build.argtypes = [C.c_char_p, C.POINTER(BuildOptions), C.POINTER(vp), C.c_char_p, C.c_size_t]
    L.fcg_model_build_on.argtypes = [vp, C.c_char_p, C.POINTER(BuildOptions), C.POINTER(vp), C.c_char_p, C.c_size_t]
    L.fcg_model_info_get.argtypes = [vp, C.POINTER(ModelInfo)]
    L.fcg_model_arrays_get.argtypes = [vp, C.POINTER(ModelArrays)]
    L.fcg_model_conductor_name.argtypes = [vp, i32]
    L.fcg_model_conductor_name.restype = C.c_char_p
    L.fcg_model_free.argtypes = [vp]
    L.fcg_model_free.restype = None
    L.fcg_context_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.fcg_context_destroy.argtypes = [vp]
    L.fcg_context_destroy.restype = None
    L.fcg_last_error.restype = C.c_char_p
    L.fcg_problem_create.argtypes = [vp, C.POINTER(ModelArrays), C.c_int, C.POINTER(vp)]
    L.fcg_problem_create_on_stream.argtypes = [vp, C.POINTER(ModelArrays), C.c_int, vp, C.POINTER(vp)]
    L.fcg_context_stream.argtypes = [vp]
    L.fcg_context_stream.restype = vp
    L.fcg_problem_set_profiling.argtypes = [vp, C.c_int]
    L.fcg_problem_set_tuning.argtypes = [vp, C.c_int]
    L.fcg_problem_get_stats.argtypes = [vp, C.POINTER(ProblemStats)]
    L.fcg_problem_reset_stats.argtypes = [vp]
    L.fcg_problem_destroy.argtypes = [vp]
    L.fcg_problem_destroy.restype = None
    L.fcg_problem_device_bytes.argtypes = [vp]
    L.fcg_problem_device_bytes.restype = i64
    L.fcg_problem_fill.argtypes = [vp]
    L.fcg_problem_get_coefficients.argtypes = [vp, vp, vp]
    L.fcg_problem_matvec.argtypes = [vp, vp, vp, C.c_int]
    L.fcg_problem_matvec_device.argtypes = [vp, vp, vp, C.c_int]
    L.fcg_problem_matvec_device_noalloc.argtypes = [vp, vp, vp, C.c_int]
    L.fcg_problem_solve.argtypes = [vp, C.POINTER(SolveOptions), vp, vp]
    L.fcg_problem_get_charges.argtypes = [vp, vp]
    L.fcg_run_command_line.argtypes = [C.c_char_p]
    L.fcg_model_concat.argtypes = [C.POINTER(vp), i32, C.POINTER(vp), vp]
    L.fcg_problem_cancel.argtypes = [vp]
    L.fcg_model_arrays_check.argtypes = [C.POINTER(ModelArrays)]
    L.fcg_problem_estimate_bytes.argtypes = [C.POINTER(ModelArrays), C.c_int, C.c_int, C.c_int]
    L.fcg_problem_estimate_bytes.restype = i64
    L.fcg_server_create.argtypes = [vp, C.POINTER(ServerConfig), C.POINTER(vp)]
    L.fcg_server_destroy.argtypes = [vp]
    L.fcg_server_destroy.restype = None
    L.fcg_server_submit.argtypes = [vp, C.POINTER(ModelArrays), C.c_int, C.POINTER(SolveOptions), C.POINTER(i64)]
    L.fcg_server_submit_file.argtypes = [vp, C.c_char_p, C.POINTER(BuildOptions), C.c_int, C.POINTER(SolveOptions),
                                         C.POINTER(i64)]
    L.fcg_server_wait.argtypes = [vp, i64, C.POINTER(JobInfo)]
    L.fcg_server_poll.argtypes = [vp, i64, C.POINTER(JobInfo)]
    L.fcg_server_result.argtypes = [vp, i64, vp, vp, C.POINTER(JobInfo)]
    L.fcg_server_cancel.argtypes = [vp, i64]
    L.fcg_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
    L.fcg_problem_set_geometries.argtypes = [vp, i32, vp]
    _lib = L
    return L


def last_error() -> str:
    return lib().fcg_last_error().decode(errors="replace")


def _check(code: int, what: str):
    if code != NORMAL_END:
        raise FCError(code, "%s: %s" % (what, last_error()))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class _NativeModel:
    """Owner of a native model: freed when the last view of its arrays (and
    the Model) is gone."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        try:
            if self.h is not None:
                lib().fcg_model_free(self.h)
                self.h = None
        except Exception:
            pass


class Model:
    """A refined panel hierarchy with its links (host memory).

    ``arrays`` holds numpy views (or owned copies for models made from
    arrays) of the flattened layout described in ``include/fastercap_gb300.h``;
    a view keeps the native model alive, so the arrays stay valid after the
    Model itself is closed or dropped.
    """

    def __init__(self, handle, arrays: dict, names: list, info: dict, owner=None):
        self._h = handle
        self._owner = owner
        self.arrays = arrays
        self.names = names
        self.info = info
        self._keep = None

    @classmethod
    def build(cls, path: str, mesh_eps: float = 0.1, eps_ratio: float = 1.0, mesh_curv: float = 3.0,
              verbose: bool = False, ctx: "Context" = None) -> "Model":
        """Build the refined hierarchy and the links of a FastCap-format file.
        With a Context the link construction runs on its GPU; the model is
        the same, link order included."""
        L = lib()
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        opt = BuildOptions(mesh_eps, eps_ratio, mesh_curv, 1 if verbose else 0)
        if ctx is not None:
            code = L.fcg_model_build_on(ctx._h, os.fsencode(path), C.byref(opt), C.byref(h), err, 512)
        else:
            code = L.fcg_model_build(os.fsencode(path), C.byref(opt), C.byref(h), err, 512)
        if code != NORMAL_END:
            raise FCError(code, "model build failed: " + err.value.decode(errors="replace"))
        return cls._from_handle(h)

    @classmethod
    def from_arrays(cls, arrays: dict, names=None) -> "Model":
        """Wrap externally produced arrays (e.g. a golden fixture) without a native handle."""
        own = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        info = {"n_nodes": len(own["node_type"]), "n_panels": len(own["leaf_diel"]), "n_links": len(own["link_src"]),
                "n_conductors": len(own["cond_is_diel"])}
        return cls(None, own, names or ["c%d" % i for i in range(info["n_conductors"])], info)

    @classmethod
    def concat(cls, models) -> tuple:
        """Concatenate independent geometries into one model (a forest with no
        link between geometries). Returns (model, geometry_of_conductor).
        Models built from files go through fcg_model_concat; models made from
        arrays are concatenated here with the same layout."""
        models = list(models)
        if not models:
            raise ValueError("no models to concatenate")
        ncond = sum(len(m.arrays["cond_is_diel"]) for m in models)
        if all(m._h is not None for m in models):
            L = lib()
            hs = (C.c_void_p * len(models))(*[m._h for m in models])
            h = C.c_void_p()
            geom = np.empty(ncond, np.int32)
            _check(L.fcg_model_concat(hs, len(models), C.byref(h), _ptr(geom)), "model concat")
            tmp = cls._from_handle(h)
            return tmp, geom
        return cls._concat_arrays(models)

    @classmethod
    def _from_handle(cls, h) -> "Model":
        L = lib()
        info_s = ModelInfo()
        _check(L.fcg_model_info_get(h, C.byref(info_s)), "model info")
        info = {f: getattr(info_s, f) for f, _ in ModelInfo._fields_}
        a = ModelArrays()
        _check(L.fcg_model_arrays_get(h, C.byref(a)), "model arrays")
        counts = {"n_nodes": a.n_nodes, "n_nodes+1": a.n_nodes + 1, "n_links": a.n_links, "n_panels": a.n_panels,
                  "n_conductors": a.n_conductors, "n_conductors+1": a.n_conductors + 1}
        owner = _NativeModel(h)
        arrays = {}
        for name, dt, key, cols in ARRAY_FIELDS:
            n = counts[key] * cols
            addr = getattr(a, name)
            if n == 0 or not addr:
                arrays[name] = np.zeros((0,) if cols == 1 else (0, cols), dtype=dt)
                continue
            buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(addr)
            buf._owner = owner  # the view's buffer keeps the native model alive
            arr = np.frombuffer(buf, dtype=dt, count=n)
            arrays[name] = arr.reshape(-1, cols) if cols > 1 else arr
        nsurf = int(arrays["cond_surf_ptr"][-1])
        buf = (C.c_char * (max(nsurf, 1) * 8)).from_address(a.cond_surf_outperm)
        buf._owner = owner
        arrays["cond_surf_outperm"] = np.frombuffer(buf, dtype=np.float64, count=max(nsurf, 1))
        names = [L.fcg_model_conductor_name(h, i).decode() for i in range(a.n_conductors)]
        return cls(h, arrays, names, info, owner)

    @classmethod
    def _concat_arrays(cls, models) -> tuple:
        out = {}
        node_off = leaf_off = link_off = surf_off = 0
        parts = {k: [] for k, _, _, _ in ARRAY_FIELDS}
        parts["cond_surf_outperm"] = []
        geom, names = [], []
        for g, m in enumerate(models):
            a = m.arrays
            nn, npan, nl = m.n_nodes, m.n_panels, m.n_links
            nc = len(a["cond_is_diel"])
            for k in ("node_type", "node_leaf_count", "node_vertices", "node_centroid", "node_normal", "node_area",
                      "node_maxside", "leaf_diel", "cond_is_diel", "cond_leaf_count", "cond_outperm", "cond_inperm"):
                parts[k].append(np.asarray(a[k]))
            for k in ("node_left", "node_right"):
                v = np.asarray(a[k]).astype(np.int32)
                parts[k].append(np.where(v >= 0, v + node_off, -1).astype(np.int32))
            parts["node_leaf_first"].append(np.asarray(a["node_leaf_first"]) + leaf_off)
            lp = np.asarray(a["link_ptr"])
            parts["link_ptr"].append((lp[:-1] if g < len(models) - 1 else lp) + link_off)
            parts["link_src"].append((np.asarray(a["link_src"]) + node_off).astype(np.int32))
            parts["cond_leaf_first"].append(np.asarray(a["cond_leaf_first"]) + leaf_off)
            sp = np.asarray(a["cond_surf_ptr"])
            parts["cond_surf_ptr"].append((sp[:-1] if g < len(models) - 1 else sp) + surf_off)
            parts["cond_surf_outperm"].append(np.asarray(a["cond_surf_outperm"])[: int(sp[-1])])
            geom += [g] * nc
            names += list(m.names)
            node_off += nn
            leaf_off += npan
            link_off += nl
            surf_off += int(sp[-1])
        for k, dt, _, _ in ARRAY_FIELDS:
            out[k] = np.ascontiguousarray(np.concatenate(parts[k]).astype(dt, copy=False))
        out["cond_surf_outperm"] = np.concatenate(parts["cond_surf_outperm"]).astype(np.float64)
        return cls.from_arrays(out, names), np.asarray(geom, np.int32)

    @property
    def n_panels(self) -> int:
        return int(len(self.arrays["leaf_diel"]))

    @property
    def n_links(self) -> int:
        return int(len(self.arrays["link_src"]))

    @property
    def n_nodes(self) -> int:
        return int(len(self.arrays["node_type"]))

    @property
    def conductor_names(self):
        return [n for n, d in zip(self.names, self.arrays["cond_is_diel"]) if not d]

    def c_arrays(self) -> ModelArrays:
        a = ModelArrays()
        a.n_nodes, a.n_panels, a.n_links = self.n_nodes, self.n_panels, self.n_links
        a.n_conductors = len(self.arrays["cond_is_diel"])
        keep = []
        for name, dt, _, _ in ARRAY_FIELDS + [("cond_surf_outperm", np.float64, None, 1)]:
            arr = np.ascontiguousarray(self.arrays[name], dtype=dt)
            keep.append(arr)
            setattr(a, name, arr.ctypes.data)
        self._keep = keep
        return a

    def check(self):
        """Structural checks of the arrays (no device needed); raises FCError."""
        arr = self.c_arrays()
        _check(lib().fcg_model_arrays_check(C.byref(arr)), "model check")

    def close(self):
        """Drop this Model's hold on the native model (its memory goes with
        the last view of its arrays)."""
        self._h = None
        self._owner = None


class Problem:
    """A model resident on the GPU (links, coefficients, sweep plan, Krylov workspace)."""

    def __init__(self, ctx: "Context", model: Model, precision: int, stream=None):
        self.model = model
        self._ctx = ctx  # the context outlives its problems
        self.precision = precision
        self.n_panels = model.n_panels
        self.n_links = model.n_links
        self.n_cond = len(model.conductor_names)
        h = C.c_void_p()
        arr = model.c_arrays()
        st = C.c_void_p(stream) if stream is not None else C.c_void_p(lib().fcg_context_stream(ctx._h))
        _check(lib().fcg_problem_create_on_stream(ctx._h, C.byref(arr), precision, st, C.byref(h)), "problem create")
        self._h = h
        self.geometries = None  # per-geometry column counts once set_geometries ran

    def set_geometries(self, geometry_of_conductor):
        """Declare independent geometries (conductor -> geometry index, as
        Model.concat returns it): every geometry gets its own GMRES solves."""
        geom = np.ascontiguousarray(geometry_of_conductor, dtype=np.int32)
        ng = int(geom.max()) + 1 if len(geom) else 0
        _check(lib().fcg_problem_set_geometries(self._h, ng, _ptr(geom)), "set geometries")
        diel = np.asarray(self.model.arrays["cond_is_diel"]) != 0
        self.geometries = [int(np.sum((geom == g) & ~diel)) for g in range(ng)]

    def set_tuning(self, on: bool):
        """Measure launch shapes and the right-hand-side width on first use (default on)."""
        _check(lib().fcg_problem_set_tuning(self._h, 1 if on else 0), "set_tuning")

    def set_profiling(self, on: bool):
        _check(lib().fcg_problem_set_profiling(self._h, 1 if on else 0), "profiling")

    def stats(self) -> dict:
        st = ProblemStats()
        _check(lib().fcg_problem_get_stats(self._h, C.byref(st)), "stats")
        return {f: getattr(st, f) for f, _ in ProblemStats._fields_}

    def reset_stats(self):
        _check(lib().fcg_problem_reset_stats(self._h), "reset stats")

    @property
    def device_bytes(self) -> int:
        return int(lib().fcg_problem_device_bytes(self._h))

    def fill(self):
        _check(lib().fcg_problem_fill(self._h), "coefficient fill")

    def coefficients(self):
        lc = np.empty(self.n_links, np.float64)
        sc = np.empty(self.n_panels, np.float64)
        _check(lib().fcg_problem_get_coefficients(self._h, _ptr(lc), _ptr(sc)), "get coefficients")
        return lc, sc

    def matvec(self, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float64)
        single = q.ndim == 1
        q2 = q.reshape(1, -1) if single else q
        v = np.empty_like(q2)
        _check(lib().fcg_problem_matvec(self._h, _ptr(q2), _ptr(v), q2.shape[0]), "matvec")
        return v[0] if single else v

    def matvec_device(self, q_ptr: int, v_ptr: int, k: int):
        _check(lib().fcg_problem_matvec_device(self._h, C.c_void_p(q_ptr), C.c_void_p(v_ptr), k), "matvec")

    def matvec_device_noalloc(self, q_ptr: int, v_ptr: int, k: int) -> int:
        """The product without any device allocation (fixed per-GPU scratch);
        returns the FC_* status instead of raising."""
        return int(lib().fcg_problem_matvec_device_noalloc(self._h, C.c_void_p(q_ptr), C.c_void_p(v_ptr), k))

    def solve(self, tol: float = 0.01, precond: int = PRECOND_JACOBI, max_iter: int = 0, allow_not_converged=False,
              rhs_width: int = 0, precond_dim: int = 0, refine: int = 0, krylov: int = KRYLOV_PAIR):
        """(C, iterations); with geometries set, lists of per-geometry C and iterations.
        refine: true-residual restarts (0 default: up to 2 in mixed precision, -1 none).
        krylov: mixed precision's basis arithmetic, KRYLOV_PAIR (FP32 pairs) or KRYLOV_FP64."""
        sizes = self.geometries or [self.n_cond]
        cap = np.empty(sum(n * n for n in sizes), np.float64)
        it = np.empty(sum(sizes), np.int32)
        opt = SolveOptions(tol, precond, max_iter, rhs_width, precond_dim, refine, krylov)
        code = lib().fcg_problem_solve(self._h, C.byref(opt), _ptr(cap), _ptr(it))
        self._last_width = int(self.stats()["rhs_width"]) or 32  # the width the solve used
        if not (code == NORMAL_END or (allow_not_converged and code == NOT_CONVERGED)):
            _check(code, "solve")
        caps, its, oc, oi = [], [], 0, 0
        for n in sizes:
            caps.append(cap[oc:oc + n * n].reshape(n, n))
            its.append(it[oi:oi + n])
            oc += n * n
            oi += n
        if self.geometries is None:
            return caps[0], its[0]
        return caps, its

    def cancel(self):
        """Stop a running (or the next) solve at its next Arnoldi step (FCError USER_BREAK)."""
        _check(lib().fcg_problem_cancel(self._h), "cancel")

    def charges(self) -> np.ndarray:
        """Charges of the last batch of right-hand-side columns, [k][n_panels]."""
        ks = max(self.geometries or [self.n_cond])
        w = getattr(self, "_last_width", 32)
        k = ks - w * ((ks - 1) // w)
        x = np.empty((k, self.n_panels), np.float64)
        _check(lib().fcg_problem_get_charges(self._h, _ptr(x)), "get charges")
        return x

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().fcg_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One GPU."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib().fcg_context_create(device, C.byref(h)), "context create")
        self._h = h

    @property
    def stream(self) -> int:
        """The context's default cudaStream_t (as an integer handle)."""
        return int(lib().fcg_context_stream(self._h) or 0)

    def problem(self, model: Model, precision: int = PREC_MIXED, stream=None) -> Problem:
        return Problem(self, model, precision, stream)

    def server(self, slots: int = 4, memory_budget: int = 0, iterations_hint: int = 0) -> "Server":
        return Server(self, slots, memory_budget, iterations_hint)

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().fcg_context_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def estimate_bytes(model: Model, precision: int = PREC_MIXED, rhs: int = 0, iterations: int = 64) -> int:
    """Device bytes of a problem of this model after a solve (the server's admission footprint)."""
    arr = model.c_arrays()
    return int(lib().fcg_problem_estimate_bytes(C.byref(arr), precision, rhs or len(model.conductor_names), iterations))


class Job:
    """A submitted extraction; result() waits for it."""

    def __init__(self, server: "Server", jid: int, model, arrays):
        self.server, self.id, self.model = server, jid, model
        self._arrays = arrays  # the C view must outlive the job
        # a file job's matrix size is known once it is done
        self.n_cond = len(model.conductor_names) if model is not None else None
        self.info = None
        self.status = None

    def wait(self) -> dict:
        """Block until the job is done or cancelled; its description."""
        info = JobInfo()
        _check(lib().fcg_server_wait(self.server._h, self.id, C.byref(info)), "wait")
        return {f: getattr(info, f) for f, _ in JobInfo._fields_}

    def poll(self) -> dict:
        info = JobInfo()
        _check(lib().fcg_server_poll(self.server._h, self.id, C.byref(info)), "poll")
        return {f: getattr(info, f) for f, _ in JobInfo._fields_}

    def cancel(self):
        _check(lib().fcg_server_cancel(self.server._h, self.id), "cancel")

    def result(self, allow_not_converged=False):
        """(C, iterations); raises FCError if the job failed or was cancelled."""
        if self.n_cond is None:
            self.n_cond = int(self.wait()["n_cond"])
        cap = np.empty((self.n_cond, self.n_cond), np.float64)
        it = np.empty(self.n_cond, np.int32)
        info = JobInfo()
        code = lib().fcg_server_result(self.server._h, self.id, _ptr(cap), _ptr(it), C.byref(info))
        self.info = {f: getattr(info, f) for f, _ in JobInfo._fields_}
        self.status = code
        self._arrays = None
        if not (code == NORMAL_END or (allow_not_converged and code == NOT_CONVERGED)):
            _check(code, "job %d" % self.id)
        return cap, it


class Server:
    """Continuous-admission extraction server on one GPU (fcg_server_*)."""

    def __init__(self, ctx: "Context", slots: int = 4, memory_budget: int = 0, iterations_hint: int = 0):
        self._ctx = ctx
        h = C.c_void_p()
        cfg = ServerConfig(slots, memory_budget, iterations_hint)
        _check(lib().fcg_server_create(ctx._h, C.byref(cfg), C.byref(h)), "server create")
        self._h = h

    def submit(self, model: Model, precision: int = PREC_MIXED, tol: float = 0.01, precond: int = PRECOND_JACOBI,
               max_iter: int = 0, rhs_width: int = 0, precond_dim: int = 0, refine: int = 0,
               krylov: int = KRYLOV_PAIR) -> Job:
        arr = model.c_arrays()
        keep = model._keep
        opt = SolveOptions(tol, precond, max_iter, rhs_width, precond_dim, refine, krylov)
        jid = C.c_int64()
        _check(lib().fcg_server_submit(self._h, C.byref(arr), precision, C.byref(opt), C.byref(jid)), "submit")
        job = Job(self, jid.value, model, (arr, keep))
        return job

    def submit_file(self, path: str, precision: int = PREC_MIXED, tol: float = 0.01, mesh_eps: float = 0.1,
                    eps_ratio: float = 1.0, mesh_curv: float = 3.0, precond: int = PRECOND_JACOBI, max_iter: int = 0,
                    rhs_width: int = 0, precond_dim: int = 0, refine: int = 0, krylov: int = KRYLOV_PAIR) -> Job:
        """An extraction request from an input file: the slot builds its
        model on the GPU (switches -m, -d, -mc), then solves it."""
        bo = BuildOptions(mesh_eps, eps_ratio, mesh_curv, 0)
        opt = SolveOptions(tol, precond, max_iter, rhs_width, precond_dim, refine, krylov)
        jid = C.c_int64()
        _check(lib().fcg_server_submit_file(self._h, os.fsencode(path), C.byref(bo), precision, C.byref(opt),
                                            C.byref(jid)), "submit_file")
        return Job(self, jid.value, None, None)

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().fcg_server_get_stats(self._h, C.byref(st)), "server stats")
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().fcg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_command_line(cmd: str) -> int:
    """Run the headless console (reference command-line switches)."""
    return int(lib().fcg_run_command_line(cmd.encode()))
