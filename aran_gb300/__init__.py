"""aran_gb300 -- GB300-native FMM behind LibAran's 3D solver interface.

Python mirror of the reference's ``AranSolver3d`` (aran/aransolver3d.h:68-170)
on top of the C ABI of ``libaran_gpu.so`` (declared in include/aran_gpu.h).
Everything computes on the GPU; when the CUDA library or a device is missing,
the calls raise instead of falling back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libaran_gpu.so")

FLAVOUR_NORMAL, FLAVOUR_KKYLIN, FLAVOUR_ROTATE = 0, 1, 2
FLAVOURS = {"normal": 0, "kkylin": 1, "rotate": 2}
PRECISIONS = {"fp64": 0, "mixed": 1}
MEM_HOST, MEM_DEVICE = 0, 1
STAT_NAMES = ("zero", "p2p", "p2m", "m2m", "m2l", "l2l", "l2p", "p2l", "m2p",
              "p2p_remote", "m2l_remote")
STAGE_NAMES = ("total", "sort", "tree", "lists", "p2m", "m2m", "m2l", "l2l", "l2p",
               "p2p", "h2d", "d2h", "semifar_p2l", "semifar_m2p")

# exported symbols of include/aran_gpu.h
EXPORTS = (
    "aran_gpu_solver3d_create", "aran_gpu_solver3d_destroy", "aran_gpu_solver3d_solve",
    "aran_gpu_solver3d_solve_forest",
    "aran_gpu_solver3d_get_stats", "aran_gpu_solver3d_tree_info",
    "aran_gpu_solver3d_tree_lists", "aran_gpu_solver3d_expansions",
    "aran_gpu_solver3d_timings", "aran_gpu_solver3d_launches", "aran_gpu_last_error",
    "aran_gpu_version", "aran_gpu_p2p_direct_noalloc", "aran_gpu_footprint_bytes",
    "aran_gpu_server_create", "aran_gpu_server_submit", "aran_gpu_server_wait",
    "aran_gpu_server_cancel", "aran_gpu_server_destroy",
    "aran_gpu_solver2d_create", "aran_gpu_solver2d_destroy", "aran_gpu_solver2d_solve",
    "aran_gpu_solver2d_get_stats", "aran_gpu_solver2d_timings", "aran_gpu_solver2d_tree_info",
    "aran_gpu_solver2d_launches", "aran_gpu_solver3d_set_fp64_root_depth",
    "aran_gpu_plan_for_tolerance", "aran_gpu_solver3d_set_leaf_predicate",
    "aran_gpu_solver3d_set_m2l_kernel", "aran_gpu_autotune3d", "aran_gpu_tune_lookup",
)

M2L_KERNELS = {"auto": 0, "lanes": 1, "sibling": 2, "tc": 3}


class AranError(RuntimeError):
    """Raised for every non-zero status of the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"aran_gpu error {code}: {msg}")
        self.code = code


class Config3d(C.Structure):
    _fields_ = [("lb", C.c_double * 3), ("ub", C.c_double * 3), ("maxbox", C.c_int),
                ("order", C.c_int), ("flavour", C.c_int), ("field", C.c_int),
                ("precision", C.c_int), ("max_depth", C.c_int), ("semifar_threshold", C.c_int)]


class Config2d(C.Structure):
    _fields_ = [("maxbox", C.c_int), ("order", C.c_int), ("max_depth", C.c_int),
                ("precision", C.c_int)]


class NodeView(C.Structure):
    """AranGpuNodeView: a node about to be split, as a leaf predicate sees it."""
    _fields_ = [("center", C.c_double * 3), ("lbound", C.c_double * 3),
                ("ubound", C.c_double * 3), ("point_count", C.c_int64), ("depth", C.c_int)]


LEAF_PREDICATE = C.CFUNCTYPE(C.c_int, C.POINTER(NodeView), C.c_void_p)


class Request3d(C.Structure):
    _fields_ = [("cfg", Config3d), ("n", C.c_int64), ("xyz", C.c_void_p), ("q", C.c_void_p),
                ("pot", C.c_void_p), ("field", C.c_void_p), ("tolerance", C.c_double)]


class TuneResult(C.Structure):
    _fields_ = [("maxbox", C.c_int), ("m2l_kernel", C.c_int), ("m2l_nst", C.c_int),
                ("m2l_g", C.c_int), ("ms", C.c_double), ("candidates", C.c_int)]


def _tune_dict(r: "TuneResult") -> dict:
    inv = {v: k for k, v in M2L_KERNELS.items()}
    return {"maxbox": r.maxbox, "m2l_kernel": inv.get(r.m2l_kernel, r.m2l_kernel),
            "m2l_nst": r.m2l_nst, "m2l_g": r.m2l_g, "ms": r.ms, "candidates": r.candidates}


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("end_s", C.c_double), ("slot", C.c_int), ("footprint_bytes", C.c_int64),
                ("order", C.c_int), ("precision", C.c_int)]


_lib = None


def load(build_if_missing: bool = True):
    """Load libaran_gpu.so (building it in-tree when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"{LIB_PATH} is missing; run __graft_entry__.build()")
        from . import _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    i64p = C.POINTER(C.c_int64)
    L.aran_gpu_solver3d_create.argtypes = [C.POINTER(Config3d), C.POINTER(vp)]
    L.aran_gpu_solver3d_create.restype = C.c_int
    L.aran_gpu_solver3d_destroy.argtypes = [vp]
    L.aran_gpu_solver3d_destroy.restype = None
    L.aran_gpu_solver3d_solve.argtypes = [vp, C.c_int64, vp, vp, vp, vp, C.c_int]
    L.aran_gpu_solver3d_solve.restype = C.c_int
    L.aran_gpu_solver3d_solve_forest.argtypes = [vp, C.c_int, i64p, dp, vp, vp, vp, vp, C.c_int]
    L.aran_gpu_solver3d_solve_forest.restype = C.c_int
    L.aran_gpu_solver3d_set_m2l_kernel.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.aran_gpu_solver3d_set_m2l_kernel.restype = C.c_int
    L.aran_gpu_autotune3d.argtypes = [C.POINTER(Config3d), C.c_int64, vp, vp, C.c_int,
                                      C.POINTER(C.c_int), C.c_int, C.c_int, C.c_char_p,
                                      C.POINTER(TuneResult)]
    L.aran_gpu_autotune3d.restype = C.c_int
    L.aran_gpu_tune_lookup.argtypes = [C.c_char_p, C.POINTER(Config3d), C.POINTER(TuneResult)]
    L.aran_gpu_tune_lookup.restype = C.c_int
    L.aran_gpu_solver3d_get_stats.argtypes = [vp, i64p]
    L.aran_gpu_solver3d_get_stats.restype = C.c_int
    L.aran_gpu_solver3d_tree_info.argtypes = [vp, i64p]
    L.aran_gpu_solver3d_tree_info.restype = C.c_int
    L.aran_gpu_solver3d_tree_lists.argtypes = [vp] * 8
    L.aran_gpu_solver3d_tree_lists.restype = C.c_int
    L.aran_gpu_solver3d_expansions.argtypes = [vp, dp, dp]
    L.aran_gpu_solver3d_expansions.restype = C.c_int
    L.aran_gpu_solver3d_timings.argtypes = [vp, dp]
    L.aran_gpu_solver3d_timings.restype = C.c_int
    L.aran_gpu_solver3d_launches.argtypes = [vp]
    L.aran_gpu_solver3d_launches.restype = C.c_int64
    L.aran_gpu_solver3d_set_leaf_predicate.argtypes = [vp, vp, vp]
    L.aran_gpu_solver3d_set_leaf_predicate.restype = C.c_int
    L.aran_gpu_solver3d_set_fp64_root_depth.argtypes = [vp, C.c_int]
    L.aran_gpu_solver3d_set_fp64_root_depth.restype = C.c_int
    L.aran_gpu_p2p_direct_noalloc.argtypes = [C.c_int64, vp, vp, vp, vp]
    L.aran_gpu_p2p_direct_noalloc.restype = C.c_int
    L.aran_gpu_footprint_bytes.argtypes = [C.POINTER(Config3d), C.c_int64]
    L.aran_gpu_footprint_bytes.restype = C.c_int64
    L.aran_gpu_plan_for_tolerance.argtypes = [C.c_double, C.POINTER(Config3d)]
    L.aran_gpu_plan_for_tolerance.restype = C.c_double
    L.aran_gpu_server_create.argtypes = [C.c_int, C.c_double, C.POINTER(vp)]
    L.aran_gpu_server_create.restype = C.c_int
    L.aran_gpu_server_submit.argtypes = [vp, C.POINTER(Request3d), C.POINTER(C.c_int64)]
    L.aran_gpu_server_submit.restype = C.c_int
    L.aran_gpu_server_wait.argtypes = [vp, C.c_int64, C.c_double, C.POINTER(RequestInfo)]
    L.aran_gpu_server_wait.restype = C.c_int
    L.aran_gpu_server_cancel.argtypes = [vp, C.c_int64]
    L.aran_gpu_server_cancel.restype = C.c_int
    L.aran_gpu_server_destroy.argtypes = [vp]
    L.aran_gpu_server_destroy.restype = None
    L.aran_gpu_solver2d_create.argtypes = [C.POINTER(Config2d), C.POINTER(vp)]
    L.aran_gpu_solver2d_create.restype = C.c_int
    L.aran_gpu_solver2d_destroy.argtypes = [vp]
    L.aran_gpu_solver2d_destroy.restype = None
    L.aran_gpu_solver2d_solve.argtypes = [vp, C.c_int, i64p, dp, vp, vp, vp, C.c_int]
    L.aran_gpu_solver2d_solve.restype = C.c_int
    for f in (L.aran_gpu_solver2d_get_stats, L.aran_gpu_solver2d_tree_info):
        f.argtypes = [vp, i64p]
        f.restype = C.c_int
    L.aran_gpu_solver2d_timings.argtypes = [vp, dp]
    L.aran_gpu_solver2d_timings.restype = C.c_int
    L.aran_gpu_solver2d_launches.argtypes = [vp]
    L.aran_gpu_solver2d_launches.restype = C.c_int64
    L.aran_gpu_last_error.restype = C.c_char_p
    L.aran_gpu_version.restype = C.c_char_p
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise AranError(rc, load().aran_gpu_last_error().decode())


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def make_config(lbound=(0.0, 0.0, 0.0), ubound=(1.0, 1.0, 1.0), *, maxbox=64, order=12,
                flavour="rotate", field=True, precision="fp64", max_depth=21,
                semifar_threshold=0) -> Config3d:
    cfg = Config3d()
    for k in range(3):
        cfg.lb[k], cfg.ub[k] = float(lbound[k]), float(ubound[k])
    cfg.maxbox, cfg.order = int(maxbox), int(order)
    cfg.flavour = FLAVOURS[flavour] if isinstance(flavour, str) else int(flavour)
    cfg.field = int(bool(field))
    cfg.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    cfg.max_depth = int(max_depth)
    cfg.semifar_threshold = int(semifar_threshold)
    return cfg


def plan_for_tolerance(tol: float, order: int = 0) -> tuple[int, str, float]:
    """(order, precision, estimated error) the request loop picks for a
    requested relative L2 potential error (order > 0: only the precision)."""
    cfg = make_config(order=order)
    est = load().aran_gpu_plan_for_tolerance(float(tol), C.byref(cfg))
    if est < 0:
        raise AranError(-1, load().aran_gpu_last_error().decode())
    return cfg.order, ("mixed" if cfg.precision == PRECISIONS["mixed"] else "fp64"), est


def autotune(xyz, q, *, maxboxes=None, reps=3, db_path=None, **cfg_kw) -> dict:
    """Times every leaf capacity of maxboxes (None: 16 .. 128) with every M2L
    kernel serving the configuration on the sample (host arrays) and returns
    the fastest; with db_path the choice is kept in that profile database
    for solvers created with maxbox=0."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    cfg = make_config(**cfg_kw)
    res = TuneResult()
    mb = None if maxboxes is None else (C.c_int * len(maxboxes))(*[int(m) for m in maxboxes])
    _check(load().aran_gpu_autotune3d(C.byref(cfg), len(q), _ptr(xyz), _ptr(q), MEM_HOST, mb,
                                      0 if maxboxes is None else len(maxboxes), int(reps),
                                      db_path.encode() if db_path else None, C.byref(res)))
    return _tune_dict(res)


def tune_lookup(db_path=None, **cfg_kw):
    """The tuned choice for a configuration from the database (None when the
    database has none)."""
    cfg = make_config(**cfg_kw)
    res = TuneResult()
    rc = load().aran_gpu_tune_lookup(db_path.encode() if db_path else None, C.byref(cfg),
                                     C.byref(res))
    if rc < 0:
        raise AranError(rc, load().aran_gpu_last_error().decode())
    return _tune_dict(res) if rc == 1 else None


def footprint_bytes(n: int, **cfg_kw) -> int:
    """Estimated device memory of one solve (the server's admission unit)."""
    return int(load().aran_gpu_footprint_bytes(C.byref(make_config(**cfg_kw)), int(n)))


class Server:
    """Request loop for independent solves on one GPU (continuous batching).

    ``nslots`` solves run concurrently (each slot a native worker thread with
    its own streams and resident solvers); a request starts when a slot is
    free and its estimated footprint fits ``hbm_budget_bytes`` next to the
    running ones.  ``submit`` returns a ticket, ``wait`` the outputs and the
    request's timestamps (seconds since the server started)."""

    def __init__(self, nslots=4, hbm_budget_bytes=150e9):
        h = C.c_void_p()
        _check(load().aran_gpu_server_create(int(nslots), float(hbm_budget_bytes), C.byref(h)))
        self._h = h
        self._live = {}

    def submit(self, xyz, q, tolerance=0.0, **cfg_kw) -> int:
        """Queues a solve; ``tolerance`` > 0 lets the server pick the
        precision (and the order, given ``order=0``) for that relative L2
        potential error."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        n = len(q)
        cfg = make_config(**cfg_kw)
        pot = np.empty(n)
        fld = np.empty((n, 3)) if cfg.field else None
        req = Request3d(cfg, n, xyz.ctypes.data, q.ctypes.data, pot.ctypes.data,
                        fld.ctypes.data if fld is not None else None, float(tolerance))
        t = C.c_int64()
        _check(load().aran_gpu_server_submit(self._h, C.byref(req), C.byref(t)))
        self._live[t.value] = (xyz, q, pot, fld)
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        info = RequestInfo()
        rc = load().aran_gpu_server_wait(self._h, int(ticket), float(timeout), C.byref(info))
        if rc == -5:  # still running
            raise AranError(rc, load().aran_gpu_last_error().decode())
        xyz, q, pot, fld = self._live.pop(int(ticket))
        d = {"status": info.status, "submit_s": info.submit_s, "start_s": info.start_s,
             "end_s": info.end_s, "slot": info.slot, "footprint_bytes": info.footprint_bytes,
             "order": info.order,
             "precision": "mixed" if info.precision == PRECISIONS["mixed"] else "fp64"}
        _check(rc)
        return pot, fld, d

    def cancel(self, ticket: int):
        _check(load().aran_gpu_server_cancel(self._h, int(ticket)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().aran_gpu_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver3d:
    """GPU counterpart of ``AranSolver3d`` for the Newton potential/field.

    ``lbound``/``ubound``/``maxbox`` are the arguments of
    ``vsg_prtree3d_new_full``; ``order`` is p of
    ``aran_development3d_new (0, p)``; ``flavour`` picks the M2M/M2L/L2L
    family; ``field`` selects newtonfield3 (potential + field) over newtonpot3
    (potential only); ``precision`` is "fp64" (plain path) or "mixed";
    ``semifar_threshold`` > 0 turns on the semifar P2L/M2P interactions of
    ``aran_solver3d_set_functions_full`` for nodes holding more points;
    ``fp64_root_depth`` (mixed precision) keeps the expansions of depths
    <= it in FP64 (-1: none; None: the library's default, 3 from order 16).
    """

    def __init__(self, lbound=(0.0, 0.0, 0.0), ubound=(1.0, 1.0, 1.0), *, maxbox=64, order=12,
                 flavour="rotate", field=True, precision="fp64", max_depth=21,
                 semifar_threshold=0, fp64_root_depth=None):
        L = load()
        cfg = make_config(lbound, ubound, maxbox=maxbox, order=order, flavour=flavour,
                          field=field, precision=precision, max_depth=max_depth,
                          semifar_threshold=semifar_threshold)
        self.cfg = cfg
        self.order = cfg.order
        self.field = bool(field)
        h = C.c_void_p()
        _check(L.aran_gpu_solver3d_create(C.byref(cfg), C.byref(h)))
        self._h = h
        if fp64_root_depth is not None:
            _check(L.aran_gpu_solver3d_set_fp64_root_depth(h, int(fp64_root_depth)))

    def set_m2l_kernel(self, kernel="auto", nst=0, g=0):
        """M2L kernel of the FP32 part: "auto", "lanes", "sibling" (with nst
        table slots and g parents per CTA, 0 = the library's), "tc"."""
        _check(load().aran_gpu_solver3d_set_m2l_kernel(self._h, M2L_KERNELS[kernel], int(nst),
                                                       int(g)))

    def set_leaf_predicate(self, fn=None):
        """Nodes about to be split for which fn(NodeView) is true stay leaves
        (virtual leaves); None clears it."""
        self._leaf_cb = LEAF_PREDICATE(lambda v, _d: int(bool(fn(v.contents)))) if fn else None
        _check(load().aran_gpu_solver3d_set_leaf_predicate(
            self._h, C.cast(self._leaf_cb, C.c_void_p) if fn else None, None))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().aran_gpu_solver3d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- solve --------------------------------------------------------------
    def solve(self, xyz, q):
        """Host arrays in, host arrays out: (potential[n], field[n,3] or None)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        n = len(q)
        if xyz.shape != (n, 3):
            raise ValueError("xyz must be (n, 3)")
        pot = np.empty(n)
        fld = np.empty((n, 3)) if self.field else None
        _check(load().aran_gpu_solver3d_solve(self._h, n, _ptr(xyz), _ptr(q), _ptr(pot),
                                              _ptr(fld), MEM_HOST))
        return pot, fld

    def solve_device(self, n, xyz_ptr, q_ptr, pot_ptr, field_ptr=None):
        """Device pointers (ints, e.g. torch ``data_ptr()``)."""
        _check(load().aran_gpu_solver3d_solve(self._h, int(n), C.c_void_p(xyz_ptr),
                                              C.c_void_p(q_ptr),
                                              C.c_void_p(pot_ptr) if pot_ptr else None,
                                              C.c_void_p(field_ptr) if field_ptr else None,
                                              MEM_DEVICE))

    def solve_forest(self, xyz, q, offsets, boxes):
        """Independent systems in one solve: system k is particles
        offsets[k]:offsets[k+1] in box boxes[k] = (lbx, lby, lbz, ubx, uby,
        ubz), every box with the solver's extents.  Returns (potential[n],
        field[n,3] or None) in input order."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        offs = np.ascontiguousarray(offsets, dtype=np.int64)
        boxes = np.ascontiguousarray(boxes, dtype=np.float64).reshape(-1, 6)
        nsys = len(offs) - 1
        n = len(q)
        if xyz.shape != (n, 3) or len(boxes) != nsys:
            raise ValueError("xyz must be (n, 3) and boxes (nsys, 6)")
        if nsys < 1 or offs[0] != 0 or offs[-1] != n:
            raise ValueError("offsets must run from 0 to the number of particles")
        pot = np.empty(n)
        fld = np.empty((n, 3)) if self.field else None
        _check(load().aran_gpu_solver3d_solve_forest(
            self._h, nsys, offs.ctypes.data_as(C.POINTER(C.c_int64)),
            boxes.ctypes.data_as(C.POINTER(C.c_double)), _ptr(xyz), _ptr(q), _ptr(pot),
            _ptr(fld), MEM_HOST))
        return pot, fld

    # -- introspection ------------------------------------------------------
    def get_stats(self) -> dict:
        st = np.zeros(11, np.int64)
        _check(load().aran_gpu_solver3d_get_stats(self._h, st.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(zip(STAT_NAMES, st.tolist()))

    def tree_info(self) -> dict:
        info = np.zeros(5, np.int64)
        _check(load().aran_gpu_solver3d_tree_info(self._h, info.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(zip(("nodes", "far", "near", "leaves", "depth"), info.tolist()))

    def tree_lists(self) -> dict:
        info = self.tree_info()
        nn, nf, nr = info["nodes"], info["far"], info["near"]
        ids = np.zeros(nn, np.uint64)
        beg = np.zeros(nn, np.int32)
        end = np.zeros(nn, np.int32)
        leaf = np.zeros(nn, np.uint8)
        far = np.zeros((nf, 2), np.uint64)
        near = np.zeros((nr, 2), np.uint64)
        n = int(self.get_stats()["p2m"])
        perm = np.zeros(n, np.int32)
        _check(load().aran_gpu_solver3d_tree_lists(self._h, _ptr(ids), _ptr(beg), _ptr(end),
                                                   _ptr(leaf), _ptr(far), _ptr(near), _ptr(perm)))
        return dict(ids=ids, begin=beg, end=end, leaf=leaf, far=far, near=near, perm=perm)

    def expansions(self):
        nn = self.tree_info()["nodes"]
        p = self.order
        nm, nl = p * (p + 1) // 2, (p + 1) * (p + 2) // 2
        mult = np.zeros((nn, nm), np.complex128)
        loc = np.zeros((nn, nl), np.complex128)
        _check(load().aran_gpu_solver3d_expansions(
            self._h, mult.ctypes.data_as(C.POINTER(C.c_double)),
            loc.ctypes.data_as(C.POINTER(C.c_double))))
        return mult, loc

    def timings(self) -> dict:
        ms = np.zeros(16)
        _check(load().aran_gpu_solver3d_timings(self._h, ms.ctypes.data_as(C.POINTER(C.c_double))))
        return dict(zip(STAGE_NAMES, ms[:len(STAGE_NAMES)].tolist()))

    def launches(self) -> int:
        return int(load().aran_gpu_solver3d_launches(self._h))


class Solver2d:
    """GPU counterpart of ``AranSolver2d`` with the Cauchy kernel of
    tests/dummypot.c (acc_i = sum_{j != i} q_j / (z_i - z_j)), solving a
    batch of independent systems per call.

    ``order`` is p of ``aran_development2d_new (0, p)``, ``maxbox`` the leaf
    capacity of ``vsg_prtree2d_new_full``; ``precision`` "fp64" or "mixed"
    (FP32 scaled expansions and near-field arithmetic, FP64 sums)."""

    def __init__(self, *, maxbox=32, order=20, max_depth=21, precision="fp64"):
        cfg = Config2d(int(maxbox), int(order), int(max_depth), PRECISIONS[precision])
        h = C.c_void_p()
        _check(load().aran_gpu_solver2d_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.cfg = cfg

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().aran_gpu_solver2d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _meta(n, offsets, boxes):
        offs = np.ascontiguousarray([0, n] if offsets is None else offsets, dtype=np.int64)
        nsys = len(offs) - 1
        if nsys < 1 or offs[-1] != n:
            # the library trusts offs[nsys] as the particle count
            raise AranError(-1, "offsets must have nsys + 1 entries ending at n")
        if boxes is None:
            boxes = np.tile([-1.0, -1.0, 1.0, 1.0], (nsys, 1))
        boxes = np.ascontiguousarray(np.broadcast_to(np.asarray(boxes, np.float64), (nsys, 4)))
        return offs, boxes

    def solve(self, xy, q, offsets=None, boxes=None):
        """Host arrays: xy (n, 2), q (n,); offsets (nsys + 1,) split the
        particles into systems with boxes (nsys, 4) = lbx, lby, ubx, uby
        (default one system in [-1, 1]^2).  Returns complex acc (n,)."""
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        n = len(q)
        if xy.shape != (n, 2):
            raise ValueError("xy must be (n, 2)")
        offs, boxes = self._meta(n, offsets, boxes)
        acc = np.empty(n, np.complex128)
        _check(load().aran_gpu_solver2d_solve(
            self._h, len(offs) - 1, offs.ctypes.data_as(C.POINTER(C.c_int64)),
            boxes.ctypes.data_as(C.POINTER(C.c_double)), _ptr(xy), _ptr(q), _ptr(acc), MEM_HOST))
        return acc

    def solve_device(self, n, xy_ptr, q_ptr, acc_ptr, offsets=None, boxes=None):
        """Device pointers for xy, q and acc (2n doubles); host metadata."""
        offs, boxes = self._meta(n, offsets, boxes)
        _check(load().aran_gpu_solver2d_solve(
            self._h, len(offs) - 1, offs.ctypes.data_as(C.POINTER(C.c_int64)),
            boxes.ctypes.data_as(C.POINTER(C.c_double)), C.c_void_p(xy_ptr), C.c_void_p(q_ptr),
            C.c_void_p(acc_ptr), MEM_DEVICE))

    def get_stats(self) -> dict:
        st = np.zeros(11, np.int64)
        _check(load().aran_gpu_solver2d_get_stats(self._h, st.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(zip(STAT_NAMES, st.tolist()))

    def tree_info(self) -> dict:
        info = np.zeros(5, np.int64)
        _check(load().aran_gpu_solver2d_tree_info(self._h, info.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(zip(("nodes", "far", "near", "leaves", "depth"), info.tolist()))

    def timings(self) -> dict:
        ms = np.zeros(16)
        _check(load().aran_gpu_solver2d_timings(self._h, ms.ctypes.data_as(C.POINTER(C.c_double))))
        return dict(zip(STAGE_NAMES, ms[:len(STAGE_NAMES)].tolist()))

    def launches(self) -> int:
        return int(load().aran_gpu_solver2d_launches(self._h))


NOALLOC_MAX = 131072


def p2p_direct_noalloc(n: int, xyz_ptr: int, q_ptr: int, pot_ptr: int | None,
                       field_ptr: int | None = None) -> None:
    """Every-pair Newton potential/field of n <= 131072 particles from device
    pointers, without any device allocation (scratch lives in a static
    device array of the library).  For callers that may not allocate device
    memory during a call; calls that overlap on the GPU race on that array."""
    _check(load().aran_gpu_p2p_direct_noalloc(
        int(n), C.c_void_p(xyz_ptr), C.c_void_p(q_ptr),
        C.c_void_p(pot_ptr) if pot_ptr else None,
        C.c_void_p(field_ptr) if field_ptr else None))


def version() -> str:
    return load().aran_gpu_version().decode()
