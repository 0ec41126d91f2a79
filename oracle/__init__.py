"""CPU oracle for the LibAran 3D/2D FMM hot path -- TEST INFRASTRUCTURE ONLY.

The GPU path is tested against this package.  Only the test suite,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` load it;
the product library never imports, links or calls anything here.

It wraps ``liboracle.so`` (built from the C restatement in this directory by
``build()``), whose functions restate the reference algorithms with
file:line citations (see ``aran_oracle.h``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_SRC = ["or_series.c", "or_translate.c", "or_solver.c", "or_laurent.c"]

NORMAL, KKYLIN, ROTATE = 0, 1, 2
FLAVOURS = {"normal": NORMAL, "kkylin": KKYLIN, "rotate": ROTATE}
NSTATS = 11
STAT_NAMES = ("zero", "p2p", "p2m", "m2m", "m2l", "l2l", "l2p", "p2l", "m2p",
              "p2p_remote", "m2l_remote")


def build(force: bool = False) -> str:
    """Compile the C restatement into liboracle.so (gcc, no FMA contraction)."""
    srcs = [os.path.join(_HERE, s) for s in _SRC if os.path.exists(os.path.join(_HERE, s))]
    hdrs = [os.path.join(_HERE, h) for h in ("aran_oracle.h", "or_internal.h")]
    if not force and os.path.exists(_LIB):
        t = os.path.getmtime(_LIB)
        if all(os.path.getmtime(s) <= t for s in srcs + hdrs):
            return _LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off",
           "-o", _LIB + ".tmp"] + srcs + ["-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(_LIB + ".tmp", _LIB)
    return _LIB


def build_reference(force: bool = False):
    """Compile the reference's own operator layer (oracle/ref_build.py) when
    the reference tree is present; None otherwise."""
    from . import ref_build
    return ref_build.build(force)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        dp = C.POINTER(C.c_double)
        i64p = C.POINTER(C.c_int64)
        u64p = C.POINTER(C.c_uint64)
        i32p = C.POINTER(C.c_int32)
        u8p = C.POINTER(C.c_uint8)
        L.or_beta.restype = C.c_double
        L.or_beta.argtypes = [C.c_int]
        L.or_alpha.restype = C.c_double
        L.or_alpha.argtypes = [C.c_int, C.c_int]
        L.or_harmonic_norm.restype = C.c_double
        L.or_harmonic_norm.argtypes = [C.c_int, C.c_int]
        L.or_vertical_factor.restype = C.c_double
        L.or_vertical_factor.argtypes = [C.c_int, C.c_int, C.c_int]
        L.or_legendre_multiple.argtypes = [C.c_int, C.c_double, C.c_double, dp]
        L.or_legendre_special.argtypes = [C.c_int, C.c_double, C.c_double, dp, dp]
        L.or_harmonics.argtypes = [C.c_int] + [C.c_double] * 4 + [dp]
        L.or_to_spherical.argtypes = [dp, dp]
        L.or_series_size.restype = C.c_int
        L.or_series_size.argtypes = [C.c_int, C.c_int]
        L.or_p2m.argtypes = [dp, C.c_double, dp, C.c_int, dp]
        L.or_p2l.argtypes = [dp, C.c_double, dp, C.c_int, dp]
        L.or_series_evaluate.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        L.or_series_gradient.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        for f in (L.or_translate, L.or_to_local):
            f.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, C.c_int, C.c_int, dp, dp]
        for f in (L.or_rotate, L.or_rotate_inverse):
            f.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_double, C.c_double,
                          C.c_int, C.c_int, dp]
        L.or_wigner_size.restype = C.c_int
        L.or_wigner_size.argtypes = [C.c_int]
        L.or_wigner.argtypes = [C.c_double] * 3 + [C.c_int, dp]
        L.or_solve.restype = C.c_int
        L.or_solve.argtypes = [C.c_void_p, dp, dp, dp, dp, i64p]
        L.or_set_leaf_predicate.restype = None
        L.or_set_leaf_predicate.argtypes = [C.c_void_p, C.c_void_p]
        L.or_solve_threaded.restype = C.c_int
        L.or_solve_threaded.argtypes = [C.c_void_p, dp, dp, dp, dp, i64p, C.c_int]
        L.or_tree_lists.restype = C.c_int
        L.or_tree_lists.argtypes = [C.c_void_p, dp, i64p, u64p, i32p, i32p, u8p,
                                    i64p, u64p, i64p, u64p, i32p]
        L.or_morton_key.restype = C.c_uint64
        L.or_morton_key.argtypes = [dp, dp, dp]
        L.or_direct.argtypes = [C.c_int, dp, dp, C.c_int, i32p, dp, dp, C.c_int]
        L.or2_p2m.argtypes = [C.c_double] * 5 + [C.c_int, dp]
        L.or2_p2l.argtypes = [C.c_double] * 5 + [C.c_int, dp]
        for f in (L.or2_translate, L.or2_to_taylor):
            f.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_double, C.c_int, C.c_int,
                          dp, C.c_double, C.c_double]
        L.or2_evaluate.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_double, dp]
        L.or2_solve.restype = C.c_int
        L.or2_solve.argtypes = [C.c_void_p, C.c_int, i64p, dp, dp, dp, dp, i64p]
        L.or2_direct.argtypes = [C.c_int, dp, dp, C.c_int, i32p, dp]
        _lib = L
    return _lib


class NodeView(C.Structure):
    """OrNodeView: a node about to be split, as a leaf predicate sees it."""
    _fields_ = [("center", C.c_double * 3), ("lbound", C.c_double * 3),
                ("ubound", C.c_double * 3), ("point_count", C.c_int64), ("depth", C.c_int)]


LEAF_PREDICATE = C.CFUNCTYPE(C.c_int, C.POINTER(NodeView), C.c_void_p)


class leaf_predicate:
    """Context manager: tree builds inside it keep as leaves the nodes for
    which fn(node_view) is true (virtual leaves)."""

    def __init__(self, fn):
        self._cb = LEAF_PREDICATE(lambda v, _d: int(bool(fn(v.contents))))

    def __enter__(self):
        lib().or_set_leaf_predicate(C.cast(self._cb, C.c_void_p), None)
        return self

    def __exit__(self, *a):
        lib().or_set_leaf_predicate(None, None)


class SolveConfig(C.Structure):
    _fields_ = [("n", C.c_int), ("maxbox", C.c_int), ("order", C.c_int),
                ("flavour", C.c_int), ("field", C.c_int), ("max_depth", C.c_int),
                ("lb", C.c_double * 3), ("ub", C.c_double * 3),
                ("semifar_threshold", C.c_int)]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _cfg(n, maxbox, order, flavour, field, lb, ub, max_depth=21, semifar_threshold=0):
    if isinstance(flavour, str):
        flavour = FLAVOURS[flavour]
    c = SolveConfig()
    c.n, c.maxbox, c.order, c.flavour = n, maxbox, order, flavour
    c.field, c.max_depth = int(field), max_depth
    for k in range(3):
        c.lb[k], c.ub[k] = lb[k], ub[k]
    c.semifar_threshold = int(semifar_threshold)
    return c


# ---------------------------------------------------------------- operators
def series_size(posdeg: int, negdeg: int) -> int:
    return ((posdeg + 1) * (posdeg + 2) + negdeg * (negdeg + 1)) // 2


def zeros_series(posdeg: int, negdeg: int) -> np.ndarray:
    return np.zeros(series_size(posdeg, negdeg), dtype=np.complex128)


def p2m(x, q, center, deg, out=None):
    out = zeros_series(0, deg) if out is None else out
    lib().or_p2m(_dp(np.ascontiguousarray(x, np.float64)), float(q),
                 _dp(np.ascontiguousarray(center, np.float64)), deg, _dp(out.view(np.float64)))
    return out


def p2l(x, q, center, deg, out=None):
    out = zeros_series(deg, 0) if out is None else out
    lib().or_p2l(_dp(np.ascontiguousarray(x, np.float64)), float(q),
                 _dp(np.ascontiguousarray(center, np.float64)), deg, _dp(out.view(np.float64)))
    return out


def evaluate(posdeg, negdeg, coefs, xrel) -> complex:
    o = np.zeros(2)
    lib().or_series_evaluate(posdeg, negdeg, _dp(np.ascontiguousarray(coefs).view(np.float64)),
                             _dp(np.ascontiguousarray(xrel, np.float64)), _dp(o))
    return complex(o[0], o[1])


def gradient(posdeg, negdeg, coefs, xrel) -> np.ndarray:
    o = np.zeros(3)
    lib().or_series_gradient(posdeg, negdeg, _dp(np.ascontiguousarray(coefs).view(np.float64)),
                             _dp(np.ascontiguousarray(xrel, np.float64)), _dp(o))
    return o


def translate(flavour, sdeg, src, xs, ddeg, dst, xd):
    """dst += M2M/L2L(src); sdeg/ddeg are (posdeg, negdeg)."""
    if isinstance(flavour, str):
        flavour = FLAVOURS[flavour]
    lib().or_translate(flavour, sdeg[0], sdeg[1], _dp(src.view(np.float64)),
                       _dp(np.asarray(xs, np.float64)), ddeg[0], ddeg[1],
                       _dp(dst.view(np.float64)), _dp(np.asarray(xd, np.float64)))
    return dst


def to_local(flavour, sdeg, src, xs, ddeg, dst, xd):
    """dst += M2L(src)."""
    if isinstance(flavour, str):
        flavour = FLAVOURS[flavour]
    lib().or_to_local(flavour, sdeg[0], sdeg[1], _dp(src.view(np.float64)),
                      _dp(np.asarray(xs, np.float64)), ddeg[0], ddeg[1],
                      _dp(dst.view(np.float64)), _dp(np.asarray(xd, np.float64)))
    return dst


def rotate(sdeg, src, a, b, g, ddeg, dst, inverse=False):
    f = lib().or_rotate_inverse if inverse else lib().or_rotate
    f(sdeg[0], sdeg[1], _dp(src.view(np.float64)), a, b, g, ddeg[0], ddeg[1],
      _dp(dst.view(np.float64)))
    return dst


def wigner(alpha, beta, gamma, lmax) -> np.ndarray:
    n = lib().or_wigner_size(lmax)
    out = np.zeros(n, dtype=np.complex128)
    lib().or_wigner(alpha, beta, gamma, lmax, _dp(out.view(np.float64)))
    return out


def wigner_index(l, mp, m):
    return (l * (l + 1) * (4 * l - 1)) // 6 + mp * (2 * l + 1) + l + m


def legendre(l, x, s=None):
    s = np.sqrt(1 - x * x) if s is None else s
    out = np.zeros((l + 1) * (l + 2) // 2)
    lib().or_legendre_multiple(l, x, s, _dp(out))
    return out


def harmonics(l, theta, phi):
    out = np.zeros((l + 1) * (l + 2) // 2, dtype=np.complex128)
    lib().or_harmonics(l, np.cos(theta), np.sin(theta), np.cos(phi), np.sin(phi),
                       _dp(out.view(np.float64)))
    return out


# ------------------------------------------------------------------- solver
def solve(xyz, q, *, order, maxbox, flavour="rotate", field=False,
          lb=(0.0, 0.0, 0.0), ub=(1.0, 1.0, 1.0), max_depth=21, semifar_threshold=0,
          nthreads=1):
    """Full CPU FMM solve; returns (potential or field, stats dict).
    semifar_threshold > 0 turns on P2L/M2P for nodes holding more points;
    nthreads != 1 spreads the per-node/per-leaf work over host threads (0:
    all cores) with the same results."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    n = len(q)
    cfg = _cfg(n, maxbox, order, flavour, field, lb, ub, max_depth, semifar_threshold)
    pot = np.zeros(n)
    fld = np.zeros((n, 3))
    st = np.zeros(NSTATS, dtype=np.int64)
    stp = st.ctypes.data_as(C.POINTER(C.c_int64))
    if nthreads == 1:
        rc = lib().or_solve(C.byref(cfg), _dp(xyz), _dp(q), _dp(pot), _dp(fld), stp)
    else:
        rc = lib().or_solve_threaded(C.byref(cfg), _dp(xyz), _dp(q), _dp(pot), _dp(fld), stp,
                                     int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle solve failed")
    return (fld if field else pot), dict(zip(STAT_NAMES, st.tolist()))


def tree_lists(xyz, *, maxbox, lb=(0.0, 0.0, 0.0), ub=(1.0, 1.0, 1.0), max_depth=21):
    """Node ids/ranges/leaf flags, unordered far and near pairs, permutation."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    n = len(xyz)
    cfg = _cfg(n, maxbox, 1, 0, 0, lb, ub, max_depth)
    L = lib()
    nn, nf, nr = C.c_int64(), C.c_int64(), C.c_int64()
    null = None
    L.or_tree_lists(C.byref(cfg), _dp(xyz), C.byref(nn), null, null, null, null,
                    C.byref(nf), null, C.byref(nr), null, null)
    ids = np.zeros(nn.value, np.uint64)
    beg = np.zeros(nn.value, np.int32)
    end = np.zeros(nn.value, np.int32)
    leaf = np.zeros(nn.value, np.uint8)
    far = np.zeros((nf.value, 2), np.uint64)
    near = np.zeros((nr.value, 2), np.uint64)
    perm = np.zeros(n, np.int32)
    L.or_tree_lists(C.byref(cfg), _dp(xyz), C.byref(nn),
                    ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                    beg.ctypes.data_as(C.POINTER(C.c_int32)),
                    end.ctypes.data_as(C.POINTER(C.c_int32)),
                    leaf.ctypes.data_as(C.POINTER(C.c_uint8)),
                    C.byref(nf), far.ctypes.data_as(C.POINTER(C.c_uint64)),
                    C.byref(nr), near.ctypes.data_as(C.POINTER(C.c_uint64)),
                    perm.ctypes.data_as(C.POINTER(C.c_int32)))
    return dict(ids=ids, begin=beg, end=end, leaf=leaf, far=far, near=near, perm=perm)


def morton_key(x, lb, ub) -> int:
    return int(lib().or_morton_key(_dp(np.asarray(x, np.float64)),
                                   _dp(np.asarray(lb, np.float64)),
                                   _dp(np.asarray(ub, np.float64))))


def direct(xyz, q, targets=None, nthreads=0):
    """FP64 compensated direct sum; returns (potential, field) at targets."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    n = len(q)
    if targets is None:
        targets_arr = None
        nt = n
    else:
        targets_arr = np.ascontiguousarray(targets, np.int32)
        nt = len(targets_arr)
    pot = np.zeros(nt)
    fld = np.zeros((nt, 3))
    tp = None if targets_arr is None else targets_arr.ctypes.data_as(C.POINTER(C.c_int32))
    lib().or_direct(n, _dp(xyz), _dp(q), nt, tp, _dp(pot), _dp(fld), nthreads)
    return pot, fld


# ------------------------------------------------------------------------ 2D
class Solve2Config(C.Structure):
    _fields_ = [("maxbox", C.c_int), ("order", C.c_int), ("max_depth", C.c_int)]


def laurent(posdeg: int, negdeg: int) -> np.ndarray:
    """Zero Laurent series; index posdeg - i holds the term of degree i."""
    return np.zeros(posdeg + negdeg + 1, dtype=np.complex128)


def p2m2d(z, q, center, negdeg, out=None):
    out = laurent(0, negdeg) if out is None else out
    lib().or2_p2m(float(np.real(z)), float(np.imag(z)), float(q), float(np.real(center)),
                  float(np.imag(center)), negdeg, _dp(out.view(np.float64)))
    return out


def p2l2d(z, q, center, posdeg, out=None):
    out = laurent(posdeg, 0) if out is None else out
    lib().or2_p2l(float(np.real(z)), float(np.imag(z)), float(q), float(np.real(center)),
                  float(np.imag(center)), posdeg, _dp(out.view(np.float64)))
    return out


def _laurent_op(f, src, sdeg, zsrc, ddeg, zdst, out):
    sp, sn = sdeg
    dp_, dn = ddeg
    out = laurent(dp_, dn) if out is None else out
    src = np.ascontiguousarray(src, np.complex128)
    f(sp, sn, _dp(src.view(np.float64)), float(np.real(zsrc)), float(np.imag(zsrc)), dp_, dn,
      _dp(out.view(np.float64)), float(np.real(zdst)), float(np.imag(zdst)))
    return out


def translate2d(src, sdeg, zsrc, ddeg, zdst, out=None):
    """aran_laurent_seriesd_translate (M2M / L2L)."""
    return _laurent_op(lib().or2_translate, src, sdeg, zsrc, ddeg, zdst, out)


def to_taylor2d(src, sdeg, zsrc, ddeg, zdst, out=None):
    """aran_laurent_seriesd_to_taylor (M2L)."""
    return _laurent_op(lib().or2_to_taylor, src, sdeg, zsrc, ddeg, zdst, out)


def evaluate2d(s, deg, z) -> complex:
    out = np.zeros(2)
    s = np.ascontiguousarray(s, np.complex128)
    lib().or2_evaluate(deg[0], deg[1], _dp(s.view(np.float64)), float(np.real(z)),
                       float(np.imag(z)), _dp(out))
    return complex(out[0], out[1])


def solve2d(xy, q, offsets, boxes, maxbox, order, max_depth=21):
    """2D FMM of sum_j q_j/(z_i - z_j) over independent systems.

    xy (n, 2), q (n,), offsets (nsys + 1,), boxes (nsys, 4) = lbx, lby, ubx, uby.
    Returns (complex accumulators (n,), stats dict summed over systems)."""
    xy = np.ascontiguousarray(xy, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    offs = np.ascontiguousarray(offsets, np.int64)
    boxes = np.ascontiguousarray(boxes, np.float64)
    acc = np.zeros(2 * len(q))
    st = np.zeros(NSTATS, np.int64)
    c = Solve2Config(maxbox, order, max_depth)
    rc = lib().or2_solve(C.byref(c), len(offs) - 1, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                         _dp(xy), _dp(q), _dp(boxes), _dp(acc),
                         st.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc != 0:
        raise ValueError("or2_solve rejected the configuration")
    return acc.view(np.complex128), dict(zip(STAT_NAMES, st.tolist()))


def direct2d(xy, q, targets=None):
    """FP64 direct sum of sum_{j != i} q_j/(z_i - z_j) for one system."""
    xy = np.ascontiguousarray(xy, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    if targets is None:
        nt, tp = len(q), None
    else:
        targets = np.ascontiguousarray(targets, np.int32)
        nt, tp = len(targets), targets.ctypes.data_as(C.POINTER(C.c_int32))
    acc = np.zeros(2 * nt)
    lib().or2_direct(len(q), _dp(xy), _dp(q), nt, tp, _dp(acc))
    return acc.view(np.complex128)
