"""TEST INFRASTRUCTURE: ctypes access to the reference's own operator code.

oracle/ref_build.py compiles LibAran's operator layer unmodified against
small glib/libvsg shims into oracle/_ref/libaranref.so.  This module calls
it through the reference's public API (aran_development{2,3}d_*,
aran_spherical_seriesd_*, aran_laurent_seriesd_*, aran_wigner_*) and returns
the coefficients in the oracle's array layout, so tests can compare the
oracle (the CPU restatement the GPU parity tests rely on) with the
reference term by term.  Only the CPU pinning tests import it; it is
unavailable (available() is False) where the reference tree is absent.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ref_build

_lib = None


def available() -> bool:
    return ref_build.available()


class Vec3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class Vec2(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double)]


class NodeInfo3(C.Structure):
    _fields_ = [("center", Vec3), ("lbound", Vec3), ("ubound", Vec3), ("point_list", C.c_void_p),
                ("point_count", C.c_uint), ("isleaf", C.c_int), ("depth", C.c_uint),
                ("user_data", C.c_void_p), ("father_info", C.c_void_p), ("id", C.c_uint)]


class NodeInfo2(C.Structure):
    _fields_ = [("center", Vec2), ("lbound", Vec2), ("ubound", Vec2), ("point_list", C.c_void_p),
                ("point_count", C.c_uint), ("isleaf", C.c_int), ("depth", C.c_uint),
                ("user_data", C.c_void_p), ("father_info", C.c_void_p), ("id", C.c_uint)]


class Devel(C.Structure):
    _fields_ = [("multipole", C.c_void_p), ("local", C.c_void_p)]


class Cplx(C.Structure):
    """gcomplex128 returned by value (the same registers as two doubles)."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = ref_build.build()
        if path is None:
            raise OSError("the reference tree is not available")
        L = C.CDLL(path)
        vp, dp = C.c_void_p, C.c_double
        u8 = C.c_uint8
        cplx_p = C.POINTER(C.c_double * 2)
        for name in ("aran_development3d_new", "aran_development2d_new"):
            getattr(L, name).argtypes = [u8, u8]
            getattr(L, name).restype = C.POINTER(Devel)
        L.aran_development3d_free.argtypes = [vp]
        L.aran_development2d_free.argtypes = [vp]
        L.aran_spherical_seriesd_get_term.argtypes = [vp, C.c_int, C.c_int]
        L.aran_spherical_seriesd_get_term.restype = cplx_p
        L.aran_spherical_seriesd_new.argtypes = [u8, u8]
        L.aran_spherical_seriesd_new.restype = vp
        L.aran_spherical_seriesd_free.argtypes = [vp]
        L.aran_laurent_seriesd_get_term.argtypes = [vp, C.c_int]
        L.aran_laurent_seriesd_get_term.restype = cplx_p
        for name in ("aran_development3d_p2m", "aran_development3d_p2l"):
            getattr(L, name).argtypes = [C.POINTER(Vec3), dp, C.POINTER(NodeInfo3), vp]
        for name in ("aran_development2d_p2m", "aran_development2d_p2l"):
            getattr(L, name).argtypes = [C.POINTER(Vec2), dp, C.POINTER(NodeInfo2), vp]
        for f in ("", "_kkylin", "_rotate"):
            for op in ("m2m", "m2l", "l2l"):
                getattr(L, f"aran_development3d_{op}{f}").argtypes = [
                    C.POINTER(NodeInfo3), vp, C.POINTER(NodeInfo3), vp]
        for op in ("m2m", "m2l", "l2l"):
            getattr(L, f"aran_development2d_{op}").argtypes = [
                C.POINTER(NodeInfo2), vp, C.POINTER(NodeInfo2), vp]
        L.aran_development3d_local_evaluate.argtypes = [C.POINTER(NodeInfo3), vp, C.POINTER(Vec3)]
        L.aran_development3d_local_evaluate.restype = Cplx
        L.aran_development3d_multipole_evaluate.argtypes = [C.POINTER(NodeInfo3), vp,
                                                             C.POINTER(Vec3)]
        L.aran_development3d_multipole_evaluate.restype = Cplx
        L.aran_development3d_local_gradient_evaluate.argtypes = [
            C.POINTER(NodeInfo3), vp, C.POINTER(Vec3), C.POINTER(Vec3)]
        L.aran_development2d_local_evaluate.argtypes = [C.POINTER(NodeInfo2), vp, C.POINTER(Vec2)]
        L.aran_development2d_local_evaluate.restype = Cplx
        L.aran_spherical_seriesd_rotate.argtypes = [vp, dp, dp, dp, vp]
        L.aran_spherical_seriesd_rotate_inverse.argtypes = [vp, dp, dp, dp, vp]
        L.aran_wigner_new.argtypes = [dp, dp, dp, C.c_int]
        L.aran_wigner_new.restype = vp
        L.aran_wigner_free.argtypes = [vp]
        L.aran_wigner_term.argtypes = [vp, C.c_uint, C.c_uint, C.c_int]
        L.aran_wigner_term.restype = cplx_p
        _lib = L
    return _lib


FLAVOUR_SUFFIX = {"normal": "", "kkylin": "_kkylin", "rotate": "_rotate"}


def node3(center) -> NodeInfo3:
    n = NodeInfo3()
    n.center = Vec3(*[float(v) for v in center])
    return n


def node2(center) -> NodeInfo2:
    n = NodeInfo2()
    n.center = Vec2(float(np.real(center)), float(np.imag(center)))
    return n


# ---------------------------------------------------------------- 3D series
def read_series(ptr, posdeg, negdeg) -> np.ndarray:
    """Reference series -> the oracle's layout: local terms (l, m), l <=
    posdeg, at l(l+1)/2 + m, then multipole terms of degree -(l+1), l <
    negdeg, at (posdeg+1)(posdeg+2)/2 + l(l+1)/2 + m."""
    L = lib()
    out = np.zeros(((posdeg + 1) * (posdeg + 2) + negdeg * (negdeg + 1)) // 2, np.complex128)
    k = 0
    for l in range(posdeg + 1):
        for m in range(l + 1):
            t = L.aran_spherical_seriesd_get_term(ptr, l, m).contents
            out[k] = complex(t[0], t[1])
            k += 1
    for l in range(negdeg):
        for m in range(l + 1):
            t = L.aran_spherical_seriesd_get_term(ptr, -l - 1, m).contents
            out[k] = complex(t[0], t[1])
            k += 1
    return out


def write_series(ptr, posdeg, negdeg, arr) -> None:
    L = lib()
    k = 0
    for l in range(posdeg + 1):
        for m in range(l + 1):
            t = L.aran_spherical_seriesd_get_term(ptr, l, m).contents
            t[0], t[1] = arr[k].real, arr[k].imag
            k += 1
    for l in range(negdeg):
        for m in range(l + 1):
            t = L.aran_spherical_seriesd_get_term(ptr, -l - 1, m).contents
            t[0], t[1] = arr[k].real, arr[k].imag
            k += 1


class Development3d:
    """aran_development3d_new (posdeg, negdeg) of the reference."""

    def __init__(self, posdeg, negdeg):
        self.posdeg, self.negdeg = posdeg, negdeg
        self.ptr = lib().aran_development3d_new(posdeg, negdeg)

    def __del__(self):
        try:
            lib().aran_development3d_free(self.ptr)
        except Exception:
            pass

    @property
    def multipole(self):
        return read_series(self.ptr.contents.multipole, self.posdeg, self.negdeg)

    @property
    def local(self):
        return read_series(self.ptr.contents.local, max(self.posdeg, self.negdeg), 0)

    def set_local(self, arr):
        write_series(self.ptr.contents.local, max(self.posdeg, self.negdeg), 0, arr)

    def set_multipole(self, arr):
        write_series(self.ptr.contents.multipole, self.posdeg, self.negdeg, arr)


def p2m(x, q, center, p) -> np.ndarray:
    d = Development3d(0, p)
    lib().aran_development3d_p2m(C.byref(Vec3(*x)), float(q), C.byref(node3(center)), d.ptr)
    return d.multipole


def p2l(x, q, center, p) -> np.ndarray:
    d = Development3d(0, p)
    lib().aran_development3d_p2l(C.byref(Vec3(*x)), float(q), C.byref(node3(center)), d.ptr)
    return d.local


def operator(op, flavour, p, src_mult, src_loc, xs, xd):
    """aran_development3d_{m2m,m2l,l2l}{flavour} from a development (0, p)
    holding (src_mult, src_loc) at xs into a zero development at xd;
    returns (multipole, local) of the destination."""
    s = Development3d(0, p)
    d = Development3d(0, p)
    if src_mult is not None:
        s.set_multipole(src_mult)
    if src_loc is not None:
        s.set_local(src_loc)
    f = getattr(lib(), f"aran_development3d_{op}{FLAVOUR_SUFFIX[flavour]}")
    f(C.byref(node3(xs)), s.ptr, C.byref(node3(xd)), d.ptr)
    return d.multipole, d.local


def local_evaluate(p, loc, center, x):
    d = Development3d(0, p)
    d.set_local(loc)
    r = lib().aran_development3d_local_evaluate(C.byref(node3(center)), d.ptr,
                                                 C.byref(Vec3(*x)))
    return complex(r.re, r.im)


def multipole_evaluate(p, mult, center, x):
    d = Development3d(0, p)
    d.set_multipole(mult)
    r = lib().aran_development3d_multipole_evaluate(C.byref(node3(center)), d.ptr,
                                                     C.byref(Vec3(*x)))
    return complex(r.re, r.im)


def local_gradient(p, loc, center, x) -> np.ndarray:
    d = Development3d(0, p)
    d.set_local(loc)
    g = Vec3()
    lib().aran_development3d_local_gradient_evaluate(C.byref(node3(center)), d.ptr,
                                                     C.byref(Vec3(*x)), C.byref(g))
    return np.array([g.x, g.y, g.z])


def rotate(posdeg, negdeg, src, a, b, g, inverse=False) -> np.ndarray:
    L = lib()
    s = L.aran_spherical_seriesd_new(posdeg, negdeg)
    d = L.aran_spherical_seriesd_new(posdeg, negdeg)
    write_series(s, posdeg, negdeg, src)
    write_series(d, posdeg, negdeg, np.zeros_like(src))
    f = L.aran_spherical_seriesd_rotate_inverse if inverse else L.aran_spherical_seriesd_rotate
    f(s, a, b, g, d)
    out = read_series(d, posdeg, negdeg)
    L.aran_spherical_seriesd_free(s)
    L.aran_spherical_seriesd_free(d)
    return out


def wigner_term(alpha, beta, gamma, lmax, l, mp, m) -> complex:
    L = lib()
    w = L.aran_wigner_new(alpha, beta, gamma, lmax)
    t = L.aran_wigner_term(w, l, mp, m).contents
    v = complex(t[0], t[1])
    L.aran_wigner_free(w)
    return v


def wigner_all(alpha, beta, gamma, lmax) -> dict:
    L = lib()
    w = L.aran_wigner_new(alpha, beta, gamma, lmax)
    out = {}
    for l in range(lmax + 1):
        for mp in range(l + 1):
            for m in range(-l, l + 1):
                t = L.aran_wigner_term(w, l, mp, m).contents
                out[(l, mp, m)] = complex(t[0], t[1])
    L.aran_wigner_free(w)
    return out


# ---------------------------------------------------------------- 2D series
def read_laurent(ptr, posdeg, negdeg) -> np.ndarray:
    """Reference Laurent series -> the oracle's layout (index posdeg - i
    holds the term of degree i)."""
    L = lib()
    out = np.zeros(posdeg + negdeg + 1, np.complex128)
    for i in range(posdeg, -negdeg - 1, -1):
        t = L.aran_laurent_seriesd_get_term(ptr, i).contents
        out[posdeg - i] = complex(t[0], t[1])
    return out


def write_laurent(ptr, posdeg, negdeg, arr) -> None:
    L = lib()
    for i in range(posdeg, -negdeg - 1, -1):
        t = L.aran_laurent_seriesd_get_term(ptr, i).contents
        t[0], t[1] = arr[posdeg - i].real, arr[posdeg - i].imag


class Development2d:
    def __init__(self, posdeg, negdeg):
        self.posdeg, self.negdeg = posdeg, negdeg
        self.ptr = lib().aran_development2d_new(posdeg, negdeg)

    def __del__(self):
        try:
            lib().aran_development2d_free(self.ptr)
        except Exception:
            pass

    @property
    def multipole(self):
        return read_laurent(self.ptr.contents.multipole, self.posdeg, self.negdeg)

    @property
    def local(self):
        return read_laurent(self.ptr.contents.local, max(self.posdeg, self.negdeg), 0)


def p2m2d(z, q, center, p):
    d = Development2d(0, p)
    lib().aran_development2d_p2m(C.byref(Vec2(z.real, z.imag)), float(q),
                                 C.byref(node2(center)), d.ptr)
    return d.multipole


def p2l2d(z, q, center, p):
    d = Development2d(0, p)
    lib().aran_development2d_p2l(C.byref(Vec2(z.real, z.imag)), float(q),
                                 C.byref(node2(center)), d.ptr)
    return d.local


def operator2d(op, p, src_mult, src_loc, zs, zd):
    s = Development2d(0, p)
    d = Development2d(0, p)
    if src_mult is not None:
        write_laurent(s.ptr.contents.multipole, 0, p, src_mult)
    if src_loc is not None:
        write_laurent(s.ptr.contents.local, p, 0, src_loc)
    getattr(lib(), f"aran_development2d_{op}")(C.byref(node2(zs)), s.ptr, C.byref(node2(zd)),
                                               d.ptr)
    return d.multipole, d.local
