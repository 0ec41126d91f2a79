"""LibAran's 3D series and development operators called one at a time
(include/aran/aransphericalseriesd.h, arandevelopment3d.h), against the
oracle's restatement of the same operators.

Each call runs on the GPU (one launch); the results must equal the oracle's
to FP64 rounding: P2M, P2L, M2M/L2L translations and M2L in the normal,
kkylin and rotate flavours, rotations with and without phases, evaluation
and gradient of multipole and local series.  The series layout is the
reference's, so the oracle's arrays and the library's containers hold the
same numbers.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class V3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class Z(C.Structure):   # gcomplex128 returned by value (two doubles)
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class NodeInfo(C.Structure):
    _fields_ = [("center", V3), ("lbound", V3), ("ubound", V3), ("point_list", C.c_void_p),
                ("point_count", C.c_uint), ("isleaf", C.c_int), ("depth", C.c_uint),
                ("user_data", C.c_void_p), ("father_info", C.c_void_p), ("id", C.c_uint)]


class Dev3(C.Structure):
    _fields_ = [("multipole", C.c_void_p), ("local", C.c_void_p)]


@pytest.fixture(scope="module")
def L(aran):
    lib = C.CDLL(aran.LIB_PATH)
    vp = C.c_void_p
    lib.aran_spherical_seriesd_new.restype = vp
    lib.aran_spherical_seriesd_new.argtypes = [C.c_uint8, C.c_uint8]
    lib.aran_spherical_seriesd_free.argtypes = [vp]
    lib.aran_spherical_seriesd_get_term.restype = C.POINTER(C.c_double)
    lib.aran_spherical_seriesd_get_term.argtypes = [vp, C.c_int, C.c_int]
    for f in ("rotate", "rotate_inverse"):
        getattr(lib, "aran_spherical_seriesd_" + f).argtypes = [vp] + [C.c_double] * 3 + [vp]
    for f in ("translate", "to_local", "translate_kkylin", "to_local_kkylin",
              "translate_rotate", "to_local_rotate"):
        getattr(lib, "aran_spherical_seriesd_" + f).argtypes = [vp, C.POINTER(V3), vp,
                                                                 C.POINTER(V3)]
    lib.aran_spherical_seriesd_evaluate.restype = Z
    lib.aran_spherical_seriesd_evaluate.argtypes = [vp, C.POINTER(V3)]
    lib.aran_spherical_seriesd_gradient_evaluate.argtypes = [vp, C.POINTER(V3), C.POINTER(V3)]
    lib.aran_development3d_new.restype = C.POINTER(Dev3)
    lib.aran_development3d_new.argtypes = [C.c_uint8, C.c_uint8]
    lib.aran_development3d_free.argtypes = [C.POINTER(Dev3)]
    for f in ("p2m", "p2l"):
        getattr(lib, "aran_development3d_" + f).argtypes = [C.POINTER(V3), C.c_double,
                                                            C.POINTER(NodeInfo), C.POINTER(Dev3)]
    return lib


def size(pd, nd):
    return ((pd + 1) * (pd + 2) + nd * (nd + 1)) // 2


def to_array(L, s, pd, nd):
    base = L.aran_spherical_seriesd_get_term(s, 0, 0)
    return np.ctypeslib.as_array(base, (2 * size(pd, nd),)).view(np.complex128).copy()


def from_array(L, a, pd, nd):
    s = L.aran_spherical_seriesd_new(pd, nd)
    base = L.aran_spherical_seriesd_get_term(s, 0, 0)
    np.ctypeslib.as_array(base, (2 * size(pd, nd),))[:] = np.asarray(a, np.complex128).view(
        np.float64)
    return s


def v3(x):
    return V3(*map(float, x))


def node(c):
    n = NodeInfo()
    n.center = v3(c)
    return n


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("p", [8, 20])
def test_p2m_p2l(L, oracle, p):
    rng = np.random.default_rng(p)
    d = L.aran_development3d_new(0, p)
    c = rng.uniform(-1, 1, 3)
    ref_m = oracle.zeros_series(0, p)
    ref_l = oracle.zeros_series(p, 0)
    for _ in range(5):
        x = c + rng.uniform(-0.3, 0.3, 3)
        y = c + rng.uniform(2, 3, 3)
        q = rng.uniform(-1, 1)
        L.aran_development3d_p2m(C.byref(v3(x)), q, C.byref(node(c)), d)
        L.aran_development3d_p2l(C.byref(v3(y)), q, C.byref(node(c)), d)
        oracle.p2m(x, q, c, p, out=ref_m)
        oracle.p2l(y, q, c, p, out=ref_l)
    assert rel(to_array(L, d.contents.multipole, 0, p), ref_m) < 1e-13
    assert rel(to_array(L, d.contents.local, p, 0), ref_l) < 1e-13
    L.aran_development3d_free(d)


def multipole(oracle, p, c, rng):
    m = oracle.zeros_series(0, p)
    for _ in range(4):
        oracle.p2m(c + rng.uniform(-0.2, 0.2, 3), rng.uniform(-1, 1), c, p, out=m)
    return m


FLAVOURS = [("normal", ""), ("kkylin", "_kkylin"), ("rotate", "_rotate")]


@pytest.mark.parametrize("p", [8, 16])
@pytest.mark.parametrize("flavour,suffix", FLAVOURS)
def test_translations_match_oracle(L, oracle, p, flavour, suffix):
    rng = np.random.default_rng(3 * p)
    xs = np.array([0.1, -0.2, 0.3])
    # M2M (parent above and below: both signs of the z component)
    for xd in (xs + [0.4, 0.3, 0.5], xs + [-0.3, 0.2, -0.6]):
        m = multipole(oracle, p, xs, rng)
        ref = oracle.translate(flavour, (0, p), m, xs, (0, p), oracle.zeros_series(0, p), xd)
        s = from_array(L, m, 0, p)
        d = L.aran_spherical_seriesd_new(0, p)
        getattr(L, "aran_spherical_seriesd_translate" + suffix)(s, C.byref(v3(xs)), d,
                                                                 C.byref(v3(xd)))
        assert rel(to_array(L, d, 0, p), ref) < 1e-12, (flavour, "m2m")
        # M2L
        xl = xd + np.array([3.0, -2.5, 2.0])
        refl = oracle.to_local(flavour, (0, p), m, xs, (p, 0), oracle.zeros_series(p, 0), xl)
        dl = L.aran_spherical_seriesd_new(p, 0)
        getattr(L, "aran_spherical_seriesd_to_local" + suffix)(s, C.byref(v3(xs)), dl,
                                                                C.byref(v3(xl)))
        assert rel(to_array(L, dl, p, 0), refl) < 1e-12, (flavour, "m2l")
        # L2L
        xl2 = xl + np.array([0.2, 0.1, -0.3])
        refl2 = oracle.translate(flavour, (p, 0), refl, xl, (p, 0), oracle.zeros_series(p, 0),
                                 xl2)
        dl2 = L.aran_spherical_seriesd_new(p, 0)
        getattr(L, "aran_spherical_seriesd_translate" + suffix)(dl, C.byref(v3(xl)), dl2,
                                                                 C.byref(v3(xl2)))
        assert rel(to_array(L, dl2, p, 0), refl2) < 1e-12, (flavour, "l2l")
        for h in (s, d, dl, dl2):
            L.aran_spherical_seriesd_free(h)


@pytest.mark.parametrize("angles", [(0.3, 1.1, -0.7), (0.0, 2.0, 0.0), (1e-7, 0.4, 2.5)])
def test_rotations_match_oracle(L, oracle, angles):
    p = 12
    rng = np.random.default_rng(5)
    a = rng.normal(size=size(p, p)) + 1j * rng.normal(size=size(p, p))
    s = from_array(L, a, p, p)
    for inv, name in ((False, "rotate"), (True, "rotate_inverse")):
        ref = oracle.rotate((p, p), a, *angles, (p, p), oracle.zeros_series(p, p), inverse=inv)
        d = L.aran_spherical_seriesd_new(p, p)
        getattr(L, "aran_spherical_seriesd_" + name)(s, *angles, d)
        assert rel(to_array(L, d, p, p), ref) < 1e-12, name
        L.aran_spherical_seriesd_free(d)
    L.aran_spherical_seriesd_free(s)


def test_evaluate_and_gradient_match_oracle(L, oracle):
    p = 14
    rng = np.random.default_rng(9)
    for pd, nd in ((p, 0), (0, p), (6, 9)):
        a = rng.normal(size=size(pd, nd)) + 1j * rng.normal(size=size(pd, nd))
        s = from_array(L, a, pd, nd)
        for x in (rng.uniform(-1, 1, 3), np.array([0.0, 0.0, 0.7])):
            z = L.aran_spherical_seriesd_evaluate(s, C.byref(v3(x)))
            ref = oracle.evaluate(pd, nd, a, x)
            assert abs(complex(z.re, z.im) - ref) <= 1e-12 * max(1.0, abs(ref))
            g = V3()
            L.aran_spherical_seriesd_gradient_evaluate(s, C.byref(v3(x)), C.byref(g))
            gref = oracle.gradient(pd, nd, a, x)
            assert np.allclose([g.x, g.y, g.z], gref, rtol=1e-11, atol=1e-12 * np.abs(gref).max())
        L.aran_spherical_seriesd_free(s)
