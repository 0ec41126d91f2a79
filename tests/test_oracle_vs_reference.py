"""The oracle pinned to LibAran's own operator code, term by term.

oracle/ref_build.py compiles the reference's operator layer unmodified (its
own aran/*.c files, against glib/libvsg shims) and oracle/ref.py calls it
through its public API.  Every operator the GPU parity tests rely on through
the oracle is compared here with the reference at orders 4-20:

* P2M and P2L (aran_development3d_p2m/p2l, arandevelopment3d.c:169-277);
* M2M, M2L, L2L in the normal, kkylin and rotate flavours
  (arandevelopment3d.c:288-451 and the series translations behind them);
* local and multipole evaluation, local gradient
  (aransphericalseriesd.c:312-546);
* rotation and inverse rotation (aransphericalseriesd-rotate.c:93-153) and
  the Wigner D terms (aranwigner.c:83-313);
* the 2D Laurent operators (arandevelopment2d.c:167-346).

Coefficients agree to 1e-14 of the largest one (both are FP64, compiled
without FMA contraction; they differ only in summation order).  Skipped
where the reference tree is not mounted.

One reference defect is pinned rather than followed: _buffer_rotate
(aransphericalseriesd-rotate.c:34-80) declares gcomplex128 src_l[deg] and
src_l_neg[deg] but fills them for m = 0..deg, one element past their end, so
the top degree of every rotated series (l = negdeg-1 of a multipole, l =
posdeg of a local) is computed from overwritten stack memory.  The rotate
flavour's translations inherit it (M2M in its top degree, M2L and L2L in
every degree through the vertical translation).  The oracle and the GPU
apply the intended operator: the rotate flavour is checked against the
reference's normal flavour (the same linear operator) and the reference's
rotation on every degree but the top one; test_rotate_overflow shows the
out-of-bounds write with the bounds sanitizer.
"""
import os
import shutil
import subprocess
import math

import numpy as np
import pytest

from oracle import ref

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference tree not mounted")

ORDERS = [4, 8, 12, 16, 20]
TOL = 1e-14


def close(a, b, tol=TOL):
    scale = max(np.max(np.abs(a)), np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale) <= tol


def charges(seed, n=6, spread=0.3):
    rng = np.random.default_rng(seed)
    return rng.uniform(-spread, spread, (n, 3)), rng.uniform(-1, 1, n)


@pytest.mark.parametrize("p", ORDERS)
def test_p2m_p2l(oracle, p):
    xs, qs = charges(p)
    c = np.array([0.05, -0.02, 0.01])
    far = np.array([2.0, 1.5, -1.0])
    for x, q in zip(xs, qs):
        assert close(oracle.p2m(x, q, c, p), ref.p2m(x, q, c, p))
        assert close(oracle.p2l(x + far, q, c, p), ref.p2l(x + far, q, c, p))


def source_multipole(oracle, p, center, seed):
    xs, qs = charges(seed)
    m = oracle.zeros_series(0, p)
    for x, q in zip(xs, qs):
        oracle.p2m(x + center, q, center, p, out=m)
    return m


def source_local(oracle, p, center, seed):
    xs, qs = charges(seed)
    loc = oracle.zeros_series(p, 0)
    for x, q in zip(xs, qs):
        oracle.p2l(x * 0.2 + center + np.array([3.0, -2.0, 2.5]), q, center, p, out=loc)
    return loc


@pytest.mark.parametrize("flavour", ["normal", "kkylin", "rotate"])
@pytest.mark.parametrize("p", ORDERS)
def test_m2m_m2l_l2l(oracle, flavour, p):
    """Each oracle flavour against the reference: normal and kkylin against
    their own reference flavour, rotate against the reference's normal
    flavour (the same operator; the reference's rotate code carries the
    _buffer_rotate overflow) and, for M2M, against the reference's rotate
    code below the top degree."""
    ref_flavour = "normal" if flavour == "rotate" else flavour
    xs = np.array([0.1, -0.2, 0.05])
    # M2M: child centre to parent centre (an octant offset)
    m = source_multipole(oracle, p, xs, 10 + p)
    xd = xs + np.array([0.25, 0.25, -0.25])
    om = oracle.translate(flavour, (0, p), m, xs, (0, p), oracle.zeros_series(0, p), xd)
    rm, _ = ref.operator("m2m", ref_flavour, p, m, None, xs, xd)
    assert close(om, rm)
    if flavour == "rotate":
        rr, _ = ref.operator("m2m", "rotate", p, m, None, xs, xd)
        below_top = 1 + (p - 1) * p // 2          # the (0, 0) slot, degrees < p-1
        assert close(om[:below_top], rr[:below_top])
    # M2L: a far offset (two boxes away, off-axis) and one along z
    for off in (np.array([1.0, -0.5, 1.5]), np.array([0.0, 0.0, 2.0])):
        ol = oracle.to_local(flavour, (0, p), m, xs, (p, 0), oracle.zeros_series(p, 0), xs + off)
        _, rl = ref.operator("m2l", ref_flavour, p, m, None, xs, xs + off)
        assert close(ol, rl)
    # L2L: parent centre to child centre
    loc = source_local(oracle, p, xs, 20 + p)
    xc = xs + np.array([-0.125, 0.125, 0.125])
    ol = oracle.translate(flavour, (p, 0), loc, xs, (p, 0), oracle.zeros_series(p, 0), xc)
    _, rl = ref.operator("l2l", ref_flavour, p, None, loc, xs, xc)
    assert close(ol, rl)


@pytest.mark.parametrize("p", ORDERS)
def test_evaluate_and_gradient(oracle, p):
    c = np.array([0.3, 0.1, -0.2])
    loc = source_local(oracle, p, c, 30 + p)
    m = source_multipole(oracle, p, c, 40 + p)
    rng = np.random.default_rng(p)
    for _ in range(5):
        x = c + rng.uniform(-0.2, 0.2, 3)
        assert abs(oracle.evaluate(p, 0, loc, x - c) - ref.local_evaluate(p, loc, c, x)) <= \
            TOL * 10 * abs(ref.local_evaluate(p, loc, c, x))
        g_o = oracle.gradient(p, 0, loc, x - c)
        g_r = ref.local_gradient(p, loc, c, x)
        assert np.linalg.norm(g_o - g_r) <= 1e-13 * np.linalg.norm(g_r)
        xf = c + rng.uniform(1.5, 2.5, 3)
        vo = oracle.evaluate(0, p, m, xf - c)
        vr = ref.multipole_evaluate(p, m, c, xf)
        assert abs(vo - vr) <= 1e-13 * abs(vr)


@pytest.mark.parametrize("p", ORDERS)
def test_rotations_and_wigner(oracle, p):
    rng = np.random.default_rng(50 + p)
    src = rng.standard_normal(oracle.series_size(p, p)) + 1j * rng.standard_normal(
        oracle.series_size(p, p))
    # the slots of every degree but the top one of each part: local degrees
    # < p, multipole degrees < p-1 (the reference's _buffer_rotate fills the
    # top degree from memory past its buffers)
    nl = (p + 1) * (p + 2) // 2
    keep = np.r_[0:p * (p + 1) // 2, nl:nl + (p - 1) * p // 2]
    for a, b, g in ((0.3, 1.1, -0.7), (-2.0, 0.4, 0.0), (0.0, math.pi / 2, 1.3)):
        for inverse in (False, True):
            o = oracle.rotate((p, p), src, a, b, g, (p, p), np.zeros_like(src), inverse=inverse)
            r = ref.rotate(p, p, src, a, b, g, inverse=inverse)
            assert close(o[keep], r[keep], 1e-13), (a, b, g, inverse)
        w_o = oracle.wigner(a, b, g, p)
        w_r = ref.wigner_all(a, b, g, p)
        got = np.array([w_o[oracle.wigner_index(l, mp, m)] for (l, mp, m) in w_r])
        assert close(got, np.array(list(w_r.values())), 1e-13)


@pytest.mark.parametrize("p", [4, 10, 20])
def test_laurent_2d(oracle, p):
    rng = np.random.default_rng(60 + p)
    zc = 0.1 - 0.2j
    zs = [zc + complex(*rng.uniform(-0.2, 0.2, 2)) for _ in range(5)]
    qs = rng.uniform(-1, 1, 5)
    m_o = oracle.laurent(0, p)
    m_r = np.zeros_like(m_o)
    for z, q in zip(zs, qs):
        oracle.p2m2d(z, q, zc, p, out=m_o)
        m_r += ref.p2m2d(z, q, zc, p)
    assert close(m_o, m_r)
    zfar = zc + 3.0 + 2.0j
    l_o = oracle.p2l2d(zfar, 0.7, zc, p)
    assert close(l_o, ref.p2l2d(zfar, 0.7, zc, p))
    zp = zc + 0.25 + 0.25j
    assert close(oracle.translate2d(m_o, (0, p), zc, (0, p), zp),
                 ref.operator2d("m2m", p, m_o, None, zc, zp)[0])
    zt = zc + 2.0 - 1.0j
    assert close(oracle.to_taylor2d(m_o, (0, p), zc, (p, 0), zt),
                 ref.operator2d("m2l", p, m_o, None, zc, zt)[1])
    zchild = zc - 0.125 + 0.125j
    assert close(oracle.translate2d(l_o, (p, 0), zc, (p, 0), zchild),
                 ref.operator2d("l2l", p, None, l_o, zc, zchild)[1])


SANITIZE_DRIVER = r"""
#include <aran/aransphericalseriesd.h>
int main (void)
{
  AranSphericalSeriesd *a = aran_spherical_seriesd_new (6, 6);
  AranSphericalSeriesd *b = aran_spherical_seriesd_new (6, 6);
  *aran_spherical_seriesd_get_term (a, 2, 1) = 1.;
  aran_spherical_seriesd_rotate (a, 0.3, 1.1, -0.7, b);
  return 0;
}
"""


def test_rotate_overflow(tmp_path):
    """The reference's rotation built with the undefined-behaviour
    sanitizer's bounds checks reports the index past the end of
    _buffer_rotate's variable-length buffers."""
    from oracle import ref_build
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    drv = tmp_path / "rot.c"
    drv.write_text(SANITIZE_DRIVER)
    gen = ref_build.generate()
    exe = tmp_path / "rot"
    here = os.path.dirname(ref_build.__file__)
    srcs = [os.path.join(ref_build.REF, "aran", f) for f in
            ("aransphericalseriesd.c", "aransphericalseriesd-rotate.c",
             "aransphericalseriesd-translate.c", "aranwigner.c", "aranwignerrepo.c",
             "aransphericalharmonic.c", "aranlegendre.c", "aranbinomial.c")]
    cmd = ["gcc", "-std=gnu99", "-O0", "-g", "-fsanitize=bounds", "-w",
           "-I" + os.path.join(here, "refshim"), "-I" + ref_build.GEN, "-I" + ref_build.REF,
           "-I" + os.path.join(ref_build.REF, "aran"), str(drv)] + srcs + gen + \
          [os.path.join(here, "refshim", "shim.c"), "-lm", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no sanitizer build: " + r.stderr[-300:])
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert "aransphericalseriesd-rotate.c" in r.stderr and "out of bounds" in r.stderr, r.stderr
