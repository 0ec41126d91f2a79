"""Known-answer tests of the reference, restated against the CPU oracle.

The reference's operator tests (tests/legendre.c, sphericalharmonic.c,
wigner.c, rotation.c, m2l3.c, multipole3.c, taylor3.c, gradient3.c, p2l3.c)
check each operator against closed forms or against 1/r on spherical grids,
with the same geometry and tolerances used here.  Several of them only print
their failures; here every check is an assertion.  These tests pin the
oracle that the GPU parity tests rely on.
"""
import math

import numpy as np
import pytest

N = 10  # grid size of the reference checks (tests/m2l3.c:31)


def sph_grid(radius_lo, radius_hi, n=N):
    """(r, theta, phi) grid of the reference checks: phi in [0, 2pi],
    theta in [0, pi], r from radius_lo to radius_hi (tests/m2l3.c:42-66)."""
    out = []
    for i in range(n):
        p = 2 * math.pi * i / (n - 1)
        for j in range(n):
            t = math.pi * j / (n - 1)
            for k in range(n):
                r = radius_lo + (radius_hi - radius_lo) * k / (n - 1)
                out.append((r * math.sin(t) * math.cos(p), r * math.sin(t) * math.sin(p),
                            r * math.cos(t)))
    return np.array(out)


def newton(x, src):
    return 1.0 / np.linalg.norm(x - src)


def newton_grad(x, src):
    d = x - src
    return -d / np.linalg.norm(d) ** 3


# ---------------------------------------------------------------- Legendre
def plm_closed(l, m, x):
    """Closed forms of P_l^m with the Condon-Shortley phase (l <= 3)."""
    s = math.sqrt(1 - x * x)
    table = {
        (0, 0): 1.0, (1, 0): x, (1, 1): -s,
        (2, 0): 0.5 * (3 * x * x - 1), (2, 1): -3 * x * s, (2, 2): 3 * (1 - x * x),
        (3, 0): 0.5 * (5 * x ** 3 - 3 * x), (3, 1): -1.5 * (5 * x * x - 1) * s,
        (3, 2): 15 * x * (1 - x * x), (3, 3): -15 * s ** 3,
    }
    return table[(l, m)]


def test_legendre_closed_forms(oracle):
    # tests/legendre.c: closed forms to 1e-10
    for x in np.linspace(-1, 1, 21):
        leg = oracle.legendre(3, x)
        for l in range(4):
            for m in range(l + 1):
                ref = plm_closed(l, m, x)
                got = leg[l * (l + 1) // 2 + m]
                err = abs(got - ref) / (abs(ref) if ref != 0 else 1.0)
                assert err < 1e-10, (l, m, x, got, ref)


def test_legendre_multiple_vs_recurrence(oracle):
    # tests/legendre.c multiple_check: all (l, m) up to 50 against a plain recursion
    L = 50
    for x in np.linspace(-0.95, 0.95, 9):
        leg = oracle.legendre(L, x)
        P = np.zeros((L + 1, L + 1))
        P[0, 0] = 1.0
        s = math.sqrt(1 - x * x)
        for l in range(1, L + 1):
            P[l, l] = -(2 * l - 1) * s * P[l - 1, l - 1]
            for m in range(l):
                P[l, m] = ((2 * l - 1) * x * P[l - 1, m] - (l + m - 1) * (P[l - 2, m] if l >= 2 else 0)) / (l - m)
        for l in range(L + 1):
            for m in range(l + 1):
                ref, got = P[l, m], leg[l * (l + 1) // 2 + m]
                assert abs(got - ref) <= 1e-10 * max(abs(ref), 1.0), (l, m, x)


def test_spherical_harmonics_closed_forms(oracle):
    # tests/sphericalharmonic.c: Y_l^m closed forms for l <= 2 (m >= 0 stored)
    def yref(l, m, t, p):
        e = np.exp(1j * m * p)
        st, ct = math.sin(t), math.cos(t)
        if (l, m) == (0, 0):
            return 0.5 / math.sqrt(math.pi)
        if (l, m) == (1, 0):
            return 0.5 * math.sqrt(3 / math.pi) * ct
        if (l, m) == (1, 1):
            return -0.5 * math.sqrt(1.5 / math.pi) * st * e
        if (l, m) == (2, 0):
            return 0.25 * math.sqrt(5 / math.pi) * (3 * ct * ct - 1)
        if (l, m) == (2, 1):
            return -0.5 * math.sqrt(7.5 / math.pi) * st * ct * e
        if (l, m) == (2, 2):
            return 0.25 * math.sqrt(7.5 / math.pi) * st * st * e
        if (l, m) == (3, 3):
            return -0.125 * math.sqrt(35 / math.pi) * st ** 3 * e
        if (l, m) == (3, 0):
            return 0.25 * math.sqrt(7 / math.pi) * (5 * ct * ct - 3) * ct
        raise KeyError
    for t in np.linspace(0, math.pi, 7):
        for p in np.linspace(0, 2 * math.pi, 7):
            h = oracle.harmonics(3, t, p)
            for (l, m) in [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2), (3, 0), (3, 3)]:
                ref = yref(l, m, t, p)
                got = h[l * (l + 1) // 2 + m]
                assert abs(got - ref) <= 1e-10 * max(abs(ref), 1.0), (l, m, t, p)


# ------------------------------------------------------------------ Wigner
def wigner_closed(l, m1, m2, beta):
    """Wigner small-d by the explicit sum over k (tests/wigner.c:89-145)."""
    lf = lambda n: math.lgamma(n + 1)
    a = 0.5 * (lf(l + m1) + lf(l - m1) + lf(l + m2) + lf(l - m2))
    cb2, sb2 = math.cos(beta / 2), math.sin(beta / 2)
    res = 0.0
    for k in range(max(0, m2 - m1), min(l - m1, l + m2) + 1):
        b = lf(k) + lf(l - m1 - k) + lf(l + m2 - k) + lf(m1 - m2 + k)
        c = cb2 ** (2 * l - m1 + m2 - 2 * k)
        d = sb2 ** (m1 - m2 + 2 * k)
        res += (-1) ** (m1 - m2 + k) * math.exp(a - b) * c * d
    return res


@pytest.mark.parametrize("beta", [i * math.pi / 30 for i in range(0, 30, 3)]
                         + [math.pi / 2, 0.84106867056793033])
def test_wigner_closed_form(oracle, beta):
    # tests/wigner.c: L = 20, 1e-6 relative
    L = 20
    w = oracle.wigner(0.0, beta, 0.0, L)
    faults = 0
    for l in range(L + 1):
        for mp in range(l + 1):
            for m in range(-l, l + 1):
                got = w[oracle.wigner_index(l, mp, m)].real
                ref = wigner_closed(l, m, mp, beta)
                err = abs(got - ref)
                if abs(ref) > 1e-6:
                    err /= abs(ref)
                faults += not (err < 1e-6)
    assert faults == 0


# ---------------------------------------------------------------- rotation
def taylor(oracle, deg, center, src):
    return oracle.p2l(src, 1.0, center, deg)


@pytest.mark.parametrize("i", range(0, 29, 4))
def test_rotation_inverse_is_identity(oracle, i):
    # tests/rotation.c: rotate then rotate_inverse gives back the series (L=29, 1e-7)
    L = 29
    beta = i * math.pi / 10
    for alpha in (0.0, 0.7):
        s = taylor(oracle, L, np.zeros(3), np.array([3.0, 3.0, 3.0]))
        rot = oracle.zeros_series(L, 0)
        back = oracle.zeros_series(L, 0)
        oracle.rotate((L, 0), s, alpha, beta, 0.0, (L, 0), rot)
        oracle.rotate((L, 0), rot, alpha, beta, 0.0, (L, 0), back, inverse=True)
        err = np.abs(back - s) / np.maximum(np.abs(s), 1e-7)
        assert err.max() < 1e-7


def test_rotation_aligns_direction_with_z(oracle):
    # rotation.c's "rotated series == series of the rotated point": rotating by
    # (-phi, theta, 0) must give the Taylor series of (0, 0, |p|); this is the
    # property the rotate-flavour M2L/M2M/L2L rely on.
    L = 20
    for p in ([3.0, 3.0, 3.0], [1.0, -2.0, 0.5], [-0.3, 0.2, 2.0]):
        p = np.array(p)
        r = np.linalg.norm(p)
        theta = math.acos(p[2] / r)
        phi = math.atan2(p[1], p[0])
        s = taylor(oracle, L, np.zeros(3), p)
        rot = oracle.zeros_series(L, 0)
        oracle.rotate((L, 0), s, -phi, theta, 0.0, (L, 0), rot)
        chk = taylor(oracle, L, np.zeros(3), np.array([0.0, 0.0, r]))
        assert np.abs(rot - chk).max() < 1e-7 * np.abs(chk).max()


# -------------------------------------------------------------- translations
M2L_TRANSLATIONS = [(5, 5, 5), (5, 5, -5), (0, 0, -5), (0, 0, 5), (5, 0, 5), (0, 5, 5),
                    (-5, -5, 5)]


@pytest.mark.parametrize("flavour", ["normal", "kkylin", "rotate"])
def test_m2l3(oracle, flavour):
    # tests/m2l3.c: multipole of a unit charge at (0.1,0.2,0.3), degree 26,
    # M2L to degree 25 at 7 translations, checked against 1/r within radius 1
    # of the target (1e-7 relative)
    deg = 25
    p = np.array([0.1, 0.2, 0.3])
    M = oracle.p2m(p, 1.0, np.zeros(3), deg + 1)
    pts = sph_grid(0.0, 1.0)
    for tr in M2L_TRANSLATIONS:
        tr = np.array(tr, float)
        Lc = oracle.zeros_series(deg, 0)
        oracle.to_local(flavour, (0, deg + 1), M, np.zeros(3), (deg, 0), Lc, tr)
        for v in pts:
            ref = newton(tr + v, p)
            got = oracle.evaluate(deg, 0, Lc, v)
            assert abs(got - ref) / abs(ref) < 1e-7, (flavour, tr, v)


@pytest.mark.parametrize("flavour", ["normal", "kkylin", "rotate"])
def test_multipole3(oracle, flavour):
    # tests/multipole3.c: P2M degree 30 of a unit charge at (0.1,0.2,0.3),
    # M2M by (1,1.1,1.2); potential and gradient checked for 5 <= r <= 10
    # (1e-7)
    deg = 30
    p = np.array([0.1, 0.2, 0.3])
    tr = np.array([1.0, 1.1, 1.2])
    M = oracle.p2m(p, 1.0, np.zeros(3), deg)
    T = oracle.zeros_series(0, deg)
    oracle.translate(flavour, (0, deg), M, np.zeros(3), (0, deg), T, tr)
    for S, c in ((M, np.zeros(3)), (T, tr)):
        for v in sph_grid(5.0, 10.0):
            ref = newton(c + v, p)
            got = oracle.evaluate(0, deg, S, v)
            assert abs(got - ref) / abs(ref) < 1e-7
            g = oracle.gradient(0, deg, S, v)
            gr = newton_grad(c + v, p)
            assert np.linalg.norm(g - gr) / np.linalg.norm(gr) < 1e-7


@pytest.mark.parametrize("flavour", ["normal", "kkylin", "rotate"])
def test_taylor3(oracle, flavour):
    # tests/taylor3.c: P2L degree 29 of a unit charge at (3,0,0) about (5,0,0),
    # L2L to (4.5,0,0); potential within radius 1 (resp. 0.5), 1e-9
    deg = 29
    src = np.array([3.0, 0.0, 0.0])
    c = np.array([5.0, 0.0, 0.0])
    tr = np.array([4.5, 0.0, 0.0])
    Lc = oracle.p2l(src, 1.0, c, deg)
    T = oracle.zeros_series(deg, 0)
    oracle.translate(flavour, (deg, 0), Lc, c, (deg, 0), T, tr)
    for S, cc, rad in ((Lc, c, 1.0), (T, tr, 0.5)):
        for v in sph_grid(0.0, rad):
            ref = newton(cc + v, src)
            got = oracle.evaluate(deg, 0, S, v)
            assert abs(got - ref) / abs(ref) < 1e-9


@pytest.mark.parametrize("flavour", ["normal", "kkylin", "rotate"])
def test_gradient3(oracle, flavour):
    # tests/gradient3.c: source (3,-1,-1), degree 29, local gradient about
    # (5,0,0) and after L2L to (4.5,0,0), 1e-9
    deg = 29
    src = np.array([3.0, -1.0, -1.0])
    c = np.array([5.0, 0.0, 0.0])
    tr = np.array([4.5, 0.0, 0.0])
    Lc = oracle.p2l(src, 1.0, c, deg)
    T = oracle.zeros_series(deg, 0)
    oracle.translate(flavour, (deg, 0), Lc, c, (deg, 0), T, tr)
    for S, cc, rad in ((Lc, c, 1.0), (T, tr, 0.5)):
        for v in sph_grid(0.0, rad):
            gr = newton_grad(cc + v, src)
            g = oracle.gradient(deg, 0, S, v)
            assert np.linalg.norm(g - gr) / np.linalg.norm(gr) < 1e-9


def test_p2l3(oracle):
    # tests/p2l3.c: P2L degree 29 and the local gradient, radius 1, 1e-9
    deg = 29
    src = np.array([3.0, -1.0, -1.0])
    c = np.array([5.0, 0.0, 0.0])
    Lc = oracle.p2l(src, 1.0, c, deg)
    for v in sph_grid(0.0, 1.0):
        gr = newton_grad(c + v, src)
        g = oracle.gradient(deg, 0, Lc, v)
        assert np.linalg.norm(g - gr) / np.linalg.norm(gr) < 1e-9


# --------------------------------------------------------------- end to end
def circle(n):
    """tests/newtonfield3.c:472-493: n charges 1/n on a circle of radius 0.999"""
    R = 0.999
    a = 2 * math.pi * np.arange(n) / n
    x = np.stack([R * np.cos(a), R * np.sin(a), np.zeros(n)], axis=1)
    return x, np.full(n, 1.0 / n)


def random_cube(n, seed):
    """uniform in [-0.999, 0.999]^3, charges in [0, 2/n] (tests/newtonfield3.c:495-541)"""
    rng = np.random.default_rng(seed)
    R = 0.999
    return rng.uniform(-R, R, (n, 3)), rng.uniform(0, 2.0 / n, n)


E2E_CASES = [  # (np, p, maxbox, distribution) of tests/newtonpot3.at / newtonfield3.at
    (12, 20, 1, "circle"), (24, 24, 1, "circle"), (24, 24, 1, "random"),
    (240, 24, 10, "circle"), (2400, 24, 100, "circle"),
]


@pytest.mark.parametrize("case", E2E_CASES)
@pytest.mark.parametrize("field", [False, True])
def test_newton_e2e_rotate(oracle, case, field):
    """newtonpot3/newtonfield3 (rotate): every particle within 1e-3 of the
    direct sum (relative, per particle; tests/newtonpot3.c:678-715,
    tests/newtonfield3.c:650-693)"""
    n, p, maxbox, dist = case
    x, q = circle(n) if dist == "circle" else random_cube(n, 0)
    out, stats = oracle.solve(x, q, order=p, maxbox=maxbox, flavour="rotate", field=field,
                              lb=(-1, -1, -1), ub=(1, 1, 1))
    ref_p, ref_f = oracle.direct(x, q)
    if field:
        err = np.linalg.norm(out - ref_f, axis=1) / np.linalg.norm(ref_f, axis=1)
    else:
        err = np.abs(out - ref_p) / np.maximum(np.abs(out), np.abs(ref_p))
    assert err.max() < 1e-3
    assert stats["p2m"] == n and stats["l2p"] == n


@pytest.mark.parametrize("flavour", ["normal", "kkylin"])
def test_newton_e2e_other_flavours(oracle, flavour):
    n, p, maxbox = 240, 12, 10
    x, q = circle(n)
    out, _ = oracle.solve(x, q, order=p, maxbox=maxbox, flavour=flavour, field=False,
                          lb=(-1, -1, -1), ub=(1, 1, 1))
    ref_p, _ = oracle.direct(x, q)
    err = np.abs(out - ref_p) / np.maximum(np.abs(out), np.abs(ref_p))
    assert err.max() < 1e-3


def test_flavours_agree(oracle):
    """The three flavours compute the same expansions up to rounding."""
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, (3000, 3))
    q = rng.uniform(-1, 1, 3000)
    outs = [oracle.solve(x, q, order=8, maxbox=20, flavour=f, field=True)[0]
            for f in ("normal", "kkylin", "rotate")]
    for o in outs[1:]:
        assert np.linalg.norm(o - outs[0]) / np.linalg.norm(outs[0]) < 1e-12


def test_direct_sum_small(oracle):
    """The compensated direct sum against a plain numpy sum."""
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 1, (300, 3))
    q = rng.uniform(-1, 1, 300)
    pot, fld = oracle.direct(x, q)
    d = x[:, None, :] - x[None, :, :]
    r = np.linalg.norm(d, axis=2)
    np.fill_diagonal(r, np.inf)
    ref_p = (q[None, :] / r).sum(1)
    ref_f = (-q[None, :, None] * d / r[:, :, None] ** 3).sum(1)
    assert np.allclose(pot, ref_p, rtol=1e-12, atol=0)
    assert np.allclose(fld, ref_f, rtol=1e-10, atol=1e-12)


# ------------------------------------------------------------------------ 2D
# tests/laurent.c: the series of 1/(z-1) (a_{-i} = 1, order 24) checked in
# rings outside radius 2, translated to 2i (ring radius 4) and re-expanded as
# a Taylor series at 6i (disk of radius 2), tolerance 1e-7.
def _rings(oracle, s, deg, center, radius, f, inner):
    worst = 0.0
    pts = [0j] if inner else []
    for i in range(11):
        r = i * radius / 10 + (0 if inner else radius)
        pts += [r * np.exp(2j * np.pi * j / i) for j in range(i)]
    for z in pts:
        ref = f(z + center)
        worst = max(worst, abs((ref - oracle.evaluate2d(s, deg, z)) / ref))
    return worst


def test_laurent_series_of_inverse_z_minus_one(oracle):
    order = 24
    f = lambda z: 1 / (z - 1)
    als = oracle.laurent(0, order)
    als[1:] = 1.0
    assert _rings(oracle, als, (0, order), 0, 2.0, f, False) < 1e-7
    alst = oracle.translate2d(als, (0, order), 0, (0, order), 2j)
    assert _rings(oracle, alst, (0, order), 2j, 4.0, f, False) < 1e-7
    alstt = oracle.to_taylor2d(als, (0, order), 0, (order, 0), 6j)
    assert _rings(oracle, alstt, (order, 0), 6j, 2.0, f, True) < 1e-7


def test_laurent_storage_order(oracle):
    # degree i of a (posdeg, negdeg) series sits at posdeg - i
    s = oracle.p2m2d(0.3 + 0.1j, 2.0, 0.0, 5)
    d = 0.3 + 0.1j
    assert s[0] == 0
    np.testing.assert_allclose(s[1:5], 2.0 * d ** np.arange(4), rtol=1e-15)
    assert s[5] == 0  # a_{-negdeg} is never filled (loop i < negdeg)


def test_p2l2d_is_the_cauchy_kernel(oracle):
    # tests/p2l2.c: source (3, -1), charge 1, centre (5, 0), degree 29,
    # points of the half disk of radius 1 (N = 10 x 10); the local value is
    # 1/(z - zp) (the p2l2.c check compares its negation and never fails)
    zp, c, deg = 3 - 1j, 5 + 0j, 29
    loc = oracle.p2l2d(zp, 1.0, c, deg)
    worst = 0.0
    for j in range(10):
        t = np.pi * j / 9
        for k in range(10):
            w = (k / 9) * np.exp(1j * t)
            ref = 1 / (w + c - zp)
            worst = max(worst, abs(oracle.evaluate2d(loc, (deg, 0), w) - ref) / abs(ref))
    assert worst < 1e-9


def _circle(n, r=0.9):
    t = 2 * np.pi * np.arange(n) / n
    return np.stack([r * np.cos(t), r * np.sin(t)], 1)


# tests/dummypot.at: (np, order, maxbox, err); distribution circle of radius
# 0.9 unless "random" (uniform in [-0.9, 0.9]^2), unit densities, box [-1,1]^2
DUMMYPOT_AT = [
    ("circle", 12, 20, 1, 1e-6),
    ("circle", 2400, 20, 1, 1e-6),
    ("circle", 240, 40, 1, 1e-8),
    ("random", 240, 20, 1, 1e-6),
    ("circle", 240, 20, 10, 1e-8),
    ("circle", 2400, 20, 10, 1e-6),
]


@pytest.mark.parametrize("dist,n,order,maxbox,tol", DUMMYPOT_AT)
def test_dummypot_cases(oracle, dist, n, order, maxbox, tol):
    xy = _circle(n) if dist == "circle" else np.random.default_rng(0).uniform(-0.9, 0.9, (n, 2))
    q = np.ones(n)
    acc, st = oracle.solve2d(xy, q, [0, n], [[-1, -1, 1, 1]], maxbox, order)
    ref = oracle.direct2d(xy, q)
    err = np.abs(acc - ref) / np.maximum(np.abs(acc), np.abs(ref))
    assert err.max() < tol
    assert st["p2m"] == n and st["l2p"] == n


def test_solve2d_systems_are_independent(oracle):
    rng = np.random.default_rng(3)
    sizes = [300, 1, 0, 1200]
    xy = rng.uniform(-1, 1, (sum(sizes), 2))
    q = rng.uniform(-1, 1, sum(sizes))
    offs = np.concatenate([[0], np.cumsum(sizes)])
    boxes = np.tile([-1.0, -1.0, 1.0, 1.0], (len(sizes), 1))
    acc, _ = oracle.solve2d(xy, q, offs, boxes, 16, 20)
    for s in range(len(sizes)):
        a, b = offs[s], offs[s + 1]
        if b > a:
            one, _ = oracle.solve2d(xy[a:b], q[a:b], [0, b - a], boxes[s:s + 1], 16, 20)
            np.testing.assert_array_equal(acc[a:b], one)


def test_semifar_keeps_the_accuracy(oracle):
    # semifar P2L/M2P replaces P2P between a coarse leaf and deep nodes that
    # do not touch it; the error against the direct sum stays that of the FMM
    from aran_gb300 import workloads as W
    x, q = W.plummer(6000, 21)
    lb, ub = (-1, -1, -1), (1, 1, 1)
    rp, rf = oracle.direct(x, q)
    base, st0 = oracle.solve(x, q, order=10, maxbox=16, field=True, lb=lb, ub=ub)
    semi, st1 = oracle.solve(x, q, order=10, maxbox=16, field=True, lb=lb, ub=ub,
                             semifar_threshold=4)
    e0 = np.linalg.norm(base - rf) / np.linalg.norm(rf)
    e1 = np.linalg.norm(semi - rf) / np.linalg.norm(rf)
    assert st1["p2l"] > 0 and st1["p2l"] == st1["m2p"] and st0["p2l"] == 0
    assert st1["p2p"] < st0["p2p"]
    assert e1 < 2 * e0 + 1e-9


@pytest.mark.parametrize("flavour", ["rotate", "kkylin"])
@pytest.mark.parametrize("field", [False, True])
def test_threaded_solve_equals_serial(oracle, flavour, field):
    """The threaded oracle solve (the CPU baseline's) gives every target its
    terms in the single-threaded order: same counters, results equal to
    rounding, also with coincident points."""
    from aran_gb300 import workloads as W
    x, q = W.plummer(6000, 8)
    x[5990:] = x[:10]
    kw = dict(order=8, maxbox=16, field=field, flavour=flavour, lb=(-1, -1, -1), ub=(1, 1, 1))
    a, sa = oracle.solve(x, q, **kw)
    b, sb = oracle.solve(x, q, nthreads=4, **kw)
    assert sa == sb
    assert np.all(np.isfinite(b))
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a)
