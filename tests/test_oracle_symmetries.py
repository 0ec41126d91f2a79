"""Identities the lane-parallel M2L kernel is built on, checked on the
oracle's FP64 operators (CPU only).

* Mirror symmetry of the translation: for a reflection sigma of some axes,
  T_d = S T_{sigma d} S, with S acting on a series as (-1)^{l+m} for a z
  flip, conjugation for a y flip and (-1)^m conjugation for an x flip (the
  kernel maps the eight children of a parent onto child 0's offsets with
  it).
* Transpose symmetry of the even/odd Wigner blocks of a rotation by beta:
  E[m][m'] = (-1)^{m-m'} E[m'][m] and O likewise for m, m' > 0,
  E[0][m] = 2 (-1)^m E[m][0], O[0][m] = 0 (the kernel stores lower triangles).
* Symmetry of the vertical M2L factors: with the source and target series
  scaled by 1/beta_n and (-1)^{j+m} beta_j, beta_l = sqrt(4 pi / (2l+1)),
  the translation along z is a symmetric matrix in the degrees (j, n) for
  each order m.
"""
import numpy as np
import pytest

P = 8


def tri(l, m=0):
    return l * (l + 1) // 2 + m


def mirror(a, pd, nd, bits):
    """S for the axes set in bits (x = 1, y = 2, z = 4) on a series stored
    LibAran-style (local degrees 0..pd, then multipole degrees 0..nd-1)."""
    bx, by, bz = bits & 1, (bits >> 1) & 1, (bits >> 2) & 1
    out = np.array(a, dtype=np.complex128)
    base = 0
    for deg in (pd + 1, nd):
        for l in range(deg):
            for m in range(l + 1):
                k = base + tri(l, m)
                v = out[k]
                if bx ^ by:
                    v = np.conj(v)
                if (bz and (l + m) & 1) ^ (bx and m & 1):
                    v = -v
                out[k] = v
        base += tri(deg)
    return out


def random_multipole(oracle, c, rng):
    m = oracle.zeros_series(0, P)
    for _ in range(5):
        oracle.p2m(c + rng.uniform(-0.2, 0.2, 3), rng.uniform(-1, 1), c, P, out=m)
    return m


@pytest.mark.parametrize("bits", range(1, 8))
def test_m2l_mirror_identity(oracle, bits):
    rng = np.random.default_rng(bits)
    sig = np.array([-1.0 if bits & 1 else 1.0, -1.0 if bits & 2 else 1.0,
                    -1.0 if bits & 4 else 1.0])
    xs = np.array([0.1, 0.25, -0.3])
    for d in ([3.0, 0.0, 0.0], [-2.0, 2.0, 1.0], [2.0, -3.0, -2.0], [0.0, 0.0, 3.0]):
        xl = xs + np.array(d)
        m = random_multipole(oracle, xs, rng)
        direct = oracle.to_local("rotate", (0, P), m, xs, (P, 0), oracle.zeros_series(P, 0), xl)
        sm = mirror(m, 0, P, bits)
        loc = oracle.to_local("rotate", (0, P), sm, sig * xs, (P, 0),
                              oracle.zeros_series(P, 0), sig * xl)
        via = mirror(loc, P, 0, bits)
        assert np.linalg.norm(via - direct) <= 1e-12 * np.linalg.norm(direct), (bits, d)


def wigner_blocks(oracle, beta, L):
    """E and O blocks of the rotation by (0, beta, 0), degree L, read off the
    oracle's rotation of unit real / imaginary coefficients."""
    E = np.zeros((L + 1, L + 1))
    O = np.zeros((L + 1, L + 1))
    for m in range(L + 1):
        for part, M in ((1.0, E), (1j, O)):
            a = oracle.zeros_series(L, 0)
            a[tri(L, m)] = part
            d = oracle.rotate((L, 0), a, 0.0, beta, 0.0, (L, 0), oracle.zeros_series(L, 0))
            col = d[tri(L):tri(L) + L + 1]
            M[:, m] = col.real if part == 1.0 else col.imag
    return E, O


@pytest.mark.parametrize("beta", [0.4, 1.3, 2.6])
def test_wigner_block_transpose_symmetry(oracle, beta):
    for L in (1, 5, 8):
        E, O = wigner_blocks(oracle, beta, L)
        for mp in range(1, L + 1):
            for m in range(1, L + 1):
                s = -1.0 if (m - mp) & 1 else 1.0
                assert abs(E[m, mp] - s * E[mp, m]) <= 1e-13
                assert abs(O[m, mp] - s * O[mp, m]) <= 1e-13
        for m in range(1, L + 1):
            s = -1.0 if m & 1 else 1.0
            assert abs(E[0, m] - 2 * s * E[m, 0]) <= 1e-13
            assert abs(O[0, m]) <= 1e-13


def test_vertical_translation_scaled_symmetry(oracle):
    """Translation of a multipole along +z into a local: with the scalings
    above, the coefficient map between degrees is symmetric per order."""
    beta = lambda l: np.sqrt(4 * np.pi / (2 * l + 1))
    xs = np.zeros(3)
    xl = np.array([0.0, 0.0, 2.5])
    for m in range(0, 4):
        n_deg = range(m, P)
        j_deg = range(m, P)
        A = np.zeros((len(j_deg), len(n_deg)))
        for b, n in enumerate(n_deg):
            a = oracle.zeros_series(0, P)
            a[tri(1) + tri(n, m)] = beta(n)   # scaled unit source, after the local term
            loc = oracle.to_local("rotate", (0, P), a, xs, (P, 0), oracle.zeros_series(P, 0), xl)
            for r, j in enumerate(j_deg):
                s = -1.0 if (j + m) & 1 else 1.0
                A[r, b] = (s / beta(j)) * loc[tri(j, m)].real
        assert np.allclose(A, A.T, rtol=1e-11, atol=1e-13 * np.abs(A).max()), m
