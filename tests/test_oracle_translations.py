"""Pins the oracle's translation path before the GPU coefficients are checked against it.

* Gaunt coefficients against the reference's own gaunt.c (compiled from its
  sources into oracle/_ref by oracle/build_oracle.py) and against sympy's exact
  Wigner 3j, and through the defining product expansion with scipy's lpmv.
* Legendre functions against scipy, spherical Bessel/Hankel against mpmath
  (real and complex argument, all four kinds, the orders the configs use).
* The reference's single-vs-array test (tests/single_translations_vs_calc.c:
  lMax 3, 10 points with sigma 12, 3 norms x CS bit x J = 1..4, RTOL 1e-8,
  ATOL 1e-14), with numpy's seeded generator standing in for GSL ranlxs0.
* Multiplier-table sizes and the r = 0 NaN semantics of translations.c:641-649.
"""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_multiplier_counts(orc):
    # ragged table sizes of translations.c:439-508 (gaunt_q_max, gauntB_Q_max)
    assert orc.TransCalculator(2).n_multipliers == (109, 133)
    assert orc.TransCalculator(3).n_multipliers == (467, 547)
    assert orc.TransCalculator(6).n_multipliers == (7435, 8219)


def _ref_gaunt():
    from oracle import build_oracle
    path = build_oracle.build_ref()
    if path is None:
        pytest.skip("reference tree absent: gaunt.c not compiled")
    lib = C.CDLL(path)
    lib.gaunt_xu.argtypes = [C.c_int] * 5 + [C.POINTER(C.c_double), C.POINTER(C.c_int)]
    return lib


def test_gaunt_vs_reference_gaunt_c(orc):
    ref = _ref_gaunt()
    worst = 0.0
    for n in range(1, 8):
        for nu in range(1, 8):
            for m in range(-n, n + 1):
                for mu in range(-nu, nu + 1):
                    a = orc.gaunt(m, n, mu, nu)
                    b = np.zeros_like(a)
                    err = C.c_int(0)
                    ref.gaunt_xu(m, n, mu, nu, len(a) - 1, b.ctypes.data_as(C.POINTER(C.c_double)),
                                 C.byref(err))
                    assert err.value == 0
                    ra, rb = a / a[0], b / b[0]
                    worst = max(worst, np.max(np.abs(ra - rb)) / np.max(np.abs(rb)))
    # the reference recurrence itself drifts ~1e-13 at n, nu = 7 (exact 3j is closer)
    assert worst < 1e-12, worst


def test_gaunt_exact_sympy(orc):
    sympy = pytest.importorskip("sympy")
    from sympy.physics.wigner import wigner_3j
    from sympy import factorial, sqrt, N
    rng = np.random.default_rng(5)
    for _ in range(60):
        n, nu = rng.integers(1, 7, size=2)
        m = int(rng.integers(-n, n + 1))
        mu = int(rng.integers(-nu, nu + 1))
        n, nu = int(n), int(nu)
        a = orc.gaunt(m, n, mu, nu)
        M = m + mu
        for q in range(len(a)):
            p = n + nu - 2 * q
            v = ((-1) ** M * (2 * p + 1)
                 * sqrt(factorial(n + m) * factorial(nu + mu) * factorial(p - M)
                        / (factorial(n - m) * factorial(nu - mu) * factorial(p + M)))
                 * wigner_3j(n, nu, p, 0, 0, 0) * wigner_3j(n, nu, p, m, mu, -M))
            assert abs(a[q] - float(N(v, 25))) <= 1e-14 * max(1.0, abs(a[0]))


def test_gaunt_product_expansion(orc):
    from scipy.special import lpmv
    x = np.linspace(-0.95, 0.95, 7)
    for (m, n, mu, nu) in [(1, 2, -1, 3), (-2, 3, 1, 2), (0, 4, 2, 3), (3, 3, -2, 5), (-1, 1, -1, 1)]:
        a = orc.gaunt(m, n, mu, nu)
        lhs = lpmv(m, n, x) * lpmv(mu, nu, x)
        rhs = sum(a[q] * lpmv(m + mu, n + nu - 2 * q, x) for q in range(len(a)))
        np.testing.assert_allclose(rhs, lhs, rtol=1e-11, atol=1e-11 * np.max(np.abs(lhs)))


def test_legendre_vs_scipy(orc):
    from scipy.special import lpmv
    L = 13
    for x in (-0.99, -0.3, 0.0, 0.41, 0.999):
        arr = orc.legendre_array(L, x, -1.0)
        for l in range(L + 1):
            for m in range(l + 1):
                ref = lpmv(m, l, x)  # scipy includes the Condon-Shortley phase
                assert abs(arr[l * (l + 1) // 2 + m] - ref) <= 1e-13 * max(1.0, abs(ref))


def _mp_sph(J, l, z):
    import mpmath as mp
    z = mp.mpc(z)
    pref = mp.sqrt(mp.pi / (2 * z))
    if J == 1:
        return complex(pref * mp.besselj(l + 0.5, z))
    if J == 2:
        return complex(pref * mp.bessely(l + 0.5, z))
    j = pref * mp.besselj(l + 0.5, z)
    y = pref * mp.bessely(l + 0.5, z)
    return complex(j + 1j * y) if J == 3 else complex(j - 1j * y)


@pytest.mark.parametrize("J", [1, 2, 3, 4])
def test_sph_bessel_vs_mpmath(orc, J):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    pts = [0.61, 1.7, 6.3, 19.0, 198.0, 0.7 + 0.0007j, 3.1 + 0.002j, 12.5 + 0.01j, 150.0 + 0.15j,
           2.0 + 1.5j]
    lmax = 13
    for z in pts:
        got = orc.sph_bessel(J, lmax, z)
        for l in range(lmax + 1):
            ref = _mp_sph(J, l, z)
            scale = abs(ref)
            if J in (3, 4):
                scale = max(scale, abs(_mp_sph(2, l, z)))
            assert abs(got[l] - ref) <= 2e-13 * scale, (J, z, l, got[l], ref)


def test_single_vs_array(orc):
    """tests/single_translations_vs_calc.c, restated (numpy seed 666)."""
    rng = np.random.default_rng(666)
    sigma = 12.0
    pts = np.zeros((10, 3))
    pts[0, 0] = pts[1, 1] = pts[2, 2] = sigma
    pts[3:] = rng.normal(0, sigma, size=(7, 3))
    RTOL, ATOL = 1e-8, 1e-14
    lMax = 3
    fails = 0
    for cs in (0, 8):
        for normbits in (65536 * 3, 65536 * 1, 65536 * 2):
            norm = normbits | cs
            c = orc.TransCalculator(lMax, norm)
            for J in (1, 2, 3, 4):
                for p in pts:
                    r = np.linalg.norm(p)
                    th = np.arccos(p[2] / r)
                    ph = np.arctan2(p[1], p[0])
                    A, B = c.get_AB_arrays_single(r, th, ph, False, J)
                    # ATOL scaled by the array magnitude: NORM_NONE entries reach ~1e3,
                    # so analytically-zero B entries carry ~1e-14 rounding in the
                    # closed form while the array form gives an exact 0.
                    atol = ATOL * max(1.0, np.max(np.abs(A)), np.max(np.abs(B)))
                    for yd in range(c.nelem):
                        nd = int(np.sqrt(yd + 1)); md = yd - (nd * (nd + 1) - 1)
                        for ys in range(c.nelem):
                            ns = int(np.sqrt(ys + 1)); ms = ys - (ns * (ns + 1) - 1)
                            a1 = orc.trans_single("A", norm, md, nd, ms, ns, r, th, ph, 0, J)
                            b1 = orc.trans_single("B", norm, md, nd, ms, ns, r, th, ph, 0, J)
                            for s, arr in ((a1, A[yd, ys]), (b1, B[yd, ys])):
                                if abs(s - arr) > atol + RTOL * 0.5 * (abs(s) + abs(arr)):
                                    fails += 1
    assert fails == 0


def test_r_zero_nan(orc):
    c = orc.TransCalculator(2)
    A, B = c.get_AB_arrays_single(0.0, 0.3, 0.2, False, 3)
    assert np.all(np.isnan(A)) and np.all(np.isnan(B))
    A, B = c.get_AB_arrays_single(0.0, 0.3, 0.2, True, 3)  # r_ge_d forces J = 1
    assert np.all(np.isfinite(A))
