"""Pins the oracle's 2D Ewald sums before they serve as the checker.

* The reference's own eta-invariance test (tests/test_scalar_ewald32.c with the
  seven parameter sets of tests/CMakeLists.txt:87-120): sigma_total = sigma_S +
  sigma_L (+ sigma0) must agree across eta in {1.5, 1.6, 2.5, 2.6} within
  |a - b| <= 1e-8 + 1e-10 (|a| + |b|)/2 (argv[13] = atol, argv[14] = rtol).
* The short-range integrals against mpmath quadrature, the complex incomplete
  gamma against mpmath.gammainc, the Gauss-Kronrod constants on polynomials.
"""
import numpy as np
import pytest

SETS = [  # k, beta, particle_shift, maxR  (b1 = (1,0), b2 = (0,1), lMax 3, maxK 160, csphase -1)
    (2.3, (2.7, 1), (0.5, 0.1325), 20), (2.3, (2.7, 1), (0.0, 0.0), 20),
    (2.3 + 0.1j, (2.7, 1), (0.5, 0.1325), 20), (2.3 - 0.1j, (2.7, 1), (0.5, 0.1325), 20),
    (2.3 + 0.1j, (2.7, 1), (0.0, 0.0), 20), (2.3 - 0.1j, (2.7, 1), (0.0, 0.0), 20),
    (2.3, (0.0, 0.0), (0.5, 0.1325), 40)]


@pytest.mark.parametrize("k,beta,shift,maxR", SETS)
def test_eta_invariance(orc, k, beta, shift, maxR):
    atol, rtol = 1e-8, 1e-10
    res = [orc.ewald_sigma_xy(3, eta, k, (1, 0), (0, 1), beta, shift, maxR, 160)[0]
           for eta in (1.5, 1.6, 2.5, 2.6)]
    for i in range(4):
        for j in range(i + 1, 4):
            a, b = res[i], res[j]
            assert (np.abs(a - b) <= atol + rtol * 0.5 * (np.abs(a) + np.abs(b))).all()


def test_sr_integral_vs_mpmath(orc):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    for (r, k, n, eta) in [(1.0, 2.3, 0, 1.5), (1.3, 2.3 + 0.1j, 3, 2.5), (0.6, 3.0, 2, 1.6), (2.0, 1.0, 7, 1.2)]:
        f = lambda x: mp.e ** (-(r * x) ** 2 + (mp.mpc(k) / x) ** 2 / 4) * x ** (2 * n)
        ref = complex(mp.quad(f, mp.linspace(eta, eta * 6, 12) + [mp.inf]))
        got = orc.ewald_sr_integral(r, k, n, eta)
        assert abs(got - ref) <= 1e-12 * abs(ref)


def test_gamma_inc_vs_mpmath(orc):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    for (a, x) in [(0.5, 2.0), (-0.5, 2.0 + 1j), (-1.5, -0.3 + 0.2j), (-2.5, 5.0), (0.5, 0.3 - 0.1j),
                   (-0.5, 12.0 + 3j)]:
        ref = complex(mp.gammainc(a, mp.mpc(x)))
        assert abs(orc.complex_gamma_inc(a, x) - ref) <= 1e-13 * abs(ref)


def test_sigma_parts_consistency(orc):
    """sigma_total == sigma_S + sigma_L (+ sigma0 only for zero shift)."""
    tot, s, l = orc.ewald_sigma_xy(3, 1.6, 2.3, (1, 0), (0, 1), (2.7, 1), (0.5, 0.1325), 20, 160)
    assert np.allclose(tot, s + l, rtol=0, atol=1e-15 * np.abs(tot).max())
    tot0, s0, l0 = orc.ewald_sigma_xy(3, 1.6, 2.3, (1, 0), (0, 1), (2.7, 1), (0, 0), 20, 160)
    d = tot0 - s0 - l0
    assert abs(d[0]) > 0 and np.allclose(d[1:], 0, atol=1e-15 * np.abs(tot0).max())


def test_adjusted_eta(orc):
    """qpms_ss_adjusted_eta (scatsystem.c:68-80): max(sqrt(pi / A),
    sqrt(|kappa^2 - |k|^2| (lMax + 1/2) / 16)) for kappa^2 >= |k|^2, else sqrt(pi / A)."""
    A = 580e-9 ** 2 * np.sqrt(3) / 2
    for kap, kv in [(1.9e7, (5e5, 1e6, 0)), (1.2e7 + 3e5j, (0, 0, 0)), (1e6, (4e6, 0, 0))]:
        k2 = sum(x * x for x in kv)
        exp = np.sqrt(np.pi / A)
        if abs(kap) ** 2 >= k2:
            exp = max(exp, np.sqrt(abs(abs(kap) ** 2 - k2) * (3 + 0.5) / 16))
        assert abs(orc.adjusted_eta(A, kap, kv, 3) - exp) <= 1e-14 * exp
