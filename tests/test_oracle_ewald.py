"""Pins the oracle's 2D Ewald sums before the GPU sums are checked against them.

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


# ---- layers at different heights (particle_shift.z != 0) ----
OBLIQUE = ((1.0, 0.0), (0.3, 1.1))


@pytest.mark.parametrize("k,shift", [(2.3 + 0.9j, (0.31, -0.2, 0.37)), (4.1 + 1.1j, (0.0, 0.0, -0.5)),
                                     (2.3 + 0.9j, (0.1, 0.2, 0.05)), (3.0 + 1.0j, (0.5, 0.55, -1.2))])
def test_shifted_vs_direct_sum(orc, k, shift):
    """The shifted Ewald sums against the lattice sum they represent, summed
    directly (converges exponentially for Im k > 0), all (n, m) to lMax_e 5.
    eta |z| <= 1.2 (the Delta series loses e^(2 eta^2 z^2) to cancellation)."""
    d = orc.sigma_direct(5, k, *OBLIQUE, (0.7, -0.4), shift, 70)
    eta = min(1.6, 1.2 / abs(shift[2]))
    e = orc.ewald_sigma_xy(5, eta, k, *OBLIQUE, (0.7, -0.4), shift, 20, 160)[0]
    assert np.abs(d - e).max() <= 1e-13 * np.abs(d).max()
    assert np.abs(d[1::2]).max() > 1e-3 * np.abs(d).max()   # the odd-parity terms are present


@pytest.mark.parametrize("k,shift", [(2.3, (0.31, -0.2, 0.37)), (5.3, (0.0, 0.0, 0.45)),
                                     (5.3, (0.2, 0.5, -0.8)), (2.3 - 0.1j, (0.5, 0.1325, 0.2))])
def test_shifted_eta_invariance(orc, k, shift):
    """Real k (propagating diffraction orders: the branch of Gamma and of the
    Kambe Delta series) and a lossy k with Im k < 0: sigma independent of eta."""
    res = [orc.ewald_sigma_xy(5, eta, k, *OBLIQUE, (0.7, -0.4), shift, 20, 160)[0] for eta in (1.2, 1.6, 2.2)]
    scale = np.abs(res[0]).max()
    for r in res[1:]:
        assert np.abs(r - res[0]).max() <= 1e-12 * scale


def test_shifted_limit_and_parity(orc):
    """shift.z -> 0 joins the xy sums; the even terms are even and the odd
    terms odd in shift.z (reflection through the lattice plane)."""
    args = (1.6, 2.3, (1, 0), (0, 1), (2.7, 1))
    e0 = orc.ewald_sigma_xy(3, *args, (0.5, 0.1325), 20, 160)[0]
    ez = orc.ewald_sigma_xy(3, *args, (0.5, 0.1325, 1e-12), 20, 160)[0]
    assert np.abs(ez - e0).max() <= 1e-10 * np.abs(e0).max()
    p = orc.ewald_sigma_xy(3, *args, (0.5, 0.1325, 0.3), 20, 160)[0]
    q = orc.ewald_sigma_xy(3, *args, (0.5, 0.1325, -0.3), 20, 160)[0]
    n = np.floor(np.sqrt(np.arange(16))).astype(int)
    m = np.arange(16) - n * (n + 1)
    odd = (n + m) % 2 == 1
    sc = np.abs(p).max()
    assert np.abs(p[~odd] - q[~odd]).max() <= 1e-13 * sc
    assert np.abs(p[odd] + q[odd]).max() <= 1e-13 * sc and np.abs(p[odd]).max() > 1e-3 * sc


@pytest.mark.parametrize("k,shift", [(3.0 + 1.0j, (0.5, 0.55, -1.2)), (4.1 + 0.5j, (0.1, 0.2, 0.9)),
                                     (9.0 + 1.0j, (0.3, 0.1, -0.5))])
def test_spectral_vs_direct_sum(orc, k, shift):
    """Distant layers: the pure reciprocal-lattice (Weyl) sum, the eta -> inf
    limit of the shifted sums with Delta_j(0, z) from half-integer Bessel K,
    against the direct lattice sum."""
    d = orc.sigma_direct(5, k, *OBLIQUE, (0.7, -0.4), shift, 90)
    sp = orc.ewald_sigma_xy(5, np.inf, k, *OBLIQUE, (0.7, -0.4), shift, 20, 160)[0]
    assert np.abs(d - sp).max() <= 1e-13 * np.abs(d).max()


@pytest.mark.parametrize("k,shift", [(3.0, (0.5, 0.55, -1.2)), (5.3, (0.2, 0.5, -0.8)), (4.0 - 0.1j, (0.3, 0.1, 0.7))])
def test_spectral_vs_ewald_real_k(orc, k, shift):
    """Real k (propagating orders: the outgoing branch e^{i k_z |z|}): the
    reciprocal-lattice sum against the Ewald sums at eta |z| = 1."""
    ew = orc.ewald_sigma_xy(5, 1.0 / abs(shift[2]), k, *OBLIQUE, (0.7, -0.4), shift, 30, 160)[0]
    sp = orc.ewald_sigma_xy(5, np.inf, k, *OBLIQUE, (0.7, -0.4), shift, 20, 160)[0]
    assert np.abs(ew - sp).max() <= 1e-12 * np.abs(ew).max()
