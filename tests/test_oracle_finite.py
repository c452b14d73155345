"""Pins the oracle's finite mode-problem path (T, S, a_inc, M = I - T S, LU, sigma_ext).

The reference's finite full-matrix builder aborts in the snapshot
(scatsystem.c:1293), and its irrep-packed builders need GSL/LAPACKE, so the
pins are physical identities that any correct implementation satisfies:
* Mie T-matrix == (-a_n, -b_n) of Bohren & Huffman (scipy Bessel functions);
* one sphere at the origin: -Re(a^H f)/k^2 == Mie extinction (2 pi/k^2) sum (2n+1) Re(a_n + b_n);
* lossless cluster: extinction == scattering, sigma_scat = Re(f^H (I + S_reg) f)/k^2
  (misc/finiterectlat-scatter.py:104-111), i.e. energy conservation through
  the whole assembled system;
* LU/solve (zgetrf/zgetrs semantics) against numpy.
"""
import numpy as np
import pytest
from scipy.special import spherical_jn, spherical_yn

from qpms_gb300.workloads import EV, HBAR, C0

EPS_I = -12 + 1.2j
EPS_E = 2.25


def _bh(n, x, m):
    def psi(z):
        return z * spherical_jn(n, z)

    def dpsi(z):
        return spherical_jn(n, z) + z * spherical_jn(n, z, derivative=True)

    def xi(z):
        return z * (spherical_jn(n, z) + 1j * spherical_yn(n, z))

    def dxi(z):
        return (spherical_jn(n, z) + 1j * spherical_yn(n, z)) + z * (
            spherical_jn(n, z, True) + 1j * spherical_yn(n, z, True))

    an = (m * psi(m * x) * dpsi(x) - psi(x) * dpsi(m * x)) / (m * psi(m * x) * dxi(x) - xi(x) * dpsi(m * x))
    bn = (psi(m * x) * dpsi(x) - m * psi(x) * dpsi(m * x)) / (psi(m * x) * dxi(x) - m * xi(x) * dpsi(m * x))
    return an, bn


@pytest.mark.parametrize("E", [1.6, 2.1, 2.6])
@pytest.mark.parametrize("eps_i", [EPS_I, 4.0])
def test_mie_vs_bohren_huffman(orc, E, eps_i):
    lMax, a = 4, 60e-9
    om = E * EV / HBAR
    T = orc.tmatrix_sphere_diag(lMax, a, om, eps_i, EPS_E)
    ke, ki = np.sqrt(EPS_E) * om / C0, np.sqrt(complex(eps_i)) * om / C0
    ne = lMax * (lMax + 2)
    for n in range(1, lMax + 1):
        an, bn = _bh(n, ke * a, ki / ke)
        y = n * (n + 1) - 1
        assert abs(T[y] + an) <= 1e-12 * abs(an)
        assert abs(T[ne + y] + bn) <= 1e-12 * abs(bn)


def test_single_sphere_extinction(orc):
    lMax, a = 3, 50e-9
    c = orc.TransCalculator(lMax)
    for E in (1.6, 2.0, 2.6):
        om = E * EV / HBAR
        f, ainc, sig = orc.finite_sphere_scatter(c, np.zeros((1, 3)), a, EPS_I, EPS_E, om)
        ke, ki = np.sqrt(EPS_E) * om / C0, np.sqrt(EPS_I) * om / C0
        ref = 2 * np.pi / ke ** 2 * sum((2 * n + 1) * (sum(_bh(n, ke * a, ki / ke))).real
                                        for n in range(1, lMax + 1))
        assert abs(sig - ref) <= 1e-12 * abs(ref)


def square_array(nx, ny, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)], axis=1)


def test_energy_conservation_lossless_cluster(orc):
    lMax, a = 2, 50e-9
    pos = square_array(4, 4, 400e-9)
    c = orc.TransCalculator(lMax)
    for E in (1.7, 2.3):
        om = E * EV / HBAR
        ke = np.sqrt(EPS_E) * om / C0
        f, ainc, sig = orc.finite_sphere_scatter(c, pos, a, 4.0, EPS_E, om)
        S1 = orc.finite_translation_matrix(c, pos, ke, 1)
        sig_scat = np.vdot(f, (S1 + np.eye(len(f))) @ f).real / ke ** 2
        assert abs(sig - sig_scat) <= 1e-10 * abs(sig)
        # lossy spheres absorb: extinction > scattering
        f, ainc, sig = orc.finite_sphere_scatter(c, pos, a, EPS_I, EPS_E, om)
        sig_scat = np.vdot(f, (S1 + np.eye(len(f))) @ f).real / ke ** 2
        assert sig > sig_scat > 0


def test_lu_vs_numpy(orc):
    rng = np.random.default_rng(4)
    for n in (1, 7, 64):
        M = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        b = rng.normal(size=(n, 3)) + 1j * rng.normal(size=(n, 3))
        a, ipiv, info = orc.lu_factor(M)
        assert info == 0
        x = orc.lu_solve(a, ipiv, b)
        np.testing.assert_allclose(x, np.linalg.solve(M, b), rtol=1e-10, atol=1e-12)


def test_modeproblem_structure(orc):
    """M = I - T S: identity diagonal blocks, off-diagonal blocks = -T_R S(R<-C)."""
    lMax, a = 2, 50e-9
    pos = square_array(2, 2, 400e-9)
    c = orc.TransCalculator(lMax)
    om = 2.0 * EV / HBAR
    ke = np.sqrt(EPS_E) * om / C0
    Td = orc.tmatrix_sphere_diag(lMax, a, om, EPS_I, EPS_E)
    n = Td.size
    T = np.zeros((4, n, n), dtype=complex)
    for p in range(4):
        T[p] = np.diag(Td)
    M = orc.finite_modeproblem(c, pos, T, ke)
    S = orc.finite_translation_matrix(c, pos, ke, 3)
    Tb = np.kron(np.eye(4), np.diag(Td))
    np.testing.assert_allclose(M, np.eye(4 * n) - Tb @ S, rtol=0, atol=1e-14)
