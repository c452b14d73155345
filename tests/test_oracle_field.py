"""Pins the oracle's scattered-field evaluation (qpms_scatsys_scattered_E,
scatsystem.c:2013-2039; VSWFs of vswf.c:230-288).

The reference marks the function QPMS_UNTESTED and ships no test or fixture
for it, so the pins are identities any correct implementation satisfies:
* regular waves (J = 1) with the plane-wave coefficients of the oracle's
  incident-field expansion reproduce E0 exp(i k.r) near the origin
  (truncation below 1e-11 at |k r| <= 1, lMax 10), including the origin
  itself (the r = 0 branch of qpms_vswf_fill_csph) and points on the polar
  axis (the |cos theta| = 1 branch of legendre.c);
* outgoing waves (J = 3) with f = T a of one sphere reproduce the scattered
  field of Bohren & Huffman (4.45), (4.50), (4.46)-(4.47) evaluated with
  scipy's spherical Bessel functions, near field and far field.
"""
import numpy as np
import pytest
from scipy.special import spherical_jn, spherical_yn

from qpms_gb300.workloads import EV, HBAR, C0


def _ball_points(rng, n, radius):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    return v * radius * rng.uniform(0.05, 1.0, size=(n, 1)) ** (1 / 3)


@pytest.mark.parametrize("kdir,E0", [
    ((0, 0, 1), (1, 0, 0)),
    ((0, 0, -1), (0, 1j, 0)),
    ((0.3, -0.5, 0.8), None),
])
def test_regular_plane_wave_reexpansion(orc, kdir, E0):
    lMax, k = 10, 2.0e7
    kd = np.asarray(kdir, dtype=float)
    kd = kd / np.linalg.norm(kd)
    if E0 is None:  # elliptic polarisation perpendicular to k
        e1 = np.cross(kd, [0, 0, 1.0])
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(kd, e1)
        E0 = e1 + (0.4 - 0.7j) * e2
    E0 = np.asarray(E0, dtype=complex)
    a = orc.planewave_full(lMax, np.zeros((1, 3)), k * kd, E0)
    rng = np.random.default_rng(3)
    pts = _ball_points(rng, 40, 1.0 / k)
    pts = np.vstack([pts, [[0, 0, 0], [0, 0, 0.7 / k], [0, 0, -0.4 / k], [0.5 / k, 0, 0]]])
    E = orc.scattered_E(lMax, np.zeros((1, 3)), 1, k, a, pts)
    ref = E0[None, :] * np.exp(1j * k * (pts @ kd))[:, None]
    assert np.abs(E - ref).max() <= 1e-9 * np.abs(E0).max()


def _bh_pitau(nmax, mu):
    pi = np.zeros((nmax + 1,) + mu.shape)
    tau = np.zeros_like(pi)
    pi[1] = 1.0
    for n in range(1, nmax + 1):
        if n >= 2:
            pi[n] = (2 * n - 1) / (n - 1) * mu * pi[n - 1] - n / (n - 1) * pi[n - 2]
        tau[n] = n * mu * pi[n] - (n + 1) * pi[n - 1]
    return pi, tau


def _bh_an_bn(n, x, m):
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


def _bh_scattered(nmax, k, radius, m, pts):
    """Scattered field of an x-polarised plane wave exp(ikz) on a sphere at the
    origin, Bohren & Huffman (4.45) with the vector harmonics (4.50), cartesian."""
    x, y, z = pts.T
    r = np.linalg.norm(pts, axis=1)
    th = np.arccos(z / r)
    ph = np.arctan2(y, x)
    rho = k * r
    pi, tau = _bh_pitau(nmax, np.cos(th))
    Es = np.zeros((3, pts.shape[0]), dtype=complex)  # (r, theta, phi)
    for n in range(1, nmax + 1):
        an, bn = _bh_an_bn(n, k * radius, m)
        En = 1j ** n * (2 * n + 1) / (n * (n + 1))
        h = spherical_jn(n, rho) + 1j * spherical_yn(n, rho)
        hm1 = spherical_jn(n - 1, rho) + 1j * spherical_yn(n - 1, rho)
        dxi = hm1 - n * h / rho  # [rho h_n]' / rho
        M_th = np.cos(ph) * pi[n] * h
        M_ph = -np.sin(ph) * tau[n] * h
        N_r = np.cos(ph) * n * (n + 1) * np.sin(th) * pi[n] * h / rho
        N_th = np.cos(ph) * tau[n] * dxi
        N_ph = -np.sin(ph) * pi[n] * dxi
        Es[0] += En * (1j * an * N_r)
        Es[1] += En * (1j * an * N_th - bn * M_th)
        Es[2] += En * (1j * an * N_ph - bn * M_ph)
    st, ct, sf, cf = np.sin(th), np.cos(th), np.sin(ph), np.cos(ph)
    return np.stack([st * cf * Es[0] + ct * cf * Es[1] - sf * Es[2],
                     st * sf * Es[0] + ct * sf * Es[1] + cf * Es[2],
                     ct * Es[0] - st * Es[1]], axis=1)


@pytest.mark.parametrize("eps_i", [-12 + 1.2j, 4.0])
def test_single_sphere_field_vs_bohren_huffman(orc, eps_i):
    lMax, radius, eps_e = 6, 80e-9, 2.25
    om = 2.0 * EV / HBAR
    k = np.sqrt(eps_e) * om / C0
    T = orc.tmatrix_sphere_diag(lMax, radius, om, eps_i, eps_e)
    a = orc.planewave_full(lMax, np.zeros((1, 3)), np.array([0, 0, k]), np.array([1, 0, 0], dtype=complex))
    f = T * a
    rng = np.random.default_rng(5)
    v = rng.normal(size=(60, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    pts = v * radius * rng.uniform(1.05, 40.0, size=(60, 1))
    E = orc.scattered_E(lMax, np.zeros((1, 3)), 3, k, f, pts)
    ref = _bh_scattered(lMax, k, radius, np.sqrt(complex(eps_i)) / np.sqrt(eps_e), pts)
    err = np.linalg.norm(E - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() <= 1e-10, err.max()
