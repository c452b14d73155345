"""Pins the oracle's Beyn eigensolver (oracle/beyn.py) before the GPU eigenvalues are checked against it.

* The reference's own Beyn test problems, with eigenvalues known independently:
  tests/tbeyn2.c (Beyn's example 4.9, a random quadratic eigenproblem
  T0 + z T1 + z^2 T2, dim 60, L 30, 150 nodes, circle radius 0.3) and
  tests/tbeyn.c (Beyn's section 4.11 "loaded string", a rational problem, dim
  400, L 10, 50 nodes, centre 150+2i, half-axes 148).  The exact eigenvalues
  inside the contour come from a companion linearisation (scipy.linalg.eigvals).
* The contour itself (beyn.c:69-86): trapezoid rule on the ellipse.
* A physical case: every eigenvalue the oracle returns for a 2 x 2 sphere
  cluster with a rank-gap tolerance makes M(z) singular (sigma_min / sigma_max
  at roundoff level).
"""
import numpy as np
import pytest

from oracle import beyn
from qpms_gb300.workloads import EV, HBAR


def quadratic_problem(dim=60, seed=1):
    rng = np.random.default_rng(seed)
    T0, T1, T2 = (rng.normal(size=(dim, dim)) for _ in range(3))
    return T0, T1, T2


def quadratic_exact(T0, T1, T2):
    sl = pytest.importorskip("scipy.linalg")
    n = T0.shape[0]
    A = np.block([[np.zeros((n, n)), np.eye(n)], [-T0, -T1]])
    B = np.block([[np.eye(n), np.zeros((n, n))], [np.zeros((n, n)), T2]])
    return sl.eigvals(A, B)


def loaded_string(m):
    """tbeyn.c:6-19 as matrices: M(z) = K - z Mm + z / (z - 1) e_m e_m^T."""
    K = np.diag(np.full(m, 2.0 * m)) + np.diag(np.full(m - 1, -1.0 * m), 1) + np.diag(np.full(m - 1, -1.0 * m), -1)
    Mm = (np.diag(np.full(m, 4.0)) + np.diag(np.ones(m - 1), 1) + np.diag(np.ones(m - 1), -1)) / (6.0 * m)
    K[-1, -1] /= 2
    Mm[-1, -1] /= 2
    E = np.zeros((m, m))
    E[-1, -1] = 1

    def M(z):
        return K - z * Mm + (z / (z - 1)) * E
    return M, K, Mm, E


def test_contour_ellipse():
    z, dz = beyn.contour_ellipse(2 + 1j, 0.5, 0.2, 64)
    t = np.arange(64) * 2 * np.pi / 64
    assert np.allclose(z, 2 + 1j + 0.5 * np.cos(t) + 0.2j * np.sin(t), rtol=0, atol=1e-15)
    # trapezoid rule on a closed analytic contour: (1/2 pi i) sum dz / (z - c) = 1, sum dz = 0
    assert abs(np.sum(dz / (z - (2 + 1j))) / (2j * np.pi) - 1) < 1e-10   # error ~ exp(-64 artanh(0.4))
    assert abs(np.sum(dz)) < 1e-14


def test_quadratic_tbeyn2():
    T0, T1, T2 = quadratic_problem()
    Mf = lambda z: T0 + z * T1 + z * z * T2
    rng = np.random.default_rng(2)
    V = rng.normal(size=(60, 30)) + 1j * rng.normal(size=(60, 30))
    r = beyn.beyn_solve(Mf, 60, 30, beyn.ellipse(0, 0.3, 0.3, 150), V, 1e-4, 1, 1e-4)
    ex = quadratic_exact(T0, T1, T2)
    ex = ex[np.abs(ex) < 0.3]
    assert r["neig"] == len(ex) >= 3
    for e in ex:  # quadrature-limited accuracy of the reference's own setup
        assert np.min(np.abs(r["eigval"] - e)) < 2e-7
    assert (r["residuals"] <= 1e-4).all()


def test_loaded_string_tbeyn():
    m = 400
    M, K, Mm, E = loaded_string(m)
    # (z - 1) M(z) = -Mm z^2 + (K + Mm + E) z - K
    ex = quadratic_exact(-K, K + Mm + E, -Mm)
    ex = ex[np.isfinite(ex) & (np.abs(ex - 1) > 1e-6)]       # z = 1 is the pole, not an eigenvalue
    inside = ex[np.abs(ex - (150 + 2j)) < 148]
    rng = np.random.default_rng(3)
    V = rng.normal(size=(m, 10)) + 1j * rng.normal(size=(m, 10))
    r = beyn.beyn_solve(M, m, 10, beyn.ellipse(150 + 2j, 148, 148, 50), V, 1e-4, 1, 1e-4)
    assert len(inside) == 5
    for e in inside:          # every eigenvalue inside is found
        assert np.min(np.abs(r["eigval"] - e)) < 1e-6 * abs(e)
    for z in r["eigval"]:     # everything found is an eigenvalue (two lie outside, where accuracy drops)
        assert np.min(np.abs(ex - z)) < 1e-5 * abs(z)


def test_sphere_cluster_modes_are_singular(orc):
    xs = np.array([-200e-9, 200e-9])
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), np.zeros(4)], 1)
    Mf = beyn.finite_sphere_M(orc, pos, 60e-9, -12 + 1.2j, 2.25, 2)
    m = 64
    rng = np.random.default_rng(0)
    V = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    c = beyn.ellipse((2.52 - 0.3j) * EV / HBAR, 0.1 * EV / HBAR, 0.1 * EV / HBAR, 64)
    r0 = beyn.beyn_solve(Mf, m, m, c, V, 1e300, 1, 0)          # rank_sel_min = 1: only the first singular value
    tol = 1e-10 * r0["ranktest_SV"][0]
    r = beyn.beyn_solve(Mf, m, m, c, V, tol, 1, 0)
    assert r["neig"] == 3
    for z in r["eigval"]:
        s = np.linalg.svd(Mf(z), compute_uv=False)
        assert s[-1] / s[0] < 1e-12
    for z, v in zip(r["eigval"], r["eigvec"]):
        assert np.linalg.norm(Mf(z) @ v) < 1e-10 * np.linalg.norm(Mf(z))
