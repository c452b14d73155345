"""Pins the oracle's axially symmetric T-matrices (extended-boundary-condition
method, tmatrices.c:615-894) before the GPU results are checked against them:

* a sphere given as an arc reproduces the Mie T-matrix (Bohren-Huffman-pinned
  oracle) at every l, for a metal and a dielectric: 1e-12;
* lossless spheroids (prolate and oblate): the scattering matrix S = I + 2T
  of the power-normalised waves is unitary, T + T^H + 2 T^H T = 0, to the
  truncation error, which falls as lMaxQR grows;
* reciprocity T_(t l m),(t' l' m') = (-1)^(m + m') T_(t' l' -m'),(t l -m) of the
  same waves, to the truncation error (1e-5 at lMaxQR 6, spheroids);
* the arc parametrisations (r, beta) against the shapes' geometry.
"""
import numpy as np
import pytest

C0 = 299792458.0
OM = 2.1 * 1.602176634e-19 / 1.054571817e-34


def _idx(lMax):
    return [(t, l, m) for t in range(2) for l in range(1, lMax + 1) for m in range(-l, l + 1)]


@pytest.mark.parametrize("lMax", [1, 3, 5])
@pytest.mark.parametrize("eps_i", [-12 + 1.2j, 4.0])
def test_sphere_as_arc_is_mie(orc, lMax, eps_i):
    k, ki = np.sqrt(2.25) * OM / C0, np.sqrt(eps_i) * OM / C0
    T = orc.tmatrix_axialsym(lMax, k, ki, "sphere", [50e-9], lMaxQR=lMax + 1)
    Td = orc.tmatrix_sphere_diag(lMax, 50e-9, OM, eps_i, 2.25)
    assert np.abs(np.diag(T) - Td).max() <= 1e-12 * np.abs(Td).max()
    assert np.abs(T - np.diag(np.diag(T))).max() <= 1e-14 * np.abs(Td).max()


@pytest.mark.parametrize("par", [(40e-9, 80e-9), (70e-9, 35e-9)])
def test_spheroid_unitarity_and_reciprocity(orc, par):
    k, ki = OM / C0, 2 * OM / C0
    res = []
    for lq in (3, 6):
        T = orc.tmatrix_axialsym(3, k, ki, "spheroid", par, lMaxQR=lq)
        res.append(np.abs(T + T.conj().T + 2 * T.conj().T @ T).max() / np.abs(T).max())
    assert res[1] <= 3e-6 and res[1] < 0.05 * res[0], res
    idx = _idx(3)
    worst = 0.0
    for i, (t1, l1, m1) in enumerate(idx):
        for j, (t2, l2, m2) in enumerate(idx):
            jj, ii = idx.index((t2, l2, -m2)), idx.index((t1, l1, -m1))
            worst = max(worst, abs(T[i, j] - (-1) ** (m1 + m2) * T[jj, ii]))
    assert worst <= 1e-5 * np.abs(T).max()


def test_cylinder_block_structure(orc):
    """Only m = m' couples; the cylinder's mirror symmetry z -> -z couples
    (t, l) to (t', l') only when l + l' + [t != t'] is even."""
    k, ki = np.sqrt(2.25) * OM / C0, np.sqrt(-12 + 1.2j) * OM / C0
    T = orc.tmatrix_axialsym(3, k, ki, "cylinder", [50e-9, 100e-9], lMaxQR=4)
    idx = _idx(3)
    sc = np.abs(T).max()
    for i, (t1, l1, m1) in enumerate(idx):
        for j, (t2, l2, m2) in enumerate(idx):
            if m1 != m2 or (l1 + l2 + (t1 != t2)) % 2:
                assert abs(T[i, j]) <= 1e-12 * sc, (idx[i], idx[j], T[i, j])


def test_arcs(orc):
    R, h = 50e-9, 100e-9
    th = np.arctan(2 * R / h)
    for theta in np.linspace(0.01, np.pi - 0.01, 37):
        r, b = orc.arc("cylinder", [R, h], theta)
        z, rho = r * np.cos(theta), r * np.sin(theta)
        if theta < th:
            assert abs(z - h / 2) < 1e-20 and abs(b + theta) < 1e-15
        elif theta > np.pi - th:
            assert abs(z + h / 2) < 1e-20
        else:
            assert abs(rho - R) < 1e-20
        a, c = 40e-9, 80e-9
        r, b = orc.arc("spheroid", [a, c], theta)
        x, z = r * np.sin(theta), r * np.cos(theta)
        assert abs((x / a) ** 2 + (z / c) ** 2 - 1) < 1e-14
        nx, nz = x / a ** 2, z / c ** 2                     # outward normal
        cosb = (nx * np.sin(theta) + nz * np.cos(theta)) / np.hypot(nx, nz)
        assert abs(np.cos(b) - cosb) < 1e-14
