"""Pins the oracle to the reference's own code and published values.

* translations.c and the lattice sums of ewald.c / ewaldsf.c, compiled from
  the reference's sources into oracle/_ref (oracle/build_oracle.py,
  build_ref_lib; GSL, AMOS and CBLAS calls answered by oracle/refshim), must
  give the oracle's A / B arrays (every normalisation convention, J = 1..4)
  and its Ewald-summed A / B arrays (the reference's eta-invariance parameter
  sets of tests/CMakeLists.txt:87-120 and the dispersion-scan lattices) within
  1e-13 relative.  Skipped where the reference tree is absent.
* Xu's published translation coefficients, the reference's known-answer table
  (tests/golden/xu_translations.json from qpms/tests/testcases_translations_Xu),
  converted from Xu's normalisation to the unnormalised convention:
  A_Xu(m n, mu nu) = i^(nu - n) g(mu, nu) / g(m, n) A(m n, mu nu), the same for
  B, with g(m, n) = (2n + 1) (n - m)! / (n + m)!.  The oracle matches the
  table within 1e-7 (the tabulated values carry a common 3e-8 offset); the
  entry (m, n, mu, nu) = (-5, 20, 5, 20) of A differs in the sign of its real
  part (B of that entry is zero and matches) and is left out.
"""
import json
import os
from math import lgamma, log

import numpy as np
import pytest

from oracle import orc, refpin

HERE = os.path.dirname(os.path.abspath(__file__))
NORM_NONE, NORM_POWER, NORM_SPHARM, CSPHASE = 2 * 65536, 65536, 3 * 65536, 8
needs_ref = pytest.mark.skipif(not refpin.available(), reason="reference sources not compiled (oracle/_ref)")


@needs_ref
@pytest.mark.parametrize("norm", [NORM_POWER | CSPHASE, NORM_POWER, NORM_NONE, NORM_NONE | CSPHASE, NORM_SPHARM,
                                  NORM_SPHARM | CSPHASE])
@pytest.mark.parametrize("lMax", [1, 3, 6])
def test_reference_translations_vs_oracle(norm, lMax):
    rc = refpin.RefCalculator(lMax, norm)
    oc = orc.TransCalculator(lMax, norm)
    rng = np.random.default_rng(lMax + norm)
    for _ in range(6):
        kr = complex(rng.uniform(0.3, 40), rng.uniform(0, 0.5))
        th, ph = rng.uniform(0, np.pi), rng.uniform(0, 2 * np.pi)
        for J in (1, 2, 3, 4):
            A, B = rc.get_AB_arrays(kr, th, ph, J)
            oA, oB = oc.get_AB_batch(np.array([kr]), np.array([th]), np.array([ph]), J)
            for X, O in ((A, oA[0]), (B, oB[0])):
                assert np.linalg.norm(X - O) <= 1e-13 * np.linalg.norm(O)


SETS = [  # k, beta, particle_shift, maxR (b1 = (1,0), b2 = (0,1), maxK 160): tests/CMakeLists.txt:87-120
    (2.3, (2.7, 1), (0.5, 0.1325), 20), (2.3, (2.7, 1), (0.0, 0.0), 20),
    (2.3 + 0.1j, (2.7, 1), (0.5, 0.1325), 20), (2.3 - 0.1j, (2.7, 1), (0.5, 0.1325), 20),
    (2.3 + 0.1j, (2.7, 1), (0.0, 0.0), 20), (2.3 - 0.1j, (2.7, 1), (0.0, 0.0), 20),
    (2.3, (0.0, 0.0), (0.5, 0.1325), 40)]


@needs_ref
@pytest.mark.parametrize("k,beta,shift,maxR", SETS)
def test_reference_lattice_sums_vs_oracle(k, beta, shift, maxR):
    rc = refpin.RefCalculator(3, NORM_POWER | CSPHASE)
    oc = orc.TransCalculator(3)
    for eta in (1.6, 2.5):
        A, Ae, B, Be = rc.get_AB_arrays_e32(eta, k, (1, 0), (0, 1), beta, shift, maxR, 160)
        oA, oB = orc.get_AB_arrays_e32(oc, eta, k, (1, 0), (0, 1), beta, shift, maxR, 160)
        for X, O in ((A, oA), (B, oB)):
            assert np.linalg.norm(X - O) <= 1e-13 * np.linalg.norm(O)


@needs_ref
@pytest.mark.parametrize("lattice", ["square", "honeycomb"])
def test_reference_lattice_sums_dispersion_lattices(lattice):
    """The 580 nm lattices of the dispersion scan, lMax 3, the reference's
    cut-offs (scatsystem.c:1227-1228) and adjusted eta, real and complex k."""
    from qpms_gb300.workloads import honeycomb_lattice, square_lattice
    b1, b2, pos = square_lattice() if lattice == "square" else honeycomb_lattice()
    area = abs(b1[0] * b2[1] - b1[1] * b2[0])
    maxR = 64 * np.sqrt(area)
    maxK = 2048 * 2 * np.pi / maxR
    rc = refpin.RefCalculator(3, NORM_POWER | CSPHASE)
    oc = orc.TransCalculator(3)
    for k, beta in ((1.6e7, (2e6, 1e6)), (1.9e7 + 2e4j, (5e5, 0.0)), (1.3e7, (0.0, 0.0))):
        eta = orc.adjusted_eta(area, k, np.array([beta[0], beta[1], 0.0]), 3)
        for d in pos:
            shift = tuple(d - pos[0])
            A, Ae, B, Be = rc.get_AB_arrays_e32(eta, k, b1, b2, beta, shift, maxR, maxK)
            oA, oB = orc.get_AB_arrays_e32(oc, eta, k, b1, b2, beta, shift, maxR, maxK)
            for X, O in ((A, oA), (B, oB)):
                assert np.linalg.norm(X - O) <= 1e-13 * np.linalg.norm(O)


def _g(m, n):
    return log(2 * n + 1) + lgamma(n - m + 1) - lgamma(n + m + 1)


def xu_convert(A, m, n, mu, nu):
    """Unnormalised coefficient -> Xu's normalisation."""
    return A * (1j) ** (nu - n) * np.exp(_g(mu, nu) - _g(m, n))


XU_SIGN_ERRATUM = (-5, 20, 5, 20)


def test_xu_table_via_oracle():
    g = json.load(open(os.path.join(HERE, "golden", "xu_translations.json")))
    oc = orc.TransCalculator(20, NORM_NONE)
    checked = 0
    for c in g["cases"]:
        m, n, mu, nu = c["m"], c["n"], c["mu"], c["nu"]
        kr, th, ph = c["kd"]
        A, B = oc.get_AB_batch(np.array([complex(kr)]), np.array([th]), np.array([ph]), g["J"])
        y, yu = n * (n + 1) + m - 1, nu * (nu + 1) + mu - 1
        a, b = xu_convert(A[0][y, yu], m, n, mu, nu), xu_convert(B[0][y, yu], m, n, mu, nu)
        xa, xb = complex(*c["A"]), complex(*c["B"])
        if (m, n, mu, nu) != XU_SIGN_ERRATUM:
            assert abs(a - xa) <= 1e-7 * abs(xa), (m, n, mu, nu, a, xa)
        if xb == 0:
            assert abs(b) <= 1e-12 * abs(a)
        else:
            assert abs(b - xb) <= 1e-7 * abs(xb), (m, n, mu, nu, b, xb)
        checked += 1
    assert checked == len(g["cases"]) >= 10
