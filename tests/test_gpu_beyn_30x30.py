"""Beyn at the benchmark's size: the 30 x 30 sphere array (14,400 unknowns),
64 contour nodes, 64 probe columns, against the FP64 oracle.

* Eigenfrequencies inside the ellipse below the Rayleigh anomaly (the four
  highest-Q modes of the array) match the oracle's (tests/golden/beyn_30x30.json,
  made by tests/golden/make_beyn_30x30.py with numpy LAPACK) within 1e-8
  relative, with the relative rank test giving the same K.
* The benchmark's own ellipse (2.1 eV, half-axes 0.05 / 0.005 eV) holds no
  eigenfrequency: with the relative rank test K = 0 and every singular value
  of A0 is below 1e-10 of the quadrature scale.
* The plain FP64 and mixed-precision node solves give the same partial
  quadrature sums (4 nodes; 1e-9 relative, Frobenius: both node solves are
  refined to a 1e-12 relative residual, and the sums can differ by the
  condition number near the modes times that): the eigenvalue check of the
  mixed path then carries over to the plain one.
"""
import json
import os

import numpy as np
import pytest

from oracle import beyn as ob
from qpms_gb300.workloads import EV, HBAR

pytestmark = pytest.mark.gpu
EIG_RTOL = 1e-8
HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "beyn_30x30.json")


@pytest.fixture(scope="module")
def sys30():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    if not os.path.exists(GOLDEN):
        pytest.skip("fixture tests/golden/beyn_30x30.json not generated")
    g = json.load(open(GOLDEN))
    xs = (np.arange(g["nx"]) - (g["nx"] - 1) / 2) * g["pitch"]
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)
    ss = qpms_gb300.ScatteringSystem(pos, g["radius"], complex(*g["eps_inside"]), g["eps_medium"], g["lMax"])
    assert ss.fecv_size == g["m"]
    return ss, g


def test_eigenfrequencies_vs_oracle_fixture(sys30):
    ss, g = sys30
    c = complex(*g["centre_eV"]) * EV / HBAR
    r = ss.find_modes(c, g["rRe_eV"] * EV / HBAR, g["rIm_eV"] * EV / HBAR, contour_points=g["nodes"],
                      rank_tol=g["rank_tol"], rank_min_sel=g["rank_sel_min"], l=g["l"], seed=g["seed"], mode=1)
    ref = np.array([complex(*x) for x in g["eigval"]])
    got = np.asarray(r["eigval"])
    assert got.size == ref.size and ref.size >= 1
    for e in ref:
        d = np.min(np.abs(got - e))
        assert d <= EIG_RTOL * abs(e), (e / (EV / HBAR), d / abs(e))
    assert r["node_residual_max"] <= 1e-11


def test_configured_contour_holds_no_eigenvalue(sys30):
    ss, g = sys30
    c, rr, ri = 2.1 * EV / HBAR, 0.05 * EV / HBAR, 0.005 * EV / HBAR
    import qpms_gb300
    r = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=-1e-10, rank_min_sel=0, l=64, seed=12345, mode=1)
    assert r["eigval"].size == 0
    _, dz = ob.contour_ellipse(c, rr, ri, 64)
    scale = ob.rank_scale(dz, qpms_gb300.beyn.probe_matrix(ss.fecv_size, 64, 12345))
    assert np.max(r["ranktest_SV"]) <= 1e-10 * scale


def test_plain_and_mixed_partial_sums_agree(sys30):
    from qpms_gb300 import beyn as qb
    ss, g = sys30
    c = complex(*g["centre_eV"]) * EV / HBAR
    args = (ss.s, ss.fecv_size, c, g["rRe_eV"] * EV / HBAR, g["rIm_eV"] * EV / HBAR, g["nodes"], 0, 4, 16)
    plain = qb.scatsys_quadrature(*args, seed=g["seed"], mode=0)
    mixed = qb.scatsys_quadrature(*args, seed=g["seed"], mode=1)
    for p, m in zip(plain[:2], mixed[:2]):
        assert np.linalg.norm(p - m) <= 1e-9 * np.linalg.norm(p)
