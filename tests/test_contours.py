"""Half-ellipse and kidney integration contours (beyn_contour_halfellipse,
beyn_contour_kidney; beyn.c:117-226) of the library against the oracle's
restatement, and the properties a closed contour must have: the nodes' dz
sum to zero and the quadrature of 1/(z - p) is 2 pi i for p inside, 0
outside (to the discretisation error of the midpoint rule, 1e-3 at 400
nodes).  Host-only geometry: no GPU is used.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import beyn as ob

ORIENT = {"re+": 3, "re-": 1, "im+": 0, "im-": 2}
# a point well inside each orientation's contour, relative to centre with half-axes (2, 1)
INSIDE = {"re+": 1.0, "re-": -1.0, "im+": 0.5j, "im-": -0.5j}


@pytest.fixture(scope="module")
def qb():
    from qpms_gb300 import beyn
    return beyn


def _lib_contour(qb, centre, rr, ri, n, shape):
    p = qb.make_contour(centre, rr, ri, n, shape)
    try:
        return qb.contour_nodes(p)
    finally:
        C.CDLL(None).free(C.c_void_p(p))


@pytest.mark.parametrize("o", list(ORIENT))
@pytest.mark.parametrize("kind", ["halfellipse", "kidney"])
def test_contour_vs_oracle_and_closed(qb, kind, o):
    centre, rr, ri, n = 3.0 - 0.5j, 2.0, 1.0, 400
    shape = ("halfellipse", ORIENT[o]) if kind == "halfellipse" else ("kidney", 0.25, ORIENT[o])
    z, dz = _lib_contour(qb, centre, rr, ri, n, shape)
    if kind == "halfellipse":
        zr, dzr, _ = ob.halfellipse(centre, rr, ri, n, ORIENT[o])
    else:
        zr, dzr, _ = ob.kidney(centre, rr, ri, 0.25, n, ORIENT[o])
    assert np.abs(z - zr).max() <= 1e-14 * abs(centre) + 1e-14
    assert np.abs(dz - dzr).max() <= 1e-14
    assert abs(dz.sum()) <= 1e-3 * np.abs(dz).sum()
    wind_in = np.sum(dz / (z - (centre + INSIDE[o]))) / (2j * np.pi)
    wind_out = np.sum(dz / (z - (centre - INSIDE[o]))) / (2j * np.pi)
    assert abs(wind_in - 1) <= 1e-3 and abs(wind_out) <= 1e-3


def test_zero_signs_on_the_straight_side(qb):
    # the straight side of an RE_MINUS half-ellipse centred on the imaginary
    # axis carries Re z = -0.0 (beyn.c:88-115)
    z, _ = _lib_contour(qb, 0j, 1.0, 1.0, 8, ("halfellipse", ORIENT["re-"]))
    side = z[4:]
    assert np.all(side.real == 0) and np.all(np.signbit(side.real))


def test_kidney_rejects_rounding(qb):
    from qpms_gb300._lib import QpmsGpuError
    with pytest.raises(QpmsGpuError):
        qb.make_contour(0j, 1.0, 1.0, 10, ("kidney", 0.5, 0))
