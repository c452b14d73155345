"""The library's complex erfc (Weideman's Faddeeva approximation, evaluated by
the same host/device source) against scipy.special.wofz / erfc, over the
arguments the Ewald sums use (short range: R eta +- i k / 2 eta; long range:
real x and -i c)."""
import ctypes as C
import os

import numpy as np
import pytest
from scipy.special import wofz

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "qpms_gb300", "libqpms_gb300.so")),
                                reason="library not built")


def _cerfc(z):
    import qpms_gb300
    out = np.zeros(2)
    qpms_gb300.lib().qpms_gpu_debug_cerfc(z.real, z.imag, out.ctypes.data)
    return out[0] + 1j * out[1]


def test_cerfc_vs_scipy():
    zs = [x + 1j * y for x in np.linspace(0.5, 8, 16) for y in np.linspace(-3.5, 3.5, 15)]
    zs += [x + 0j for x in np.linspace(0, 7, 15)] + [-1j * c for c in np.linspace(0, 3.5, 15)]
    zs += [-0.7 + 0.2j, -2 - 1j]
    worst = 0
    for z in zs:
        ref = np.exp(-z * z) * wofz(1j * z) if z.real >= 0 else 2 - np.exp(-z * z) * wofz(-1j * z)
        got = _cerfc(z)
        worst = max(worst, abs(got - ref) / abs(ref))
    assert worst < 2e-13, worst
