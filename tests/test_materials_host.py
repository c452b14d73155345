"""Lorentz-Drude permittivities (materials.c:156-176) on the host, no GPU:
the library's model against the formula restated in numpy, and its metal
tables against the published fits they restate (Rakic et al., Appl. Opt. 37,
5271 (1998): gold, omega_p = 9.03 eV, first term f = 0.760, gamma = 0.053 eV;
silver omega_p = 9.01 eV), eV converted with GSL's CODATA-2006 constants as the
reference does."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "qpms_gb300", "libqpms_gb300.so")),
                                reason="libqpms_gb300.so not built")
EH = 1.602176487e-19 / 1.05457162825e-34


def _params(model):
    n = C.c_size_t.from_address(model.ptr + 24).value
    omega_p = C.c_double.from_address(model.ptr + 16).value
    tr = np.frombuffer((C.c_double * (3 * n)).from_address(model.ptr + 32), dtype=np.float64).reshape(n, 3)
    return omega_p, tr.copy()


def lorentzdrude_np(omega, omega_p, tr):
    return sum(f * omega_p ** 2 / (w ** 2 - omega ** 2 - 1j * omega * g) for f, w, g in tr)


def test_tables_and_formula():
    from qpms_gb300.materials import LorentzDrude, lorentz_drude
    au_wp, au = _params(lorentz_drude["Au"])
    ag_wp, _ = _params(lorentz_drude["Ag"])
    assert abs(au_wp - 9.03 * EH) <= 1e-15 * au_wp and abs(ag_wp - 9.01 * EH) <= 1e-15 * ag_wp
    assert au.shape == (6, 3) and au[0, 0] == 0.76 and au[0, 1] == 0 and abs(au[0, 2] - 0.053 * EH) < 1e-3
    for name in ("Au", "Ag", "Cu", "Al", "Cr"):
        m = lorentz_drude[name]
        wp, tr = _params(m)
        for E in (1.2, 2.1, 3.0 + 0.05j):
            w = E * EH
            ref = lorentzdrude_np(w, wp, tr)
            assert abs(m(w) - ref) <= 1e-14 * abs(ref)
    own = LorentzDrude(1, 9.0 * EH, [0.5, 0.3], [0.0, 2.0 * EH], [0.05 * EH, 0.4 * EH])
    w = 2.2 * EH
    assert abs(own(w) - lorentzdrude_np(w, 9.0 * EH, [(0.5, 0, 0.05 * EH), (0.3, 2 * EH, 0.4 * EH)])) < 1e-12
    # gold at 2 eV: a plasmonic metal (Re eps < 0, Im eps > 0)
    e = lorentz_drude["Au"](2.0 * EH)
    assert e.real < -8 and 0 < e.imag < 5
