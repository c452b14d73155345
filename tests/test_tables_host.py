"""Host-side parity of the library's translation multiplier tables (no GPU).

The library computes the Gaunt coefficients by Gauss-Legendre projection and
the 3j symbols by the Racah sum in long double; the oracle by exact-3j Gaunt
coefficients.  Both restate translations.c:313-437; they must agree to 1e-13
relative (max-norm over the table) for every normalisation the reference's
translation code accepts, and obey the structure the kernel relies on (A real,
B imaginary).  Also checks that the C-ABI library loads and exports every
symbol declared in include/qpms_gb300.h.
"""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NORMS = [65536 | 8, 65536, 65536 * 3, 65536 * 3 | 8, 65536 * 2, 65536 * 2 | 8]


def _have_lib():
    return os.path.exists(os.path.join(ROOT, "qpms_gb300", "libqpms_gb300.so"))


pytestmark = pytest.mark.skipif(not _have_lib(), reason="libqpms_gb300.so not built")


def test_library_exports_header_symbols():
    import ctypes
    from qpms_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    hdr_dir = os.path.join(ROOT, "include")
    names = set()
    for fn in os.listdir(hdr_dir):
        if fn.endswith(".h"):
            txt = open(os.path.join(hdr_dir, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            for m in re.finditer(r"\b(qpms_\w+|beyn_\w+)\s*\((?!\*)", txt):
                names.add(m.group(1))
    assert names, "no declarations found"
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("lMax", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("norm", NORMS)
def test_multiplier_tables_vs_oracle(orc, lMax, norm):
    from qpms_gb300.translations import multipliers_export
    A, B = multipliers_export(lMax, norm)
    oA, oB = orc.TransCalculator(lMax, norm).multipliers()
    assert A.shape == oA.shape and B.shape == oB.shape
    assert np.max(np.abs(A - oA)) <= 1e-13 * np.max(np.abs(oA))
    assert np.max(np.abs(B - oB)) <= 1e-13 * np.max(np.abs(oB))
    assert np.all(A.imag == 0) and np.all(B.real == 0)


def test_lmax8_tables_vs_oracle(orc):
    from qpms_gb300.translations import multipliers_export
    A, B = multipliers_export(8)
    oA, oB = orc.TransCalculator(8).multipliers()
    assert np.max(np.abs(A - oA)) <= 1e-12 * np.max(np.abs(oA))
    assert np.max(np.abs(B - oB)) <= 1e-12 * np.max(np.abs(oB))
