"""The library against the reference's own code and Xu's published table.

* tests/golden/ref_vectors.npz holds A/B arrays and Ewald-summed A/B arrays
  computed by the reference's own translations.c, ewald.c and ewaldsf.c
  (compiled from its sources into oracle/_ref; made by
  tests/golden/make_ref_vectors.py).  The batched GPU kernel and the
  lattice-sum drop-in (qpms_trans_calculator_get_AB_arrays_e32) match them
  within the translation tolerance, 1e-11 relative (Frobenius per matrix).
* Xu's published coefficients (tests/golden/xu_translations.json, the
  reference's known-answer table) through the library's unnormalised
  convention at lMax 10 and the conversion to Xu's normalisation stated in
  tests/test_oracle_refpin.py: within 1e-7 (the table's own precision).
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
RTOL = 1e-11
NORM_DEFAULT, NORM_NONE = 65536 | 8, 2 * 65536


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return torch, qpms_gb300, np.load(os.path.join(HERE, "golden", "ref_vectors.npz"))


def _device_AB(torch, q, lMax, kd, J, norm=NORM_DEFAULT):
    dev = torch.device("cuda:0")
    c = q.trans_calculator(lMax, norm)
    ne = c.nelem()
    n = kd.shape[0]
    A = torch.empty((n, ne, ne), dtype=torch.complex128, device=dev)
    B = torch.empty_like(A)
    t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (kd[:, 0], kd[:, 1].real, kd[:, 2].real)]
    c.get_AB_arrays_device(t[0], t[1], t[2], J, A, B)
    torch.cuda.synchronize()
    return A.cpu().numpy(), B.cpu().numpy()


@pytest.mark.parametrize("lMax", [3, 6])
@pytest.mark.parametrize("J", [1, 3])
def test_translations_vs_reference_code(env, lMax, J):
    torch, q, g = env
    A, B = _device_AB(torch, q, lMax, g["AB_l%d_kd" % lMax], J)
    for G, R in ((A, g["AB_l%d_J%d_A" % (lMax, J)]), (B, g["AB_l%d_J%d_B" % (lMax, J)])):
        err = np.linalg.norm((G - R).reshape(len(R), -1), axis=1) / np.linalg.norm(R.reshape(len(R), -1), axis=1)
        assert err.max() <= RTOL, err.max()


class _Cplx(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class _Cart2(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double)]


class _Cart3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


def test_lattice_sums_vs_reference_code(env):
    torch, q, g = env
    L = C.CDLL(q.lib()._name)  # private handle: argtypes set here stay out of the package's
    f = L.qpms_trans_calculator_get_AB_arrays_e32
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_ssize_t, C.c_double,
                  _Cplx, _Cart2, _Cart2, _Cart2, _Cart3, C.c_double, C.c_double]
    calc = q.trans_calculator(3, NORM_DEFAULT)
    ne = 15
    for p, RA, RB in zip(g["e32_params"], g["e32_A"], g["e32_B"]):
        eta, kr, ki, b1x, b1y, b2x, b2y, bx, by, sx, sy, sz, maxR, maxK = p
        A = np.zeros((ne, ne), dtype=np.complex128)
        B = np.zeros_like(A)
        rc = f(calc.c, A.ctypes.data, None, B.ctypes.data, None, ne, 1, eta, _Cplx(kr, ki), _Cart2(b1x, b1y),
               _Cart2(b2x, b2y), _Cart2(bx, by), _Cart3(sx, sy, sz), maxR, maxK)
        assert rc == 0, q.last_error()
        for G, R in ((A, RA), (B, RB)):
            assert np.linalg.norm(G - R) <= RTOL * np.linalg.norm(R), (p, np.linalg.norm(G - R) / np.linalg.norm(R))


def test_xu_table_through_library(env):
    from math import lgamma, log
    torch, q, _ = env
    g = json.load(open(os.path.join(HERE, "golden", "xu_translations.json")))
    cases = [c for c in g["cases"] if c["n"] <= 10 and c["nu"] <= 10]
    assert len(cases) >= 4
    kd = np.array([[complex(c["kd"][0]), complex(c["kd"][1]), complex(c["kd"][2])] for c in cases])
    A, B = _device_AB(torch, q, 10, kd, g["J"], NORM_NONE)

    def conv(x, m, n, mu, nu):
        gg = lambda mm, nn: log(2 * nn + 1) + lgamma(nn - mm + 1) - lgamma(nn + mm + 1)
        return x * (1j) ** (nu - n) * np.exp(gg(mu, nu) - gg(m, n))

    for i, c in enumerate(cases):
        m, n, mu, nu = c["m"], c["n"], c["mu"], c["nu"]
        y, yu = n * (n + 1) + m - 1, nu * (nu + 1) + mu - 1
        a, b = conv(A[i][y, yu], m, n, mu, nu), conv(B[i][y, yu], m, n, mu, nu)
        xa, xb = complex(*c["A"]), complex(*c["B"])
        assert abs(a - xa) <= 1e-7 * abs(xa), (m, n, mu, nu)
        assert (abs(b) <= 1e-12 * abs(a)) if xb == 0 else (abs(b - xb) <= 1e-7 * abs(xb)), (m, n, mu, nu)
