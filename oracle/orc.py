"""ctypes binding of the oracle library (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle as _b

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _b.build_oracle()
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


def _declare(L):
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    L.orc_wigner3j.restype = C.c_double
    L.orc_wigner3j.argtypes = [C.c_int] * 6
    L.orc_gaunt.restype = C.c_int
    L.orc_gaunt.argtypes = [C.c_int] * 4 + [dp]
    L.orc_gaunt_q_max.restype = C.c_int
    L.orc_gaunt_q_max.argtypes = [C.c_int] * 4
    L.orc_legendre_array.restype = None
    L.orc_legendre_array.argtypes = [C.c_int, C.c_double, C.c_double, dp]
    L.orc_sph_bessel_fill_ri.restype = C.c_int
    L.orc_sph_bessel_fill_ri.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, vp]
    L.orc_trans_calculator_init.restype = vp
    L.orc_trans_calculator_init.argtypes = [C.c_int, C.c_int]
    L.orc_trans_calculator_free.restype = None
    L.orc_trans_calculator_free.argtypes = [vp]
    L.orc_trans_calculator_nA.restype = C.c_size_t
    L.orc_trans_calculator_nA.argtypes = [vp]
    L.orc_trans_calculator_nB.restype = C.c_size_t
    L.orc_trans_calculator_nB.argtypes = [vp]
    L.orc_trans_calculator_get_AB_arrays_ri.restype = C.c_int
    L.orc_trans_calculator_get_AB_arrays_ri.argtypes = [
        vp, vp, vp, C.c_size_t, C.c_size_t, C.c_double, C.c_double, C.c_double, C.c_double,
        C.c_int, C.c_int]
    L.orc_trans_AB_batch.restype = C.c_int
    L.orc_trans_AB_batch.argtypes = [vp, C.c_size_t, vp, vp, vp, C.c_int, vp, vp]
    for f in (L.orc_trans_single_A_out, L.orc_trans_single_B_out):
        f.restype = None
        f.argtypes = [C.c_int] * 5 + [C.c_double] * 4 + [C.c_int, C.c_int, vp]
    L.orc_num_threads.restype = C.c_int
    L.orc_num_threads.argtypes = []


def num_threads():
    return lib().orc_num_threads()


NORMALISATION_DEFAULT = 65536 | 8  # QPMS_NORMALISATION_NORM_POWER | CSPHASE


def wigner3j(*a):
    return lib().orc_wigner3j(*[int(x) for x in a])


def gaunt(m, n, mu, nu):
    L = lib()
    qmax = L.orc_gaunt_q_max(m, n, mu, nu)
    out = np.zeros(qmax + 1)
    L.orc_gaunt(m, n, mu, nu, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def legendre_array(L_, x, csphase=-1.0):
    out = np.zeros((L_ + 1) * (L_ + 2) // 2)
    lib().orc_legendre_array(L_, x, csphase, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def sph_bessel(J, lmax, x):
    x = complex(x)
    out = np.zeros(lmax + 1, dtype=np.complex128)
    r = lib().orc_sph_bessel_fill_ri(J, lmax, x.real, x.imag, out.ctypes.data)
    if r:
        raise ValueError("orc_sph_bessel_fill failed")
    return out


class TransCalculator:
    """Oracle counterpart of the reference's trans_calculator (cytranslations.pyx:318)."""

    def __init__(self, lMax, normalisation=NORMALISATION_DEFAULT):
        self._L = lib()
        self.lMax = lMax
        self.nelem = lMax * (lMax + 2)
        self.normalisation = normalisation
        self.ptr = self._L.orc_trans_calculator_init(lMax, normalisation)
        if not self.ptr:
            raise ValueError("lMax has to be greater than 0.")

    def __del__(self):
        if getattr(self, "ptr", None):
            self._L.orc_trans_calculator_free(self.ptr)
            self.ptr = None

    @property
    def n_multipliers(self):
        return (self._L.orc_trans_calculator_nA(self.ptr), self._L.orc_trans_calculator_nB(self.ptr))

    def multipliers(self):
        """Ragged A/B multiplier tables (A_multipliers[0][...], B_multipliers[0][...])."""
        class _S(C.Structure):
            _fields_ = [("norm", C.c_int), ("lMax", C.c_int), ("nelem", C.c_int),
                        ("A", C.POINTER(C.POINTER(C.c_double))), ("B", C.POINTER(C.POINTER(C.c_double)))]
        s = _S.from_address(self.ptr)
        nA, nB = self.n_multipliers
        A = np.ctypeslib.as_array(s.A[0], shape=(2 * nA,)).view(np.complex128).copy()
        B = np.ctypeslib.as_array(s.B[0], shape=(2 * nB,)).view(np.complex128).copy()
        return A, B

    def get_AB_arrays_single(self, kr, theta, phi, r_ge_d, J):
        ne = self.nelem
        A = np.empty((ne, ne), dtype=np.complex128)
        B = np.empty((ne, ne), dtype=np.complex128)
        kr = complex(kr)
        self._L.orc_trans_calculator_get_AB_arrays_ri(
            self.ptr, A.ctypes.data, B.ctypes.data, ne, 1, kr.real, kr.imag, float(theta),
            float(phi), int(bool(r_ge_d)), int(J))
        return A, B

    def get_AB_batch(self, kr, theta, phi, J):
        kr = np.ascontiguousarray(kr, dtype=np.complex128)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        n = kr.shape[0]
        ne = self.nelem
        A = np.empty((n, ne, ne), dtype=np.complex128)
        B = np.empty((n, ne, ne), dtype=np.complex128)
        self._L.orc_trans_AB_batch(self.ptr, n, kr.ctypes.data, theta.ctypes.data, phi.ctypes.data,
                                   int(J), A.ctypes.data, B.ctypes.data)
        return A, B


def trans_single(which, norm, m, n, mu, nu, kr, theta, phi, r_ge_d, J):
    """Closed-form single coefficient (translations.c:135-286)."""
    L = lib()
    f = L.orc_trans_single_A_out if which == "A" else L.orc_trans_single_B_out
    out = np.zeros(1, dtype=np.complex128)
    kr = complex(kr)
    f(norm, m, n, mu, nu, kr.real, kr.imag, float(theta), float(phi), int(r_ge_d), int(J),
      out.ctypes.data)
    return out[0]
