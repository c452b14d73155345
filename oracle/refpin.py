"""The reference's own translation and lattice-sum code, compiled from its
sources into oracle/_ref/libqpms_ref.so by oracle/build_oracle.py
(build_ref_lib), for pinning the oracle's restatement to it.  Test
infrastructure only: present where the reference tree is (not on machines
without it), never used by the library.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libqpms_ref.so")
_L = None


def available():
    return os.path.exists(LIB)


def lib():
    global _L
    if _L is None:
        L = C.CDLL(LIB)
        d, vp, sz, ci = C.c_double, C.c_void_p, C.c_size_t, C.c_int
        L.refpin_trans_calculator_init.restype = vp
        L.refpin_trans_calculator_init.argtypes = [ci, ci]
        L.refpin_trans_calculator_free.restype = None
        L.refpin_trans_calculator_free.argtypes = [vp]
        L.refpin_get_AB_arrays.restype = ci
        L.refpin_get_AB_arrays.argtypes = [vp, vp, vp, sz, d, d, d, d, ci, ci]
        L.refpin_get_AB_arrays_e32.restype = ci
        L.refpin_get_AB_arrays_e32.argtypes = [vp, vp, vp, vp, vp, sz] + [d] * 14
        _L = L
    return _L


class RefCalculator:
    """qpms_trans_calculator of the reference (translations.c:439-508)."""

    def __init__(self, lMax, normalisation):
        self.lMax = lMax
        self.nelem = lMax * (lMax + 2)
        self.ptr = lib().refpin_trans_calculator_init(lMax, normalisation)
        if not self.ptr:
            raise RuntimeError("reference calculator init failed")

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().refpin_trans_calculator_free(self.ptr)
            self.ptr = None

    def get_AB_arrays(self, kr, theta, phi, J, r_ge_d=False):
        """qpms_trans_calculator_get_AB_arrays (translations.c:610-698): A, B
        as nelem x nelem arrays (destination y, source yu)."""
        ne = self.nelem
        A = np.zeros((ne, ne), dtype=np.complex128)
        B = np.zeros_like(A)
        kr = complex(kr)
        rc = lib().refpin_get_AB_arrays(self.ptr, A.ctypes.data, B.ctypes.data, ne, kr.real, kr.imag, float(theta),
                                        float(phi), int(bool(r_ge_d)), int(J))
        if rc:
            raise RuntimeError("reference get_AB_arrays returned %d" % rc)
        return A, B

    def get_AB_arrays_e32(self, eta, k, b1, b2, beta, shift, maxR, maxK):
        """qpms_trans_calculator_get_AB_arrays_e32 (translations.c:926-1078),
        full Ewald sums: A, Aerr, B, Berr."""
        ne = self.nelem
        A = np.zeros((ne, ne), dtype=np.complex128)
        B = np.zeros_like(A)
        Ae = np.zeros((ne, ne))
        Be = np.zeros((ne, ne))
        k = complex(k)
        sh = list(shift) + [0.0] * (3 - len(shift))
        rc = lib().refpin_get_AB_arrays_e32(self.ptr, A.ctypes.data, Ae.ctypes.data, B.ctypes.data, Be.ctypes.data,
                                            ne, float(eta), k.real, k.imag, b1[0], b1[1], b2[0], b2[1], beta[0],
                                            beta[1], sh[0], sh[1], sh[2], float(maxR), float(maxK))
        if rc:
            raise RuntimeError("reference get_AB_arrays_e32 returned %d" % rc)
        return A, Ae, B, Be
