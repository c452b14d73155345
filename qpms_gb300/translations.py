"""Python mirror of the reference's ``trans_calculator`` (cytranslations.pyx:318-557).

``trans_calculator(lMax, normalization).get_AB_arrays(r, theta, phi, r_ge_d, J)``
returns ``(a, b)`` with two trailing nelem x nelem axes, like the Cython
wrapper, computed by the GPU kernel through the C-ABI.  ``r`` may be complex
(kr with absorbing media), which the reference's numpy loop could not take
(translations_python.c:110 casts r to double).
"""
import numpy as np

from . import _lib

QPMS_NORMALISATION_DEFAULT = 65536 | 8
QPMS_BESSEL_REGULAR, QPMS_BESSEL_SINGULAR, QPMS_HANKEL_PLUS, QPMS_HANKEL_MINUS = 1, 2, 3, 4


class trans_calculator:
    def __init__(self, lMax, normalization=QPMS_NORMALISATION_DEFAULT):
        if lMax <= 0:
            raise ValueError("lMax has to be greater than 0.")
        self._L = _lib.lib()
        self.c = self._L.qpms_trans_calculator_init(int(lMax), int(normalization))
        if not self.c:
            raise _lib.QpmsGpuError("qpms_trans_calculator_init: " + _lib.last_error())
        self._lMax = int(lMax)
        self._nelem = self._lMax * (self._lMax + 2)

    def __del__(self):
        c = getattr(self, "c", None)
        if c:
            self._L.qpms_trans_calculator_free(c)
            self.c = None

    def lMax(self):
        return self._lMax

    def nelem(self):
        return self._nelem

    def n_multipliers(self):
        f = self._L.qpms_gpu_trans_calculator_n_multipliers
        return f(self.c, 0), f(self.c, 1)

    def get_AB_arrays(self, r, theta, phi, r_ge_d, J):
        """Broadcast r (kr, real or complex), theta, phi, r_ge_d; returns (a, b)
        of shape broadcast_shape + (nelem, nelem), complex128 (host arrays)."""
        r, theta, phi, r_ge_d = np.broadcast_arrays(np.asarray(r), np.asarray(theta), np.asarray(phi),
                                                    np.asarray(r_ge_d))
        shape = r.shape
        kr = np.ascontiguousarray(r.reshape(-1), dtype=np.complex128)
        th = np.ascontiguousarray(theta.reshape(-1), dtype=np.float64)
        ph = np.ascontiguousarray(phi.reshape(-1), dtype=np.float64)
        rg = np.ascontiguousarray(r_ge_d.reshape(-1), dtype=np.uint8)
        n = kr.shape[0]
        ne = self._nelem
        a = np.empty((n, ne, ne), dtype=np.complex128)
        b = np.empty((n, ne, ne), dtype=np.complex128)
        rc = self._L.qpms_gpu_trans_AB_arrays_batch_host(self.c, n, kr.ctypes.data, th.ctypes.data,
                                                         ph.ctypes.data, rg.ctypes.data, int(J),
                                                         a.ctypes.data, b.ctypes.data)
        _lib.check(rc, "qpms_gpu_trans_AB_arrays_batch_host")
        return a.reshape(shape + (ne, ne)), b.reshape(shape + (ne, ne))

    def get_AB_arrays_device(self, kr, theta, phi, J, A, B, r_ge_d=None, stream=0):
        """Device-pointer batch: torch CUDA tensors kr (complex128, n), theta,
        phi (float64, n); writes A, B (complex128, n x nelem x nelem).
        Asynchronous on ``stream`` (a CUDA stream handle, 0 = default)."""
        n = kr.shape[0]
        rg = 0 if r_ge_d is None else r_ge_d.data_ptr()
        rc = self._L.qpms_gpu_trans_AB_arrays_batch(self.c, n, kr.data_ptr(), theta.data_ptr(),
                                                    phi.data_ptr(), rg, int(J), A.data_ptr(),
                                                    B.data_ptr(), stream)
        _lib.check(rc, "qpms_gpu_trans_AB_arrays_batch")

    def get_AB_arrays_single(self, kr, theta, phi, r_ge_d, J):
        """qpms_trans_calculator_get_AB_arrays_ext for one translation."""
        ne = self._nelem
        A = np.empty((ne, ne), dtype=np.complex128)
        B = np.empty((ne, ne), dtype=np.complex128)
        kr = complex(kr)
        rc = self._L.qpms_trans_calculator_get_AB_arrays_ext(self.c, A.ctypes.data, B.ctypes.data, ne, 1,
                                                             kr.real, kr.imag, float(theta), float(phi),
                                                             int(bool(r_ge_d)), int(J))
        _lib.check(rc, "qpms_trans_calculator_get_AB_arrays_ext")
        return A, B


def multipliers_export(lMax, normalization=QPMS_NORMALISATION_DEFAULT):
    """Host-side A/B multiplier tables of the library (no GPU needed), in the
    reference's ragged A_multipliers[0] / B_multipliers[0] order."""
    import ctypes as C
    L = _lib.lib()
    nA, nB = C.c_size_t(0), C.c_size_t(0)
    _lib.check(L.qpms_gpu_trans_multipliers_export(int(lMax), int(normalization), None, C.byref(nA), None,
                                                   C.byref(nB)), "qpms_gpu_trans_multipliers_export")
    A = np.zeros(nA.value, dtype=np.complex128)
    B = np.zeros(nB.value, dtype=np.complex128)
    _lib.check(L.qpms_gpu_trans_multipliers_export(int(lMax), int(normalization), A.ctypes.data, C.byref(nA),
                                                   B.ctypes.data, C.byref(nB)), "qpms_gpu_trans_multipliers_export")
    return A, B
