"""Tabulated T-matrices on the C-ABI: the reference's TMatrixInterpolator
(qpms/cytmatrices.pyx:12-66 over tmatrices.c:287-490) — a SCUFF-EM
T-matrix file, or arrays, interpolated in frequency (natural cubic spline by
default, as gsl_interp_cspline).  Pass one as an element of ``eps_inside`` to
``ScatteringSystem`` to make a particle kind with that T-matrix.
"""
import ctypes as C

import numpy as np

from ._lib import QpmsGpuError, last_error, lib
from .materials import interp_type


class _TM(C.Structure):
    _fields_ = [("spec", C.c_void_p), ("m", C.c_void_p), ("owns_m", C.c_bool)]


def declare(L):
    vp, sz, cd, ci = C.c_void_p, C.c_size_t, C.c_double, C.c_int
    L.qpms_vswf_set_spec_from_lMax.restype = vp
    L.qpms_vswf_set_spec_from_lMax.argtypes = [ci, ci]
    L.qpms_vswf_set_spec_free.restype = None
    L.qpms_vswf_set_spec_free.argtypes = [vp]
    L.qpms_tmatrix_interpolator_create.restype = vp
    L.qpms_tmatrix_interpolator_create.argtypes = [sz, vp, vp, vp]
    L.qpms_tmatrix_interpolator_free.restype = None
    L.qpms_tmatrix_interpolator_free.argtypes = [vp]
    L.qpms_tmatrix_interpolator_eval.restype = C.POINTER(_TM)
    L.qpms_tmatrix_interpolator_eval.argtypes = [vp, cd]
    L.qpms_tmatrix_interpolator_eval_fill.restype = ci
    L.qpms_tmatrix_interpolator_eval_fill.argtypes = [vp, vp, cd]
    L.qpms_tmatrix_free.restype = None
    L.qpms_tmatrix_free.argtypes = [vp]
    L.qpms_tmatrix_init.restype = C.POINTER(_TM)
    L.qpms_tmatrix_init.argtypes = [vp]
    L.qpms_tmatrix_interpolator_bspec.restype = vp
    L.qpms_tmatrix_interpolator_bspec.argtypes = [vp]
    L.qpms_gpu_tmatrix_interpolator_eval_batch.restype = ci
    L.qpms_gpu_tmatrix_interpolator_eval_batch.argtypes = [vp, sz, vp, vp, vp]
    L.qpms_load_scuff_tmatrix.restype = ci
    L.qpms_load_scuff_tmatrix.argtypes = [C.c_char_p, vp, C.POINTER(sz), C.POINTER(vp), C.POINTER(vp),
                                          C.POINTER(vp), C.POINTER(vp)]


QPMS_NORMALISATION_DEFAULT = 65536 | 8
QPMS_NAN_ENCOUNTERED = 1024


class BaseSpec:
    """The default VSWF set of lMax (vswf.c:76-92): electric block, then magnetic."""

    def __init__(self, lMax):
        self._L = lib()
        self.lMax = int(lMax)
        self.ptr = self._L.qpms_vswf_set_spec_from_lMax(self.lMax, QPMS_NORMALISATION_DEFAULT)
        if not self.ptr:
            raise QpmsGpuError("qpms_vswf_set_spec_from_lMax: " + last_error())
        self.n = 2 * self.lMax * (self.lMax + 2)

    def __len__(self):
        return self.n

    def __del__(self):
        p = getattr(self, "ptr", None)
        if p:
            self._L.qpms_vswf_set_spec_free(p)
            self.ptr = None


def load_scuff_tmatrix(filename, lMax):
    """Frequencies (rad/s), T-matrices [nfreq, n, n] of a SCUFF-EM file in the
    default lMax basis (tmatrices.c:367-490), and whether an element of the
    basis was missing (NaN in the data)."""
    L = lib()
    spec = BaseSpec(lMax)
    nf = C.c_size_t(0)
    fr, fsu, tma, data = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
    rc = L.qpms_load_scuff_tmatrix(str(filename).encode(), spec.ptr, C.byref(nf), C.byref(fr), C.byref(fsu),
                                   C.byref(tma), C.byref(data))
    if rc and not (rc & QPMS_NAN_ENCOUNTERED):
        raise IOError("Could not read T-matrix from %s: %s" % (filename, last_error()))
    n = spec.n
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    try:
        freqs = np.ctypeslib.as_array(C.cast(fr, C.POINTER(C.c_double)), (nf.value,)).copy()
        T = np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_double)), (nf.value * n * n * 2,)).copy()
    finally:
        for p in (fr, fsu, tma, data):
            if p.value:
                libc.free(p)
    return freqs, T.view(np.complex128).reshape(nf.value, n, n), bool(rc & QPMS_NAN_ENCOUNTERED)


class TMatrixInterpolator:
    """T(omega) interpolated from tabulated T-matrices in the default lMax basis.

    ``TMatrixInterpolator(filename, lMax)`` reads a SCUFF-EM T-matrix file;
    ``TMatrixInterpolator.from_arrays(freqs, tmatrices, lMax)`` takes arrays."""

    def __init__(self, filename=None, lMax=None, kind="cspline", _arrays=None):
        if _arrays is None:
            freqs, T, has_nan = load_scuff_tmatrix(filename, lMax)
            if has_nan:
                raise IOError("T-matrix file %s lacks elements of the lMax = %d basis" % (filename, lMax))
        else:
            freqs, T = _arrays
        self._L = lib()
        self.spec = BaseSpec(lMax)
        n = self.spec.n
        self.freqs = np.ascontiguousarray(freqs, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.complex128)
        if T.shape != (self.freqs.size, n, n):
            raise ValueError("T-matrices must have shape (%d, %d, %d)" % (self.freqs.size, n, n))
        self._T = T
        tms = (_TM * self.freqs.size)()
        for i in range(self.freqs.size):
            tms[i].spec = self.spec.ptr
            tms[i].m = T[i].ctypes.data
            tms[i].owns_m = False
        self.ptr = self._L.qpms_tmatrix_interpolator_create(self.freqs.size, self.freqs.ctypes.data,
                                                            C.addressof(tms), interp_type(kind))
        if not self.ptr:
            raise QpmsGpuError("T-matrix interpolator: " + last_error())

    @classmethod
    def from_arrays(cls, freqs, tmatrices, lMax, kind="cspline"):
        return cls(lMax=lMax, kind=kind, _arrays=(freqs, tmatrices))

    def __del__(self):
        p = getattr(self, "ptr", None)
        if p:
            self._L.qpms_tmatrix_interpolator_free(p)
            self.ptr = None

    def __call__(self, freq):
        if freq < self.freqs[0] or freq > self.freqs[-1]:
            raise ValueError("input frequency %g is outside the interpolator domain (%g, %g)"
                             % (freq, self.freqs[0], self.freqs[-1]))
        t = self._L.qpms_tmatrix_interpolator_eval(self.ptr, float(freq))
        n = self.spec.n
        try:
            m = np.ctypeslib.as_array(C.cast(t.contents.m, C.POINTER(C.c_double)), (n * n * 2,)).copy()
        finally:
            self._L.qpms_tmatrix_free(C.cast(t, C.c_void_p))
        return m.view(np.complex128).reshape(n, n)

    def eval_batch_device(self, freqs, out=None, stream=None):
        """T at every frequency of the CUDA tensor ``freqs`` (float64), on the
        GPU: returns a complex128 tensor [nfreq, n, n]."""
        import torch
        n = self.spec.n
        if out is None:
            out = torch.empty((freqs.numel(), n, n), dtype=torch.complex128, device=freqs.device)
        if stream is None:
            stream = torch.cuda.current_stream(freqs.device)
        rc = self._L.qpms_gpu_tmatrix_interpolator_eval_batch(self.ptr, freqs.numel(), freqs.data_ptr(),
                                                              out.data_ptr(), stream.cuda_stream)
        if rc:
            raise QpmsGpuError("qpms_gpu_tmatrix_interpolator_eval_batch: " + last_error())
        return out

    @property
    def freq_interval(self):
        return [self.freqs[0], self.freqs[-1]]

    @property
    def omega_table(self):
        return self.freqs.copy()
