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


class _Cplx(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class _EpsMu(C.Structure):
    _fields_ = [("eps", _Cplx), ("mu", _Cplx)]


class _ArcRet(C.Structure):
    _fields_ = [("r", C.c_double), ("beta", C.c_double)]


_ARCCB = C.CFUNCTYPE(None, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)


class _ArcCB(C.Structure):
    """qpms_arc_callback_params_t"""
    _fields_ = [("fn", C.c_void_p), ("user", C.c_void_p)]


class _Arc(C.Structure):
    _fields_ = [("function", C.c_void_p), ("params", C.c_void_p)]


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
    L.qpms_gpu_tmatrix_axialsym_batch.restype = ci
    L.qpms_gpu_tmatrix_axialsym_batch.argtypes = [vp, ci, _Arc, sz, vp, vp, vp, vp]
    L.qpms_tmatrix_axialsym_RQ_transposed_fill.restype = ci
    L.qpms_tmatrix_axialsym_RQ_transposed_fill.argtypes = [vp, _Cplx, _EpsMu, _EpsMu, _Arc, ci, ci, ci]
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


# ---------------- axially symmetric particles ----------------

class ArcFunction:
    """qpms_arc_function_t (cytmatrices.pyx:149-191): the surface of a particle
    with C_inf symmetry about z as r(theta) and the angle beta between the
    surface normal and the radial direction.  The library's sphere and
    cylinder (as the reference) and spheroid, or a Python callable
    theta -> (r, beta) (slow: called at every quadrature node)."""

    def __init__(self, function_name=None, params=(), callable_=None):
        self._L = lib()
        if callable_ is not None:
            def _f(theta, r, b, _user):
                rr, bb = callable_(theta)
                r[0], b[0] = float(rr), float(bb)
            self._cb = _ARCCB(_f)
            self._par = _ArcCB(C.cast(self._cb, C.c_void_p).value, None)
            self.arc = _Arc(C.cast(self._L.qpms_arc_callback, C.c_void_p).value, C.addressof(self._par))
        else:
            self._par = (C.c_double * len(params))(*[float(x) for x in params])
            fn = getattr(self._L, function_name)
            self.arc = _Arc(C.cast(fn, C.c_void_p).value, C.addressof(self._par))

    @staticmethod
    def sphere(r):
        return ArcFunction("qpms_arc_sphere", (r,))

    @staticmethod
    def cylinder(r, h):
        return ArcFunction("qpms_arc_cylinder", (r, h))

    @staticmethod
    def spheroid(a, c):
        """Equatorial semi-axis a, polar (z) semi-axis c."""
        return ArcFunction("qpms_arc_spheroid", (a, c))

    @staticmethod
    def custom(fn):
        return ArcFunction(callable_=fn)


def _epsmu(medium, omega):
    """Constant permittivity, (eps, mu), or a callable omega -> eps (the
    materials models)."""
    if isinstance(medium, tuple):
        e, mu = complex(medium[0]), complex(medium[1])
    elif callable(medium):
        e, mu = complex(medium(omega.real if isinstance(omega, complex) else omega)), 1.0
    else:
        e, mu = complex(medium), 1.0
    return _EpsMu(_Cplx(e.real, e.imag), _Cplx(mu.real, mu.imag))


class TMatrixGenerator:
    """T-matrices of an axially symmetric particle by the extended-boundary-
    condition method on the GPU (cytmatrices.pyx:193-384: the axialsym
    __AxialSymParams generators; sphere_asarc, cylinder).  outside / inside:
    constant permittivity, (eps, mu) or a materials model."""

    def __init__(self, outside, inside, shape, lMax_extend=None):
        self._L = lib()
        self.outside, self.inside, self.shape = outside, inside, shape
        self.lMax_extend = int(lMax_extend) if lMax_extend else 1

    @staticmethod
    def sphere_asarc(outside, inside, r, lMax_extend=None):
        return TMatrixGenerator(outside, inside, ArcFunction.sphere(r), lMax_extend)

    @staticmethod
    def cylinder(outside, inside, r, h, lMax_extend=None):
        return TMatrixGenerator(outside, inside, ArcFunction.cylinder(r, h), lMax_extend)

    @staticmethod
    def spheroid(outside, inside, a, c, lMax_extend=None):
        return TMatrixGenerator(outside, inside, ArcFunction.spheroid(a, c), lMax_extend)

    def batch(self, spec, omegas):
        """T [len(omegas), n, n] in the basis spec (a BaseSpec or lMax)."""
        if not isinstance(spec, BaseSpec):
            spec = BaseSpec(spec)
        om = np.ascontiguousarray(np.atleast_1d(omegas), dtype=np.complex128)
        nw = om.shape[0]
        outs = (_EpsMu * nw)(*[_epsmu(self.outside, complex(w)) for w in om])
        ins = (_EpsMu * nw)(*[_epsmu(self.inside, complex(w)) for w in om])
        T = np.empty((nw, spec.n, spec.n), dtype=np.complex128)
        rc = self._L.qpms_gpu_tmatrix_axialsym_batch(spec.ptr, self.lMax_extend, self.shape.arc, nw, om.ctypes.data,
                                                     C.addressof(outs), C.addressof(ins), T.ctypes.data)
        if rc:
            raise QpmsGpuError("qpms_gpu_tmatrix_axialsym_batch: " + last_error())
        return T

    def __call__(self, spec, omega):
        return self.batch(spec, [omega])[0]

    def _rq(self, omega, norm, J):
        L = max(self.lMax_extend, 1)
        n = 2 * L * (L + 2)
        out = np.empty((n, n), dtype=np.complex128)
        w = complex(omega)
        rc = self._L.qpms_tmatrix_axialsym_RQ_transposed_fill(out.ctypes.data, _Cplx(w.real, w.imag),
                                                              _epsmu(self.outside, w), _epsmu(self.inside, w),
                                                              self.shape.arc, L, int(norm), J)
        if rc:
            raise QpmsGpuError("qpms_tmatrix_axialsym_RQ_transposed_fill: " + last_error())
        return out

    def Q_transposed(self, omega, norm=QPMS_NORMALISATION_DEFAULT):
        """target[i1 + i2 n] as tmatrices.c:896-956 writes it (a C-ordered array
        whose [i2, i1] element is Q(i1, i2))."""
        return self._rq(omega, norm, 3)

    def R_transposed(self, omega, norm=QPMS_NORMALISATION_DEFAULT):
        return self._rq(omega, norm, 1)
