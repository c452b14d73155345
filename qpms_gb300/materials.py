"""Optical properties of materials on the C-ABI: the reference's Lorentz-Drude
model (qpms/cymaterials.pyx:80-160 over materials.c:156-176) and its tabulated
permittivity interpolator (cymaterials.pyx:251-275 over materials.c:11-153).

``LorentzDrude(eps_inf, omega_p, f, omega, gamma)`` builds a parameter block;
``lorentz_drude["Au"]`` etc. are the library's fits of Rakic et al. (1998);
``MaterialInterpolator(path)`` reads a refractiveindex.info table.
Pass such objects as ``eps_inside`` to ``ScatteringSystem``.
"""
import ctypes as C

import numpy as np

from ._lib import QpmsGpuError, last_error, lib


class _Triple(C.Structure):
    _fields_ = [("f", C.c_double), ("omega", C.c_double), ("gamma", C.c_double)]


def declare(L):
    vp, sz, cd = C.c_void_p, C.c_size_t, C.c_double
    L.qpms_permittivity_interpolator_create.restype = vp
    L.qpms_permittivity_interpolator_create.argtypes = [sz, vp, vp, vp, vp]
    L.qpms_permittivity_interpolator_from_yml.restype = vp
    L.qpms_permittivity_interpolator_from_yml.argtypes = [C.c_char_p, vp]
    L.qpms_permittivity_interpolator_free.restype = None
    L.qpms_permittivity_interpolator_free.argtypes = [vp]
    L.qpms_permittivity_interpolator_eps_at_omega.restype = _Cplx
    L.qpms_permittivity_interpolator_eps_at_omega.argtypes = [vp, cd]
    L.qpms_permittivity_interpolator_omega_min.restype = cd
    L.qpms_permittivity_interpolator_omega_min.argtypes = [vp]
    L.qpms_permittivity_interpolator_omega_max.restype = cd
    L.qpms_permittivity_interpolator_omega_max.argtypes = [vp]
    L.qpms_lorentzdrude_eps.restype = _Cplx
    L.qpms_lorentzdrude_eps.argtypes = [_Cplx, C.c_void_p]
    L.qpms_gpu_scatsys_create_spheres_ld.restype = C.c_void_p
    L.qpms_gpu_scatsys_create_spheres_ld.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p,
                                                     C.c_void_p]


class _Cplx(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class LorentzDrude:
    """eps(omega) = sum_j f_j omega_p^2 / (omega_j^2 - omega^2 - i omega gamma_j)
    (eps_inf is carried but, as in the reference, not added)."""

    def __init__(self, eps_inf, omega_p, f_arr, omega_arr, gamma_arr, _ptr=None):
        if _ptr is not None:          # a parameter block owned by the library
            self.ptr = _ptr
            self._buf = None
            return
        n = len(f_arr)
        if n != len(omega_arr) or n != len(gamma_arr):
            raise ValueError("f_arr, omega_arr and gamma_arr must have equal lengths")

        class Block(C.Structure):
            _fields_ = [("eps_inf", _Cplx), ("omega_p", C.c_double), ("n", C.c_size_t), ("data", _Triple * n)]
        e = complex(eps_inf)
        self._buf = Block(_Cplx(e.real, e.imag), float(omega_p), n,
                          (_Triple * n)(*[_Triple(float(a), float(b), float(c))
                                          for a, b, c in zip(f_arr, omega_arr, gamma_arr)]))
        self.ptr = C.addressof(self._buf)

    def __call__(self, omega):
        w = complex(omega)
        r = lib().qpms_lorentzdrude_eps(_Cplx(w.real, w.imag), self.ptr)
        return complex(r.re, r.im)


def _library_models():
    L = lib()
    out = {}
    for name in ("Au", "Ag", "Cu", "Al", "Cr"):
        p = C.c_void_p.in_dll(L, "QPMS_LDPARAMS_" + name.upper()).value
        out[name] = LorentzDrude(None, None, [], [], [], _ptr=p)
    return out


class _Models(dict):
    def __missing__(self, key):
        self.update(_library_models())
        return dict.__getitem__(self, key)


lorentz_drude = _Models()


def interp_type(kind):
    """The library's stand-in for gsl_interp_linear / gsl_interp_cspline."""
    if kind not in ("linear", "cspline"):
        raise ValueError("interpolation kind must be 'linear' or 'cspline'")
    return C.c_void_p.in_dll(lib(), "qpms_interp_" + kind).value


class MaterialInterpolator:
    """Tabulated refractive index n + i k over vacuum wavelength, interpolated
    (natural cubic spline by default, as the reference's gsl_interp_cspline);
    ``mi(omega)`` is the permittivity (n + i k)^2 at angular frequency omega."""

    def __init__(self, filename=None, kind="cspline", _ptr=None):
        L = lib()
        self._L = L
        if _ptr is None:
            _ptr = L.qpms_permittivity_interpolator_from_yml(str(filename).encode(), interp_type(kind))
            if not _ptr:
                raise IOError("Could not load permittivity data from %s: %s" % (filename, last_error()))
        self.ptr = _ptr
        self.omegamin = L.qpms_permittivity_interpolator_omega_min(self.ptr)
        self.omegamax = L.qpms_permittivity_interpolator_omega_max(self.ptr)

    @classmethod
    def from_arrays(cls, wavelength_m, n, k, kind="cspline"):
        w = np.ascontiguousarray(wavelength_m, dtype=np.float64)
        nn = np.ascontiguousarray(n, dtype=np.float64)
        kk = np.ascontiguousarray(k, dtype=np.float64)
        p = lib().qpms_permittivity_interpolator_create(w.size, w.ctypes.data, nn.ctypes.data, kk.ctypes.data,
                                                        interp_type(kind))
        if not p:
            raise QpmsGpuError("permittivity interpolator: " + last_error())
        return cls(_ptr=p)

    def __del__(self):
        p = getattr(self, "ptr", None)
        if p:
            self._L.qpms_permittivity_interpolator_free(p)
            self.ptr = None

    def __call__(self, freq):
        if freq < self.omegamin or freq > self.omegamax:
            raise ValueError("Input frequency %g is outside the interpolator domain (%g, %g)."
                             % (freq, self.omegamin, self.omegamax))
        r = self._L.qpms_permittivity_interpolator_eps_at_omega(self.ptr, float(freq))
        return complex(r.re, r.im)

    @property
    def freq_interval(self):
        return [self.omegamin, self.omegamax]
