"""Optical properties of materials: the reference's Lorentz-Drude model
(qpms/cymaterials.pyx:80-160 over materials.c:156-176) on the C-ABI.

``LorentzDrude(eps_inf, omega_p, f, omega, gamma)`` builds a parameter block;
``lorentz_drude["Au"]`` etc. are the library's fits of Rakic et al. (1998).
Pass such objects as ``eps_inside`` to ``ScatteringSystem``.
"""
import ctypes as C

import numpy as np

from ._lib import lib


class _Triple(C.Structure):
    _fields_ = [("f", C.c_double), ("omega", C.c_double), ("gamma", C.c_double)]


def declare(L):
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
