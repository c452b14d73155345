"""ctypes binding of the oracle library (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only to check results.
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
    _declare_scatsys(L)
    _declare_ewald(L)


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


def _declare_scatsys(L):
    vp, ci, cd, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    L.orc_tmatrix_sphere_diag_ri.restype = None
    L.orc_tmatrix_sphere_diag_ri.argtypes = [ci, cd, cd, cd, cd, cd, cd, cd, vp]
    L.orc_finite_modeproblem_ri.restype = ci
    L.orc_finite_modeproblem_ri.argtypes = [vp, ci, vp, vp, cd, cd, vp]
    L.orc_finite_translation_matrix_ri.restype = ci
    L.orc_finite_translation_matrix_ri.argtypes = [vp, ci, vp, cd, cd, ci, vp]
    L.orc_finite_sphere_scatter_ri.restype = ci
    L.orc_finite_sphere_scatter_ri.argtypes = [vp, ci, vp, cd, cd, cd, cd, cd, cd, vp, vp, vp, vp, vp, vp]
    L.orc_planewave_full.restype = None
    L.orc_planewave_full.argtypes = [ci, ci, vp, vp, vp, vp]
    L.orc_lu_factor.restype = ci
    L.orc_lu_factor.argtypes = [sz, vp, vp]
    L.orc_lu_solve.restype = None
    L.orc_lu_solve.argtypes = [sz, vp, vp, vp, sz]
    L.orc_spline_eval.restype = None
    L.orc_spline_eval.argtypes = [ci, ci, vp, vp, ci, vp, vp]
    L.orc_scattered_E_ri.restype = None
    L.orc_scattered_E_ri.argtypes = [ci, ci, vp, ci, cd, cd, vp, ci, vp, vp]


C0 = 299792458.0


def tmatrix_sphere_diag(lMax, radius, omega, eps_i, eps_e):
    L = lib()
    out = np.zeros(2 * lMax * (lMax + 2), dtype=np.complex128)
    om, ei, ee = complex(omega), complex(eps_i), complex(eps_e)
    L.orc_tmatrix_sphere_diag_ri(lMax, radius, om.real, om.imag, ei.real, ei.imag, ee.real, ee.imag,
                                 out.ctypes.data)
    return out


def finite_modeproblem(calc, pos, T, k):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.complex128)
    np_ = pos.shape[0]
    N = np_ * 2 * calc.nelem
    M = np.empty((N, N), dtype=np.complex128)
    k = complex(k)
    lib().orc_finite_modeproblem_ri(calc.ptr, np_, pos.ctypes.data, T.ctypes.data, k.real, k.imag,
                                    M.ctypes.data)
    return M


def finite_translation_matrix(calc, pos, k, J):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    np_ = pos.shape[0]
    N = np_ * 2 * calc.nelem
    S = np.empty((N, N), dtype=np.complex128)
    k = complex(k)
    lib().orc_finite_translation_matrix_ri(calc.ptr, np_, pos.ctypes.data, k.real, k.imag, J, S.ctypes.data)
    return S


def planewave_full(lMax, pos, k_cart, E_cart):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    kc = np.ascontiguousarray(k_cart, dtype=np.float64)
    Ec = np.ascontiguousarray(E_cart, dtype=np.complex128)
    out = np.empty(pos.shape[0] * 2 * lMax * (lMax + 2), dtype=np.complex128)
    lib().orc_planewave_full(lMax, pos.shape[0], pos.ctypes.data, kc.ctypes.data, Ec.ctypes.data,
                             out.ctypes.data)
    return out


def spline_eval(kind, x, y, xq):
    """kind 0 linear, 1 natural cubic spline (the reference's gsl_interp_cspline)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    q = np.ascontiguousarray(np.atleast_1d(xq), dtype=np.float64)
    out = np.empty(q.size)
    lib().orc_spline_eval(int(kind), x.size, x.ctypes.data, y.ctypes.data, q.size, q.ctypes.data, out.ctypes.data)
    return out


def scattered_E(lMax, pos, J, k, cvf, where):
    """Field of the full coefficient vector cvf at points where [..., 3]
    (qpms_scatsys_scattered_E, scatsystem.c:2013-2039); returns [..., 3] complex."""
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(where, dtype=np.float64)
    shape = w.shape
    w = w.reshape(-1, 3)
    cv = np.ascontiguousarray(cvf, dtype=np.complex128)
    assert cv.size == pos.shape[0] * 2 * lMax * (lMax + 2)
    E = np.empty((w.shape[0], 3), dtype=np.complex128)
    k = complex(k)
    lib().orc_scattered_E_ri(lMax, pos.shape[0], pos.ctypes.data, int(J), k.real, k.imag, cv.ctypes.data,
                             w.shape[0], w.ctypes.data, E.ctypes.data)
    return E.reshape(shape)


def finite_sphere_scatter(calc, pos, radius, eps_i, eps_e, omega, k_dir=(0, 0, 1), E_cart=(1, 0, 0),
                          want_M=False):
    """One frequency: returns (f, a_inc, sigma_ext[, M])."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    np_ = pos.shape[0]
    N = np_ * 2 * calc.nelem
    f = np.empty(N, dtype=np.complex128)
    a = np.empty(N, dtype=np.complex128)
    sig = np.zeros(1)
    M = np.empty((N, N), dtype=np.complex128) if want_M else None
    kd = np.ascontiguousarray(k_dir, dtype=np.float64)
    Ec = np.ascontiguousarray(E_cart, dtype=np.complex128)
    ei, ee = complex(eps_i), complex(eps_e)
    info = lib().orc_finite_sphere_scatter_ri(calc.ptr, np_, pos.ctypes.data, radius, ei.real, ei.imag,
                                              ee.real, ee.imag, float(omega), kd.ctypes.data, Ec.ctypes.data,
                                              f.ctypes.data, a.ctypes.data, sig.ctypes.data,
                                              M.ctypes.data if want_M else None)
    if info:
        raise ArithmeticError("singular mode-problem matrix (info=%d)" % info)
    return (f, a, float(sig[0]), M) if want_M else (f, a, float(sig[0]))


def lu_factor(M):
    a = np.array(M, dtype=np.complex128, order="C", copy=True)
    ipiv = np.zeros(a.shape[0], dtype=np.int32)
    info = lib().orc_lu_factor(a.shape[0], a.ctypes.data, ipiv.ctypes.data)
    return a, ipiv, info


def lu_solve(a, ipiv, b):
    b = np.array(b, dtype=np.complex128, order="C", copy=True)
    nrhs = 1 if b.ndim == 1 else b.shape[1]
    lib().orc_lu_solve(a.shape[0], a.ctypes.data, ipiv.ctypes.data, b.ctypes.data, nrhs)
    return b


def _declare_ewald(L):
    vp, ci, cd = C.c_void_p, C.c_int, C.c_double
    L.orc_ewald3_sigma_xy_ri.restype = None
    L.orc_ewald3_sigma_xy_ri.argtypes = [ci, ci, cd, cd, cd, vp, vp, vp, cd, cd, ci, vp, vp, vp]
    L.orc_get_AB_arrays_e32_ri.restype = ci
    L.orc_get_AB_arrays_e32_ri.argtypes = [vp, vp, vp, cd, cd, cd, vp, vp, vp, cd, cd, ci]
    L.orc_tmatrix_axialsym_ri.restype = None
    L.orc_tmatrix_axialsym_ri.argtypes = [ci, ci, vp, ci, vp, cd, vp, vp, vp, vp]
    L.orc_arc_ri.restype = None
    L.orc_arc_ri.argtypes = [ci, vp, cd, vp]
    L.orc_sigma_direct_ri.restype = None
    L.orc_sigma_direct_ri.argtypes = [ci, ci, cd, cd, vp, vp, vp, ci, vp]
    L.orc_periodic_modeproblem_ri.restype = ci
    L.orc_periodic_modeproblem_ri.argtypes = [vp, ci, vp, vp, cd, cd, vp, vp, cd, vp]
    L.orc_complex_gamma_inc_ri.restype = None
    L.orc_complex_gamma_inc_ri.argtypes = [cd, cd, cd, ci, vp]
    L.orc_ewald_sr_integral_ri.restype = None
    L.orc_ewald_sr_integral_ri.argtypes = [cd, cd, cd, ci, cd, vp]
    L.orc_adjusted_eta.restype = cd
    # double complex by value = two doubles (same registers on x86-64 and aarch64)
    L.orc_adjusted_eta.argtypes = [cd, cd, cd, vp, ci]


def ewald_sigma_xy(lMax_e, eta, k, b1, b2, beta, shift, maxR, maxK, parts=7, csphase=-1):
    """(sigma_total, sigma_short, sigma_long) of the 2D xy Ewald sum, nelem_sc each."""
    L = lib()
    ne = lMax_e * (lMax_e + 2) + 1
    out = [np.zeros(ne, dtype=np.complex128) for _ in range(3)]
    b12 = np.array([b1[0], b1[1], b2[0], b2[1]], dtype=np.float64)
    be = np.array(beta[:2], dtype=np.float64)
    sh = np.array(list(shift[:3]) + [0.0] * (3 - len(shift[:3])), dtype=np.float64)
    k = complex(k)
    L.orc_ewald3_sigma_xy_ri(lMax_e, csphase, float(eta), k.real, k.imag, b12.ctypes.data, be.ctypes.data,
                             sh.ctypes.data, float(maxR), float(maxK), int(parts), out[0].ctypes.data,
                             out[1].ctypes.data, out[2].ctypes.data)
    return tuple(out)


def get_AB_arrays_e32(calc, eta, k, b1, b2, beta, shift, maxR, maxK, parts=7):
    L = lib()
    ne = calc.nelem
    A = np.zeros((ne, ne), dtype=np.complex128)
    B = np.zeros((ne, ne), dtype=np.complex128)
    b12 = np.array([b1[0], b1[1], b2[0], b2[1]], dtype=np.float64)
    be = np.array(beta[:2], dtype=np.float64)
    sh = np.array(list(shift[:3]) + [0.0] * (3 - len(shift[:3])), dtype=np.float64)
    k = complex(k)
    L.orc_get_AB_arrays_e32_ri(calc.ptr, A.ctypes.data, B.ctypes.data, float(eta), k.real, k.imag, b12.ctypes.data,
                               be.ctypes.data, sh.ctypes.data, float(maxR), float(maxK), int(parts))
    return A, B


def periodic_modeproblem(calc, pos, T, k, b1, b2, kvec, eta):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.complex128)
    np_ = pos.shape[0]
    N = np_ * 2 * calc.nelem
    M = np.empty((N, N), dtype=np.complex128)
    b12 = np.array([b1[0], b1[1], b2[0], b2[1]], dtype=np.float64)
    kv = np.array(kvec[:2], dtype=np.float64)
    k = complex(k)
    lib().orc_periodic_modeproblem_ri(calc.ptr, np_, pos.ctypes.data, T.ctypes.data, k.real, k.imag,
                                      b12.ctypes.data, kv.ctypes.data, float(eta), M.ctypes.data)
    return M


def sigma_direct(lMax_e, k, b1, b2, beta, shift, nlayers, csphase=-1):
    """Direct (non-Ewald) lattice sum of h_n(k r) leg_nm e^{i m phi} e^{i beta.(R - s)},
    |i|, |j| <= nlayers; converges for Im k > 0."""
    out = np.zeros((lMax_e + 1) ** 2, dtype=np.complex128)
    b12 = np.array([b1[0], b1[1], b2[0], b2[1]], dtype=np.float64)
    be = np.array(beta[:2], dtype=np.float64)
    sh = np.array(list(shift[:3]) + [0.0] * (3 - len(shift[:3])), dtype=np.float64)
    k = complex(k)
    lib().orc_sigma_direct_ri(lMax_e, csphase, k.real, k.imag, b12.ctypes.data, be.ctypes.data, sh.ctypes.data,
                              int(nlayers), out.ctypes.data)
    return out


def complex_gamma_inc(a, x, m=0):
    out = np.zeros(1, dtype=np.complex128)
    x = complex(x)
    lib().orc_complex_gamma_inc_ri(float(a), x.real, x.imag, int(m), out.ctypes.data)
    return out[0]


def ewald_sr_integral(r, k, n, eta):
    out = np.zeros(1, dtype=np.complex128)
    k = complex(k)
    lib().orc_ewald_sr_integral_ri(float(r), k.real, k.imag, int(n), float(eta), out.ctypes.data)
    return out[0]


def adjusted_eta(area, wavenumber, kvec, lMax):
    kv = np.zeros(3)
    kv[:len(kvec)] = kvec
    w = complex(wavenumber)
    return lib().orc_adjusted_eta(float(area), w.real, w.imag, kv.ctypes.data, int(lMax))


SHAPES = {"sphere": 0, "cylinder": 1, "spheroid": 2}


def tmatrix_axialsym(lMax, k, kin, shape, par, lMaxQR=None, zr=None, rtol=1e-10, want_QR=False):
    """T-matrix (default normalisation, bspec order) of an axially symmetric
    particle by the extended-boundary-condition method; zr = z / z_in defaults
    to kin / k (non-magnetic media).  Optionally Q, R at lMaxQR."""
    L = lib()
    lq = max(lMax, lMaxQR or lMax)
    n, nq = 2 * lMax * (lMax + 2), 2 * lq * (lq + 2)
    T = np.zeros((n, n), dtype=np.complex128)
    Q = np.zeros((nq, nq), dtype=np.complex128)
    R = np.zeros((nq, nq), dtype=np.complex128)
    k, kin = complex(k), complex(kin)
    zr = complex(kin / k if zr is None else zr)
    kk = np.array([k.real, k.imag, kin.real, kin.imag, zr.real, zr.imag])
    pr = np.ascontiguousarray(par, dtype=np.float64)
    rc = np.zeros(1, dtype=np.int32)
    L.orc_tmatrix_axialsym_ri(lMax, lq, kk.ctypes.data, SHAPES.get(shape, shape), pr.ctypes.data, float(rtol),
                              T.ctypes.data, Q.ctypes.data, R.ctypes.data, rc.ctypes.data)
    if rc[0]:
        raise ArithmeticError("singular Q block")
    return (T, Q, R) if want_QR else T


def arc(shape, par, theta):
    out = np.zeros(2)
    lib().orc_arc_ri(SHAPES.get(shape, shape), np.ascontiguousarray(par, dtype=np.float64).ctypes.data,
                     float(theta), out.ctypes.data)
    return tuple(out)
