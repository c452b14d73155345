"""Reference-API convenience entry points beside the hot path (qg_dropins.cu),
through the C-ABI:

* sphere T-matrices (qpms_mie_coefficients_reflection, qpms_tmatrix_spherical*,
  qpms_tmatrix_generator_sphere; tmatrices.c:500-606) against the oracle's Mie
  diagonal, 1e-12 relative;
* generator / copy / isclose / apply helpers (tmatrices.c:49-75, 257-271, 608-619);
* plane-wave coefficients (qpms_planewave2vswf_fill_*, qpms_incfield_planewave,
  qpms_scatsys_incident_field_vector_full; vswf.c:445-530, scatsystem.c:1970-1983)
  against the oracle's plane-wave vector, 1e-9 (the excitation tolerance);
* single translation coefficients against the oracle's closed form, 1e-11;
* Beyn with the half-ellipse and kidney contours against the oracle's solver on
  the same contour, eigenvalues 1e-8.
"""
import ctypes as C

import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0

pytestmark = pytest.mark.gpu
OM = 2.1 * EV / HBAR
NDEF = 65536 | 8  # QPMS_NORMALISATION_DEFAULT


class Cplx(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def cx(z):
    z = complex(z)
    return Cplx(z.real, z.imag)


def pz(c):
    return complex(c.re, c.im)


class EpsMu(C.Structure):
    _fields_ = [("eps", Cplx), ("mu", Cplx)]


class Spec(C.Structure):
    _fields_ = [("n", C.c_size_t), ("ilist", C.POINTER(C.c_ulonglong)), ("lMax", C.c_int), ("lMax_M", C.c_int),
                ("lMax_N", C.c_int), ("lMax_L", C.c_int), ("capacity", C.c_size_t), ("norm", C.c_int)]


class TM(C.Structure):
    _fields_ = [("spec", C.POINTER(Spec)), ("m", C.POINTER(Cplx)), ("owns_m", C.c_bool)]


class Cart3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class CCart3(C.Structure):
    _fields_ = [("x", Cplx), ("y", Cplx), ("z", Cplx)]


class Sph(C.Structure):
    _fields_ = [("r", C.c_double), ("theta", C.c_double), ("phi", C.c_double)]


class CSphVec(C.Structure):
    _fields_ = [("rc", Cplx), ("thetac", Cplx), ("phic", Cplx)]


class CSph(C.Structure):
    _fields_ = [("r", Cplx), ("theta", C.c_double), ("phi", C.c_double)]


class _KU(C.Union):
    _fields_ = [("cart", CCart3), ("sph", CSph)]


class _EU(C.Union):
    _fields_ = [("cart", CCart3), ("sph", CSphVec)]


class PWParams(C.Structure):
    _fields_ = [("use_cartesian", C.c_bool), ("k", _KU), ("E", _EU)]


EPSMU_FN = C.CFUNCTYPE(EpsMu, Cplx, C.c_void_p)  # declared only for the struct layout


class EpsMuGen(C.Structure):
    _fields_ = [("function", C.c_void_p), ("params", C.c_void_p)]


class SphereParam(C.Structure):
    _fields_ = [("outside", EpsMuGen), ("inside", EpsMuGen), ("radius", C.c_double)]


class TMGen(C.Structure):
    _fields_ = [("function", C.c_void_p), ("params", C.c_void_p)]


INCFIELD = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, Cart3, C.c_void_p, C.c_bool)


@pytest.fixture(scope="module")
def L():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qpms_gb300._lib import lib
    L = C.CDLL(lib()._name)  # private handle: argtypes set here stay out of the package's
    vp, cd, ci, sz = C.c_void_p, C.c_double, C.c_int, C.c_size_t
    PT, PS = C.POINTER(TM), C.POINTER(Spec)
    L.qpms_vswf_set_spec_from_lMax.restype = PS
    L.qpms_vswf_set_spec_from_lMax.argtypes = [ci, ci]
    L.qpms_vswf_set_spec_free.argtypes = [PS]
    L.qpms_tmatrix_free.argtypes = [PT]
    L.qpms_mie_coefficients_reflection.restype = vp
    L.qpms_mie_coefficients_reflection.argtypes = [vp, PS, cd, Cplx, Cplx, Cplx, Cplx, ci, ci]
    L.qpms_tmatrix_spherical.restype = PT
    L.qpms_tmatrix_spherical.argtypes = [PS, cd, Cplx, Cplx, Cplx, Cplx]
    L.qpms_tmatrix_spherical_mu0.restype = PT
    L.qpms_tmatrix_spherical_mu0.argtypes = [PS, cd, cd, Cplx, Cplx]
    L.qpms_tmatrix_init_from_generator.restype = PT
    L.qpms_tmatrix_init_from_generator.argtypes = [PS, TMGen, Cplx]
    L.qpms_tmatrix_copy.restype = PT
    L.qpms_tmatrix_copy.argtypes = [PT]
    L.qpms_tmatrix_mv.restype = PT
    L.qpms_tmatrix_mv.argtypes = [PT, PT]
    L.qpms_tmatrix_isclose.restype = C.c_bool
    L.qpms_tmatrix_isclose.argtypes = [PT, PT, cd, cd]
    L.qpms_apply_tmatrix.restype = vp
    L.qpms_apply_tmatrix.argtypes = [vp, vp, PT]
    L.qpms_wavenumber.restype = Cplx
    L.qpms_wavenumber.argtypes = [Cplx, EpsMu]
    L.qpms_lorentzdrude_epsmu.restype = EpsMu
    L.qpms_lorentzdrude_epsmu.argtypes = [Cplx, vp]
    L.qpms_lorentzdrude_eps.restype = Cplx
    L.qpms_lorentzdrude_eps.argtypes = [Cplx, vp]
    L.qpms_drude_epsilon.restype = Cplx
    L.qpms_drude_epsilon.argtypes = [Cplx, Cplx, Cplx, Cplx]
    L.qpms_planewave2vswf_fill_cart.restype = ci
    L.qpms_planewave2vswf_fill_cart.argtypes = [Cart3, CCart3, vp, vp, vp, ci, ci]
    L.qpms_planewave2vswf_fill_sph.restype = ci
    L.qpms_planewave2vswf_fill_sph.argtypes = [Sph, CSphVec, vp, vp, vp, ci, ci]
    L.qpms_scatsys_incident_field_vector_full.restype = vp
    L.qpms_scatsys_incident_field_vector_full.argtypes = [vp, vp, vp, vp, C.c_bool]
    L.qpms_trans_calculator_init.restype = vp
    L.qpms_trans_calculator_init.argtypes = [ci, ci]
    L.qpms_trans_calculator_free.argtypes = [vp]
    L.qpms_trans_calculator_get_A_ext.restype = Cplx
    L.qpms_trans_calculator_get_A_ext.argtypes = [vp, ci, ci, ci, ci, Cplx, cd, cd, ci, ci]
    L.qpms_trans_calculator_get_B_ext.restype = Cplx
    L.qpms_trans_calculator_get_B_ext.argtypes = [vp, ci, ci, ci, ci, Cplx, cd, cd, ci, ci]
    L.qpms_trans_calculator_get_AB_p.restype = ci
    L.qpms_trans_calculator_get_AB_p.argtypes = [vp, vp, vp, ci, ci, ci, ci, CSph, C.c_bool, ci]
    L.qpms_trans_single_A.restype = Cplx
    L.qpms_trans_single_A.argtypes = [ci, ci, ci, ci, ci, CSph, C.c_bool, ci]
    L.qpms_trans_single_B.restype = Cplx
    L.qpms_trans_single_B.argtypes = [ci, ci, ci, ci, ci, CSph, C.c_bool, ci]
    return L


def _mat(t):
    n = t.contents.spec.contents.n
    return np.ctypeslib.as_array(C.cast(t.contents.m, C.POINTER(C.c_double)), (n * n * 2,)).view(
        np.complex128).reshape(n, n).copy()


@pytest.mark.parametrize("lMax", [1, 3, 6, 10])
@pytest.mark.parametrize("eps_i", [-12 + 1.2j, 4.0])
def test_sphere_tmatrix_vs_oracle(L, orc, lMax, eps_i):
    a, eps_e = 50e-9, 2.25
    Td = orc.tmatrix_sphere_diag(lMax, a, OM, eps_i, eps_e)
    sp = L.qpms_vswf_set_spec_from_lMax(lMax, NDEF)
    k_i, k_e = np.sqrt(complex(eps_i)) * OM / C0, np.sqrt(eps_e) * OM / C0
    d = np.empty(sp.contents.n, dtype=np.complex128)
    assert L.qpms_mie_coefficients_reflection(d.ctypes.data, sp, a, cx(k_i), cx(k_e), cx(1), cx(1), 1, 3)
    assert np.abs(d - Td).max() <= 1e-12 * np.abs(Td).max()
    t1 = L.qpms_tmatrix_spherical(sp, a, cx(k_i), cx(k_e), cx(1), cx(1))
    t2 = L.qpms_tmatrix_spherical_mu0(sp, a, OM, cx(eps_i), cx(eps_e))
    # the generator with constant media (qpms_epsmu_const_g)
    em_o, em_i = EpsMu(cx(eps_e), cx(1)), EpsMu(cx(eps_i), cx(1))
    g = C.cast(L.qpms_epsmu_const_g, C.c_void_p).value
    par = SphereParam(EpsMuGen(g, C.addressof(em_o)), EpsMuGen(g, C.addressof(em_i)), a)
    t3 = L.qpms_tmatrix_init_from_generator(
        sp, TMGen(C.cast(L.qpms_tmatrix_generator_sphere, C.c_void_p).value, C.addressof(par)), cx(OM))
    try:
        M1, M2, M3 = _mat(t1), _mat(t2), _mat(t3)
        assert np.array_equal(np.diag(M1), d) and np.count_nonzero(M1 - np.diag(d)) == 0
        assert np.abs(M2 - M1).max() <= 1e-13 * np.abs(Td).max()
        assert np.abs(M3 - M1).max() <= 1e-13 * np.abs(Td).max()
        assert L.qpms_tmatrix_isclose(t1, t3, 1e-12, 0) and L.qpms_tmatrix_isclose(t1, t2, 1e-12, 0)
        t4 = L.qpms_tmatrix_copy(t1)
        t5 = L.qpms_tmatrix_init_from_generator(
            sp, TMGen(C.cast(L.qpms_tmatrix_generator_constant, C.c_void_p).value, C.cast(t1, C.c_void_p).value),
            cx(OM))
        assert np.array_equal(_mat(t4), M1) and np.array_equal(_mat(t5), M1)
        L.qpms_tmatrix_mv(t4, t2)
        assert np.array_equal(_mat(t4), M2)
        assert not L.qpms_tmatrix_isclose(t1, t4, 0, 0) or np.array_equal(M1, M2)
        rng = np.random.default_rng(lMax)
        av = rng.normal(size=d.size) + 1j * rng.normal(size=d.size)
        f = np.empty_like(av)
        assert L.qpms_apply_tmatrix(f.ctypes.data, av.ctypes.data, t1)
        assert np.abs(f - M1 @ av).max() <= 1e-15 * np.abs(M1).max() * np.abs(av).sum()
        for t in (t4, t5):
            L.qpms_tmatrix_free(t)
    finally:
        for t in (t1, t2, t3):
            L.qpms_tmatrix_free(t)
        L.qpms_vswf_set_spec_free(sp)
    # J_ext == J_scat is refused
    assert not L.qpms_mie_coefficients_reflection(None, L.qpms_vswf_set_spec_from_lMax(2, NDEF), a, cx(k_i),
                                                  cx(k_e), cx(1), cx(1), 1, 1)


def test_materials(L):
    em = EpsMu(cx(2.25), cx(1.0))
    assert abs(pz(L.qpms_wavenumber(cx(OM), em)) - 1.5 * OM / C0) <= 1e-15 * OM / C0
    for name in ("AU", "AG"):
        p = C.c_void_p.in_dll(L, "QPMS_LDPARAMS_" + name).value
        e = L.qpms_lorentzdrude_epsmu(cx(OM), p)
        assert pz(e.eps) == pz(L.qpms_lorentzdrude_eps(cx(OM), p)) and pz(e.mu) == 1
    wp, g = 9.0 * EV / HBAR, 0.07 * EV / HBAR
    assert abs(pz(L.qpms_drude_epsilon(cx(1), cx(wp), cx(g), cx(OM))) - (1 - wp ** 2 / (OM * (OM + 1j * g)))) \
        <= 1e-13 * wp ** 2 / OM ** 2


@pytest.mark.parametrize("lMax", [2, 5])
def test_planewave_coefficients(L, orc, lMax):
    from qpms_gb300.scatsystem import ScatteringSystem
    rng = np.random.default_rng(7)
    pos = rng.uniform(-400e-9, 400e-9, size=(4, 3))
    kdir = np.array([0.3, -0.4, 0.866])
    kdir /= np.linalg.norm(kdir)
    kv = 1.5 * OM / C0 * kdir
    Ec = np.cross(kdir, [1.0, 0.2, 0.0]) * (1 + 0.5j)
    ref = orc.planewave_full(lMax, pos, kv, Ec)
    ne = lMax * (lMax + 2)
    # one particle at the origin: fill_cart gives the per-particle block
    el, mg, lc = (np.empty(ne, dtype=np.complex128) for _ in range(3))
    assert L.qpms_planewave2vswf_fill_cart(Cart3(*kdir), CCart3(*map(cx, Ec)), lc.ctypes.data, mg.ctypes.data,
                                           el.ctypes.data, lMax, NDEF) == 0
    ref0 = orc.planewave_full(lMax, np.zeros((1, 3)), kv, Ec)
    assert np.abs(np.concatenate([el, mg]) - ref0).max() <= 1e-9 * np.abs(ref0).max()
    assert np.abs(lc).max() <= 1e-12 * np.abs(Ec).max()   # transverse amplitude
    # the same wave given in spherical coordinates
    th, ph = np.arccos(kdir[2]), np.arctan2(kdir[1], kdir[0])
    st, ct, sf, cf = np.sin(th), np.cos(th), np.sin(ph), np.cos(ph)
    Es = [0.0, Ec[0] * ct * cf + Ec[1] * ct * sf - Ec[2] * st, -Ec[0] * sf + Ec[1] * cf]
    el2, mg2 = np.empty(ne, dtype=np.complex128), np.empty(ne, dtype=np.complex128)
    assert L.qpms_planewave2vswf_fill_sph(Sph(1.0, th, ph), CSphVec(*map(cx, Es)), None, mg2.ctypes.data,
                                          el2.ctypes.data, lMax, NDEF) == 0
    assert np.abs(el2 - el).max() <= 1e-12 * np.abs(el).max() and np.abs(mg2 - mg).max() <= 1e-12 * np.abs(mg).max()
    # the incident vector of a system through the reference's callback interface
    ss = ScatteringSystem(pos, 50e-9, 4.0, 2.25, lMax)
    prm = PWParams(True, _KU(cart=CCart3(*map(cx, kv))), _EU(cart=CCart3(*map(cx, Ec))))
    fn = C.cast(L.qpms_incfield_planewave, C.c_void_p).value
    out = np.empty(ss.fecv_size, dtype=np.complex128)
    assert L.qpms_scatsys_incident_field_vector_full(out.ctypes.data, ss.s, fn, C.addressof(prm), False)
    assert np.abs(out - ref).max() <= 1e-9 * np.abs(ref).max()
    assert np.abs(out - ss.planewave_full(kv, Ec)).max() <= 1e-12 * np.abs(ref).max()
    # add = true doubles it
    assert L.qpms_scatsys_incident_field_vector_full(out.ctypes.data, ss.s, fn, C.addressof(prm), True)
    assert np.abs(out - 2 * ref).max() <= 2e-9 * np.abs(ref).max()


def test_single_translation_coefficients(L, orc):
    lMax, norm = 4, NDEF
    c = L.qpms_trans_calculator_init(lMax, norm)
    try:
        rng = np.random.default_rng(3)
        for J in (1, 3):
            for _ in range(12):
                n, nu = (int(v) for v in rng.integers(1, lMax + 1, size=2))
                m, mu = int(rng.integers(-n, n + 1)), int(rng.integers(-nu, nu + 1))
                kr = complex(rng.uniform(0.5, 6), 0.0 if J == 3 else rng.uniform(-0.2, 0.2))
                th, ph = rng.uniform(0, np.pi), rng.uniform(-np.pi, np.pi)
                for which, get in (("A", L.qpms_trans_calculator_get_A_ext), ("B", L.qpms_trans_calculator_get_B_ext)):
                    ref = orc.trans_single(which, norm, m, n, mu, nu, kr, th, ph, 0, J)
                    got = pz(get(c, int(m), int(n), int(mu), int(nu), cx(kr), th, ph, 0, J))
                    assert abs(got - ref) <= 1e-11 * max(abs(ref), 1e-3), (which, m, n, mu, nu, J)
                    single = L.qpms_trans_single_A if which == "A" else L.qpms_trans_single_B
                    g2 = pz(single(norm, int(m), int(n), int(mu), int(nu), CSph(cx(kr), th, ph), False, J))
                    assert abs(g2 - ref) <= 1e-11 * max(abs(ref), 1e-3)
                A, B = Cplx(), Cplx()
                assert L.qpms_trans_calculator_get_AB_p(c, C.addressof(A), C.addressof(B), int(m), int(n), int(mu),
                                                        int(nu), CSph(cx(kr), th, ph), False, J) == 0
                assert abs(pz(B) - orc.trans_single("B", norm, m, n, mu, nu, kr, th, ph, 0, J)) <= \
                    1e-11 * max(abs(pz(B)), 1e-3)
        assert L.qpms_trans_calculator_get_AB_p(c, None, None, 0, lMax + 1, 0, 1, CSph(cx(1), 0, 0), False, 1) != 0
    finally:
        L.qpms_trans_calculator_free(c)


def _pencil(n=40, seed=11):
    """complex quadratic pencil T0 + z T1 + z^2 T2 and its eigenvalues (linearised)"""
    import scipy.linalg as sl
    rng = np.random.default_rng(seed)
    T = [rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)) for _ in range(3)]
    I, Z = np.eye(n), np.zeros((n, n))
    lam = sl.eigvals(np.block([[Z, I], [-T[0], -T[1]]]), np.block([[I, Z], [Z, T[2]]]))
    return T, lam[np.isfinite(lam)]


def _radius(lam, curved_side):
    """a radius between two eigenvalue moduli (a 15 % gap) enclosing at least
    two eigenvalues on the curved side of the straight edge, none near it"""
    c = np.sort(np.abs(lam[curved_side(lam)]))
    for k in range(2, c.size):
        if c[k] > 1.15 * c[k - 1]:
            return 0.5 * (c[k - 1] + c[k])
    raise AssertionError("no gap")


@pytest.mark.parametrize("shape", [("halfellipse", 0), ("halfellipse", 3), ("kidney", 0.2, 0)])
def test_beyn_on_halfplane_contours(shape):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import beyn as ob
    from qpms_gb300 import beyn as qb
    (T0, T1, T2), lam = _pencil()
    Mf = lambda z: T0 + z * T1 + z * z * T2
    orient = shape[-1]
    side = (lambda z: z.imag > 0) if orient == 0 else (lambda z: z.real > 0)
    R = _radius(lam, side)
    n = 320
    if shape[0] == "halfellipse":
        contour = ob.halfellipse(0.0, R, R, n, orient)
    else:
        contour = ob.kidney(0.0, R, R, shape[1], n, orient)
    V = np.random.default_rng(5).normal(size=(40, 20)) + 1j * np.random.default_rng(6).normal(size=(40, 20))
    ref = ob.beyn_solve(Mf, 40, 20, contour, V, 1e-4, 1, 1e-4)
    got = qb.beyn_solve(Mf, 40, 20, 0.0, R, R, n, 1e-4, 1, 1e-4, Vhat=V, mode=0, shape=shape)
    assert got["eigval"].size == ref["neig"] >= 2
    for e in ref["eigval"]:
        assert np.min(np.abs(got["eigval"] - e)) <= 1e-8 * max(abs(e), 1e-3)
        assert np.min(np.abs(lam - e)) <= 1e-3 * abs(e)   # a true eigenvalue (to the quadrature error)
