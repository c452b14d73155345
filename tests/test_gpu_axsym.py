"""GPU parity of the axially symmetric T-matrices (extended-boundary-condition
method; qpms_tmatrix_axialsym_fill and relatives, tmatrices.c:615-976) against
the oracle, through the C-ABI.

Tolerances: sphere as an arc against the Mie T-matrix 1e-12 (relative to
max |T|); cylinders and spheroids against the oracle's adaptive quadrature
1e-10 (the GPU integrates on fixed Gauss-Legendre panels); lossless spheroid
unitarity T + T^H + 2 T^H T = 0 to the truncation error; Q and R in the
reference's transposed layout 1e-10 (relative to the largest entry of the m
block); batches bit-identical to single frequencies.
"""
import ctypes as C

import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0

pytestmark = pytest.mark.gpu

OM = 2.1 * EV / HBAR


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _gen(shape, par, eps_o, eps_i, lq):
    from qpms_gb300.tmatrices import TMatrixGenerator
    if shape == "sphere":
        return TMatrixGenerator.sphere_asarc(eps_o, eps_i, par[0], lq)
    if shape == "cylinder":
        return TMatrixGenerator.cylinder(eps_o, eps_i, par[0], par[1], lq)
    return TMatrixGenerator.spheroid(eps_o, eps_i, par[0], par[1], lq)


@pytest.mark.parametrize("lMax,lq", [(1, 1), (2, 4), (4, 4), (6, 8), (3, 12)])
@pytest.mark.parametrize("eps_i", [-12 + 1.2j, 4.0])
def test_sphere_asarc_is_mie(gpu, orc, lMax, lq, eps_i):
    T = _gen("sphere", [50e-9], 2.25, eps_i, lq)(lMax, OM)
    Td = orc.tmatrix_sphere_diag(lMax, 50e-9, OM, eps_i, 2.25)
    assert np.abs(np.diag(T) - Td).max() <= 1e-12 * np.abs(Td).max()
    assert np.abs(T - np.diag(np.diag(T))).max() <= 1e-14 * np.abs(Td).max()


CASES = [("cylinder", (50e-9, 100e-9), -12 + 1.2j), ("cylinder", (60e-9, 40e-9), 4.0),
         ("spheroid", (40e-9, 80e-9), 4.0), ("spheroid", (70e-9, 35e-9), -12 + 1.2j)]


@pytest.mark.parametrize("shape,par,eps_i", CASES)
def test_vs_oracle(gpu, orc, shape, par, eps_i):
    lMax, lq = 3, 5
    T = _gen(shape, par, 2.25, eps_i, lq)(lMax, OM)
    k, ki = np.sqrt(2.25) * OM / C0, np.sqrt(eps_i + 0j) * OM / C0
    O = orc.tmatrix_axialsym(lMax, k, ki, shape, par, lMaxQR=lq)
    assert np.abs(T - O).max() <= 1e-10 * np.abs(O).max(), np.abs(T - O).max() / np.abs(O).max()


def test_complex_frequency_and_batch(gpu, orc):
    """A batch over real and complex frequencies (the Beyn contour case)
    equals the single-frequency calls bit for bit, and the oracle to 1e-10."""
    g = _gen("cylinder", (50e-9, 100e-9), 2.25, -12 + 1.2j, 4)
    oms = OM * np.array([1.0, 0.95 + 0.02j, 1.07 - 0.01j, 1.2])
    Tb = g.batch(3, oms)
    for w, om in enumerate(oms):
        assert np.array_equal(Tb[w], g(3, om))
    k, ki = np.sqrt(2.25) * oms[1] / C0, np.sqrt(-12 + 1.2j) * oms[1] / C0
    O = orc.tmatrix_axialsym(3, k, ki, "cylinder", (50e-9, 100e-9), lMaxQR=4)
    assert np.abs(Tb[1] - O).max() <= 1e-10 * np.abs(O).max()


def test_lossless_unitarity(gpu):
    g = _gen("spheroid", (40e-9, 80e-9), 1.0, 4.0, 8)
    T = g(3, OM)
    U = T + T.conj().T + 2 * T.conj().T @ T
    assert np.abs(U).max() <= 1e-7 * np.abs(T).max()


@pytest.mark.parametrize("J", [3, 1])
def test_RQ_transposed_vs_oracle(gpu, orc, J):
    """qpms_tmatrix_axialsym_RQ_transposed_fill: target[i1 + i2 n] = Q or R
    (i1 outside wave (t, l, m), i2 inside wave (t', l', -m))."""
    lq = 3
    g = _gen("cylinder", (50e-9, 100e-9), 2.25, -12 + 1.2j, lq)
    G = (g.Q_transposed if J == 3 else g.R_transposed)(OM)      # [i2, i1]
    k, ki = np.sqrt(2.25) * OM / C0, np.sqrt(-12 + 1.2j) * OM / C0
    _, Qo, Ro = orc.tmatrix_axialsym(lq, k, ki, "cylinder", (50e-9, 100e-9), lMaxQR=lq, want_QR=True)
    O = Qo if J == 3 else Ro        # [i1][(t', l', m)] holding the (t', l', -m) inside wave
    idx = [(t, l, m) for t in range(2) for l in range(1, lq + 1) for m in range(-l, l + 1)]
    ref = np.zeros_like(O)
    for i1, (t, l, m) in enumerate(idx):
        for j, (t2, l2, m2) in enumerate(idx):
            if m2 == m:
                ref[i1, idx.index((t2, l2, -m))] = O[i1, j]
    got = G.T
    for m in range(-lq, lq + 1):
        rows = [i for i, x in enumerate(idx) if x[2] == m]
        cols = [i for i, x in enumerate(idx) if x[2] == -m]
        blk, rb = got[np.ix_(rows, cols)], ref[np.ix_(rows, cols)]
        assert np.abs(blk - rb).max() <= 1e-10 * np.abs(rb).max(), m
    zero = np.ones_like(got, dtype=bool)
    for m in range(-lq, lq + 1):
        rows = [i for i, x in enumerate(idx) if x[2] == m]
        cols = [i for i, x in enumerate(idx) if x[2] == -m]
        zero[np.ix_(rows, cols)] = False
    assert np.all(got[zero] == 0)


def test_user_arc_and_generator(gpu, orc):
    """A Python arc function (the reference's userarc) and the C generator
    entry with epsmu generators give the library's spheroid T."""
    from qpms_gb300.tmatrices import ArcFunction, TMatrixGenerator, _EpsMu, _Cplx, _TM, BaseSpec
    a, c = 40e-9, 80e-9
    ref = _gen("spheroid", (a, c), 2.25, 4.0, 4)(3, OM)
    L = C.CDLL(gpu.lib()._name)  # private handle: argtypes set here stay out of the package's
    arc_lib = ArcFunction.spheroid(a, c)

    def f(theta):
        rb = L.qpms_arc_spheroid(C.c_double(theta), C.c_void_p(arc_lib.arc.params))
        return rb.r, rb.beta
    from qpms_gb300.tmatrices import _ArcRet
    L.qpms_arc_spheroid.restype = _ArcRet   # a C call returning a struct is supported
    L.qpms_arc_spheroid.argtypes = [C.c_double, C.c_void_p]
    user = TMatrixGenerator(2.25, 4.0, ArcFunction.custom(f), 4)(3, OM)
    assert np.abs(user - ref).max() <= 1e-13 * np.abs(ref).max()

    # qpms_tmatrix_generator_axialsym with constant epsmu generators (qpms_epsmu_const_g)
    eo, ei = _EpsMu(_Cplx(2.25, 0), _Cplx(1, 0)), _EpsMu(_Cplx(4.0, 0), _Cplx(1, 0))
    cg = C.cast(L.qpms_epsmu_const_g, C.c_void_p).value

    class _EMG(C.Structure):
        _fields_ = [("function", C.c_void_p), ("params", C.c_void_p)]

    from qpms_gb300.tmatrices import _Arc

    class _Par(C.Structure):
        _fields_ = [("outside", _EMG), ("inside", _EMG), ("shape", _Arc), ("lMax_extend", C.c_int)]

    par = _Par(_EMG(cg, C.addressof(eo)), _EMG(cg, C.addressof(ei)), arc_lib.arc, 4)
    spec = BaseSpec(3)
    L.qpms_tmatrix_init.restype = C.POINTER(_TM)
    tm = L.qpms_tmatrix_init(spec.ptr)
    L.qpms_tmatrix_generator_axialsym.restype = C.c_int
    L.qpms_tmatrix_generator_axialsym.argtypes = [C.c_void_p, _Cplx, C.c_void_p]
    assert L.qpms_tmatrix_generator_axialsym(tm, _Cplx(OM, 0), C.byref(par)) == 0, gpu.last_error()
    n = spec.n
    T = np.ctypeslib.as_array((C.c_double * (2 * n * n)).from_address(tm.contents.m)).view(np.complex128)
    assert np.array_equal(T.reshape(n, n), ref)
    L.qpms_tmatrix_free(tm)


def test_errors(gpu):
    from qpms_gb300 import QpmsGpuError
    with pytest.raises(QpmsGpuError):
        _gen("cylinder", (50e-9, 100e-9), 2.25, 4.0, 13)(3, OM)       # lMax_extend above 12
    with pytest.raises(QpmsGpuError):
        _gen("cylinder", (-50e-9, 100e-9), 2.25, 4.0, 4)(3, OM)       # R <= 0


# ---- axially symmetric particles in scattering systems ----

def _cyl_system(gpu, lattice=None, lq=5):
    from qpms_gb300.tmatrices import TMatrixGenerator
    a = 580e-9
    if lattice is None:
        pos = np.array([[0, 0, 0], [a, 0, 0], [0, 1.1 * a, 0], [a, 1.1 * a, 0.2 * a]])
    else:
        pos = np.array([[0, 0, 0], [0.5 * a, 0.5 * a, 0.25 * a]])
    gens = [TMatrixGenerator.cylinder(2.25, -12 + 1.2j, 50e-9, 100e-9, lq),
            TMatrixGenerator.spheroid(2.25, 4.0, 40e-9, 80e-9, lq)]
    kinds = np.arange(len(pos)) % 2
    ss = gpu.ScatteringSystem(pos, 0.0, gens, 2.25, 3, kinds=kinds, lattice=lattice)
    return ss, pos, kinds


def _oracle_T(orc, om, lq=5):
    k = np.sqrt(2.25) * om / C0
    return [orc.tmatrix_axialsym(3, k, np.sqrt(-12 + 1.2j) * om / C0, "cylinder", (50e-9, 100e-9), lMaxQR=lq),
            orc.tmatrix_axialsym(3, k, 2.0 * om / C0, "spheroid", (40e-9, 80e-9), lMaxQR=lq)]


@pytest.mark.parametrize("om", [OM, OM * (1 + 0.01j)])
def test_system_of_cylinders_vs_oracle(gpu, orc, om):
    """Mode problem M = I - T S of cylinders and spheroids (dense T formed on
    the GPU at omega) against the oracle's with the oracle's T."""
    ss, pos, kinds = _cyl_system(gpu)
    M = ss(om).modeproblem_matrix_full()
    To = _oracle_T(orc, om)
    T = np.stack([To[t] for t in kinds])
    calc = orc.TransCalculator(3)
    O = orc.finite_modeproblem(calc, pos, T, np.sqrt(2.25) * om / C0)
    I = np.eye(len(M))
    assert np.linalg.norm(M - O) <= 1e-10 * np.linalg.norm(O - I)


def test_lattice_of_cylinders_vs_oracle(gpu, orc):
    a = 580e-9
    ss, pos, kinds = _cyl_system(gpu, lattice=((a, 0.0), (0.0, a)))
    kv = (2e6, -1e6)
    k = np.sqrt(2.25) * OM / C0
    eta = ss.adjusted_eta(k, kv)
    M = ss(OM).modeproblem_matrix_full(k=kv)
    To = _oracle_T(orc, OM)
    T = np.stack([To[t] for t in kinds])
    O = orc.periodic_modeproblem(orc.TransCalculator(3), pos, T, k, (a, 0.0), (0.0, a), kv, eta)
    I = np.eye(len(M))
    assert np.linalg.norm(M - O) <= 1e-9 * np.linalg.norm(O - I)


def test_sphere_as_arc_kind_equals_sphere_kind(gpu):
    """The same spheres as Mie kinds and as arc kinds: extinction of a plane
    wave agrees (the arc kind takes the dense-T path)."""
    from qpms_gb300.tmatrices import TMatrixGenerator
    a = 580e-9
    pos = np.array([[0, 0, 0], [a, 0, 0], [0, a, 0], [a, a, 0]])
    s1 = gpu.ScatteringSystem(pos, 50e-9, -12 + 1.2j, 2.25, 3)
    s2 = gpu.ScatteringSystem(pos, 0.0, [TMatrixGenerator.sphere_asarc(2.25, -12 + 1.2j, 50e-9, 3)], 2.25, 3)
    oms = OM * np.array([0.9, 1.0, 1.1])
    r1 = s1.planewave_scatter_batch(oms, mode=0)
    r2 = s2.planewave_scatter_batch(oms, mode=0)
    np.testing.assert_allclose(r2["sigma_ext"], r1["sigma_ext"], rtol=1e-11)
