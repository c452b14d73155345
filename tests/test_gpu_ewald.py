"""GPU parity of the 2D-periodic (Ewald) mode-problem path against the oracle.

Tolerances: mode-problem matrices 1e-10 Frobenius-relative on M and 1e-9 on
the lattice part M - I (that part carries the Ewald sums, whose short- and
long-range pieces cancel); eta invariance of M - I to 1e-9 (the reference's
own check is 1e-10 rel / 1e-8 abs on sigma, tests/test_scalar_ewald32.c);
log|det M| to 1e-9 absolute; plane-wave solves to a 1e-10 residual.
"""
import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0, square_lattice, honeycomb_lattice

pytestmark = pytest.mark.gpu

EPS_I = -12 + 1.2j
EPS_E = 2.25
RAD = 80e-9


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _oracle_M(orc, lMax, pos, b1, b2, om, kv, eta):
    c = orc.TransCalculator(lMax)
    Td = orc.tmatrix_sphere_diag(lMax, RAD, om, EPS_I, EPS_E)
    T = np.stack([np.diag(Td)] * len(pos))
    ke = np.sqrt(EPS_E) * om / C0
    return orc.periodic_modeproblem(c, pos, T, ke, b1, b2, kv, eta)


CASES = [("square", 1.6, (0.0, 0.0)), ("square", 2.1, (3e6, 1e6)), ("square", 2.6, (5.4e6, 5.4e6)),
         ("honeycomb", 1.7, (0.0, 0.0)), ("honeycomb", 2.3, (4e6, -2e6)), ("honeycomb", 2.55, (7.2e6, 0.0))]


@pytest.mark.parametrize("lat,E,kv", CASES)
def test_periodic_M_vs_oracle(gpu, orc, lat, E, kv):
    lMax = 3
    b1, b2, pos = square_lattice() if lat == "square" else honeycomb_lattice()
    ss = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax, lattice=(b1, b2))
    om = E * EV / HBAR
    ke = np.sqrt(EPS_E) * om / C0
    eta = ss.adjusted_eta(ke, kv)
    M = ss(om).modeproblem_matrix_full(k=kv)
    O = _oracle_M(orc, lMax, pos, b1, b2, om, kv, eta)
    I = np.eye(len(M))
    assert np.linalg.norm(M - O) <= 1e-10 * np.linalg.norm(O)
    assert np.linalg.norm(M - O) <= 1e-9 * np.linalg.norm(O - I), np.linalg.norm(M - O) / np.linalg.norm(O - I)


CASES_COMPLEX = [("square", 1.72 + 0.05j, (0.0, 0.0)), ("square", 1.909 - 0.0788j, (0.0, 0.0)),
                 ("square", 2.1 + 0.02j, (3e6, 1e6)), ("honeycomb", 2.3 + 0.05j, (0.0, 0.0)),
                 ("honeycomb", 2.3 - 0.05j, (4e6, -2e6))]


@pytest.mark.parametrize("lat,E,kv", CASES_COMPLEX)
def test_periodic_M_complex_omega(gpu, orc, lat, E, kv):
    """Complex frequencies (Beyn contours), both signs of Im omega, Bloch
    vectors on and off a reciprocal lattice point; plus eta invariance."""
    lMax = 3
    b1, b2, pos = square_lattice() if lat == "square" else honeycomb_lattice()
    ss = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax, lattice=(b1, b2))
    om = E * EV / HBAR
    ke = np.sqrt(EPS_E) * om / C0
    eta = ss.adjusted_eta(ke, kv)
    M = ss(om).modeproblem_matrix_full(k=kv)
    M2 = ss(om).modeproblem_matrix_full(k=kv, eta=1.3 * eta)
    O = _oracle_M(orc, lMax, pos, b1, b2, om, kv, eta)
    I = np.eye(len(M))
    assert np.linalg.norm(M - O) <= 1e-10 * np.linalg.norm(O)
    assert np.linalg.norm(M - O) <= 1e-9 * np.linalg.norm(O - I)
    assert np.linalg.norm(M2 - M) <= 1e-9 * np.linalg.norm(M - I)


def test_eta_invariance_gpu(gpu):
    lMax = 3
    b1, b2, pos = honeycomb_lattice()
    ss = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax, lattice=(b1, b2))
    om = 2.0 * EV / HBAR
    ke = np.sqrt(EPS_E) * om / C0
    kv = (2e6, 1e6)
    eta0 = ss.adjusted_eta(ke, kv)
    ssw = ss(om)
    Ms = [ssw.modeproblem_matrix_full(k=kv, eta=f * eta0) for f in (1.0, 1.3, 1.7)]
    I = np.eye(len(Ms[0]))
    for Mx in Ms[1:]:
        assert np.linalg.norm(Mx - Ms[0]) <= 1e-9 * np.linalg.norm(Ms[0] - I)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("lat", ["square", "honeycomb"])
def test_dispersion_scan_vs_oracle(gpu, orc, lat, mode):
    """mode 0: complex128 LU; mode 1: complex64 LU + FP64 refinement, with
    log|det| from complex128 factors of the same FP64 matrices in both modes
    (1e-9 absolute against the oracle's LAPACK slogdet)."""
    lMax = 3
    b1, b2, pos = square_lattice() if lat == "square" else honeycomb_lattice()
    ss = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax, lattice=(b1, b2))
    om = np.array([1.65, 2.05, 2.45]) * EV / HBAR
    kvs = np.array([[0.0, 0.0], [2.5e6, 0.0], [4e6, 3e6]])
    out = ss.dispersion_scan(om, kvs, want_f=True, mode=mode)
    assert (out["residual"] <= 1e-10).all(), out["residual"].max()
    ld_tol = 1e-9
    c = orc.TransCalculator(lMax)
    for i, w in enumerate(om):
        ke = np.sqrt(EPS_E) * w / C0
        for j, kv in enumerate(kvs):
            eta = ss.adjusted_eta(ke, kv)
            O = _oracle_M(orc, lMax, pos, b1, b2, w, kv, eta)
            sgn, ld = np.linalg.slogdet(O)
            assert abs(out["logdet"][i, j] - ld) <= ld_tol, (out["logdet"][i, j], ld)
            # plane wave with in-plane k = Bloch vector, E = x projected perpendicular to k
            kz = np.sqrt(ke ** 2 - kv[0] ** 2 - kv[1] ** 2)
            kd = np.array([kv[0], kv[1], kz])
            E = np.array([1.0, 0, 0]) - (kd[0] / ke) * kd / ke
            E /= np.linalg.norm(E)
            a = orc.planewave_full(lMax, pos, kd, E)
            Td = orc.tmatrix_sphere_diag(lMax, RAD, w, EPS_I, EPS_E)
            f = np.linalg.solve(O, np.tile(Td, len(pos)) * a)
            assert np.linalg.norm(out["f"][i, j] - f) <= 1e-9 * np.linalg.norm(f)
            sig = -np.vdot(a, f).real / ke ** 2
            assert abs(out["sigma_ext"][i, j] - sig) <= 1e-9 * abs(sig)


@pytest.mark.parametrize("norm", [65536 | 8, 65536, 65536 * 3 | 8])
@pytest.mark.parametrize("k,beta,shift", [(2.3, (2.7, 1.0), (0.5, 0.1325, 0.0)),
                                          (2.3 + 0.1j, (2.7, 1.0), (0.0, 0.0, 0.0)),
                                          (2.3 - 0.1j, (0.3, -0.2), (0.25, 0.4, 0.0)),
                                          # layers at different heights
                                          (2.3, (2.7, 1.0), (0.5, 0.1325, 0.3)),
                                          (2.3 + 0.1j, (0.3, -0.2), (0.0, 0.0, -0.45)),
                                          # |k z| >= 2.5: the reciprocal-lattice sum
                                          (5.3, (0.7, -0.4), (0.2, 0.5, -0.8)),
                                          (2.3 + 0.1j, (0.3, -0.2), (0.1, 0.3, 1.7))])
def test_AB_arrays_e32_vs_oracle(gpu, orc, norm, k, beta, shift):
    """qpms_trans_calculator_get_AB_arrays_e32 (unit square lattice, lMax 3,
    eta 1.6: the reference's eta-invariance parameter sets) against the oracle,
    for several normalisations (csphase on and off); particle_shift.z != 0
    takes the shifted-layer sums."""
    import ctypes as C

    class Cplx(C.Structure):
        _fields_ = [("re", C.c_double), ("im", C.c_double)]

    class Cart2(C.Structure):
        _fields_ = [("x", C.c_double), ("y", C.c_double)]

    class Cart3(C.Structure):
        _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]

    L = C.CDLL(gpu.lib()._name)  # private handle: argtypes set here stay out of the package's
    f = L.qpms_trans_calculator_get_AB_arrays_e32
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_ssize_t, C.c_double,
                  Cplx, Cart2, Cart2, Cart2, Cart3, C.c_double, C.c_double]
    lMax = 3
    calc = gpu.trans_calculator(lMax, norm)
    ne = lMax * (lMax + 2)
    A = np.zeros((ne, ne), dtype=np.complex128)
    B = np.zeros((ne, ne), dtype=np.complex128)
    kc = complex(k)
    rc = f(calc.c, A.ctypes.data, None, B.ctypes.data, None, ne, 1, 1.6, Cplx(kc.real, kc.imag), Cart2(1, 0),
           Cart2(0, 1), Cart2(*beta), Cart3(*shift), 20.0, 160.0)
    assert rc == 0, gpu.last_error()
    oc = orc.TransCalculator(lMax, norm)
    Ao, Bo = orc.get_AB_arrays_e32(oc, 1.6, kc, (1, 0), (0, 1), beta, shift, 20, 160)
    assert np.linalg.norm(A - Ao) <= 1e-11 * np.linalg.norm(Ao)
    assert np.linalg.norm(B - Bo) <= 1e-11 * np.linalg.norm(Bo)


LAYERED = [  # positions in units of the square lattice constant 580 nm
    ((0, 0, 0), (0.5, 0.3, 0.4)),
    ((0, 0, 0), (0, 0, 0.35)),                     # second layer straight above (rho = 0 branch)
    ((0, 0, 0), (0.5, 0.5, 0.25), (0.1, -0.2, -0.3)),
]


@pytest.mark.parametrize("cell", LAYERED)
@pytest.mark.parametrize("E,kv", [(1.9, (0.0, 0.0)), (2.3, (4e6, -2e6)), (2.1 + 0.03j, (2e6, 1e6))])
def test_layered_lattice_M_vs_oracle(gpu, orc, cell, E, kv):
    """Particles of a square lattice at different heights (a bilayer and a
    three-layer cell): the pairs of layers go through the shifted-layer Ewald
    sums.  Same tolerances as the single-plane lattices."""
    lMax = 2
    a = 580e-9
    b1, b2 = (a, 0.0), (0.0, a)
    pos = np.array(cell, dtype=float) * a
    ss = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax, lattice=(b1, b2))
    om = E * EV / HBAR
    ke = np.sqrt(EPS_E) * om / C0
    eta = ss.adjusted_eta(ke, kv)
    M = ss(om).modeproblem_matrix_full(k=kv)
    O = _oracle_M(orc, lMax, pos, b1, b2, om, kv, eta)
    I = np.eye(len(M))
    assert np.linalg.norm(M - O) <= 1e-10 * np.linalg.norm(O)
    assert np.linalg.norm(M - O) <= 1e-9 * np.linalg.norm(O - I), np.linalg.norm(M - O) / np.linalg.norm(O - I)
    # the sums do not depend on eta (the kernel lowers eta for distant layers)
    M2 = ss(om).modeproblem_matrix_full(k=kv, eta=0.7 * eta)
    assert np.linalg.norm(M2 - M) <= 1e-9 * np.linalg.norm(M - I)


def test_periodic_translation_matrix_dropins(gpu, orc):
    """qpms_scatsys_periodic_build_translation_matrix_full and
    qpms_scatsyswk_build_translation_matrix_full (scatsystem.c:1252-1281): W of
    the unit cell (here a bilayer cell) against the oracle's I + W (T = -1)
    minus I; the finite qpms_scatsys_build_translation_matrix_full equals the
    _e_full form with outgoing waves."""
    import ctypes as C

    class Cplx(C.Structure):
        _fields_ = [("re", C.c_double), ("im", C.c_double)]

    class Cart3(C.Structure):
        _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]

    L = C.CDLL(gpu.lib()._name)  # private handle: argtypes set here stay out of the package's
    lMax, a = 2, 580e-9
    pos = np.array([[0, 0, 0], [0.5, 0.3, 0.4]]) * a
    ss = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax, lattice=((a, 0.0), (0.0, a)))
    om = 2.0 * EV / HBAR
    k = np.sqrt(EPS_E) * om / C0
    kv = (3e6, -1e6)
    eta = ss.adjusted_eta(k, kv)
    N = ss.fecv_size
    f = L.qpms_scatsys_periodic_build_translation_matrix_full
    f.restype = C.c_void_p
    f.argtypes = [C.c_void_p, C.c_void_p, Cplx, C.POINTER(Cart3), C.c_double]
    W = np.zeros((N, N), dtype=np.complex128)
    assert f(W.ctypes.data, ss.s, Cplx(k, 0.0), C.byref(Cart3(kv[0], kv[1], 0.0)), 0.0), gpu.last_error()
    n = 2 * lMax * (lMax + 2)
    T = np.ascontiguousarray(np.broadcast_to(-np.eye(n), (2, n, n)), dtype=complex)
    X = orc.periodic_modeproblem(orc.TransCalculator(lMax), pos, T, k, (a, 0.0), (0.0, a), kv, eta)
    ref = X - np.eye(N)
    assert np.linalg.norm(W - ref) <= 1e-10 * np.linalg.norm(ref)
    # finite: the J = 3 shorthand
    fin = gpu.ScatteringSystem(pos, RAD, EPS_I, EPS_E, lMax)
    g = L.qpms_scatsys_build_translation_matrix_full
    g.restype = C.c_void_p
    g.argtypes = [C.c_void_p, C.c_void_p, Cplx]
    h = L.qpms_scatsys_build_translation_matrix_e_full
    h.restype = C.c_void_p
    h.argtypes = [C.c_void_p, C.c_void_p, Cplx, C.c_int]
    S1 = np.zeros((N, N), dtype=np.complex128)
    S3 = np.zeros((N, N), dtype=np.complex128)
    assert g(S1.ctypes.data, fin.s, Cplx(k, 0.0)) and h(S3.ctypes.data, fin.s, Cplx(k, 0.0), 3)
    assert np.array_equal(S1, S3)


def test_symmetry_from_reference_group_object(gpu):
    """qpms_gpu_scatsys_set_symmetry_group reads the group's name, the first
    member of the reference's qpms_finite_group_t."""
    import ctypes as C

    class FG(C.Structure):
        _fields_ = [("name", C.c_char_p), ("order", C.c_int)]

    a = 400e-9
    pos = np.array([[x, y, 0.0] for x in (-a / 2, a / 2) for y in (-a / 2, a / 2)])
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, 2)
    L = C.CDLL(gpu.lib()._name)  # private handle: argtypes set here stay out of the package's
    L.qpms_gpu_scatsys_set_symmetry_group.restype = C.c_int
    L.qpms_gpu_scatsys_set_symmetry_group.argtypes = [C.c_void_p, C.c_void_p]
    grp = FG(b"D4h", 16)
    assert L.qpms_gpu_scatsys_set_symmetry_group(ss.s, C.byref(grp)) == 0, gpu.last_error()
    assert ss.nirreps == 10


def test_AB_arrays_e32_cutoffs_and_error_estimate(gpu, orc):
    """The caller's maxR / maxK (translations.c:960-1000: PGen_xyWeb layers,
    latticegens.c:449-568).  Unit square lattice, eta 1.6, shift (0.5,
    0.1325): the points with |R - s| eta <= 6 reach the diamond layer
    |i| + |j| = 5, of height 5 / sqrt(2) = 3.536, so maxR 3.6 keeps the full
    sum (matching the oracle's sum over those layers) and maxR 3.5 asks for a
    truncated one (QPMS_EINVAL).  Aerr / Berr hold |A(eta) - A(1.25 eta)|."""
    import ctypes as C

    class Cplx(C.Structure):
        _fields_ = [("re", C.c_double), ("im", C.c_double)]

    class Cart2(C.Structure):
        _fields_ = [("x", C.c_double), ("y", C.c_double)]

    class Cart3(C.Structure):
        _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]

    L = C.CDLL(gpu.lib()._name)  # private handle: argtypes set here stay out of the package's
    f = L.qpms_trans_calculator_get_AB_arrays_e32
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_ssize_t, C.c_double,
                  Cplx, Cart2, Cart2, Cart2, Cart3, C.c_double, C.c_double]
    lMax, ne = 3, 15
    calc = gpu.trans_calculator(lMax)
    oc = orc.TransCalculator(lMax)
    beta, shift = (2.7, 1.0), (0.5, 0.1325, 0.0)

    def run(maxR, maxK, err=False):
        A = np.zeros((ne, ne), dtype=np.complex128)
        B = np.zeros_like(A)
        Ae = np.full((ne, ne), np.nan) if err else None
        Be = np.full((ne, ne), np.nan) if err else None
        rc = f(calc.c, A.ctypes.data, None if Ae is None else Ae.ctypes.data, B.ctypes.data,
               None if Be is None else Be.ctypes.data, ne, 1, 1.6, Cplx(2.3, 0.0), Cart2(1, 0), Cart2(0, 1),
               Cart2(*beta), Cart3(*shift), maxR, maxK)
        return rc, A, B, Ae, Be

    rc, A, B, Ae, Be = run(3.6, 160.0, err=True)
    assert rc == 0, gpu.last_error()
    Ao, Bo = orc.get_AB_arrays_e32(oc, 1.6, 2.3, (1, 0), (0, 1), beta, shift, 3.6, 160)
    assert np.linalg.norm(A - Ao) <= 1e-11 * np.linalg.norm(Ao)
    assert np.linalg.norm(B - Bo) <= 1e-11 * np.linalg.norm(Bo)
    for G, E in ((A, Ae), (B, Be)):
        assert np.all(np.isfinite(E)) and np.all(E >= 0)
        assert E.max() <= 1e-10 * np.abs(G).max()
    assert Ae.max() > 0  # a second evaluation, not a zero fill
    rc, *_ = run(3.5, 160.0)
    assert rc == 22 and "maxR" in gpu.last_error()
    # |K + beta|^2 - |k|^2 <= 36 (2 eta)^2 reaches |K| ~ 22.8: maxK 10 truncates
    rc, *_ = run(20.0, 10.0)
    assert rc == 22 and "maxK" in gpu.last_error()
