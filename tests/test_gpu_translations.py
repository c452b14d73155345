"""GPU parity of the batched translation kernel against the oracle, through the C-ABI.

Tolerance (translation coefficients, 1e-11 relative): for every translation
and each of A, B: ||G - O||_F <= 1e-11 ||O||_F, and element-wise
|g - o| <= 1e-11 |o| + 1e-13 max|O|.  The absolute floor (1e-13 of the
matrix's largest element) covers elements that are small only because their
q-terms, each of order max|O|, cancel: their rounding error is set by the
terms, not by the sum, in the reference (AMOS/GSL) as much as here.
"""
import numpy as np
import pytest

from qpms_gb300.workloads import translation_vectors

pytestmark = pytest.mark.gpu

RTOL = 1e-11
ATOL_REL = 1e-13


def _check(G, O, what):
    G = G.reshape(-1, G.shape[-2] * G.shape[-1])
    O = O.reshape(-1, O.shape[-2] * O.shape[-1])
    fro = np.linalg.norm(G - O, axis=1) / np.linalg.norm(O, axis=1)
    assert np.all(np.isfinite(fro)), what
    assert fro.max() <= RTOL, (what, fro.max())
    bound = RTOL * np.abs(O) + ATOL_REL * np.abs(O).max(axis=1, keepdims=True)
    excess = (np.abs(G - O) / bound).max()
    assert excess <= 1.0, (what, excess)
    return fro.max(), excess


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _inputs(n, seed):
    kr, th, ph = translation_vectors(n, seed=seed)
    # mix in real kr (the GSL real-argument branch of qpms_sph_bessel_fill)
    kr[::7] = kr[::7].real
    # and a few large / small arguments at the edges of the range
    kr[1] = 0.6
    kr[2] = 198.0 + 0.1j
    th[3] = 0.0
    th[4] = np.pi
    return kr, th, ph


@pytest.mark.parametrize("lMax", [1, 2, 3, 4, 6, 8])
@pytest.mark.parametrize("J", [1, 2, 3, 4])
def test_batch_device_vs_oracle(torch_cuda, orc, lMax, J):
    torch = torch_cuda
    import qpms_gb300
    n = 300 if lMax <= 4 else 60
    kr, th, ph = _inputs(n, seed=100 + lMax * 10 + J)
    c = qpms_gb300.trans_calculator(lMax)
    ne = c.nelem()
    dev = torch.device("cuda:0")
    tkr = torch.from_numpy(kr).to(dev)
    tth = torch.from_numpy(th).to(dev)
    tph = torch.from_numpy(ph).to(dev)
    A = torch.empty((n, ne, ne), dtype=torch.complex128, device=dev)
    B = torch.empty_like(A)
    c.get_AB_arrays_device(tkr, tth, tph, J, A, B)
    torch.cuda.synchronize()
    oA, oB = orc.TransCalculator(lMax).get_AB_batch(kr, th, ph, J)
    _check(A.cpu().numpy(), oA, "A")
    _check(B.cpu().numpy(), oB, "B")


def test_host_api_and_variants_agree(torch_cuda, orc, monkeypatch):
    import qpms_gb300
    kr, th, ph = _inputs(1000, seed=7)
    c = qpms_gb300.trans_calculator(3)
    a0, b0 = c.get_AB_arrays(kr, th, ph, False, 3)  # pageable numpy buffers
    monkeypatch.setenv("QPMS_GB300_TRANS_VARIANT", "1")
    a1, b1 = c.get_AB_arrays(kr, th, ph, False, 3)
    assert np.array_equal(a0, a1) and np.array_equal(b0, b1)
    oA, oB = orc.TransCalculator(3).get_AB_batch(kr, th, ph, 3)
    _check(a0, oA, "A")
    _check(b0, oB, "B")


def test_single_dropin_strides_and_r_zero(torch_cuda, orc):
    import qpms_gb300
    c = qpms_gb300.trans_calculator(2)
    o = orc.TransCalculator(2)
    A, B = c.get_AB_arrays_single(3.3 + 0.01j, 0.7, 1.9, False, 3)
    oA, oB = o.get_AB_arrays_single(3.3 + 0.01j, 0.7, 1.9, False, 3)
    _check(A[None], oA[None], "A")
    _check(B[None], oB[None], "B")
    # r == 0 with a singular kind -> NaN arrays (translations.c:641-649)
    A, B = c.get_AB_arrays_single(0.0, 0.3, 0.2, False, 3)
    assert np.all(np.isnan(A)) and np.all(np.isnan(B))
    # r_ge_d forces the regular kind
    A, B = c.get_AB_arrays_single(0.0, 0.3, 0.2, True, 3)
    oA, oB = o.get_AB_arrays_single(0.0, 0.3, 0.2, True, 3)
    assert np.allclose(A, oA, rtol=0, atol=1e-14)
    # broadcasting like the Cython wrapper
    a, b = c.get_AB_arrays(np.array([[1.0, 2.0]]), np.array([0.3]), 0.1, False, 1)
    assert a.shape == (1, 2, 8, 8)


def test_empty_batch(torch_cuda):
    import qpms_gb300
    c = qpms_gb300.trans_calculator(3)
    a, b = c.get_AB_arrays(np.zeros(0), np.zeros(0), np.zeros(0), False, 3)
    assert a.shape == (0, 15, 15)


def test_full_size_parity_symmetry(torch_cuda, orc):
    """10^6 translations at lMax 3: a seeded 1% subsample against the oracle,
    and on the whole batch the inversion symmetry r -> -r
    (A -> (-1)^(n+nu) A, B -> (-1)^(n+nu+1) B) between two launches."""
    torch = torch_cuda
    import qpms_gb300
    n = 1_000_000
    kr, th, ph = translation_vectors(n, seed=11)
    c = qpms_gb300.trans_calculator(3)
    ne = 15
    dev = torch.device("cuda:0")
    tkr = torch.from_numpy(kr).to(dev)
    A = torch.empty((n, ne, ne), dtype=torch.complex128, device=dev)
    B = torch.empty_like(A)
    c.get_AB_arrays_device(tkr, torch.from_numpy(th).to(dev), torch.from_numpy(ph).to(dev), 3, A, B)
    A2 = torch.empty_like(A)
    B2 = torch.empty_like(A)
    th2 = np.pi - th
    ph2 = np.mod(ph + np.pi, 2 * np.pi)
    c.get_AB_arrays_device(tkr, torch.from_numpy(th2).to(dev), torch.from_numpy(ph2).to(dev), 3, A2, B2)
    nn = np.array([int(np.sqrt(y + 1)) for y in range(ne)])
    sgn = torch.from_numpy(((-1.0) ** (nn[:, None] + nn[None, :]))).to(dev)
    dA = (A2 - sgn * A).abs().amax(dim=(1, 2)) / A.abs().amax(dim=(1, 2))
    dB = (B2 + sgn * B).abs().amax(dim=(1, 2)) / B.abs().amax(dim=(1, 2))
    assert float(dA.max()) < 1e-10 and float(dB.max()) < 1e-10
    idx = np.random.default_rng(3).choice(n, 10_000, replace=False)
    oA, oB = orc.TransCalculator(3).get_AB_batch(kr[idx], th[idx], ph[idx], 3)
    tidx = torch.from_numpy(idx).to(dev)
    _check(A[tidx].cpu().numpy(), oA, "A")
    _check(B[tidx].cpu().numpy(), oB, "B")


def test_trans_array_lc3p_vs_oracle(torch_cuda, orc):
    """qpms_trans_calculator_get_trans_array_lc3p: a full bspec (N then M
    waves, lMax 3) between two positions, against the oracle's A/B arranged by
    qpms_trans_array_from_AB (translations_inlines.h:8-35)."""
    import ctypes as C
    import qpms_gb300

    class Cplx(C.Structure):
        _fields_ = [("re", C.c_double), ("im", C.c_double)]

    class Cart3(C.Structure):
        _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]

    class Spec(C.Structure):
        _fields_ = [("n", C.c_size_t), ("ilist", C.c_void_p), ("lMax", C.c_int), ("lMax_M", C.c_int),
                    ("lMax_N", C.c_int), ("lMax_L", C.c_int), ("capacity", C.c_size_t), ("norm", C.c_int)]

    lMax = 3
    L = C.CDLL(qpms_gb300.lib()._name)  # private handle: argtypes set here stay out of the package's
    L.qpms_trans_calculator_get_trans_array_lc3p.restype = C.c_int
    L.qpms_trans_calculator_get_trans_array_lc3p.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(Spec), C.c_size_t,
                                                              C.POINTER(Spec), C.c_size_t, Cplx, Cart3, Cart3, C.c_int]
    ys = [(t, n * (n + 1) + m) for t in (2, 1) for n in range(1, lMax + 1) for m in range(-n, n + 1)]
    il = np.array([t + 4 * y for t, y in ys], dtype=np.uint64)
    spec = Spec(len(ys), il.ctypes.data, lMax, lMax, lMax, -1, len(ys), 65536 | 8)
    calc = qpms_gb300.trans_calculator(lMax)
    rng = np.random.default_rng(5)
    c = orc.TransCalculator(lMax)
    for _ in range(4):
        d = rng.normal(size=3) * 400e-9
        k = complex(1.2e7, rng.uniform(0, 1e4))
        for J in (1, 3):
            out = np.zeros((len(ys), len(ys)), dtype=np.complex128)
            rc = L.qpms_trans_calculator_get_trans_array_lc3p(calc.c, out.ctypes.data, C.byref(spec), len(ys),
                                                              C.byref(spec), 1, Cplx(k.real, k.imag),
                                                              Cart3(*d), Cart3(0, 0, 0), J)
            assert rc == 0, qpms_gb300.last_error()
            r = np.linalg.norm(d)
            A, B = c.get_AB_arrays_single(k * r, np.arccos(d[2] / r), np.arctan2(d[1], d[0]), False, J)
            ref = np.empty_like(out)
            for di, (td, yd) in enumerate(ys):
                for si, (ts, y2) in enumerate(ys):
                    ref[di, si] = (A if ts == td else B)[yd - 1, y2 - 1]
            assert np.linalg.norm(out - ref) <= RTOL * np.linalg.norm(ref)
