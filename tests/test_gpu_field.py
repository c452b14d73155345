"""GPU parity of the scattered-field evaluation (qpms_scatsys_scattered_E,
scatsystem.c:2013-2039) against the oracle, through the C-ABI.

Tolerance: per point, |E_gpu - E_oracle| <= 1e-10 |E_oracle| + 1e-13 max|E_oracle|
(the oracle is pinned against Bohren & Huffman and the plane-wave
re-expansion identity).  Covered: outgoing (J = 3), regular (J = 1) and
incoming (J = 4) waves, real and complex wavenumbers, points on the polar axis
of a particle (the |cos theta| = 1 branch), in the particle plane, at a
particle centre for regular waves (the r = 0 branch), far away, the split
over particles with its fixed-order reduction, the single-point drop-ins
(direct, __alt, at-omega), the device-buffer entry and an empty point list.
"""
import ctypes as C

import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0, jittered_square_cluster

pytestmark = pytest.mark.gpu

EPS_I = -12 + 1.2j
EPS_E = 2.25


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _close(G, O, rtol=1e-10, floor=1e-13):
    G = np.asarray(G).reshape(-1, 3)
    O = np.asarray(O).reshape(-1, 3)
    d = np.linalg.norm(G - O, axis=1)
    n = np.linalg.norm(O, axis=1)
    bound = rtol * n + floor * n.max()
    assert (d <= bound).all(), (d / bound).max()


def _points(pos, rng, n):
    lo, hi = pos.min(0) - 3e-7, pos.max(0) + 3e-7
    pts = rng.uniform(lo, hi, size=(n, 3))
    pts[: n // 4, 2] = 0.0                                       # particle plane
    axis = pos[: 6] + np.array([0, 0, 1.7e-7])                   # above particles: polar axis
    below = pos[6: 10] - np.array([0, 0, 2.3e-7])                # below: cos theta = -1
    far = rng.normal(size=(8, 3)) * 5e-5
    return np.vstack([pts, axis, below, far])


@pytest.fixture(scope="module")
def solved(gpu):
    rng = np.random.default_rng(21)
    pos = jittered_square_cluster(20, rng)
    lMax = 3
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    om = 2.2 * EV / HBAR
    r = ss.planewave_scatter_batch(np.array([om]), mode=1, want_f=True)
    f = r["f"][0]
    k = np.sqrt(EPS_E) * om / C0
    return ss, pos, lMax, f, k, rng


@pytest.mark.parametrize("J", [3, 1, 4])
def test_field_vs_oracle(gpu, orc, solved, J):
    ss, pos, lMax, f, k, rng = solved
    pts = _points(pos, np.random.default_rng(J), 400)
    if J == 1:
        pts = np.vstack([pts, pos[:3]])                          # particle centres: r = 0 branch
    E = ss.scattered_E(k, f, pts, btyp=J)
    O = orc.scattered_E(lMax, pos, J, k, f, pts)
    assert np.isfinite(E).all()
    _close(E, O)


def test_field_complex_wavenumber(gpu, orc, solved):
    ss, pos, lMax, f, k, rng = solved
    kc = k * (1 + 0.03j)
    pts = _points(pos, np.random.default_rng(7), 200)
    _close(ss.scattered_E(kc, f, pts), orc.scattered_E(lMax, pos, 3, kc, f, pts))


@pytest.mark.parametrize("lMax", [1, 2, 4, 6])
def test_field_lmax(gpu, orc, lMax):
    rng = np.random.default_rng(40 + lMax)
    pos = jittered_square_cluster(6, rng)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    f = rng.normal(size=ss.fecv_size) + 1j * rng.normal(size=ss.fecv_size)
    k = 1.7e7
    pts = _points(pos, rng, 150)[:150]
    _close(ss.scattered_E(k, f, pts), orc.scattered_E(lMax, pos, 3, k, f, pts))


def test_split_over_particles(gpu, orc):
    """Few points, many particles: the particle list is split over grid.y and
    the partial sums are reduced in a fixed order (deterministic)."""
    rng = np.random.default_rng(9)
    pos = jittered_square_cluster(400, rng)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, 2)
    f = rng.normal(size=ss.fecv_size) + 1j * rng.normal(size=ss.fecv_size)
    k = 1.7e7
    pts = rng.uniform(pos.min(0), pos.max(0), size=(5, 3)) + np.array([0, 0, 1e-7])
    E1 = ss.scattered_E(k, f, pts)
    E2 = ss.scattered_E(k, f, pts)
    assert np.array_equal(E1, E2)
    _close(E1, orc.scattered_E(2, pos, 3, k, f, pts))


def test_single_point_dropins(gpu, solved):
    from qpms_gb300.scatsystem import _Cart3
    ss, pos, lMax, f, k, rng = solved
    L = gpu.lib()
    w = np.array([1.3e-7, -2.1e-7, 0.9e-7])
    ref = ss.scattered_E(k, f, w[None, :])[0]
    fc = np.ascontiguousarray(f)
    for name in ("qpms_scatsys_scattered_E", "qpms_scatsys_scattered_E__alt"):
        r = getattr(L, name)(ss.s, 3, k.real, k.imag, fc.ctypes.data, _Cart3(*w))
        v = np.array(r.v[:]).view(np.complex128)
        assert np.array_equal(v, ref), name
    ssw = ss(2.2 * EV / HBAR)
    assert abs(ssw.wavenumber() - k) <= 1e-15 * abs(k)
    for name in ("qpms_scatsysw_scattered_E", "qpms_scatsysw_scattered_E__alt"):
        r = getattr(L, name)(ssw.ssw, 3, fc.ctypes.data, _Cart3(*w))
        v = np.array(r.v[:]).view(np.complex128)
        np.testing.assert_allclose(v, ref, rtol=1e-14, atol=0)
    np.testing.assert_allclose(ssw.scattered_E(f, w), ref, rtol=1e-14, atol=0)
    # shape handling as qpms_c.pyx: [..., 3] in, [..., 3] out
    grid = np.stack(np.meshgrid(np.linspace(-3e-7, 3e-7, 4), np.linspace(-3e-7, 3e-7, 5), [1e-7],
                                indexing="ij"), -1)
    assert ss.scattered_E(k, f, grid).shape == grid.shape
    assert ss.scattered_E(k, f, np.zeros((0, 3))).shape == (0, 3)


def test_device_entry(gpu, solved):
    import torch
    ss, pos, lMax, f, k, rng = solved
    pts = _points(pos, np.random.default_rng(11), 300)
    dev = torch.device("cuda:0")
    tf = torch.from_numpy(f).to(dev)
    tp = torch.from_numpy(np.ascontiguousarray(pts)).to(dev)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        E = ss.scattered_E_device(k, tf, tp, stream=s)
    s.synchronize()
    assert np.array_equal(E.cpu().numpy(), ss.scattered_E(k, f, pts))


def test_errors(gpu):
    from qpms_gb300 import QpmsGpuError
    from qpms_gb300.workloads import square_lattice
    b1, b2, p1 = square_lattice()
    lat = gpu.ScatteringSystem(p1, 80e-9, EPS_I, EPS_E, 2, lattice=(b1, b2))
    with pytest.raises(QpmsGpuError):
        lat.scattered_E(1.7e7, np.zeros(lat.fecv_size, complex), np.zeros((2, 3)))
    fin = gpu.ScatteringSystem(np.zeros((1, 3)), 50e-9, EPS_I, EPS_E, 2)
    with pytest.raises(QpmsGpuError):
        fin.scattered_E(1.7e7, np.zeros(fin.fecv_size, complex), np.ones((2, 3)), btyp=7)
    with pytest.raises(ValueError):
        fin.scattered_E(1.7e7, np.zeros(3, complex), np.ones((2, 3)))


def test_periodic_field_vs_oracle(gpu, orc):
    """Field of a 2D lattice at points in and off the particles' plane
    (qpms_scatsyswk_scattered_E; off-plane points use the shifted-layer sums):
    the lattice-summed translation W(point <- particle) applied to f, of which
    the regular electric dipole waves give the field at the point.  Oracle:
    the same blocks from its Ewald mode-problem builder with the point as an
    extra particle (T = -1), and its regular-wave field at r = 0."""
    from qpms_gb300 import QpmsGpuError
    from qpms_gb300.workloads import honeycomb_lattice
    lMax = 2
    b1, b2, pos = honeycomb_lattice()
    ss = gpu.ScatteringSystem(pos, 80e-9, EPS_I, EPS_E, lMax, lattice=(b1, b2))
    om = 2.1 * EV / HBAR
    k = np.sqrt(EPS_E) * om / C0
    kxy = (0.13 * np.pi / 580e-9, 0.05 * np.pi / 580e-9)
    kv = np.array([kxy[0], kxy[1], 0.0])
    rng = np.random.default_rng(17)
    f = rng.normal(size=ss.fecv_size) + 1j * rng.normal(size=ss.fecv_size)
    pts = np.zeros((16, 3))
    pts[:, :2] = rng.uniform(-700e-9, 700e-9, size=(16, 2))
    pts[12:, 2] = [150e-9, -90e-9, 400e-9, -1e-6]                 # off the particles' plane
    eta = orc.adjusted_eta(abs(b1[0] * b2[1] - b1[1] * b2[0]), k, kv, lMax)
    E = ss(om).scattered_E(f, pts, k=kxy, eta=eta)
    calc = orc.TransCalculator(lMax)
    n = 2 * lMax * (lMax + 2)
    for q, r in enumerate(pts):
        pa = np.vstack([pos, r])
        T = np.ascontiguousarray(np.broadcast_to(-np.eye(n), (3, n, n)), dtype=complex)
        X = orc.periodic_modeproblem(calc, pa, T, k, b1, b2, kv, eta)   # I + W
        a = sum(X[2 * n:3 * n, p * n:(p + 1) * n] @ f[p * n:(p + 1) * n] for p in range(2))
        ref = orc.scattered_E(lMax, r[None, :], 1, k, a, r[None, :])[0]
        assert np.linalg.norm(E[q] - ref) <= 1e-9 * np.linalg.norm(ref), (q, E[q], ref)
    # the errors
    with pytest.raises(QpmsGpuError):
        ss(om).scattered_E(f, pts[:1], k=kxy, btyp=1)                 # Hankel waves only
