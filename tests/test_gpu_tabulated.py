"""Tabulated data on the GPU: T(omega) batch evaluation, and scattering
systems whose particle kinds carry tabulated T-matrices or tabulated
permittivities, against the oracle (same interpolated T, the oracle's
M = I - T S and LAPACK-style solve).

Tolerances as for the other finite paths: mode-problem matrices 1e-10
(Frobenius), excitation coefficients and sigma_ext 1e-9.
"""
import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0

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


def square_array(nx, ny, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)], axis=1)


def _table(orc, lMax, radius, offdiag=0.0, seed=0):
    """T-matrices of a sphere (Mie) on a frequency grid, optionally with a
    fixed non-diagonal part (an arbitrary anisotropic particle)."""
    fr = np.linspace(1.5, 2.7, 41) * EV / HBAR
    n = 2 * lMax * (lMax + 2)
    rng = np.random.default_rng(seed)
    extra = offdiag * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    np.fill_diagonal(extra, 0)
    T = np.empty((fr.size, n, n), complex)
    for i, w in enumerate(fr):
        d = orc.tmatrix_sphere_diag(lMax, radius, w, EPS_I, EPS_E)
        T[i] = np.diag(d) + extra * np.abs(d).mean()
    return fr, T


def _oracle_T(orc, fr, T, w):
    n = T.shape[1]
    out = np.zeros((n, n), complex)
    for i in range(n):
        for j in range(n):
            if np.any(T[:, i, j].real):
                out[i, j] += orc.spline_eval(1, fr, T[:, i, j].real, [w])[0]
            if np.any(T[:, i, j].imag):
                out[i, j] += 1j * orc.spline_eval(1, fr, T[:, i, j].imag, [w])[0]
    return out


def _oracle_scatter(orc, lMax, pos, Tp, w):
    calc = orc.TransCalculator(lMax)
    k = np.sqrt(EPS_E) * w / C0
    M = orc.finite_modeproblem(calc, pos, Tp, k)
    a = orc.planewave_full(lMax, pos, np.array([0, 0, k]), np.array([1, 0, 0], dtype=complex))
    n = Tp.shape[1]
    rhs = (Tp @ a.reshape(pos.shape[0], n, 1)).reshape(-1)
    f = np.linalg.solve(M, rhs)
    return M, f, -np.real(np.vdot(a, f)) / k ** 2


def test_device_batch_matches_host(gpu, orc):
    import torch
    from qpms_gb300.tmatrices import TMatrixInterpolator
    fr, T = _table(orc, 2, 60e-9, offdiag=0.1)
    ti = TMatrixInterpolator.from_arrays(fr, T, 2)
    q = np.random.default_rng(1).uniform(fr[0], fr[-1], 50)
    q[:3] = fr[[0, 7, -1]]
    D = ti.eval_batch_device(torch.from_numpy(q).cuda()).cpu().numpy()
    for i, w in enumerate(q):
        H = ti(w)
        assert np.abs(D[i] - H).max() <= 1e-14 * np.abs(H).max()
        if i < 4:
            O = _oracle_T(orc, fr, T, w)
            assert np.abs(H - O).max() <= 1e-12 * np.abs(O).max()


@pytest.mark.parametrize("mode", [0, 1])
def test_tabulated_kind_scatter_vs_oracle(gpu, orc, mode):
    from qpms_gb300.tmatrices import TMatrixInterpolator
    lMax = 2
    fr, T = _table(orc, lMax, 50e-9)
    ti = TMatrixInterpolator.from_arrays(fr, T, lMax)
    pos = square_array(3, 3, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, [ti], EPS_E, lMax)
    om = np.array([1.73, 2.11, 2.49]) * EV / HBAR  # between the knots
    out = ss.planewave_scatter_batch(om, mode=mode, want_f=True)
    sph = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax).planewave_scatter_batch(om, mode=mode)
    for i, w in enumerate(om):
        Tw = _oracle_T(orc, fr, T, w)
        _, f, sig = _oracle_scatter(orc, lMax, pos, np.stack([Tw] * pos.shape[0]), w)
        assert out["residual"][i] <= 1e-12
        assert np.linalg.norm(out["f"][i] - f) <= 1e-9 * np.linalg.norm(f)
        assert abs(out["sigma_ext"][i] - sig) <= 1e-9 * abs(sig)
        # the table samples the Mie T-matrix: close to the sphere system
        assert abs(out["sigma_ext"][i] - sph["sigma_ext"][i]) <= 1e-4 * abs(sig)


def test_mixed_kinds_nondiagonal_vs_oracle(gpu, orc):
    """A sphere kind and an anisotropic tabulated kind in one system: the
    matrix M = I - T S (reference-layout path) and the batched scatter."""
    from qpms_gb300.tmatrices import TMatrixInterpolator
    lMax = 2
    fr, T = _table(orc, lMax, 60e-9, offdiag=0.05, seed=3)
    ti = TMatrixInterpolator.from_arrays(fr, T, lMax)
    pos = square_array(4, 2, 400e-9)
    kinds = np.array([0, 1, 0, 1, 1, 0, 1, 0], dtype=np.int32)
    ss = gpu.ScatteringSystem(pos, 50e-9, [EPS_I, ti], EPS_E, lMax, kinds=kinds)
    w = 2.2 * EV / HBAR
    Tw = _oracle_T(orc, fr, T, w)
    Ts = np.diag(orc.tmatrix_sphere_diag(lMax, 50e-9, w, EPS_I, EPS_E))
    Tp = np.stack([Ts if k == 0 else Tw for k in kinds])
    Mo, f, sig = _oracle_scatter(orc, lMax, pos, Tp, w)
    M = ss(w).modeproblem_matrix_full()
    assert np.linalg.norm(M - Mo) <= 1e-10 * np.linalg.norm(Mo)
    for mode in (0, 1):
        out = ss.planewave_scatter_batch(np.array([w]), mode=mode, want_f=True)
        assert np.linalg.norm(out["f"][0] - f) <= 1e-9 * np.linalg.norm(f)
        assert abs(out["sigma_ext"][0] - sig) <= 1e-9 * abs(sig)


def test_large_tabulated_dense_path(gpu, orc):
    """768 unknowns (> 512): the per-frequency dense-solver path with dense T."""
    from qpms_gb300.tmatrices import TMatrixInterpolator
    lMax = 4
    fr, T = _table(orc, lMax, 50e-9, offdiag=0.02, seed=5)
    ti = TMatrixInterpolator.from_arrays(fr, T, lMax)
    pos = square_array(4, 4, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, [ti], EPS_E, lMax)
    assert ss.fecv_size == 768
    w = 2.05 * EV / HBAR
    out = ss.planewave_scatter_batch(np.array([w]), mode=1, want_f=True, want_scat=True)
    Tw = _oracle_T(orc, fr, T, w)
    _, f, sig = _oracle_scatter(orc, lMax, pos, np.stack([Tw] * 16), w)
    assert out["residual"][0] <= 1e-12
    assert np.linalg.norm(out["f"][0] - f) <= 1e-9 * np.linalg.norm(f)
    assert abs(out["sigma_ext"][0] - sig) <= 1e-9 * abs(sig)


def test_interpolated_permittivity_sphere(gpu, orc):
    """Spheres of a tabulated material equal spheres of the interpolated
    permittivity at that frequency."""
    from qpms_gb300.materials import MaterialInterpolator
    wl = np.linspace(400e-9, 900e-9, 30)
    nn = 0.15 + 0.2 * (wl - 400e-9) / 500e-9
    kk = 2.2 + 3.0 * (wl - 400e-9) / 500e-9
    mi = MaterialInterpolator.from_arrays(wl, nn, kk)
    pos = square_array(3, 3, 400e-9)
    lMax = 2
    ss = gpu.ScatteringSystem(pos, 50e-9, [mi], EPS_E, lMax)
    for E in (1.7, 2.3):
        w = E * EV / HBAR
        eps = mi(w)
        lam = 2 * np.pi * C0 / w
        ref_eps = (orc.spline_eval(1, wl, nn, [lam])[0] + 1j * orc.spline_eval(1, wl, kk, [lam])[0]) ** 2
        assert abs(eps - ref_eps) <= 1e-12 * abs(ref_eps)
        a = ss.planewave_scatter_batch(np.array([w]), mode=1, want_f=True)
        b = gpu.ScatteringSystem(pos, 50e-9, eps, EPS_E, lMax).planewave_scatter_batch(np.array([w]), mode=1,
                                                                                       want_f=True)
        assert np.linalg.norm(a["f"][0] - b["f"][0]) <= 1e-12 * np.linalg.norm(b["f"][0])


def test_server_and_errors(gpu, orc):
    from qpms_gb300 import QpmsGpuError
    from qpms_gb300.serving import Server
    from qpms_gb300.tmatrices import TMatrixInterpolator
    lMax = 2
    fr, T = _table(orc, lMax, 50e-9, offdiag=0.05, seed=7)
    ti = TMatrixInterpolator.from_arrays(fr, T, lMax)
    pos = square_array(3, 3, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, [ti], EPS_E, lMax)
    w = 2.3 * EV / HBAR
    ref = ss.planewave_scatter_batch(np.array([w]), mode=1, want_f=True)["f"][0]
    srv = Server(mode=1, workers=2)
    r = srv.wait(srv.submit(ss, w))
    srv.close()
    assert r["status"] == 0
    assert np.linalg.norm(r["f"] - ref) <= 1e-9 * np.linalg.norm(ref)
    with pytest.raises(QpmsGpuError):  # basis of another lMax
        gpu.ScatteringSystem(pos, 50e-9, [ti], EPS_E, 3)


def _lattice_oracle(orc, lMax, pos, Tp, w, b1, b2, kxy):
    """Oracle M = I - T W(k) and the plane-wave solve with the incidence of
    the library's lattice paths (in-plane wavevector k, E = x projected
    perpendicular to the propagation direction)."""
    calc = orc.TransCalculator(lMax)
    k = np.sqrt(EPS_E) * w / C0
    kv = np.array([kxy[0], kxy[1], 0.0])
    eta = orc.adjusted_eta(abs(b1[0] * b2[1] - b1[1] * b2[0]), k, kv, lMax)
    M = orc.periodic_modeproblem(calc, pos, Tp, k, b1, b2, kv, eta)
    kd = np.array([kv[0], kv[1], np.sqrt(k.real ** 2 - kv[0] ** 2 - kv[1] ** 2)])
    E = np.array([1.0, 0, 0]) - kd[0] * kd / (kd @ kd)
    a = orc.planewave_full(lMax, pos, kd, E / np.linalg.norm(E))
    n = Tp.shape[1]
    rhs = (Tp @ a.reshape(pos.shape[0], n, 1)).reshape(-1)
    return M, np.linalg.solve(M, rhs)


def test_tabulated_kinds_in_a_lattice(gpu, orc):
    """Dense T in the lattice sums: X = I + W from the Ewald kernel with T = -1,
    then M = I + T - T X by a batched GEMM; the matrix (reference-layout
    path), the dispersion scan and a serving request against the oracle."""
    from qpms_gb300.serving import Server
    from qpms_gb300.tmatrices import TMatrixInterpolator
    from qpms_gb300.workloads import honeycomb_lattice
    lMax = 2
    fr, T = _table(orc, lMax, 80e-9, offdiag=0.05, seed=11)
    ti = TMatrixInterpolator.from_arrays(fr, T, lMax)
    b1, b2, pos = honeycomb_lattice()
    ss = gpu.ScatteringSystem(pos, 80e-9, [EPS_I, ti], EPS_E, lMax, kinds=[0, 1], lattice=(b1, b2))
    w = 2.15 * EV / HBAR
    kxy = (0.11 * np.pi / 580e-9, -0.07 * np.pi / 580e-9)
    Tw = _oracle_T(orc, fr, T, w)
    Ts = np.diag(orc.tmatrix_sphere_diag(lMax, 80e-9, w, EPS_I, EPS_E))
    Tp = np.stack([Ts, Tw])
    Mo, fo = _lattice_oracle(orc, lMax, pos, Tp, w, b1, b2, kxy)
    M = ss(w).modeproblem_matrix_full(k=kxy)
    assert np.linalg.norm(M - Mo) <= 1e-10 * np.linalg.norm(Mo)
    for mode in (0, 1):
        r = ss.dispersion_scan(np.array([w]), np.array([kxy]), want_f=True, mode=mode)
        assert r["residual"][0, 0] <= 1e-12
        assert np.linalg.norm(r["f"][0, 0] - fo) <= 1e-9 * np.linalg.norm(fo)
    srv = Server(mode=1, workers=2)
    res = srv.wait(srv.submit(ss, w, kxy))
    srv.close()
    assert res["status"] == 0
    assert np.linalg.norm(res["f"] - fo) <= 1e-9 * np.linalg.norm(fo)
