"""GPU parity of the finite mode-problem path against the oracle, through the C-ABI.

Tolerances (from the path's specification):
  mode-problem matrices M = I - T S   1e-10 Frobenius-relative (and element-wise
                                      1e-10 |o| + 1e-12 max|O|)
  translation matrices S              same
  excitation coefficients f           1e-9 relative (2-norm)
  sigma_ext                           1e-9 relative
  solve residual ||M f - T a||/||T a|| <= 1e-10 in both the FP64 and the mixed mode
"""
import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0

pytestmark = pytest.mark.gpu

EPS_I = -12 + 1.2j
EPS_E = 2.25


def square_array(nx, ny, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)], axis=1)


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _mat_close(G, O, rtol=1e-10, atol_rel=1e-12):
    fro = np.linalg.norm(G - O) / np.linalg.norm(O)
    assert fro <= rtol, fro
    bound = rtol * np.abs(O) + atol_rel * np.abs(O).max()
    assert (np.abs(G - O) <= bound).all(), (np.abs(G - O) / bound).max()


@pytest.mark.parametrize("lMax", [1, 2, 3])
def test_modeproblem_matrix_vs_oracle(gpu, orc, lMax):
    pos = square_array(4, 4, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    om = 2.1 * EV / HBAR
    M = ss(om).modeproblem_matrix_full()
    c = orc.TransCalculator(lMax)
    Td = orc.tmatrix_sphere_diag(lMax, 50e-9, om, EPS_I, EPS_E)
    T = np.stack([np.diag(Td)] * len(pos))
    ke = np.sqrt(EPS_E) * om / C0
    O = orc.finite_modeproblem(c, pos, T, ke)
    _mat_close(M, O)


@pytest.mark.parametrize("J", [1, 3])
def test_translation_matrix_vs_oracle(gpu, orc, J):
    pos = square_array(3, 2, 400e-9) + np.array([0, 0, 30e-9]) * np.arange(6)[:, None]
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, 2)
    k = 1.7e7 + 2e4j
    S = ss.translation_matrix_full(k, J)
    O = orc.finite_translation_matrix(orc.TransCalculator(2), pos, k, J)
    _mat_close(S, O)


def test_planewave_and_solve_vs_oracle(gpu, orc):
    lMax = 2
    pos = square_array(4, 4, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    om = 1.9 * EV / HBAR
    ke = np.sqrt(EPS_E) * om / C0
    a = ss.planewave_full([0, 0, ke], [1, 0, 0])
    oa = orc.planewave_full(lMax, pos, [0, 0, ke], [1, 0, 0])
    assert np.linalg.norm(a - oa) <= 1e-12 * np.linalg.norm(oa)
    # oblique incidence, other polarisation
    kc = ke * np.array([np.sin(0.4) * np.cos(0.3), np.sin(0.4) * np.sin(0.3), np.cos(0.4)])
    a2 = ss.planewave_full(kc, [0, 1, 0.2j])
    oa2 = orc.planewave_full(lMax, pos, kc, [0, 1, 0.2j])
    assert np.linalg.norm(a2 - oa2) <= 1e-12 * np.linalg.norm(oa2)
    ssw = ss(om)
    Ta = ssw.apply_Tmatrices_full(a)
    f = ssw.scatter_solver()(Ta)
    of, oainc, osig = orc.finite_sphere_scatter(orc.TransCalculator(lMax), pos, 50e-9, EPS_I, EPS_E, om)
    assert np.linalg.norm(f - of) <= 1e-9 * np.linalg.norm(of)
    sig = -np.vdot(a, f).real / ke ** 2
    assert abs(sig - osig) <= 1e-9 * abs(osig)


@pytest.mark.parametrize("mode", [0, 1])
def test_config1_batch_vs_oracle(gpu, orc, mode):
    """4x4 array, pitch 400 nm, r = 50 nm, lMax 2 (256 x 256), 32 frequencies 1.6-2.6 eV."""
    lMax = 2
    pos = square_array(4, 4, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    E = np.linspace(1.6, 2.6, 32)
    om = E * EV / HBAR
    out = ss.planewave_scatter_batch(om, mode=mode, want_f=True)
    assert (out["residual"] <= 1e-10).all(), out["residual"].max()
    c = orc.TransCalculator(lMax)
    for i in range(0, 32, 5):
        of, oa, osig = orc.finite_sphere_scatter(c, pos, 50e-9, EPS_I, EPS_E, om[i])
        assert abs(out["sigma_ext"][i] - osig) <= 1e-9 * abs(osig), (i, out["sigma_ext"][i], osig)
        assert np.linalg.norm(out["f"][i] - of) <= 1e-9 * np.linalg.norm(of)


def test_energy_conservation_gpu(gpu):
    lMax = 2
    pos = square_array(3, 3, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, 4.0, EPS_E, lMax)
    om = np.array([1.8, 2.4]) * EV / HBAR
    out = ss.planewave_scatter_batch(om, mode=1, want_f=True)
    for i, w in enumerate(om):
        ke = np.sqrt(EPS_E) * w / C0
        S1 = ss.translation_matrix_full(ke, 1)
        f = out["f"][i]
        sscat = np.vdot(f, (S1 + np.eye(len(f))) @ f).real / ke ** 2
        assert abs(out["sigma_ext"][i] - sscat) <= 1e-9 * abs(sscat)


@pytest.mark.parametrize("eps_in", [4.0, EPS_I])
def test_sigma_scat_vs_oracle(gpu, orc, eps_in):
    """sigma_scat = Re(f^H (I + R) f) / k^2 (misc/finiterectlat-scatter.py:98-111)
    from the library against the oracle's regular translation matrix and f;
    lossless spheres conserve energy (sigma_ext = sigma_scat), lossy ones absorb."""
    lMax = 2
    pos = square_array(3, 3, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, eps_in, EPS_E, lMax)
    om = np.array([1.7, 2.1, 2.5]) * EV / HBAR
    out = ss.planewave_scatter_batch(om, mode=1, want_scat=True)
    c = orc.TransCalculator(lMax)
    for i, w in enumerate(om):
        ke = np.sqrt(EPS_E) * w / C0
        f, _, sig = orc.finite_sphere_scatter(c, pos, 50e-9, eps_in, EPS_E, w)
        R = orc.finite_translation_matrix(c, pos, ke, 1)
        ref = np.vdot(f, (R + np.eye(len(f))) @ f).real / ke ** 2
        assert abs(out["sigma_scat"][i] - ref) <= 1e-9 * abs(ref)
        if np.imag(eps_in) == 0:
            assert abs(out["sigma_ext"][i] - out["sigma_scat"][i]) <= 1e-9 * abs(ref)
        else:
            assert out["sigma_abs"][i] > 0


def test_lorentz_drude_spheres_vs_oracle(gpu, orc):
    """Gold spheres (Lorentz-Drude model, the permittivity following omega):
    the batched scatter against the oracle at eps(omega) evaluated by the model."""
    from qpms_gb300.materials import lorentz_drude
    au = lorentz_drude["Au"]
    lMax = 2
    pos = square_array(3, 3, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, au, EPS_E, lMax)
    om = np.array([1.7, 2.1, 2.5]) * EV / HBAR
    out = ss.planewave_scatter_batch(om, mode=1, want_f=True)
    c = orc.TransCalculator(lMax)
    for i, w in enumerate(om):
        f, _, sig = orc.finite_sphere_scatter(c, pos, 50e-9, au(w), EPS_E, w)
        assert np.linalg.norm(out["f"][i] - f) <= 1e-9 * np.linalg.norm(f)
        assert abs(out["sigma_ext"][i] - sig) <= 1e-9 * abs(sig)


@pytest.mark.parametrize("mode", [0, 1])
def test_large_system_dense_path_vs_oracle(gpu, orc, mode):
    """N = 768 > 512: each frequency runs through the dense solver (random
    butterfly + LU without pivoting, FP64 refinement) instead of the batched
    LU; f, sigma_ext and sigma_scat against the oracle's LAPACK-style solve."""
    lMax = 4
    pos = square_array(4, 4, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    assert ss.fecv_size == 768
    om = np.array([1.8, 2.3]) * EV / HBAR
    out = ss.planewave_scatter_batch(om, mode=mode, want_f=True, want_scat=True)
    c = orc.TransCalculator(lMax)
    for i, w in enumerate(om):
        ke = np.sqrt(EPS_E) * w / C0
        f, _, sig = orc.finite_sphere_scatter(c, pos, 50e-9, EPS_I, EPS_E, w)
        assert out["residual"][i] <= 1e-12
        assert np.linalg.norm(out["f"][i] - f) <= 1e-9 * np.linalg.norm(f)
        assert abs(out["sigma_ext"][i] - sig) <= 1e-9 * abs(sig)
        R = orc.finite_translation_matrix(c, pos, ke, 1)
        ref = np.vdot(f, (R + np.eye(len(f))) @ f).real / ke ** 2
        assert abs(out["sigma_scat"][i] - ref) <= 1e-9 * abs(ref)
