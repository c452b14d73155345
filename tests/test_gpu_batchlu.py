"""The library's batched LU with partial pivoting (qg_batchlu.cu) through the
reference's drop-in LU entry point, qpms_scatsysw_build_modeproblem_matrix_full_LU
(scatsystem.c:2202-2244): the factors and LAPACK's 1-based pivots must be those
of LAPACK's zgetrf on the same row-major matrix (scipy.linalg.lu_factor), and
qpms_scatsys_scatter_solve must solve with them.

Tolerances: identical pivot sequence; factors within 1e-12 of LAPACK's
(Frobenius, relative); solution within 1e-10 of numpy.linalg.solve.
"""
import ctypes as C

import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _square(nx, ny, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)


@pytest.mark.parametrize("nx,ny,lMax,omega_eV", [(4, 4, 2, 1.9), (3, 3, 3, 2.3 + 0.01j), (2, 1, 1, 2.0),
                                                 (4, 4, 3, 2.1), (8, 4, 2, 1.7)])
def test_dropin_lu_matches_lapack(gpu, nx, ny, lMax, omega_eV):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    ss = gpu.ScatteringSystem(_square(nx, ny, 400e-9), 50e-9, -12 + 1.2j, 2.25, lMax)
    ssw = ss(omega_eV * EV / HBAR)
    M = ssw.modeproblem_matrix_full()
    N = M.shape[0]
    sm = ssw.scatter_solver()
    lu = np.ctypeslib.as_array(C.cast(sm.lu.a, C.POINTER(C.c_double)), shape=(N * N * 2,)).copy()
    lu = lu.view(np.complex128).reshape(N, N)
    ipiv = np.ctypeslib.as_array(C.cast(sm.lu.ipiv, C.POINTER(C.c_int)), shape=(N,)).copy()
    ref_lu, ref_piv = scipy_linalg.lu_factor(M)
    assert np.array_equal(ipiv, ref_piv + 1)
    assert np.linalg.norm(lu - ref_lu) <= 1e-12 * np.linalg.norm(ref_lu)
    rng = np.random.default_rng(N)
    b = rng.normal(size=N) + 1j * rng.normal(size=N)
    x = sm(b)
    xr = np.linalg.solve(M, b)
    assert np.linalg.norm(x - xr) <= 1e-10 * np.linalg.norm(xr)
