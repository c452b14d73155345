"""GPU dense solver (random butterfly + blocked LU without pivoting) against numpy.

Tolerances: solution within 1e-10 relative (2-norm) of numpy.linalg.solve on
well-conditioned systems and mode-problem matrices; FP64 residual
||B - M X|| / ||B|| <= 1e-12 in both modes (the mixed mode reaches it by FP64
iterative refinement).
"""
import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _solve(torch, M, B, mode):
    import ctypes as C
    import qpms_gb300
    dev = torch.device("cuda:0")
    tM = torch.from_numpy(np.asfortranarray(M).reshape(-1, order="F")).to(dev)   # column-major
    tB = torch.from_numpy(np.asfortranarray(B).reshape(-1, order="F")).to(dev)
    tX = torch.empty_like(tB)
    res = np.zeros(1)
    it = np.zeros(1, dtype=np.int32)
    N, nrhs = B.shape
    rc = qpms_gb300.lib().qpms_gpu_dense_solve(N, nrhs, tM.data_ptr(), tB.data_ptr(), tX.data_ptr(), mode,
                                               res.ctypes.data, it.ctypes.data)
    assert rc == 0, qpms_gb300.last_error()
    X = tX.cpu().numpy().reshape((N, nrhs), order="F")
    return X, res[0], it[0]


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("N", [37, 256, 300, 1000])
def test_random_system(torch_cuda, mode, N):
    rng = np.random.default_rng(N)
    M = (rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))) / np.sqrt(N) + 2 * np.eye(N)
    B = rng.normal(size=(N, 8)) + 1j * rng.normal(size=(N, 8))
    X, res, it = _solve(torch_cuda, M, B, mode)
    ref = np.linalg.solve(M, B)
    assert np.linalg.norm(X - ref) <= 1e-10 * np.linalg.norm(ref)
    assert res <= 1e-12


@pytest.mark.parametrize("mode", [0, 1])
def test_modeproblem_system(torch_cuda, orc, mode):
    """M = I - T S of a 6 x 6 sphere array (lMax 2, N = 576) at a complex frequency."""
    lMax = 2
    xs = (np.arange(6) - 2.5) * 400e-9
    X_, Y_ = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X_.ravel(), Y_.ravel(), np.zeros(36)], 1)
    om = (2.1 + 0.003j) * EV / HBAR
    c = orc.TransCalculator(lMax)
    Td = orc.tmatrix_sphere_diag(lMax, 60e-9, om, -12 + 1.2j, 2.25)
    T = np.stack([np.diag(Td)] * 36)
    M = orc.finite_modeproblem(c, pos, T, np.sqrt(2.25) * om / C0)
    rng = np.random.default_rng(3)
    B = rng.normal(size=(M.shape[0], 16)) + 1j * rng.normal(size=(M.shape[0], 16))
    X, res, it = _solve(torch_cuda, M, B, mode)
    ref = np.linalg.solve(M, B)
    assert np.linalg.norm(X - ref) <= 1e-10 * np.linalg.norm(ref)
    assert res <= 1e-12, res


@pytest.mark.parametrize("cond", [1e2, 1e5])
def test_single_rhs_refinement(torch_cuda, cond):
    """One right-hand side: complex64 factors with TF32 trailing updates, FP64
    refinement to 1e-13 (falling back to FP32 factors if it stalls), on a
    matrix of prescribed condition number."""
    N = 768
    rng = np.random.default_rng(int(cond))
    Q1, _ = np.linalg.qr(rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)))
    Q2, _ = np.linalg.qr(rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)))
    M = (Q1 * np.logspace(0, -np.log10(cond), N)) @ Q2
    B = rng.normal(size=(N, 1)) + 1j * rng.normal(size=(N, 1))
    X, res, it = _solve(torch_cuda, M, B, 1)
    ref = np.linalg.solve(M, B)
    # FP64 attains a relative residual of about eps * cond at best
    assert res <= max(1e-12, 1e-16 * cond * 100), (res, it)
    assert np.linalg.norm(X - ref) <= cond * 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("nrhs", [1, 3, 8])
def test_one_application_of_the_sweeps(torch_cuda, nrhs):
    """Refinement capped at zero steps, complex128 factors: one application of
    the factors through the one-launch substitution sweeps must already give
    the solution to FP64 accuracy.  A tile that read a block of the right-hand
    side before the tiles writing it had finished would show here (refinement
    would hide it).  4,100 unknowns: 65 blocks of 64, the last one 4 rows wide;
    three right-hand-side sets against one matrix."""
    import scipy.linalg as sla
    import qpms_gb300
    N = 4100
    rng = np.random.default_rng(41 + nrhs)
    M = (rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))) / np.sqrt(N) + 2 * np.eye(N)
    lu = sla.lu_factor(M)
    L = qpms_gb300.lib()
    L.qpms_gpu_testing_set_max_refine(0)
    try:
        for rep in range(3):
            B = rng.normal(size=(N, nrhs)) + 1j * rng.normal(size=(N, nrhs))
            X, res, it = _solve(torch_cuda, M, B, 0)
            ref = sla.lu_solve(lu, B)
            assert it == 1
            assert np.linalg.norm(X - ref) <= 1e-11 * np.linalg.norm(ref), rep
    finally:
        L.qpms_gpu_testing_set_max_refine(-1)


_PLANES_CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import qpms_gb300
N, nrhs = 1500, 24
rng = np.random.default_rng(7)
M = (rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))) / np.sqrt(N) + 2 * np.eye(N)
B = rng.normal(size=(N, nrhs)) + 1j * rng.normal(size=(N, nrhs))
dev = torch.device("cuda:0")
tM = torch.from_numpy(np.asfortranarray(M).reshape(-1, order="F")).to(dev)
tB = torch.from_numpy(np.asfortranarray(B).reshape(-1, order="F")).to(dev)
tX = torch.empty_like(tB)
res, it = np.zeros(1), np.zeros(1, dtype=np.int32)
rc = qpms_gb300.lib().qpms_gpu_dense_solve(N, nrhs, tM.data_ptr(), tB.data_ptr(), tX.data_ptr(), 1,
                                           res.ctypes.data, it.ctypes.data)
assert rc == 0, qpms_gb300.last_error()
np.save(sys.argv[2], tX.cpu().numpy())
"""


def test_factor_planes_match_per_step_splits(torch_cuda, tmp_path):
    """Many right-hand sides: the substitutions reading the factors' digit
    planes cut once per factorisation give bit-for-bit the result of cutting
    each step's panel (the same elementwise digits, the same products), in a
    child process with the cached planes off (QPMS_GB300_FACTOR_PLANES=0)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for flag in ("1", "0"):
        env = dict(os.environ, QPMS_GB300_FACTOR_PLANES=flag)
        f = str(tmp_path / ("x%s.npy" % flag))
        subprocess.run([sys.executable, "-c", _PLANES_CHILD, root, f], env=env, check=True, timeout=600)
        out[flag] = np.load(f)
    assert np.array_equal(out["1"], out["0"])
