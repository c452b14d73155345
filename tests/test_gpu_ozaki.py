"""The dense solver's FP64 residual from bf16 digit products (qg_ozaki.cu).

* the cuBLAS bf16 GEMM with FP32 accumulation is exact for integer operands
  whose partial sums stay below 2^24 (the premise of the digit width), checked
  against int64 products at the bound;
* R = B - M X agrees with an extended-precision reference to the error bound
  of an FP64 GEMM (elementwise, relative to |M| |X|), for column- and
  row-major M, rows scaled over 16 decades, odd sizes;
* it agrees with the complex128 cuBLAS GEMM residual.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _digits(K):
    lk = int(np.ceil(np.log2(K))) if K > 1 else 0
    s = min(8, max(1, (24 - lk) // 2))
    return s


@pytest.mark.parametrize("k", [100, 4096, 14400])
def test_bf16_gemm_exact_at_the_bound(gpu, k):
    import torch
    s = _digits(k)
    rng = np.random.default_rng(k)
    m, n = 96, 40
    A = rng.integers(-2 ** (s - 1), 2 ** (s - 1) + 1, size=(m, k))
    B = rng.integers(-2 ** (s - 1), 2 ** (s - 1) + 1, size=(k, n))
    A[:4] = 2 ** s            # rows / columns at the largest first digit:
    B[:, :4] = 2 ** s         # partial sums up to k 2^(2s) <= 2^24
    A[4:8] = -2 ** s
    dev = torch.device("cuda:0")
    # column-major storage = the row-major transposes
    tA = torch.from_numpy(np.ascontiguousarray(A.T).astype(np.float32)).to(dev).to(torch.bfloat16)
    tB = torch.from_numpy(np.ascontiguousarray(B.T).astype(np.float32)).to(dev).to(torch.bfloat16)
    C = torch.empty((n, m), dtype=torch.float32, device=dev)
    assert gpu.lib().qpms_gpu_bf16_gemm(m, n, k, tA.data_ptr(), tB.data_ptr(), C.data_ptr()) == 0, \
        gpu.last_error()
    ref = A.astype(np.int64) @ B.astype(np.int64)
    assert np.abs(ref).max() <= 2 ** 24
    assert np.array_equal(C.cpu().numpy().T.astype(np.int64), ref)


def _resid(gpu, M, X, B, row_major):
    import torch
    N, nrhs = X.shape
    dev = torch.device("cuda:0")
    Mh = np.ascontiguousarray(M) if row_major else np.asfortranarray(M)
    tM = torch.from_numpy(Mh.reshape(-1, order="C" if row_major else "F").copy()).to(dev)
    tX = torch.from_numpy(np.asfortranarray(X).reshape(-1, order="F").copy()).to(dev)
    tB = torch.from_numpy(np.asfortranarray(B).reshape(-1, order="F").copy()).to(dev)
    tR = torch.empty_like(tB)
    rc = gpu.lib().qpms_gpu_ozaki_residual(N, nrhs, tM.data_ptr(), N, int(row_major), tX.data_ptr(),
                                           tB.data_ptr(), tR.data_ptr())
    assert rc == 0, gpu.last_error()
    return tR.cpu().numpy().reshape(nrhs, N).T


def _case(N, nrhs, decades, seed):
    rng = np.random.default_rng(seed)
    M = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    M *= 10.0 ** rng.uniform(-decades, decades, size=(N, 1))
    X = rng.normal(size=(N, nrhs)) + 1j * rng.normal(size=(N, nrhs))
    X[:, 0] *= 1e-5
    B = M @ X + 1e-6 * (np.abs(M) @ np.abs(X)) * (rng.normal(size=(N, nrhs)) + 1j * rng.normal(size=(N, nrhs)))
    return M, X, B


@pytest.mark.parametrize("N,nrhs,decades,row_major", [(64, 8, 0, False), (201, 9, 8, True), (201, 9, 8, False)])
def test_residual_vs_extended_precision(gpu, N, nrhs, decades, row_major):
    """Small sizes: against a long-double reference, within the bound of an
    FP64 GEMM (the digits keep 55 bits)."""
    M, X, B = _case(N, nrhs, decades, N + nrhs)
    R = _resid(gpu, M, X, B, row_major)
    ref = B.astype(np.clongdouble) - M.astype(np.clongdouble) @ X.astype(np.clongdouble)
    bound = np.abs(M) @ np.abs(X)
    err = (np.abs(R - ref) / bound).astype(np.float64)
    fp64 = (np.abs((B - M @ X) - ref) / bound).astype(np.float64)
    assert err.max() <= max(4 * fp64.max(), 2.0 ** -50), (err.max(), fp64.max())


@pytest.mark.parametrize("N,nrhs,decades,row_major", [(1000, 64, 8, False), (1000, 64, 8, True),
                                                       (2304, 64, 2, True), (4099, 16, 0, False)])
def test_residual_vs_fp64(gpu, N, nrhs, decades, row_major):
    """Larger sizes: within twice the worst-case FP64 GEMM error N u |M| |X|
    of numpy's complex128 product (both are that close to the exact one)."""
    M, X, B = _case(N, nrhs, decades, N + nrhs)
    R = _resid(gpu, M, X, B, row_major)
    bound = np.abs(M) @ np.abs(X)
    err = np.abs(R - (B - M @ X)) / bound
    assert err.max() <= 2 * N * 2.0 ** -53, err.max()


def test_dense_solve_many_rhs_uses_digits(gpu):
    """64 right-hand sides: the refinement (tensor-core residual) reaches the
    1e-13 residual and the complex128 solution."""
    import torch
    N, nrhs = 1500, 64
    rng = np.random.default_rng(2)
    M = (rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))) / np.sqrt(N) + 2 * np.eye(N)
    B = rng.normal(size=(N, nrhs)) + 1j * rng.normal(size=(N, nrhs))
    dev = torch.device("cuda:0")
    tM = torch.from_numpy(np.asfortranarray(M).reshape(-1, order="F").copy()).to(dev)
    tB = torch.from_numpy(np.asfortranarray(B).reshape(-1, order="F").copy()).to(dev)
    tX = torch.empty_like(tB)
    res = np.zeros(1)
    it = np.zeros(1, dtype=np.int32)
    assert gpu.lib().qpms_gpu_dense_solve(N, nrhs, tM.data_ptr(), tB.data_ptr(), tX.data_ptr(), 1,
                                          res.ctypes.data, it.ctypes.data) == 0, gpu.last_error()
    X = tX.cpu().numpy().reshape(nrhs, N).T
    assert res[0] <= 1e-13
    assert np.linalg.norm(X - np.linalg.solve(M, B)) <= 1e-11 * np.linalg.norm(X)
