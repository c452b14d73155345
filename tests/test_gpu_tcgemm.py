"""Tensor-core GEMMs (tcgen05, TMA) against complex128 / exact references.

qpms_gpu_tc_cgemm is the building block of the mixed-precision LU that stands
in for the reference's LAPACKE_zgetrf / zgetrs (scatsystem.c:2202-2273,
beyn.c:552-564): complex64 operands cut into nsplit bf16 digits, digit
products accumulated in FP32.  Tolerances (Frobenius-relative, random
Gaussian operands): 1 digit 1e-2, 2 digits 5e-5, 3 digits 2e-6.
qpms_gpu_tc_gemm_bf16 carries the digit products of the FP64 residual and
must be exact on integer digits whose products sum below 2^24.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {1: 1e-2, 2: 5e-5, 3: 2e-6}


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    L = qpms_gb300.lib()
    vp, sz, ci, cf = C.c_void_p, C.c_size_t, C.c_int, C.c_float
    L.qpms_gpu_tc_cgemm.restype = ci
    L.qpms_gpu_tc_cgemm.argtypes = [ci, ci, ci, vp, sz, vp, sz, cf, cf, vp, sz, vp, sz, ci, vp]
    L.qpms_gpu_tc_gemm_bf16.restype = ci
    L.qpms_gpu_tc_gemm_bf16.argtypes = [ci, ci, ci, vp, sz, vp, sz, cf, cf, vp, sz, vp, sz, vp]
    L.qpms_gpu_tc_check_error.restype = ci
    L.qpms_gpu_tc_check_error.argtypes = [vp]
    return torch, qpms_gb300, L


def _cgemm(env, m, n, k, nsplit, alpha=1.0, beta=0.0, lda_pad=0, inplace=False, seed=0):
    torch, q, L = env
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    lda, ldb, ldc = m + lda_pad, k + lda_pad, m + lda_pad
    A = torch.randn(k, lda, dtype=torch.complex64, device=dev, generator=g)  # column-major storage: [col][row]
    B = torch.randn(n, ldb, dtype=torch.complex64, device=dev, generator=g)
    Cm = torch.randn(n, ldc, dtype=torch.complex64, device=dev, generator=g)
    D = Cm if inplace else torch.full((n, ldc), float("nan"), dtype=torch.complex64, device=dev)
    ref = alpha * (A[:, :m].T.to(torch.complex128) @ B[:, :k].T.to(torch.complex128))
    if beta != 0:
        ref = ref + beta * Cm[:, :m].T.to(torch.complex128)
    st = torch.cuda.current_stream().cuda_stream
    rc = L.qpms_gpu_tc_cgemm(m, n, k, A.data_ptr(), lda, B.data_ptr(), ldb, alpha, beta, Cm.data_ptr(), ldc,
                             D.data_ptr(), ldc, nsplit, st)
    assert rc == 0, q.last_error()
    assert L.qpms_gpu_tc_check_error(st) == 0, q.last_error()
    got = D[:, :m].T.to(torch.complex128)
    err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
    return err, D, ldc


@pytest.mark.parametrize("nsplit", [1, 2, 3])
@pytest.mark.parametrize("m,n,k", [(64, 64, 64), (200, 130, 96), (37, 5, 12), (300, 257, 128), (128, 64, 300)])
def test_cgemm_vs_complex128(env, m, n, k, nsplit):
    err, _, _ = _cgemm(env, m, n, k, nsplit, seed=m + n + k)
    assert err < TOL[nsplit], err


def test_cgemm_update_in_place_padded(env):
    """C -= A B in place with leading dimensions above the sizes (the LU's
    trailing update); the padding rows stay untouched."""
    torch = env[0]
    err, D, ld = _cgemm(env, 500, 450, 128, 2, alpha=-1.0, beta=1.0, lda_pad=12, inplace=True, seed=7)
    assert err < TOL[2], err
    assert torch.isfinite(D).all()


def test_cgemm_large_update(env):
    """A trailing update of the size the 14,400-unknown LU starts with."""
    err, _, _ = _cgemm(env, 2048, 1800, 128, 2, alpha=-1.0, beta=1.0, inplace=True, seed=3)
    assert err < TOL[2], err


def test_bf16_gemm_exact_on_integers(env):
    torch, q, L = env
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    m, n, k = 333, 190, 1024
    # 5-bit signed digits: |sum| <= 1024 * 15 * 15 < 2^24
    A = torch.randint(-15, 16, (m, k), device=dev, generator=g).to(torch.bfloat16)
    B = torch.randint(-15, 16, (n, k), device=dev, generator=g).to(torch.bfloat16)
    D = torch.empty((n, m), dtype=torch.float32, device=dev)  # column-major m x n
    st = torch.cuda.current_stream().cuda_stream
    rc = L.qpms_gpu_tc_gemm_bf16(m, n, k, A.data_ptr(), k, B.data_ptr(), k, 1.0, 0.0, None, m, D.data_ptr(), m, st)
    assert rc == 0, q.last_error()
    assert L.qpms_gpu_tc_check_error(st) == 0, q.last_error()
    ref = A.cpu().to(torch.int64) @ B.cpu().to(torch.int64).T
    assert torch.equal(D.T.cpu().to(torch.int64), ref)
