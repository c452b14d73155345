"""The allocation-free translation entry point against the regular one.

qpms_gpu_trans_AB_arrays_batch_host_noalloc serves callers that cannot
allocate GPU (or pinned host) memory while they run -- processes whose device
memory belongs to a pool allocator or sits under a hard budget, real-time loops
that forbid allocation after start-up, plug-ins that must not grow their host
process.  It stages through a fixed device array instead of allocating, so it
must give the same A/B arrays as qpms_gpu_trans_AB_arrays_batch_host, call
after call (the array keeps the previous call's contents), must leave the
device's free memory unchanged, and must reject a batch that does not fit the
array.  This file runs last so that a failure here does not hide any other
test.
"""
import numpy as np
import pytest

from qpms_gb300.workloads import translation_vectors

pytestmark = pytest.mark.gpu

RTOL = 1e-11  # the translation tests' tolerance


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _call(L, f, c, n, kr, th, ph, rgd, J, ne):
    A = np.full((n, ne, ne), np.nan, dtype=np.complex128)
    B = np.full((n, ne, ne), np.nan, dtype=np.complex128)
    rc = f(c.c, n, kr.ctypes.data, th.ctypes.data, ph.ctypes.data, rgd.ctypes.data if rgd is not None else None,
           J, A.ctypes.data, B.ctypes.data)
    return rc, A, B


def _both(lib, c, n, seed, J, with_rgd):
    L = lib.lib()
    kr, th, ph = translation_vectors(n, seed=seed)
    rgd = np.zeros(n, dtype=np.uint8)
    rgd[::5] = 1
    out = []
    for f in (L.qpms_gpu_trans_AB_arrays_batch_host_noalloc, L.qpms_gpu_trans_AB_arrays_batch_host):
        rc, A, B = _call(L, f, c, n, kr, th, ph, rgd if with_rgd else None, J, c.nelem())
        assert rc == 0, lib.last_error()
        out.append((A, B))
    return out


def _close(G, O):
    G = G.reshape(G.shape[0], -1)
    O = O.reshape(O.shape[0], -1)
    assert np.all(np.isfinite(G))
    assert (np.linalg.norm(G - O, axis=1) <= RTOL * np.linalg.norm(O, axis=1)).all()


def test_noalloc_leaves_device_memory_unchanged(lib):
    import torch
    L = lib.lib()
    n = 600
    kr, th, ph = translation_vectors(n, seed=31)
    warm = lib.trans_calculator(3)
    # first call: loads the kernel and looks up the array's device address
    rc, _, _ = _call(L, L.qpms_gpu_trans_AB_arrays_batch_host_noalloc, warm, n, kr, th, ph, None, 3, warm.nelem())
    assert rc == 0, lib.last_error()
    c = lib.trans_calculator(3)  # its device tables are allocated here, before the measurement
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for seed, J in ((32, 3), (33, 1), (34, 3)):
        kr, th, ph = translation_vectors(n, seed=seed)
        rc, A, _ = _call(L, L.qpms_gpu_trans_AB_arrays_batch_host_noalloc, c, n, kr, th, ph, None, J, c.nelem())
        assert rc == 0, lib.last_error()
        assert np.all(np.isfinite(A))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_matches_regular_two_calls(lib):
    c3 = lib.trans_calculator(3)
    # two calls in a row: the second finds the first call's data in the array
    for seed, J, rgd in ((21, 3, False), (22, 1, True)):
        (a0, b0), (a1, b1) = _both(lib, c3, 700, seed, J, rgd)
        _close(a0, a1)
        _close(b0, b1)
    c6 = lib.trans_calculator(6)
    (a0, b0), (a1, b1) = _both(lib, c6, 300, 23, 3, False)
    _close(a0, a1)
    _close(b0, b1)


def test_noalloc_rejects_oversized_batch(lib):
    c = lib.trans_calculator(3)
    L = lib.lib()
    for n in (5000, 1 << 60):  # 5000 x 7.2 KB of output > 32 MiB; 2^60 would wrap a byte count
        m = min(n, 5000)
        kr, th, ph = translation_vectors(m, seed=3)
        A = np.empty((m, 15, 15), dtype=np.complex128)
        B = np.empty_like(A)
        before = L.qpms_gpu_kernel_launch_count()
        rc = L.qpms_gpu_trans_AB_arrays_batch_host_noalloc(c.c, n, kr.ctypes.data, th.ctypes.data, ph.ctypes.data,
                                                           None, 3, A.ctypes.data, B.ctypes.data)
        assert rc != 0
        assert "scratch" in lib.last_error()
        assert L.qpms_gpu_kernel_launch_count() == before


def test_wrong_device_is_rejected_before_any_launch(lib):
    """A calculator used while another device is current: both host entry
    points return an error and launch nothing (the mismatch is faked through
    the test hook, as this machine has one GPU)."""
    L = lib.lib()
    c = lib.trans_calculator(3)
    n = 16
    kr, th, ph = translation_vectors(n, seed=4)
    import torch
    home = torch.cuda.current_device()
    try:
        assert L.qpms_gpu_testing_set_calculator_device(c.c, 7) == 0
        for f in (L.qpms_gpu_trans_AB_arrays_batch_host_noalloc, L.qpms_gpu_trans_AB_arrays_batch_host):
            before = L.qpms_gpu_kernel_launch_count()
            rc, A, _ = _call(L, f, c, n, kr, th, ph, None, 3, c.nelem())
            assert rc != 0
            assert "device 7" in lib.last_error()
            assert L.qpms_gpu_kernel_launch_count() == before
            assert np.isnan(A).all()
    finally:
        L.qpms_gpu_testing_set_calculator_device(c.c, home)
    rc, A, _ = _call(L, L.qpms_gpu_trans_AB_arrays_batch_host_noalloc, c, n, kr, th, ph, None, 3, c.nelem())
    assert rc == 0 and np.isfinite(A).all()
