"""The allocation-free translation entry point against the regular one.

qpms_gpu_trans_AB_arrays_batch_host_noalloc serves callers that cannot
allocate GPU (or pinned host) memory while they run -- processes whose device
memory belongs to a pool allocator or sits under a hard budget, real-time loops
that forbid allocation after start-up, plug-ins that must not grow their host
process.  It stages through a fixed device array instead of allocating, so it
must give the same A/B arrays as qpms_gpu_trans_AB_arrays_batch_host, call
after call (the array keeps the previous call's contents), and must reject a
batch that does not fit the array.  This file runs last so that a failure here
does not hide any other test.
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


def _both(lib, c, n, seed, J, with_rgd):
    L = lib.lib()
    kr, th, ph = translation_vectors(n, seed=seed)
    rgd = np.zeros(n, dtype=np.uint8)
    rgd[::5] = 1
    ne = c.nelem()
    out = []
    for f in (L.qpms_gpu_trans_AB_arrays_batch_host_noalloc, L.qpms_gpu_trans_AB_arrays_batch_host):
        A = np.full((n, ne, ne), np.nan, dtype=np.complex128)
        B = np.full((n, ne, ne), np.nan, dtype=np.complex128)
        rc = f(c.c, n, kr.ctypes.data, th.ctypes.data, ph.ctypes.data, rgd.ctypes.data if with_rgd else None,
               J, A.ctypes.data, B.ctypes.data)
        assert rc == 0, lib.last_error()
        out.append((A, B))
    return out


def _close(G, O):
    G = G.reshape(G.shape[0], -1)
    O = O.reshape(O.shape[0], -1)
    assert np.all(np.isfinite(G))
    assert (np.linalg.norm(G - O, axis=1) <= RTOL * np.linalg.norm(O, axis=1)).all()


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
    n = 5000  # 5000 x 7.2 KB of output > 32 MiB
    kr, th, ph = translation_vectors(n, seed=3)
    A = np.empty((n, 15, 15), dtype=np.complex128)
    B = np.empty_like(A)
    rc = lib.lib().qpms_gpu_trans_AB_arrays_batch_host_noalloc(c.c, n, kr.ctypes.data, th.ctypes.data,
                                                               ph.ctypes.data, None, 3, A.ctypes.data,
                                                               B.ctypes.data)
    assert rc != 0
    assert "scratch" in lib.last_error()
