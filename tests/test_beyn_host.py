"""Host-side pieces of the library's Beyn solver (no GPU): the contour, the
seeded probe matrix and the dense post-processing (thin SVD, general
eigenproblem) that replace the reference's LAPACKE_zgesdd / LAPACKE_zgeev
(beyn.c:321-333, 404-416), checked against numpy's LAPACK.
"""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "qpms_gb300", "libqpms_gb300.so")),
                                reason="libqpms_gb300.so not built")


def test_contour_matches_oracle():
    from oracle import beyn as ob
    from qpms_gb300 import _lib
    L = _lib.lib()
    n = 40
    p = L.beyn_contour_ellipse(2.0, 1.0, 0.5, 0.2, n)
    try:
        # layout: size_t n, complex centre, function pointer, then (z, dz) pairs and the half-axes entry
        raw = np.frombuffer((C.c_char * (32 + 32 * (n + 1))).from_address(p), dtype=np.uint8)
        assert int(np.frombuffer(raw[:8].tobytes(), dtype=np.uint64)[0]) == n
        zdz = np.frombuffer(raw[32:].tobytes(), dtype=np.complex128).reshape(n + 1, 2)
    finally:
        C.CDLL(None).free(C.c_void_p(p))
    z, dz = ob.contour_ellipse(2 + 1j, 0.5, 0.2, n)
    assert np.allclose(zdz[:n, 0], z, rtol=0, atol=1e-15)
    assert np.allclose(zdz[:n, 1], dz, rtol=0, atol=1e-15)
    assert zdz[n, 0] == 0.5 and zdz[n, 1] == 0.2


def test_probe_matrix_seeded_gaussian():
    from qpms_gb300 import beyn
    a = beyn.probe_matrix(500, 64, 7)
    b = beyn.probe_matrix(500, 64, 7)
    c = beyn.probe_matrix(500, 64, 8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    x = np.concatenate([a.real.ravel(), a.imag.ravel()])
    assert abs(x.mean()) < 0.01 and abs(x.std() - 1) < 0.01


def test_probe_matrix_matches_oracle_restatement():
    from oracle import beyn as ob
    from qpms_gb300 import beyn
    for m, l, seed in ((37, 5, 12345), (300, 64, beyn.DEFAULT_SEED)):
        a = beyn.probe_matrix(m, l, seed)
        o = ob.probe_matrix(m, l, seed)
        assert np.abs(a - o).max() <= 1e-14 * np.abs(o).max()


@pytest.mark.parametrize("m,n,deficient", [(40, 10, False), (300, 64, True), (64, 64, False), (1000, 30, True)])
def test_host_svd(m, n, deficient):
    from qpms_gb300 import beyn
    rng = np.random.default_rng(m + n)
    A = rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))
    if deficient:  # numerical rank n // 2, as Beyn's A0 is
        r = n // 2
        A = A[:, :r] @ (rng.normal(size=(r, n)) + 1j * rng.normal(size=(r, n)))
        A += 1e-15 * (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n)))
    U, s, V = beyn.host_svd(A)
    s_ref = np.linalg.svd(A, compute_uv=False)
    assert np.all(np.diff(s) <= 0)
    assert np.max(np.abs(s - s_ref)) <= 1e-13 * s_ref[0]
    assert np.linalg.norm(U @ np.diag(s) @ V.conj().T - A) <= 1e-13 * np.linalg.norm(A)
    k = int(np.sum(s > 1e-10 * s[0]))
    assert np.linalg.norm(U[:, :k].conj().T @ U[:, :k] - np.eye(k)) < 1e-12
    assert np.linalg.norm(V.conj().T @ V - np.eye(n)) < 1e-12


@pytest.mark.parametrize("n", [1, 2, 7, 30, 64, 150])
def test_host_eig(n):
    from qpms_gb300 import beyn
    rng = np.random.default_rng(n)
    B = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    w, X = beyn.host_eig(B)
    wr = np.linalg.eigvals(B)
    for x in w:
        assert np.min(np.abs(wr - x)) <= 1e-12 * np.abs(wr).max()
    assert np.linalg.norm(B @ X - X * w[None, :]) <= 1e-13 * np.linalg.norm(B)
    # zgeev's normalisation: unit 2-norm, largest component real
    assert np.allclose(np.linalg.norm(X, axis=0), 1, rtol=0, atol=1e-14)
    for k in range(n):
        assert X[np.argmax(np.abs(X[:, k])), k].imag == 0


def test_host_eig_repeated():
    from qpms_gb300 import beyn
    B = np.diag([1, 1, 2, 3.0]).astype(complex)
    B[0, 1] = 1e-3
    w, _ = beyn.host_eig(B)
    assert np.allclose(np.sort(w.real), [1, 1, 2, 3]) and np.allclose(w.imag, 0)
