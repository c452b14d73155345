"""Failure handling of the serving loop and the mixed-precision solves, made
on the host (no GPU fault is provoked):

* a refinement that cannot converge -- the step cap forced to 0 through a
  test hook -- falls back to more precise factors (complex128 at the end), in
  the batched path and in the dense path, and the result says so;
* a request cancelled before it starts completes with QPMS_ECANCELED while the
  others are solved;
* a device-pool allocation that fails (test hook) fails only the request that
  needed it; the server keeps serving.

The reference aborts the process on such errors (qpms_error.c); the library
returns codes instead.
"""
import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR

pytestmark = pytest.mark.gpu
QPMS_ENOMEM, QPMS_ECANCELED = 12, 125


@pytest.fixture(scope="module")
def q():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def _cluster(q, nx, lMax):
    xs = (np.arange(nx) - (nx - 1) / 2) * 400e-9
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)
    return q.ScatteringSystem(pos, 50e-9, -12 + 1.2j, 2.25, lMax)


def test_stalled_refinement_falls_back(q):
    from qpms_gb300.serving import Server
    from qpms_gb300.workloads import square_lattice
    b1, b2, p = square_lattice()
    lat = q.ScatteringSystem(p, 80e-9, -12 + 1.2j, 2.25, 3, lattice=(b1, b2))
    small, large = _cluster(q, 3, 2), _cluster(q, 5, 2)   # 144 (batched) and 400 (dense) unknowns
    om = 2.0 * EV / HBAR
    L = q.lib()
    srv = Server(mode=1, workers=2)
    try:
        ref = {}
        for name, sysm, k in (("lat", lat, (1e6, 0.0)), ("small", small, (0, 0)), ("large", large, (0, 0))):
            ref[name] = srv.wait(srv.submit(sysm, om, k=k))
            assert ref[name]["status"] == 0 and ref[name]["fallback"] == 0
        L.qpms_gpu_testing_set_max_refine(0)
        for name, sysm, k in (("lat", lat, (1e6, 0.0)), ("small", small, (0, 0)), ("large", large, (0, 0))):
            r = srv.wait(srv.submit(sysm, om, k=k))
            assert r["status"] == 0, r.get("error")
            assert r["fallback"] == 1, name
            assert r["residual"] <= 1e-12, (name, r["residual"])
            assert np.linalg.norm(r["f"] - ref[name]["f"]) <= 1e-9 * np.linalg.norm(ref[name]["f"])
    finally:
        L.qpms_gpu_testing_set_max_refine(-1)
        srv.close()


def test_cancel_before_start(q):
    from qpms_gb300.serving import Server
    sysm = _cluster(q, 6, 3)   # 1080 unknowns: each solve takes a while on one worker
    oms = np.linspace(1.8, 2.4, 12) * EV / HBAR
    srv = Server(mode=1, workers=1)
    try:
        tickets = [srv.submit(sysm, w) for w in oms]
        cancelled = {t: srv.cancel(t) for t in tickets[6:]}
        assert any(cancelled.values())
        for t, c in cancelled.items():
            if c:
                assert not srv.cancel(t)  # a second cancel finds nothing pending
        for t in tickets:
            r = srv.wait(t)
            if cancelled.get(t):
                assert r["status"] == QPMS_ECANCELED and "cancel" in r["error"]
            else:
                assert r["status"] == 0 and r["residual"] <= 1e-11  # the server refines to 1e-11
        # the server still serves afterwards
        assert srv.wait(srv.submit(sysm, oms[0]))["status"] == 0
    finally:
        srv.close()


def test_failed_allocation_fails_one_request(q):
    from qpms_gb300.serving import Server
    sysm = _cluster(q, 5, 2)   # 400 unknowns: each request runs alone
    om = 2.2 * EV / HBAR
    srv = Server(mode=1, workers=1)
    L = q.lib()
    try:
        good = srv.wait(srv.submit(sysm, om))
        assert good["status"] == 0
        assert L.qpms_gpu_server_testing_fail_allocations(srv.s, 1) == 0
        bad = srv.wait(srv.submit(sysm, om))
        assert bad["status"] == QPMS_ENOMEM and "allocation" in bad["error"]
        again = srv.wait(srv.submit(sysm, om))
        assert again["status"] == 0
        assert abs(again["sigma_ext"] - good["sigma_ext"]) <= 1e-12 * abs(good["sigma_ext"])
    finally:
        L.qpms_gpu_server_testing_fail_allocations(srv.s, 0)
        srv.close()
