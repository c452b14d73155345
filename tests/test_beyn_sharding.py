"""Beyn sharded over ranks (replicas with one exchange step), on the CPU with
gloo, world size 2: each rank sums its contiguous share of the contour nodes,
the partial sums are all-reduced through host memory, rank 0 runs the
library's host post-processing.  The result must equal the post-processing of
the serial sums, and the oracle's Beyn eigenvalues within 1e-8."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "qpms_gb300", "libqpms_gb300.so")),
                                reason="libqpms_gb300.so not built")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_node_range_partition():
    from qpms_gb300.beyn import node_range
    for n in (1, 7, 64, 150):
        for w in (1, 2, 3, 8):
            parts = [node_range(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))
            assert max(e - b for b, e in parts) - min(e - b for b, e in parts) <= 1


def test_sharded_quadrature_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle import beyn as ob
    from qpms_gb300 import beyn
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import _sharding_worker as w
    env_path = os.pathsep.join([ROOT, os.path.dirname(os.path.abspath(__file__)), os.environ.get("PYTHONPATH", "")])
    os.environ["PYTHONPATH"] = env_path
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=w.worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    sharded = q.get()
    Mf, V = w.problem()
    contour = ob.ellipse(0, 0.3, 0.3, 150)
    serial = beyn.process(*ob.quadrature(Mf, contour, V, 0, 150), 0.0, 1e-4, 1)["eigval"]
    assert sharded.size == serial.size >= 3
    for e in serial:
        assert np.min(np.abs(sharded - e)) <= 1e-12 * abs(e)
    ref = ob.beyn_solve(Mf, 60, 30, contour, V, 1e-4, 1, 0.0)["eigval"]
    assert ref.size == serial.size
    for e in ref:
        assert np.min(np.abs(serial - e)) <= 1e-8 * abs(e)
