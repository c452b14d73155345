"""Worker of tests/test_beyn_sharding.py (a gloo rank on the CPU)."""
import os

import numpy as np


def problem():
    """tests/tbeyn2.c setup: quadratic T0 + z T1 + z^2 T2, dim 60, L 30."""
    rng = np.random.default_rng(1)
    T0, T1, T2 = (rng.normal(size=(60, 60)) for _ in range(3))
    V = rng.normal(size=(60, 30)) + 1j * rng.normal(size=(60, 30))
    return (lambda z: T0 + z * T1 + z * z * T2), V


def worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import beyn as ob
        from qpms_gb300 import beyn
        Mf, V = problem()
        contour = ob.ellipse(0, 0.3, 0.3, 150)
        b, e = beyn.node_range(150, rank, world)
        parts = ob.quadrature(Mf, contour, V, b, e)   # this rank's share (stands in for its GPU quadrature)
        total = beyn.allreduce_sum(parts)
        if rank == 0:
            q.put(beyn.process(*total, 0.0, 1e-4, 1)["eigval"])
    finally:
        dist.destroy_process_group()
