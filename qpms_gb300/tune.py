"""Autotuner of the library's block sizes on the GPU it runs on.

Measures the mixed dense solve (random butterfly + complex64 LU on the tensor
cores + FP64 refinement, one right-hand side: the serving loop's solve) at
several sizes with 64- and 128-wide diagonal blocks (QPMS_GB300_LU_NB), picks
the size from which 128 is faster, and writes

* qpms_gb300/csrc/qg_tuned.h  -- the constant the library is built with,
* qpms_gb300/tuning.json       -- the measurements behind it.

Run on the target GPU, then rebuild:
    python -m qpms_gb300.tune && python -c "import __graft_entry__ as g; g.build()"
"""
import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SIZES = (1024, 2048, 3072, 4096, 6144, 8192, 11008, 14400)
NBS = (64, 128)


def measure(sizes=SIZES, reps=3):
    import torch
    from . import _lib
    L = _lib.lib()
    L.qpms_gpu_dense_solve.restype = C.c_int
    L.qpms_gpu_dense_solve.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_void_p]
    dev = torch.device("cuda:0")
    out = []
    for N in sizes:
        g = torch.Generator(device=dev)
        g.manual_seed(N)
        M = torch.randn(N, N, dtype=torch.complex128, device=dev, generator=g) / N ** 0.5
        M += 2 * torch.eye(N, dtype=torch.complex128, device=dev)
        B = torch.randn(1, N, dtype=torch.complex128, device=dev, generator=g)
        X = torch.empty_like(B)
        row = {"N": N}
        for nb in NBS:
            os.environ["QPMS_GB300_LU_NB"] = str(nb)
            res = np.zeros(1)
            it = np.zeros(1, dtype=np.int32)
            ts = []
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                rc = L.qpms_gpu_dense_solve(N, 1, M.data_ptr(), B.data_ptr(), X.data_ptr(), 1, res.ctypes.data,
                                            it.ctypes.data)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
                if rc:
                    raise RuntimeError(_lib.last_error())
            row["s_nb%d" % nb] = min(ts)
            row["residual_nb%d" % nb] = float(res[0])
        os.environ.pop("QPMS_GB300_LU_NB", None)
        out.append(row)
        print(json.dumps(row), flush=True)
    return out


def crossover(rows):
    """Smallest measured size from which 128 stays at least as fast as 64."""
    for i, r in enumerate(rows):
        if all(x["s_nb128"] <= x["s_nb64"] for x in rows[i:]):
            return r["N"]
    return rows[-1]["N"] + 1


def main():
    rows = measure()
    n64 = crossover(rows)
    with open(os.path.join(HERE, "tuning.json"), "w") as f:
        json.dump({"what": "mixed dense solve, 1 right-hand side, seconds (min of 3)", "rows": rows,
                   "kTunedNb64Below": n64}, f, indent=1)
    path = os.path.join(HERE, "csrc", "qg_tuned.h")
    src = open(path).read()
    import re
    src = re.sub(r"constexpr int kTunedNb64Below = \d+;", "constexpr int kTunedNb64Below = %d;" % n64, src)
    open(path, "w").write(src)
    print("kTunedNb64Below =", n64)


if __name__ == "__main__":
    sys.exit(main())
