"""Autotuner of the library's block sizes on the GPU it runs on.

* The tensor-core GEMM: every pipeline variant (operand stages x tensor-memory
  accumulators, QPMS_GB300_GEMM_PIPE) with and without 256-wide tiles
  (QPMS_GB300_GEMM_WIDE), each in a process of its own, on trailing-update
  shapes; the fastest in total wins.
* The mixed dense solve (random butterfly + complex64 LU on the tensor cores +
  FP64 refinement, one right-hand side) at several sizes with 64- and
  128-wide diagonal blocks (QPMS_GB300_LU_NB): the size from which 128 is
  faster.

It writes

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


GEMM_SHAPES = ((8064, 8064, 128, 2), (14272, 14272, 128, 2), (4096, 4096, 128, 2))
PIPES = ("6x2", "6x3", "7x2", "7x3")


def gemm_probe():
    """Times the tensor-core GEMM on trailing-update shapes in this process
    (the variant comes from the environment): microseconds per shape."""
    import torch
    from . import _lib
    L = _lib.lib()
    vp, sz, ci, cf = C.c_void_p, C.c_size_t, C.c_int, C.c_float
    L.qpms_gpu_tc_cgemm.restype = ci
    L.qpms_gpu_tc_cgemm.argtypes = [ci, ci, ci, vp, sz, vp, sz, cf, cf, vp, sz, vp, sz, ci, vp]
    dev = torch.device("cuda:0")
    out = []
    for m, n, k, ns in GEMM_SHAPES:
        A = torch.randn(k, m, dtype=torch.complex64, device=dev)
        B = torch.randn(n, k, dtype=torch.complex64, device=dev)
        Cm = torch.randn(n, m, dtype=torch.complex64, device=dev)
        st = torch.cuda.current_stream().cuda_stream
        for rep in range(4):
            if rep == 3:
                _lib.kernel_timing(True)
            if L.qpms_gpu_tc_cgemm(m, n, k, A.data_ptr(), m, B.data_ptr(), k, -1.0, 1.0, Cm.data_ptr(), m,
                                   Cm.data_ptr(), m, ns, st):
                raise RuntimeError(_lib.last_error())
            torch.cuda.synchronize()
        kt = _lib.kernel_timing_get()
        _lib.kernel_timing(False)
        out.append(kt["tc_gemm"][0] * 1e3)
    return out


def tune_gemm():
    import subprocess
    res = {}
    for wide in ("0", "1"):
        for pipe in PIPES:
            env = dict(os.environ, QPMS_GB300_GEMM_PIPE=pipe, QPMS_GB300_GEMM_WIDE=wide)
            r = subprocess.run([sys.executable, "-m", "qpms_gb300.tune", "--gemm-probe"], env=env,
                               capture_output=True, text=True, cwd=os.path.dirname(HERE))
            if r.returncode:
                raise RuntimeError(r.stderr[-2000:])
            res["%s wide%s" % (pipe, wide)] = json.loads(r.stdout.strip().splitlines()[-1])
            print(pipe, "wide", wide, res["%s wide%s" % (pipe, wide)], flush=True)
    return (res,) + choose_gemm(res)


def choose_gemm(res):
    """Pipeline variant from the runs without wide tiles (there every shape
    runs the 128-wide kernel the variant shapes; another variant must beat the
    default 6x2 by more than 1 %); wide tiles if their best total beats the
    best total without them."""
    tot = {k: sum(v) for k, v in res.items()}
    pipe = "6x2"
    for p in PIPES:
        if tot["%s wide0" % p] < 0.99 * tot["%s wide0" % pipe]:
            pipe = p
    wide = min(tot["%s wide1" % p] for p in PIPES) < min(tot["%s wide0" % p] for p in PIPES)
    return int(pipe[0]) * 10 + int(pipe[2]), wide


def crossover(rows):
    """Smallest measured size from which 128 stays at least as fast as 64."""
    for i, r in enumerate(rows):
        if all(x["s_nb128"] <= x["s_nb64"] for x in rows[i:]):
            return r["N"]
    return rows[-1]["N"] + 1


def main():
    if "--gemm-probe" in sys.argv:
        print(json.dumps(gemm_probe()))
        return 0
    gemm, pipe, wide = tune_gemm()
    rows = measure()
    n64 = crossover(rows)
    with open(os.path.join(HERE, "tuning.json"), "w") as f:
        json.dump({"dense_solve": {"what": "mixed dense solve, 1 right-hand side, seconds (min of 3)", "rows": rows},
                   "gemm": {"what": "tensor-core GEMM, microseconds per trailing update (m, n, k, digits): %s"
                            % (GEMM_SHAPES,), "variants": gemm},
                   "kTunedNb64Below": n64, "kTunedGemmPipe": pipe, "kTunedGemmWide": wide}, f, indent=1)
    path = os.path.join(HERE, "csrc", "qg_tuned.h")
    src = open(path).read()
    import re
    src = re.sub(r"constexpr int kTunedNb64Below = \d+;", "constexpr int kTunedNb64Below = %d;" % n64, src)
    src = re.sub(r"constexpr int kTunedGemmPipe = \d+;", "constexpr int kTunedGemmPipe = %d;" % pipe, src)
    src = re.sub(r"constexpr bool kTunedGemmWide = \w+;", "constexpr bool kTunedGemmWide = %s;"
                 % ("true" if wide else "false"), src)
    open(path, "w").write(src)
    print("kTunedNb64Below =", n64, "kTunedGemmPipe =", pipe, "kTunedGemmWide =", wide)
    return 0


if __name__ == "__main__":
    sys.exit(main())
