"""The autotuner's choices (qpms_gb300/tune.py), on the host: the constants the
library is built with (csrc/qg_tuned.h) are the ones its rules pick from the
committed measurements (tuning.json), and the rules themselves behave as
documented on synthetic measurements."""
import json
import os
import re

from qpms_gb300 import tune

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_constants():
    src = open(os.path.join(ROOT, "qpms_gb300", "csrc", "qg_tuned.h")).read()
    n64 = int(re.search(r"constexpr int kTunedNb64Below = (\d+);", src).group(1))
    pipe = int(re.search(r"constexpr int kTunedGemmPipe = (\d+);", src).group(1))
    wide = re.search(r"constexpr bool kTunedGemmWide = (\w+);", src).group(1) == "true"
    return n64, pipe, wide


def test_header_matches_committed_measurements():
    d = json.load(open(os.path.join(ROOT, "qpms_gb300", "tuning.json")))
    pipe, wide = tune.choose_gemm(d["gemm"]["variants"])
    n64 = tune.crossover(d["dense_solve"]["rows"])
    assert (n64, pipe, wide) == _header_constants()
    assert (d["kTunedNb64Below"], d["kTunedGemmPipe"], d["kTunedGemmWide"]) == (n64, pipe, wide)


def _variants(times_wide0, times_wide1):
    res = {}
    for p in tune.PIPES:
        res["%s wide0" % p] = [times_wide0[p]]
        res["%s wide1" % p] = [times_wide1[p]]
    return res


def test_choose_gemm_rules():
    base = {p: 100.0 for p in tune.PIPES}
    # no variant more than 1 % faster than 6x2: 6x2 stays
    w0 = dict(base, **{"7x2": 99.5})
    assert tune.choose_gemm(_variants(w0, base)) == (62, False)
    # a variant 2 % faster wins
    w0 = dict(base, **{"7x3": 98.0})
    assert tune.choose_gemm(_variants(w0, base))[0] == 73
    # wide tiles only when their best total beats the best without them
    w1 = dict(base, **{"6x2": 90.0})
    assert tune.choose_gemm(_variants(base, w1)) == (62, True)


def test_crossover_rules():
    rows = [{"N": n, "s_nb64": a, "s_nb128": b}
            for n, a, b in ((1024, 1.0, 1.1), (2048, 2.0, 1.9), (4096, 4.0, 4.1), (8192, 8.0, 7.0), (14400, 20.0, 15.0))]
    # 128 must stay at least as fast from the crossover on: 2048 fails at 4096
    assert tune.crossover(rows) == 8192
    rows[2]["s_nb128"] = 3.9
    assert tune.crossover(rows) == 2048
    # 64 faster everywhere: past the largest measured size
    assert tune.crossover([{"N": 1024, "s_nb64": 1.0, "s_nb128": 2.0}]) == 1025
