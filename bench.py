"""Benchmark of the QPMS hot path on GB300.

Workload (one "step"): the batched translation-operator configuration --
10^6 seeded separation vectors (|r| log-uniform 50 nm..10 um, directions
uniform on the sphere, complex k with Re k = 1.5 omega/c for hbar omega in
1.6..2.6 eV and Im k in [0, 1e-3 Re k]); regular (J=1) and outgoing (J=3)
A/B arrays in complex128 at lMax 3 and lMax 6: four launches, 4e6 "solves"
(one solve = the A and B arrays of one vector for one J and one lMax).

value:  solves/s with inputs resident in HBM (CUDA events on the launching
        stream, max over ranks).
e2e:    the same through the C-ABI host entry point
        qpms_gpu_trans_AB_arrays_batch_host with pinned host inputs/outputs
        (H2D of inputs and D2H of all A/B arrays inside the timed region).
--impl reference: the CPU restatement of the reference's translation path
        (the reference itself needs GSL + AMOS, absent here) on all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s + p50/p99 latency vs plain FP64 GPU path at ≤1e-10 rel. residual"
UNIT = "solves/s"
N_VEC = 1_000_000
LMAXES = (3, 6)
JS = (1, 3)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nvec", type=int, default=N_VEC)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def config_dict(args, ws):
    return {"workload": "batched translation-operator kernel: %d seeded vectors x J in {1,3} x lMax in "
                        "{3,6}, complex128 A/B arrays" % args.nvec,
            "n_vectors_per_rank": args.nvec, "lMax": list(LMAXES), "J": list(JS),
            "parallelism": "replicas (vectors sharded by rank)" if ws > 1 else "single GPU",
            "l2": "no flush needed: each launch writes 7.2-73.7 GB of A/B, >> 129 MB L2"}


def algo_bytes(nvec, lMax):
    ne2 = (lMax * (lMax + 2)) ** 2
    return nvec * (2 * ne2 * 16 + 32)


def algo_flops(lMax):
    from qpms_gb300.translations import multipliers_export
    A, B = multipliers_export(lMax)
    return 4 * (A.size + B.size)  # two FP64 FMAs per real-coefficient x complex term


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self, dev_index=0):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9 or f[0] != str(dev_index):
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def profile_traffic(lMax):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "trans_ab_traffic.json")))
        return d.get("lmax%d" % lMax)
    except Exception:
        return None


def cpu_baseline(args, sample_sec=12.0):
    """Oracle (C restatement, OpenMP over all host cores) on a bounded sample."""
    from oracle import orc
    from qpms_gb300.workloads import translation_vectors
    threads = orc.num_threads()
    total_time = 0.0
    samples = []
    for lMax in LMAXES:
        c = orc.TransCalculator(lMax)
        for J in JS:
            n = 64
            while True:
                kr, th, ph = translation_vectors(n, seed=99)
                t0 = time.perf_counter()
                c.get_AB_batch(kr, th, ph, J)
                dt = time.perf_counter() - t0
                if dt > sample_sec / (len(LMAXES) * len(JS)) or n >= args.nvec:
                    break
                n *= 4
            rate = n / dt
            samples.append("lMax%d J%d: %d vectors in %.2fs" % (lMax, J, n, dt))
            total_time += args.nvec / rate
    solves = args.nvec * len(LMAXES) * len(JS)
    return {"value": solves / total_time, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "; ".join(samples) + " (rate scaled to the full step)"}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    cb = None
    vals = []
    for _ in range(args.warmup):
        pass
    t_all = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        cb = cpu_baseline(args, sample_sec=8.0)
        t_all.append(time.perf_counter() - t0)
        vals.append(cb["value"])
    v = float(np.median(vals))
    cb["value"] = v
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.nvec * 4 / v,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded, config shapes)", "config": config_dict(args, 1),
           "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                                       "d2h_bytes_per_step": 0},
           "note": "reference C path needs GSL + AMOS (absent); timed the oracle's C restatement"}
    print(json.dumps(out), flush=True)


def run_ours(args, ws, rank, local):
    import torch
    import qpms_gb300
    from qpms_gb300 import _lib
    from qpms_gb300.workloads import translation_vectors

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = qpms_gb300.lib()
    kr, th, ph = translation_vectors(args.nvec, seed=1000 + rank)
    tkr = torch.from_numpy(kr).to(dev)
    tth = torch.from_numpy(th).to(dev)
    tph = torch.from_numpy(ph).to(dev)
    calcs = {lm: qpms_gb300.trans_calculator(lm) for lm in LMAXES}
    outs = {}
    for lm in LMAXES:
        ne = lm * (lm + 2)
        outs[lm] = (torch.empty((args.nvec, ne, ne), dtype=torch.complex128, device=dev),
                    torch.empty((args.nvec, ne, ne), dtype=torch.complex128, device=dev))
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def step(evs=None):
        for lm in LMAXES:
            A, B = outs[lm]
            for J in JS:
                if evs is not None:
                    evs[(lm, J)][0].record(stream)
                calcs[lm].get_AB_arrays_device(tkr, tth, tph, J, A, B, stream=sh)
                if evs is not None:
                    evs[(lm, J)][1].record(stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    launches0 = L.qpms_gpu_kernel_launch_count()
    step_ms, kern = [], {(lm, J): [] for lm in LMAXES for J in JS}
    clk = ClockSampler(os.path.join(ROOT, "gpurun_out" if os.path.isdir(os.path.join(ROOT, "gpurun_out"))
                                    else "/tmp", "bench_clocks.csv"))
    with clk:
        barrier()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for _ in range(args.steps):
            evs = {k: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for k in kern}
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            step(evs)
            s1.record(stream)
            s1.synchronize()
            step_ms.append(s0.elapsed_time(s1))
            for k, (a, b) in evs.items():
                kern[k].append(a.elapsed_time(b))
        t_end.record(stream)
        barrier()
    total_ms = t_start.elapsed_time(t_end)
    launches = L.qpms_gpu_kernel_launch_count() - launches0
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    solves_per_step = args.nvec * len(LMAXES) * len(JS) * ws
    value = solves_per_step * args.steps / (total_ms / 1e3)

    # roofline of the dominant kernel (the lMax 6 launches)
    peaks = measured_peaks()
    fp64 = None
    import ctypes as C
    fp = C.c_double(0)
    if L.qpms_gpu_measure_fp64_peak(C.byref(fp)) == 0:
        fp64 = fp.value
    dom = max(kern, key=lambda k: np.mean(kern[k]))
    lm_dom = dom[0]
    dur = float(np.mean([np.mean(kern[(lm_dom, J)]) for J in JS])) / 1e3
    abytes = algo_bytes(args.nvec, lm_dom)
    aflops = algo_flops(lm_dom) * args.nvec
    achieved_gbs = abytes / dur / 1e9
    roof = {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
            "frac": achieved_gbs / peaks.get("hbm_gbs"), "traffic": profile_traffic(lm_dom),
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)" if not peaks.get("fallback")
            else "fallback 6.8 TB/s",
            "kernel": "trans_ab_kernel<%d> (lMax %d, mean of J=1,3)" % (lm_dom, lm_dom),
            "ms_per_launch": dur * 1e3,
            "fp64": {"achieved_tflops": aflops / dur / 1e12, "peak_tflops": fp64,
                     "frac": (aflops / dur / 1e12 / fp64) if fp64 else None,
                     "peak_source": "library DFMA probe qpms_gpu_measure_fp64_peak"}}
    per_kernel = {"lMax%d_J%d_ms" % k: float(np.mean(v)) for k, v in kern.items()}

    # end to end through the host C-ABI entry point (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, calcs, kr, th, ph, ws)

    if rank == 0:
        cb = None if args.no_cpu else cpu_baseline(args)
        sm = clk.summary(local)
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic (seeded; config distributions)", "config": config_dict(args, ws),
               "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                              "unit_of_latency": "one step (4e6 solves)"},
               "per_kernel": per_kernel, "roofline": roof, "cpu_baseline": cb, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": sm,
               "plain_fp64_path": "this path is FP64 throughout (the plain path itself): ratio 1"}
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _mem_available():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 16 << 30


def run_e2e(args, calcs, kr, th, ph, ws):
    """Host-buffer path: pinned inputs, pinned output buffers (reused across
    sub-batches when the host cannot hold a whole launch's output)."""
    import torch
    L = calcs[LMAXES[0]]._L
    n = args.nvec
    pk = torch.from_numpy(kr).pin_memory()
    pt = torch.from_numpy(th).pin_memory()
    pp = torch.from_numpy(ph).pin_memory()
    budget = min(8 << 30, _mem_available() // 8)
    bufs = {}
    for lm in LMAXES:
        ne2 = (lm * (lm + 2)) ** 2
        nsub = max(1, min(n, budget // (ne2 * 32)))
        bufs[lm] = (nsub, torch.empty((nsub, ne2), dtype=torch.complex128).pin_memory(),
                    torch.empty((nsub, ne2), dtype=torch.complex128).pin_memory())

    h2d = d2h = 0

    def step():
        nonlocal h2d, d2h
        h2d = d2h = 0
        for lm in LMAXES:
            nsub, hA, hB = bufs[lm]
            ne2 = hA.shape[1]
            for J in JS:
                for o in range(0, n, nsub):
                    m = min(nsub, n - o)
                    rc = L.qpms_gpu_trans_AB_arrays_batch_host(
                        calcs[lm].c, m, pk.data_ptr() + 16 * o, pt.data_ptr() + 8 * o, pp.data_ptr() + 8 * o,
                        None, J, hA.data_ptr(), hB.data_ptr())
                    if rc:
                        raise RuntimeError(calcs[lm]._L.qpms_gpu_last_error())
                    h2d += 32 * m
                    d2h += 2 * 16 * ne2 * m

    step()  # warm-up (allocates staging)
    reps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(reps):
        step()
    dt = (time.perf_counter() - t0) / reps
    solves = n * len(LMAXES) * len(JS) * ws
    return {"value": solves / dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": dt * 1e3, "host_output_buffer_vectors": {str(k): v[0] for k, v in bufs.items()},
            "path": "qpms_gpu_trans_AB_arrays_batch_host (C-ABI), pinned host buffers"}


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
