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

Secondary objects in the same JSON line (rank 0), each the other workloads of
the path measured mixed (complex64 LU + FP64 refinement) against the plain
FP64 GPU path at a <= 1e-10 relative residual:
  modeproblem - finite 4x4 sphere array, lMax 2 (256 x 256), 32 frequencies:
                assembly + LU + solve + sigma_ext per frequency;
  dispersion  - square (30 x 30) and honeycomb (60 x 60) lattices, lMax 3:
                (omega, k) points/s of assembly + LU + log|det| + excitation;
  beyn        - 30 x 30 array, lMax 2 (14,400 x 14,400), 64 contour nodes,
                64 probe columns; the plain path timed on one node x 64;
  serving     - seeded request stream (70 % clusters of 16-400 spheres,
                lMax 2-4; 30 % lattice points): solves/s and p50/p99 latency
                at saturation and at Poisson arrival rates.
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
    ap.add_argument("--sections", default="modeproblem,dispersion,beyn,serving,field,axsym",
                    help="secondary workloads reported beside the headline (comma list, or 'none')")
    ap.add_argument("--case", default=None,
                    help="run one small case for a profiler and exit: dense:N:NRHS:MODE, "
                         "scan:{square,honeycomb,bilayer}:NW:NK:MODE, finite:NX:LMAX:NW:MODE, "
                         "field:NX:NPTS:LMAX, axsym:L:NW, beyn:NX:NODES:MODE")
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
        sections = run_sections(args)
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic (seeded; config distributions)", "config": config_dict(args, ws),
               "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                              "unit_of_latency": "one step (4e6 solves)"},
               "per_kernel": per_kernel, "roofline": roof, "cpu_baseline": cb, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": sm,
               "plain_fp64_path": "this path is FP64 throughout (the plain path itself): ratio 1"}
        out.update(sections)
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


def _sq(nx, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * nx)], 1)


def section_modeproblem(args):
    """Finite 4x4 array, lMax 2, 32 frequencies: plain vs mixed, and the CPU oracle."""
    import torch
    import qpms_gb300
    from qpms_gb300.workloads import EV, HBAR
    ss = qpms_gb300.ScatteringSystem(_sq(4, 400e-9), 50e-9, -12 + 1.2j, 2.25, 2)
    om = np.linspace(1.6, 2.6, 32) * EV / HBAR
    out = {"workload": "finite 4x4 spheres, pitch 400 nm, r 50 nm, lMax 2 (256 x 256), 32 omegas, "
                       "normal incidence: assembly + LU + solve + sigma_ext"}
    for mode, name in ((0, "plain_fp64"), (1, "mixed")):
        for _ in range(3):
            ss.planewave_scatter_batch(om, mode=mode)
        ts = []
        for _ in range(10):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = ss.planewave_scatter_batch(om, mode=mode)
            ts.append(time.perf_counter() - t0)
        ts = np.array(ts)
        out[name] = {"solves_per_s": float(32 / np.median(ts)), "ms_per_32": float(np.median(ts) * 1e3),
                     "p50_ms": float(np.percentile(ts, 50) * 1e3), "p99_ms": float(np.percentile(ts, 99) * 1e3),
                     "max_residual": float(r["residual"].max())}
    out["mixed_vs_plain"] = out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    if not args.no_cpu:
        from oracle import orc
        c = orc.TransCalculator(2)
        t0 = time.perf_counter()
        for w in om:
            orc.finite_sphere_scatter(c, _sq(4, 400e-9), 50e-9, -12 + 1.2j, 2.25, w)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"solves_per_s": 32 / dt, "cores": orc.num_threads(), "kind": "port",
                               "sample": "all 32 frequencies"}
    return out


def section_dispersion(args):
    import torch
    import qpms_gb300
    from qpms_gb300.workloads import EV, HBAR, honeycomb_lattice, honeycomb_path, square_lattice, square_path
    out = {"workload": "sample of 32 omegas x 256 k of each 4096 k x 256 omega scan, lMax 3, r 80 nm, a 580 nm"}
    om = np.linspace(1.6, 2.6, 32) * EV / HBAR
    for lat in ("square", "honeycomb"):
        b1, b2, pos = square_lattice() if lat == "square" else honeycomb_lattice()
        ss = qpms_gb300.ScatteringSystem(pos, 80e-9, -12 + 1.2j, 2.25, 3, lattice=(b1, b2))
        kp = (square_path if lat == "square" else honeycomb_path)(n=256)
        ss.dispersion_scan(om[:2], kp[:8])
        d = {}
        for mode, name in ((0, "plain_fp64"), (1, "mixed")):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = ss.dispersion_scan(om, kp, mode=mode)
            dt = time.perf_counter() - t0
            d[name] = {"points_per_s": om.size * kp.shape[0] / dt, "max_residual": float(r["residual"].max()),
                       "full_scan_s": 4096 * 256 / (om.size * kp.shape[0] / dt)}
        d["mixed_vs_plain"] = d["mixed"]["points_per_s"] / d["plain_fp64"]["points_per_s"]
        out[lat] = d
    return out


def section_beyn(args):
    import qpms_gb300
    from qpms_gb300.workloads import EV, HBAR
    ss = qpms_gb300.ScatteringSystem(_sq(30, 400e-9), 60e-9, -12 + 1.2j, 2.25, 2)
    c, rr, ri = 2.1 * EV / HBAR, 0.05 * EV / HBAR, 0.005 * EV / HBAR
    r = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=1e-4, l=64, seed=12345, mode=1)
    out = {"workload": "30x30 spheres r 60 nm, lMax 2 (14400 x 14400), ellipse 2.1 eV +- 0.05 / 0.005 eV, "
                       "64 nodes, L 64",
           "mixed": {"total_s": r["total_s"], "quadrature_s": r["quadrature_s"],
                     "node_residual_max": r["node_residual_max"], "refine_iters_max": r["node_refine_iters_max"],
                     "neig": int(r["eigval"].size), "inside": int((r["eigval_inside_metric"] < 1).sum())}}
    one = {}
    for mode in (0, 1):
        q = ss.find_modes(c, rr, ri, contour_points=1, rank_tol=1e-4, l=64, seed=12345, mode=mode)
        one[mode] = q["quadrature_s"]
    out["per_node_s"] = {"plain_fp64": one[0], "mixed": one[1]}
    out["plain_fp64_estimate_s"] = 64 * one[0]
    out["mixed_vs_plain"] = 64 * one[0] / r["quadrature_s"]
    return out


def section_serving(args):
    import qpms_gb300
    from qpms_gb300.serving import Server, run_trace
    from qpms_gb300.workloads import honeycomb_lattice, poisson_arrivals, serving_requests, square_lattice
    b1, b2, p1 = square_lattice()
    h1, h2, p2 = honeycomb_lattice()
    lat = {"square": qpms_gb300.ScatteringSystem(p1, 80e-9, -12 + 1.2j, 2.25, 3, lattice=(b1, b2)),
           "honeycomb": qpms_gb300.ScatteringSystem(p2, 80e-9, -12 + 1.2j, 2.25, 3, lattice=(h1, h2))}
    n = 60
    reqs = []
    for s in serving_requests(n, seed=5):
        if s["kind"] == "finite":
            reqs.append({"system": qpms_gb300.ScatteringSystem(s["positions"], 50e-9, -12 + 1.2j, 2.25, s["lMax"]),
                         "omega": s["omega"]})
        else:
            reqs.append({"system": lat[s["lattice"]], "omega": s["omega"], "k": s["k"]})
    srv = Server(mode=1, workers=4)
    run_trace(srv, reqs[:8])
    _, sat = run_trace(srv, reqs)
    st = srv.stats()
    sweep = {}
    for rate in (5.0, 20.0):
        _, sweep[str(rate)] = run_trace(srv, reqs, poisson_arrivals(n, rate, 1))
    srv.close()
    sub = reqs[:12]
    res = {}
    for mode, name in ((0, "plain_fp64"), (1, "mixed")):
        srv = Server(mode=mode, workers=4)
        _, res[name] = run_trace(srv, sub)
        srv.close()
    return {"workload": "%d seeded requests: 70%% clusters N 16-400 spheres (jittered 400 nm grid, r 50 nm, "
                        "lMax 2-4), 30%% lattice (omega, k) solves; 4 worker streams" % n,
            "mean_unknowns": float(np.mean([r["system"].fecv_size for r in reqs])),
            "saturated": sat, "poisson": sweep, "server": st,
            "subsample_12": res,
            "mixed_vs_plain": res["mixed"]["solves_per_s"] / res["plain_fp64"]["solves_per_s"]}


def section_field(args):
    """Scattered-field map of a solved 30 x 30 sphere array (lMax 3): a 512 x 512
    grid 100 nm above the particle plane, every point summed over all 900 particles."""
    import torch
    import qpms_gb300
    from qpms_gb300.workloads import EV, HBAR
    pos = _sq(30, 400e-9)
    lMax = 3
    ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, lMax)
    om = 2.1 * EV / HBAR
    k = np.sqrt(2.25) * om / 299792458.0
    f = ss.planewave_scatter_batch(np.array([om]), mode=1, want_f=True)["f"][0]
    g = np.linspace(-6.5e-6, 6.5e-6, 512)
    X, Y = np.meshgrid(g, g, indexing="ij")
    pts = np.ascontiguousarray(np.stack([X.ravel(), Y.ravel(), np.full(X.size, 1e-7)], 1))
    npts, pairs = pts.shape[0], pts.shape[0] * pos.shape[0]
    dev = torch.device("cuda:0")
    tf = torch.from_numpy(f).to(dev)
    tp = torch.from_numpy(pts).to(dev)
    out = torch.empty((npts, 3), dtype=torch.complex128, device=dev)
    st = torch.cuda.current_stream(dev)
    for _ in range(3):
        ss.scattered_E_device(k, tf, tp, out, stream=st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        ss.scattered_E_device(k, tf, tp, out, stream=st)
    e1.record(st)
    torch.cuda.synchronize()
    dms = e0.elapsed_time(e1) / reps
    # end to end through the host API (points H2D, field D2H inside)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        E = ss.scattered_E(k, f, pts)
        ts.append(time.perf_counter() - t0)
    e2e = float(np.median(ts))
    res = {"workload": "field map: 30x30 spheres (pitch 400 nm, r 60 nm, lMax 3, solved at 2.1 eV), "
                       "512x512 points 100 nm above the array, all 900 particles per point",
           "device": {"ms_per_map": dms, "points_per_s": npts / dms * 1e3, "pairs_per_s": pairs / dms * 1e3},
           "e2e": {"ms_per_map": e2e * 1e3, "points_per_s": npts / e2e,
                   "h2d_bytes": int(pts.nbytes + f.nbytes), "d2h_bytes": int(E.nbytes)}}
    if not args.no_cpu:
        from oracle import orc
        ns = 256
        t0 = time.perf_counter()
        O = orc.scattered_E(lMax, pos, 3, k, f, pts[:ns])
        dt = time.perf_counter() - t0
        err = np.abs(E[:ns] - O).max() / np.abs(O).max()
        res["cpu_baseline"] = {"points_per_s": ns / dt, "pairs_per_s": ns * pos.shape[0] / dt, "cores": 1,
                               "kind": "port", "sample": "first %d points of the map" % ns,
                               "max_rel_diff_vs_gpu": float(err)}
        res["gpu_vs_cpu"] = res["device"]["points_per_s"] / res["cpu_baseline"]["points_per_s"]
    return res


def _axsym_flops(L, nq, zsym=True):
    """Algorithmic FP64 flops of the Q/R quadrature at lMax_extend L over nq
    nodes: per m block 2 nb^2 dot products (n x y) . v of complex 3-vectors
    (3 complex FMAs = 24 flops per node), half of them for a z-mirror
    symmetric surface (the others vanish)."""
    tot = 0
    for m in range(-L, L + 1):
        nb = 2 * (L - max(1, abs(m)) + 1)
        tot += 2 * nb * nb // (2 if zsym else 1)
    return tot * nq * 24


def section_axsym(args):
    """T-matrices of an axially symmetric particle (gold-like cylinder r 50 nm,
    h 100 nm in eps 2.25, basis lMax 3, Q/R at lMax_extend 8) at 256
    frequencies 1.6-2.6 eV: the batched EBCM kernel, device time and end to end."""
    import torch
    from qpms_gb300.tmatrices import TMatrixGenerator
    from qpms_gb300.workloads import EV, HBAR
    L, lMax, nw = 8, 3, 256
    g = TMatrixGenerator.cylinder(2.25, -12 + 1.2j, 50e-9, 100e-9, L)
    oms = np.linspace(1.6, 2.6, nw) * EV / HBAR
    for _ in range(3):
        g.batch(lMax, oms[:16])
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record(st)
    for _ in range(reps):
        T = g.batch(lMax, oms)
    e1.record(st)
    torch.cuda.synchronize()
    e2e = (time.perf_counter() - t0) / reps
    dev_ms = e0.elapsed_time(e1) / reps
    nq = (6 + 3) * 32  # cylinder, theta in [0, pi/2]: cap 6 panels, side 3 panels, 32 nodes each
    flops = _axsym_flops(L, nq) * nw
    import ctypes as C
    import qpms_gb300
    fp = C.c_double(0)
    fp64 = fp.value if qpms_gb300.lib().qpms_gpu_measure_fp64_peak(C.byref(fp)) == 0 else None
    ach = flops / (dev_ms * 1e-3) / 1e12
    res = {"workload": "cylinder r 50 nm h 100 nm, eps -12+1.2i in 2.25, lMax 3, lMax_extend 8, %d frequencies" % nw,
           "tmatrices_per_s": nw / (dev_ms * 1e-3), "ms_per_batch": dev_ms,
           "fp64": {"achieved_tflops": ach, "peak_tflops": fp64, "frac": ach / fp64 if fp64 else None,
                    "flops_per_batch": flops, "note": "device time includes the batch's H2D/D2H (host API)"},
           "e2e": {"tmatrices_per_s": nw / e2e, "h2d_bytes": 0, "d2h_bytes": int(T.nbytes)}}
    if not args.no_cpu:
        from oracle import orc
        C0 = 299792458.0
        ns = 4
        t0 = time.perf_counter()
        worst = 0.0
        for w in range(ns):
            k, ki = np.sqrt(2.25) * oms[w] / C0, np.sqrt(-12 + 1.2j) * oms[w] / C0
            O = orc.tmatrix_axialsym(lMax, k, ki, "cylinder", (50e-9, 100e-9), lMaxQR=L)
            worst = max(worst, float(np.abs(T[w] - O).max() / np.abs(O).max()))
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"tmatrices_per_s": ns / dt, "cores": 1, "kind": "port",
                               "sample": "first %d frequencies, adaptive quadrature (rtol 1e-10)" % ns,
                               "max_rel_diff_vs_gpu": worst}
        res["gpu_vs_cpu"] = res["tmatrices_per_s"] / res["cpu_baseline"]["tmatrices_per_s"]
    return res


def run_sections(args):
    out = {}
    names = [x for x in args.sections.split(",") if x and x != "none"]
    for nm in names:
        fn = globals().get("section_" + nm)
        if fn is None:
            continue
        try:
            t0 = time.perf_counter()
            out[nm] = fn(args)
            out[nm]["bench_s"] = time.perf_counter() - t0
        except Exception as e:  # a failing secondary section must not hide the headline
            out[nm] = {"error": repr(e)}
    return out


def run_case(spec):
    """One workload for a profiler (ncu) run: no timing, prints a checksum."""
    import torch
    import qpms_gb300
    from qpms_gb300.workloads import EV, HBAR
    f = spec.split(":")
    if f[0] == "finite":  # finite:nx:lMax:nw:mode -- nx x nx spheres, pitch 400 nm, plane-wave scatter
        nx, lMax, nw, mode = int(f[1]), int(f[2]), int(f[3]), int(f[4])
        ss = qpms_gb300.ScatteringSystem(_sq(nx, 400e-9), 50e-9, -12 + 1.2j, 2.25, lMax)
        r = ss.planewave_scatter_batch(np.linspace(1.6, 2.6, nw) * EV / HBAR, mode=mode)
        torch.cuda.synchronize()
        print("finite", nx, lMax, nw, "max resid", float(r["residual"].max()))
    elif f[0] == "dense":
        N, nrhs, mode = int(f[1]), int(f[2]), int(f[3])
        dev = torch.device("cuda:0")
        g = torch.Generator(device=dev)
        g.manual_seed(N)
        M = torch.randn(N, N, dtype=torch.complex128, device=dev, generator=g) / N ** 0.5
        M += 2 * torch.eye(N, dtype=torch.complex128, device=dev)
        B = torch.randn(nrhs, N, dtype=torch.complex128, device=dev, generator=g)
        X = torch.empty_like(B)
        res = np.zeros(1)
        it = np.zeros(1, dtype=np.int32)
        rc = qpms_gb300.lib().qpms_gpu_dense_solve(N, nrhs, M.data_ptr(), B.data_ptr(), X.data_ptr(), mode,
                                                  res.ctypes.data, it.ctypes.data)
        print("dense", N, nrhs, mode, "rc", rc, "resid", res[0], "iters", it[0])
    elif f[0] == "scan":
        from qpms_gb300.workloads import honeycomb_lattice, honeycomb_path, square_lattice, square_path
        lat, nw, nk, mode = f[1], int(f[2]), int(f[3]), int(f[4])
        if lat == "bilayer":  # square lattice, second particle shifted (a/2, a/2, 150 nm): layered Ewald sums
            b1, b2, pos = square_lattice()
            pos = np.array([[0.0, 0.0, 0.0], [290e-9, 290e-9, 150e-9]])
        else:
            b1, b2, pos = square_lattice() if lat == "square" else honeycomb_lattice()
        ss = qpms_gb300.ScatteringSystem(pos, 80e-9, -12 + 1.2j, 2.25, 3, lattice=(b1, b2))
        kp = (honeycomb_path if lat == "honeycomb" else square_path)(n=nk)
        r = ss.dispersion_scan(np.linspace(1.6, 2.6, nw) * EV / HBAR, kp, mode=mode)
        print("scan", lat, nw, nk, "logdet sum", float(np.sum(r["logdet"])), "max resid", float(r["residual"].max()))
    elif f[0] == "field":
        nx, npts, lMax = int(f[1]), int(f[2]), int(f[3])
        pos = _sq(nx, 400e-9)
        ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, lMax)
        rng = np.random.default_rng(1)
        cv = rng.normal(size=ss.fecv_size) + 1j * rng.normal(size=ss.fecv_size)
        pts = rng.uniform(-nx * 2e-7, nx * 2e-7, size=(npts, 3))
        E = ss.scattered_E(1.6e7, cv, pts)
        print("field", nx, npts, lMax, "sum |E|", float(np.abs(E).sum()))
    elif f[0] == "axsym":
        from qpms_gb300.tmatrices import TMatrixGenerator
        L, nw = int(f[1]), int(f[2])
        g = TMatrixGenerator.cylinder(2.25, -12 + 1.2j, 50e-9, 100e-9, L)
        T = g.batch(3, np.linspace(1.6, 2.6, nw) * EV / HBAR)
        print("axsym", L, nw, "sum |T|", float(np.abs(T).sum()))
    elif f[0] == "beyn":
        nx, nodes, mode = int(f[1]), int(f[2]), int(f[3])
        xs = (np.arange(nx) - (nx - 1) / 2) * 400e-9
        X_, Y_ = np.meshgrid(xs, xs, indexing="ij")
        pos = np.stack([X_.ravel(), Y_.ravel(), np.zeros(nx * nx)], 1)
        ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, 2)
        r = ss.find_modes(2.1 * EV / HBAR, 0.05 * EV / HBAR, 0.005 * EV / HBAR, contour_points=nodes,
                          rank_tol=1e-4, l=64, seed=12345, mode=mode)
        print("beyn", nx, nodes, "neig", r["eigval"].size, "node resid", r["node_residual_max"])
    torch.cuda.synchronize()


def main():
    args = parse()
    if args.case:
        run_case(args.case)
        return
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
