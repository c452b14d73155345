"""Benchmark of the QPMS mode-problem hot path on GB300.

Headline workload (one "step"): the serving configuration -- a seeded trace
of 60 plane-wave scattering solves (70 % finite clusters of 16-400 spheres on
a jittered 400 nm grid, r 50 nm, eps -12+1.2i in eps 2.25, lMax 2-4, i.e.
736-18,912 unknowns; 30 % single (omega, k) solves of the square and
honeycomb lattices of the dispersion configuration), all submitted at once to
the continuous-batching server (qpms_gpu_server_*, 8 worker streams).  One
solve = assembly of M = I - T S (or I - T W), LU, solve for the scattered
coefficients f at <= 1e-10 relative FP64 residual, sigma_ext.

value:   solves/s of the batched mixed-precision serving path (complex64 LU
         on the tensor cores + FP64 iterative refinement), systems resident on
         the device, results as sigma_ext and residual (CUDA events around each
         step after a device synchronise, max over ranks).
latency: p50/p99 per request (submit to done) over the timed steps, and at
         Poisson arrival rates.
plain_fp64_path: the same full trace through the plain FP64 GPU path
         (complex128 LU), one saturated pass; mixed_vs_plain = the ratio.
e2e:     the same trace through qpms_gpu_server_submit with host output
         buffers for every solution vector f (device-to-host inside the
         timed region).
roofline: the kernel with the largest device time in the timed steps, from
         the library's live per-launch CUDA-event timing.
cpu_baseline / --impl reference: the oracle (C restatement of the reference's
         assembly; numpy LAPACK zgesv for the solves, all host cores) on the
         requests of the trace in order, within a bounded time.

Secondary objects in the same JSON line (rank 0), each the other workloads of
the path: translation (10^6 vectors x J {1,3} x lMax {3,6}), modeproblem
(4x4 array, 32 omegas), dispersion (square / honeycomb lattices), beyn
(30 x 30 array, 14,400 unknowns, 64 nodes, 64 probe columns), field, axsym.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s + p50/p99 latency vs plain FP64 GPU path at ≤1e-10 rel. residual"
UNIT = "solves/s"
N_REQ = 60
TRACE_SEED = 5
WORKERS = 8
EPS_I, EPS_E = -12 + 1.2j, 2.25
C0 = 299792458.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--requests", type=int, default=N_REQ)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workers", type=int, default=WORKERS, help="worker streams of the serving loop")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 pass of the trace")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of the CPU baseline sample")
    ap.add_argument("--clocks-out", default=None, help="file for the nvidia-smi clock samples (default: a temp file)")
    ap.add_argument("--sections", default="translation,modeproblem,dispersion,beyn,field,axsym",
                    help="secondary workloads reported beside the headline (comma list, or 'none')")
    ap.add_argument("--nvec", type=int, default=1_000_000, help="translation section: vectors per launch")
    ap.add_argument("--case", default=None,
                    help="run one small case for a profiler and exit: dense:N:NRHS:MODE, "
                         "scan:{square,honeycomb,bilayer}:NW:NK:MODE, finite:NX:LMAX:NW:MODE, "
                         "field:NX:NPTS:LMAX, axsym:L:NW, beyn:NX:NODES:MODE, serve:NREQ:MODE, "
                         "trans:NVEC:LMAX")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "fallback": True}


def isolated_tc_rate(peaks):
    """The dominant kernel with the GPU to itself: one mixed dense solve of
    14,400 unknowns (random well-conditioned matrix, one right-hand side), every
    tc_gemm launch timed with CUDA events on its stream (second of two solves)."""
    import torch
    import qpms_gb300
    from qpms_gb300 import _lib
    L = qpms_gb300.lib()
    dev = torch.device("cuda:0")
    N = 14400
    g = torch.Generator(device=dev)
    g.manual_seed(N)
    M = torch.randn(N, N, dtype=torch.complex128, device=dev, generator=g) / N ** 0.5
    M += 2 * torch.eye(N, dtype=torch.complex128, device=dev)
    B = torch.randn(1, N, dtype=torch.complex128, device=dev, generator=g)
    X = torch.empty_like(B)
    res, it = np.zeros(1), np.zeros(1, dtype=np.int32)
    for rep in range(2):
        if rep == 1:
            _lib.kernel_timing(True)
        rc = L.qpms_gpu_dense_solve(N, 1, M.data_ptr(), B.data_ptr(), X.data_ptr(), 1, res.ctypes.data,
                                    it.ctypes.data)
        if rc:
            return {"error": qpms_gb300.last_error()}
    torch.cuda.synchronize()
    kt = _lib.kernel_timing_get()
    _lib.kernel_timing(False)
    del M, B, X
    if "tc_gemm" not in kt:
        return None
    ms, work, n = kt["tc_gemm"]
    ach = work / (ms * 1e-3) / 1e12
    pk = peaks.get("bf16_tflops") or 1900.0
    return {"achieved": ach, "peak": pk, "frac": ach / pk, "unit": "TFLOP/s", "launches": n,
            "ms": ms, "peak_source": "measured burst (MEASURED_PEAKS.json bf16_tflops)",
            "of": "one 14,400-unknown mixed dense solve alone on the GPU (%d tc_gemm launches)" % n}


def profile_json(name):
    """A figure from a committed ncu summary under profiles/ (json), if present."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", name)))
    except Exception:
        return None


def fp64_probe():
    import ctypes as C
    import qpms_gb300
    fp = C.c_double(0)
    return fp.value if qpms_gb300.lib().qpms_gpu_measure_fp64_peak(C.byref(fp)) == 0 else None


def _sq(nx, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * nx)], 1)


# ---------------- the serving trace ----------------
def trace_specs(n):
    from qpms_gb300.workloads import serving_requests
    return serving_requests(n, seed=TRACE_SEED)


def spec_unknowns(s):
    if s["kind"] == "finite":
        return len(s["positions"]) * 2 * s["lMax"] * (s["lMax"] + 2)
    return (1 if s["lattice"] == "square" else 2) * 30


def build_trace(specs):
    """ScatteringSystem objects of the trace (device-resident particle data) and request dicts."""
    import qpms_gb300
    from qpms_gb300.workloads import honeycomb_lattice, square_lattice
    b1, b2, p1 = square_lattice()
    h1, h2, p2 = honeycomb_lattice()
    lat = {"square": qpms_gb300.ScatteringSystem(p1, 80e-9, EPS_I, EPS_E, 3, lattice=(b1, b2)),
           "honeycomb": qpms_gb300.ScatteringSystem(p2, 80e-9, EPS_I, EPS_E, 3, lattice=(h1, h2))}
    reqs = []
    for s in specs:
        if s["kind"] == "finite":
            reqs.append({"system": qpms_gb300.ScatteringSystem(s["positions"], 50e-9, EPS_I, EPS_E, s["lMax"]),
                         "omega": s["omega"]})
        else:
            reqs.append({"system": lat[s["lattice"]], "omega": s["omega"], "k": s["k"]})
    return reqs, lat


class OracleSolver:
    """The reference path on the host for one request: M from the oracle's C
    restatement of the assembly (scatsystem.c:1283-1357 finite; the Ewald
    lattice sums for lattices), f = M^-1 T a by LAPACK zgesv (numpy, all host
    cores) as the reference's zgetrf/zgetrs (scatsystem.c:2202-2273)."""

    def __init__(self):
        from oracle import orc
        from qpms_gb300.workloads import honeycomb_lattice, square_lattice
        self.orc = orc
        self.calcs = {}
        self.lat = {"square": square_lattice(), "honeycomb": honeycomb_lattice()}

    def calc(self, lMax):
        if lMax not in self.calcs:
            self.calcs[lMax] = self.orc.TransCalculator(lMax)
        return self.calcs[lMax]

    def solve(self, s):
        orc = self.orc
        om = s["omega"]
        k = np.sqrt(EPS_E) * om / C0
        if s["kind"] == "finite":
            lMax, pos, r = s["lMax"], np.ascontiguousarray(s["positions"]), 50e-9
        else:
            lMax, r = 3, 80e-9
            b1, b2, pos = self.lat[s["lattice"]]
        Td = orc.tmatrix_sphere_diag(lMax, r, om, EPS_I, EPS_E)
        T = np.ascontiguousarray(np.broadcast_to(np.diag(Td), (pos.shape[0], Td.size, Td.size)))
        if s["kind"] == "finite":
            M = orc.finite_modeproblem(self.calc(lMax), pos, T, k)
            kvec, E = np.array([0, 0, k]), np.array([1, 0, 0])
        else:
            bx, by = s["k"]
            area = abs(b1[0] * b2[1] - b1[1] * b2[0])
            kv = np.array([bx, by, 0.0])
            eta = orc.adjusted_eta(area, k, kv, lMax)
            M = orc.periodic_modeproblem(self.calc(lMax), pos, T, k, b1, b2, kv, eta)
            kz = np.sqrt(max(k * k - bx * bx - by * by, 0.0))
            kvec = np.array([bx, by, kz])
            E = np.array([1.0, 0, 0]) - kvec[0] * kvec / max(np.dot(kvec, kvec), 1e-300)
            E = E / np.linalg.norm(E)
        a = orc.planewave_full(lMax, pos, kvec, E)
        f = np.linalg.solve(M, np.tile(Td, pos.shape[0]) * a)
        return -np.vdot(a, f).real / k ** 2


def cpu_baseline(specs, budget_s, gpu_sigma=None):
    """Oracle on the trace's requests in order until budget_s is spent."""
    from oracle import orc
    o = OracleSolver()
    t0 = time.perf_counter()
    done, unk, worst = 0, 0, 0.0
    for i, s in enumerate(specs):
        if time.perf_counter() - t0 > budget_s:
            break
        sig = o.solve(s)
        done += 1
        unk += spec_unknowns(s)
        if gpu_sigma is not None:
            worst = max(worst, abs(sig - gpu_sigma[i]) / max(abs(sig), 1e-300))
    dt = time.perf_counter() - t0
    out = {"value": done / dt, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
           "sample": "first %d of %d trace requests in order (mean %.0f unknowns; trace mean %.0f), %.1f s; "
                     "oracle C assembly + numpy LAPACK zgesv" % (done, len(specs), unk / max(done, 1),
                                                                 np.mean([spec_unknowns(x) for x in specs]), dt)}
    if gpu_sigma is not None:
        out["max_rel_diff_sigma_ext_vs_gpu"] = worst
    return out


def run_reference(args, ws, rank):
    """The reference's CPU path (the oracle's restatement; the reference itself
    needs GSL, LAPACKE and AMOS, absent here) on the serving trace: each step a
    bounded sample of the trace's requests in order."""
    if rank != 0:
        return
    specs = trace_specs(args.requests)
    budget = min(args.cpu_seconds, 20.0)
    for _ in range(args.warmup):
        cpu_baseline(specs[:2], 1e9)
    vals, cb = [], None
    t_all = time.perf_counter()
    for _ in range(max(1, args.steps)):
        cb = cpu_baseline(specs, budget)
        vals.append(cb["value"])
    v = float(np.median(vals))
    cb["value"] = v
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * (time.perf_counter() - t_all) / max(1, args.steps),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded serving trace)", "config": config_dict(args, 1, specs),
           "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference C path needs GSL + LAPACKE + AMOS (absent); timed the oracle's C restatement with "
                   "numpy LAPACK"}
    print(json.dumps(out), flush=True)


def config_dict(args, ws, specs):
    unk = [spec_unknowns(s) for s in specs]
    return {"workload": "serving trace: %d seeded plane-wave scattering requests, 70%% finite clusters of 16-400 "
                        "spheres (jittered 400 nm grid, r 50 nm, lMax 2-4), 30%% single (omega, k) solves of the "
                        "square / honeycomb lattices (a 580 nm, r 80 nm, lMax 3); all submitted at once to %d "
                        "worker streams" % (len(specs), args.workers),
            "requests": len(specs), "mean_unknowns": float(np.mean(unk)), "max_unknowns": int(max(unk)),
            "workers": args.workers, "parallelism": "replicas (one trace per rank)" if ws > 1 else "single GPU",
            "l2": "no flush needed: each step assembles and factors %.1f GB of FP64 mode-problem matrices, "
                  ">> 129 MB L2" % (16.0 * sum(u * u for u in unk) / 1e9)}


def _serve_pass(srv, reqs, want_f, arrivals=None):
    from qpms_gb300.serving import run_trace
    results, summ = run_trace(srv, reqs, arrivals, want_f=want_f)
    lat = [r["t_done"] - r["t_submit"] for r in results]
    return results, summ, lat


def run_ours(args, ws, rank, local):
    import torch
    import qpms_gb300
    from qpms_gb300 import _lib
    from qpms_gb300.serving import Server
    from qpms_gb300.workloads import poisson_arrivals

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = qpms_gb300.lib()
    specs = trace_specs(args.requests)
    reqs, _lat_systems = build_trace(specs)
    srv = Server(mode=1, workers=args.workers)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(max(3, args.warmup)):
        _serve_pass(srv, reqs, False)
    barrier()
    clk_path = args.clocks_out or os.path.join(tempfile.gettempdir(), "qpms_bench_clocks_%d.csv" % os.getpid())
    clk = ClockSampler(clk_path)
    step_ms, lat_all, resid_max, sig = [], [], 0.0, None
    launches0 = L.qpms_gpu_kernel_launch_count()
    stream = torch.cuda.current_stream(dev)
    with clk:
        barrier()
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            results, summ, lat = _serve_pass(srv, reqs, False)
            torch.cuda.synchronize()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            lat_all += lat
            resid_max = max(resid_max, summ["max_residual"])
            sig = [r["sigma_ext"] for r in results]
            if summ["failed"]:
                raise RuntimeError("serving step: %d requests failed" % summ["failed"])
        barrier()
    launches = L.qpms_gpu_kernel_launch_count() - launches0
    # one more pass with the library's per-launch CUDA-event timing on (kept out of
    # the timed steps: recording two events per launch slows the small kernels)
    _lib.kernel_timing(True)
    _serve_pass(srv, reqs, False)
    torch.cuda.synchronize()
    kt = _lib.kernel_timing_get()
    _lib.kernel_timing(False)
    total_ms = float(np.sum(step_ms))
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = len(reqs) * args.steps * ws / (total_ms / 1e3)
    st = srv.stats()

    # Poisson arrivals (continuous batching with requests arriving while others run)
    sweep = {}
    if rank == 0:
        for rate in (20.0, 60.0):
            _, summ, lat = _serve_pass(srv, reqs, False, poisson_arrivals(len(reqs), rate, 1))
            sweep["%g_per_s" % rate] = {"p50_ms": summ["p50_ms"], "p99_ms": summ["p99_ms"],
                                        "solves_per_s": summ["solves_per_s"], "mean_batch": summ["mean_batch"],
                                        "max_residual": summ["max_residual"]}

    # end to end: every solution vector back to host memory inside the timed region
    e2e = None
    if not args.no_e2e:
        ts, d2h, h2d = [], 0, 0
        for rep in range(1 + max(1, min(args.steps, 3))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            results, summ, _ = _serve_pass(srv, reqs, True)
            torch.cuda.synchronize()
            if rep:
                ts.append(time.perf_counter() - t0)
            from qpms_gb300.serving import _Request, _Result
            import ctypes
            d2h = int(sum(16 * spec_unknowns(x) + ctypes.sizeof(_Result) for x in specs))
            h2d = int(len(specs) * ctypes.sizeof(_Request))
        e2e = {"value": len(reqs) * ws / float(np.median(ts)), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": float(np.median(ts)) * 1e3,
               "path": "qpms_gpu_server_submit / _wait (C-ABI): request structs in, every solution vector f "
                       "plus sigma_ext and residual out to host memory"}
    srv.close()

    # the plain FP64 GPU path on the same full trace
    plain = None
    if rank == 0 and not args.no_plain:
        psrv = Server(mode=0, workers=args.workers)
        _serve_pass(psrv, reqs[:2], False)
        torch.cuda.synchronize()
        _, psumm, plat = _serve_pass(psrv, reqs, False)
        torch.cuda.synchronize()
        psrv.close()
        plain = {"solves_per_s": psumm["solves_per_s"], "makespan_s": psumm["makespan_s"],
                 "p50_ms": float(np.percentile(plat, 50) * 1e3), "p99_ms": float(np.percentile(plat, 99) * 1e3),
                 "max_residual": psumm["max_residual"], "requests": len(reqs),
                 "path": "same server, complex128 LU (partial pivoting batched / blocked LU without pivoting "
                         "after the random butterfly), FP64 throughout"}

    if rank == 0:
        peaks = measured_peaks()
        roof, kernels = roofline(kt, peaks)
        if roof and roof.get("bound") == "tensor":
            roof["isolated"] = isolated_tc_rate(peaks)
        cb = None if args.no_cpu else cpu_baseline(specs, args.cpu_seconds, sig)
        smry = clk.summary(local)
        sections = run_sections(args)
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
               "warmup": max(3, args.warmup), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "c64 LU + f64 refinement (f64 assembly)",
               "data": "synthetic (seeded serving trace; config distributions)",
               "config": config_dict(args, ws, specs),
               "latency_ms": {"p50": float(np.percentile(lat_all, 50) * 1e3),
                              "p99": float(np.percentile(lat_all, 99) * 1e3),
                              "of": "per request, submit to done, saturated (all %d submitted at once)" % len(reqs),
                              "poisson": sweep},
               "max_residual": resid_max,
               "plain_fp64_path": plain,
               "mixed_vs_plain": (value / ws / plain["solves_per_s"]) if plain else None,
               "kernels": kernels, "roofline": roof, "cpu_baseline": cb, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": smry, "server": st}
        out.update(sections)
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def roofline(kt, peaks):
    """Roofline object of the kernel kind with the largest device time in the
    timed steps (live CUDA-event timing of every launch on its own stream)."""
    from qpms_gb300._lib import KERNEL_KINDS  # noqa: F401
    kernels = {k: {"ms": v[0], "launches": v[2], "work": v[1]} for k, v in kt.items()}
    if not kt:
        return None, kernels
    top = max(kt, key=lambda k: kt[k][0])
    ms, work, n = kt[top]
    fp64 = None
    if top == "tc_gemm":
        ach = work / (ms * 1e-3) / 1e12
        pk = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops")
        tr = profile_json("tc_gemm_traffic.json")
        roof = {"bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s", "frac": ach / pk,
                "traffic": tr.get("bytes_per_launch") if tr else None,
                "traffic_of": tr.get("of") if tr else None,
                "peak_source": "measured (MEASURED_PEAKS.json bf16_tflops_sustained)" if not peaks.get("fallback")
                else "fallback 1.7 PFLOP/s sustained",
                "kernel": "tc_gemm_kernel (tcgen05 bf16 digit products, FP32 accumulate)",
                "launches": n, "ms_per_launch": ms / n,
                "work": "executed bf16 flops (2 x rows x cols x K per digit product)",
                "concurrency": "the worker streams run concurrently: a launch's CUDA-event duration includes the "
                               "time it shares the SMs with other requests' kernels, so this is the per-launch "
                               "rate under that sharing (the same kernel alone: 'isolated')"}
    else:
        fp64 = fp64_probe()
        ach = work / (ms * 1e-3) / 1e9
        pk = peaks.get("hbm_gbs")
        roof = {"bound": "hbm", "achieved": ach, "peak": pk, "unit": "GB/s", "frac": ach / pk, "traffic": None,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)", "kernel": top, "launches": n,
                "ms_per_launch": ms / n, "fp64_probe_tflops": fp64}
    for k, v in kernels.items():
        v["share"] = v["ms"] / sum(x["ms"] for x in kernels.values())
    return roof, kernels


# ---------------- secondary workloads ----------------
TR_LMAXES = (3, 6)
TR_JS = (1, 3)


def _trans_bytes(nvec, lMax):
    ne2 = (lMax * (lMax + 2)) ** 2
    return nvec * (2 * ne2 * 16 + 32)


def _trans_flops(lMax):
    from qpms_gb300.translations import multipliers_export
    A, B = multipliers_export(lMax)
    return 4 * (A.size + B.size)  # two FP64 FMAs per real-coefficient x complex term


def section_translation(args):
    """Batched translation coefficients: 10^6 seeded vectors (|r| log-uniform
    50 nm-10 um, complex k) x J in {1, 3} x lMax in {3, 6}, complex128 A/B
    arrays, device-resident inputs and outputs; e2e through the host entry
    point; CPU oracle on a bounded sample."""
    import torch
    import qpms_gb300
    from qpms_gb300.workloads import translation_vectors
    dev = torch.device("cuda:0")
    n = args.nvec
    kr, th, ph = translation_vectors(n, seed=1000)
    tkr, tth, tph = (torch.from_numpy(x).to(dev) for x in (kr, th, ph))
    calcs = {lm: qpms_gb300.trans_calculator(lm) for lm in TR_LMAXES}
    st = torch.cuda.current_stream(dev)
    res = {"workload": "%d seeded vectors x J {1,3} x lMax {3,6}, complex128 A/B arrays, FP64" % n}
    tot_ms, per = 0.0, {}
    for lm in TR_LMAXES:
        ne = lm * (lm + 2)
        A = torch.empty((n, ne, ne), dtype=torch.complex128, device=dev)
        B = torch.empty_like(A)
        for J in TR_JS:
            for _ in range(2):
                calcs[lm].get_AB_arrays_device(tkr, tth, tph, J, A, B, stream=st.cuda_stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            for _ in range(3):
                calcs[lm].get_AB_arrays_device(tkr, tth, tph, J, A, B, stream=st.cuda_stream)
            e1.record(st)
            torch.cuda.synchronize()
            per[(lm, J)] = e0.elapsed_time(e1) / 3
            tot_ms += per[(lm, J)]
        del A, B
        torch.cuda.empty_cache()
    solves = n * len(TR_LMAXES) * len(TR_JS)
    res["solves_per_s"] = solves / (tot_ms / 1e3)
    res["ms_per_launch"] = {"lMax%d_J%d" % k: v for k, v in per.items()}
    peaks = measured_peaks()
    fp64 = fp64_probe()
    dur = float(np.mean([per[(6, J)] for J in TR_JS])) / 1e3
    gbs = _trans_bytes(n, 6) / dur / 1e9
    tfl = _trans_flops(6) * n / dur / 1e12
    tr = profile_json("trans_ab_traffic.json")
    res["roofline"] = {"bound": "fp64", "kernel": "trans_ab_kernel<6>", "achieved": tfl, "unit": "TFLOP/s",
                       "peak": fp64, "frac": tfl / fp64 if fp64 else None,
                       "peak_source": "library DFMA probe qpms_gpu_measure_fp64_peak",
                       "hbm": {"achieved": gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                               "frac": gbs / peaks.get("hbm_gbs")},
                       "traffic": tr.get("lmax6") if tr else None}
    if not args.no_e2e:
        L = calcs[3]._L
        pk, pt, pp = (torch.from_numpy(x).pin_memory() for x in (kr, th, ph))
        nsub = min(n, 50_000)
        bufs = {lm: (torch.empty((nsub, (lm * (lm + 2)) ** 2), dtype=torch.complex128).pin_memory(),
                     torch.empty((nsub, (lm * (lm + 2)) ** 2), dtype=torch.complex128).pin_memory())
                for lm in TR_LMAXES}
        t0 = time.perf_counter()
        d2h = 0
        for lm in TR_LMAXES:
            hA, hB = bufs[lm]
            for J in TR_JS:
                for o in range(0, n, nsub):
                    m = min(nsub, n - o)
                    rc = L.qpms_gpu_trans_AB_arrays_batch_host(calcs[lm].c, m, pk.data_ptr() + 16 * o,
                                                               pt.data_ptr() + 8 * o, pp.data_ptr() + 8 * o, None, J,
                                                               hA.data_ptr(), hB.data_ptr())
                    if rc:
                        raise RuntimeError(L.qpms_gpu_last_error())
                    d2h += 2 * 16 * hA.shape[1] * m
        dt = time.perf_counter() - t0
        res["e2e"] = {"solves_per_s": solves / dt, "d2h_bytes": d2h, "h2d_bytes": 32 * n * 4,
                      "path": "qpms_gpu_trans_AB_arrays_batch_host, pinned host buffers"}
    if not args.no_cpu:
        from oracle import orc
        total = 0.0
        samples = []
        for lm in TR_LMAXES:
            c = orc.TransCalculator(lm)
            for J in TR_JS:
                m = 2000 if lm == 6 else 20000
                k2, t2, p2 = translation_vectors(m, seed=99)
                t0 = time.perf_counter()
                c.get_AB_batch(k2, t2, p2, J)
                d = time.perf_counter() - t0
                total += n * d / m
                samples.append("lMax%d J%d: %d in %.2fs" % (lm, J, m, d))
        res["cpu_baseline"] = {"solves_per_s": solves / total, "cores": orc.num_threads(), "kind": "port",
                               "sample": "; ".join(samples) + " (scaled to the full workload)"}
        res["gpu_vs_cpu"] = res["solves_per_s"] / res["cpu_baseline"]["solves_per_s"]
    return res


def section_modeproblem(args):
    """Finite 4x4 array, lMax 2, 32 frequencies: plain vs mixed, and the CPU oracle."""
    import torch
    import qpms_gb300
    from qpms_gb300.workloads import EV, HBAR
    ss = qpms_gb300.ScatteringSystem(_sq(4, 400e-9), 50e-9, EPS_I, EPS_E, 2)
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
            orc.finite_sphere_scatter(c, _sq(4, 400e-9), 50e-9, EPS_I, EPS_E, w)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"solves_per_s": 32 / dt, "cores": orc.num_threads(), "kind": "port",
                               "sample": "all 32 frequencies"}
    return out


def section_dispersion(args):
    """Square (30 x 30) and honeycomb (60 x 60) lattices, lMax 3: a 32 omega x
    256 k sample of the 4096 k x 256 omega scans, mixed and plain; CPU oracle
    on a few points; live timing of the lattice-sum kernel."""
    import torch
    import qpms_gb300
    from qpms_gb300 import _lib
    from qpms_gb300.workloads import EV, HBAR, honeycomb_lattice, honeycomb_path, square_lattice, square_path
    out = {"workload": "sample of 32 omegas x 256 k of each 4096 k x 256 omega scan, lMax 3, r 80 nm, a 580 nm"}
    om = np.linspace(1.6, 2.6, 32) * EV / HBAR
    for lat in ("square", "honeycomb"):
        b1, b2, pos = square_lattice() if lat == "square" else honeycomb_lattice()
        ss = qpms_gb300.ScatteringSystem(pos, 80e-9, EPS_I, EPS_E, 3, lattice=(b1, b2))
        kp = (square_path if lat == "square" else honeycomb_path)(n=256)
        ss.dispersion_scan(om[:2], kp[:8])
        d = {}
        for mode, name in ((0, "plain_fp64"), (1, "mixed")):
            if mode == 1:
                _lib.kernel_timing(True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = ss.dispersion_scan(om, kp, mode=mode)
            dt = time.perf_counter() - t0
            d[name] = {"points_per_s": om.size * kp.shape[0] / dt, "max_residual": float(r["residual"].max()),
                       "full_scan_s": 4096 * 256 / (om.size * kp.shape[0] / dt)}
            if mode == 1:
                kt = _lib.kernel_timing_get()
                _lib.kernel_timing(False)
                d[name]["kernels_ms"] = {k: v[0] for k, v in kt.items()}
                if "ewald" in kt:
                    ms, work, n = kt["ewald"]
                    d["roofline"] = {"bound": "fp64", "kernel": "ewald_assemble_kernel<3> (+ sr table)",
                                     "ms": ms, "launches": n, "share_of_scan": ms / (dt * 1e3),
                                     "note": "FP64-pipe bound (special functions per lattice point); "
                                             "output bytes %.2f GB/s" % (work / (ms * 1e-3) / 1e9)}
        d["mixed_vs_plain"] = d["mixed"]["points_per_s"] / d["plain_fp64"]["points_per_s"]
        if not args.no_cpu:
            o = OracleSolver()
            t0 = time.perf_counter()
            npts = 0
            for i in range(4):
                o.solve({"kind": "lattice", "lattice": lat, "omega": om[8 * i], "k": tuple(kp[60 * i])})
                npts += 1
            dt = time.perf_counter() - t0
            d["cpu_baseline"] = {"points_per_s": npts / dt, "cores": 1, "kind": "port",
                                 "sample": "%d (omega, k) points: oracle Ewald assembly (adaptive quadrature as the "
                                           "reference) + LAPACK solve" % npts}
            d["gpu_vs_cpu"] = d["mixed"]["points_per_s"] / d["cpu_baseline"]["points_per_s"]
        out[lat] = d
    return out


BEYN_RA = {"centre_eV": (2.064, -0.020), "rRe_eV": 0.006, "rIm_eV": 0.006}


def section_beyn(args):
    """30 x 30 array, r 60 nm, lMax 2 (14,400 unknowns), 64 nodes, 64 probe
    columns: the configured ellipse (2.1 eV, half-axes 0.05 / 0.005 eV) with
    the relative rank test, and the ellipse below the Rayleigh anomaly that
    holds the array's highest-Q modes, checked against the FP64 oracle's
    eigenvalues (tests/golden/beyn_30x30.json)."""
    import qpms_gb300
    from qpms_gb300 import _lib
    from qpms_gb300.workloads import EV, HBAR
    ss = qpms_gb300.ScatteringSystem(_sq(30, 400e-9), 60e-9, EPS_I, EPS_E, 2)
    N, L = ss.fecv_size, 64
    c, rr, ri = 2.1 * EV / HBAR, 0.05 * EV / HBAR, 0.005 * EV / HBAR
    Lb = qpms_gb300.lib()
    ss.find_modes(c, rr, ri, contour_points=1, rank_tol=-1e-10, rank_min_sel=0, l=L, seed=12345, mode=1)
    l0, g0 = Lb.qpms_gpu_kernel_launch_count(), Lb.qpms_gpu_graph_replay_count()
    r = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=-1e-10, rank_min_sel=0, l=L, seed=12345, mode=1)
    launches = (Lb.qpms_gpu_kernel_launch_count() - l0) / 64
    replays = (Lb.qpms_gpu_graph_replay_count() - g0) / 64
    # the same nodes with every launch issued eagerly (no CUDA graphs)
    os.environ["QPMS_GB300_GRAPHS"] = "0"
    try:
        re_ = ss.find_modes(c, rr, ri, contour_points=16, rank_tol=-1e-10, rank_min_sel=0, l=L, seed=12345, mode=1)
    finally:
        del os.environ["QPMS_GB300_GRAPHS"]
    # per-kind kernel times on a shorter contour (per-launch timing runs eagerly)
    _lib.kernel_timing(True)
    ss.find_modes(c, rr, ri, contour_points=8, rank_tol=-1e-10, rank_min_sel=0, l=L, seed=12345, mode=1)
    kt = _lib.kernel_timing_get()
    _lib.kernel_timing(False)
    from oracle import beyn as ob
    z, dz = ob.contour_ellipse(c, rr, ri, 64)
    scale = ob.rank_scale(dz, qpms_gb300.beyn.probe_matrix(N, L, 12345))
    sv = np.asarray(r["ranktest_SV"]) / scale
    node_s = r["quadrature_s"] / 64
    lu_flops = 8.0 / 3.0 * N ** 3 + 8.0 * N * N * L  # LU + forward/back substitution (real flops)
    out = {"workload": "30x30 spheres r 60 nm, lMax 2 (14400 x 14400), 64 nodes, L 64",
           "configured_contour": {"ellipse_eV": "2.1 +- 0.05 (Re) / 0.005 (Im)", "neig": int(r["eigval"].size),
                                  "rank_test": "sigma_k > 1e-10 x sum|dz| ||Vhat||_F / sqrt(L)",
                                  "sigma_over_scale_max": float(sv[0]), "sigma_over_scale_next": float(sv[1]),
                                  "total_s": r["total_s"], "quadrature_s": r["quadrature_s"],
                                  "node_s": node_s, "node_residual_max": r["node_residual_max"],
                                  "refine_iters_max": r["node_refine_iters_max"],
                                  "note": "no eigenfrequency of this array lies inside (its modes have "
                                          "Im(hbar omega) <= -0.0159 eV); K = 0 is the valid result"},
           "lu_tflops_per_node": lu_flops / node_s / 1e12,
           "graphs": {"launches_per_node": launches, "graph_replays_per_node": replays, "node_s": node_s,
                      "node_s_eager": re_["quadrature_s"] / 16,
                      "note": "the dense solver's factorisation and solve launch sequences are captured at the "
                              "second node and replayed after; eager = QPMS_GB300_GRAPHS=0, 16 nodes"}}
    if "tc_gemm" in kt:
        ms, work, n = kt["tc_gemm"]
        out["tc_gemm"] = {"ms_per_node": ms / 8, "launches_per_node": n / 8,
                          "tflops_bf16_executed": work / (ms * 1e-3) / 1e12,
                          "frac_of_sustained": work / (ms * 1e-3) / 1e12 /
                          (measured_peaks().get("bf16_tflops_sustained") or 1700.0)}
    out["kernels_ms_per_node"] = {k: v[0] / 8 for k, v in kt.items()}
    # the modes below the Rayleigh anomaly, against the FP64 oracle's eigenvalues
    cr = complex(*BEYN_RA["centre_eV"]) * EV / HBAR
    q = ss.find_modes(cr, BEYN_RA["rRe_eV"] * EV / HBAR, BEYN_RA["rIm_eV"] * EV / HBAR, contour_points=64,
                      rank_tol=-1e-4, rank_min_sel=0, l=L, seed=12345, mode=1)
    ev = np.sort_complex(q["eigval"])
    ra = {"ellipse_eV": "2.064-0.020i +- 0.006 / 0.006", "neig": int(ev.size),
          "eigval_eV": [[float(x.real * HBAR / EV), float(x.imag * HBAR / EV)] for x in ev],
          "total_s": q["total_s"]}
    try:
        g = json.load(open(os.path.join(ROOT, "tests", "golden", "beyn_30x30.json")))
        ge = np.sort_complex(np.array([complex(*x) for x in g["eigval"]]))
        if ge.size == ev.size:
            ra["max_rel_diff_vs_oracle"] = float(np.max(np.abs(ev - ge) / np.abs(ge)))
        ra["oracle_neig"] = int(ge.size)
        ra["oracle_seconds_64_nodes"] = g.get("oracle_seconds")
    except OSError:
        pass
    out["below_rayleigh_anomaly"] = ra
    one = {}
    for mode in (0, 1):
        p = ss.find_modes(c, rr, ri, contour_points=1, rank_tol=-1e-10, rank_min_sel=0, l=L, seed=12345, mode=mode)
        one[mode] = p["quadrature_s"]
    out["per_node_s"] = {"plain_fp64": one[0], "mixed": one[1], "mixed_in_64_node_run": node_s}
    out["plain_fp64_estimate_s"] = 64 * one[0]
    out["mixed_vs_plain"] = one[0] / node_s
    return out
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
        ss = qpms_gb300.ScatteringSystem(_sq(nx, 400e-9), 50e-9, EPS_I, EPS_E, lMax)
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
        ss = qpms_gb300.ScatteringSystem(pos, 80e-9, EPS_I, EPS_E, 3, lattice=(b1, b2))
        kp = (honeycomb_path if lat == "honeycomb" else square_path)(n=nk)
        r = ss.dispersion_scan(np.linspace(1.6, 2.6, nw) * EV / HBAR, kp, mode=mode)
        print("scan", lat, nw, nk, "logdet sum", float(np.sum(r["logdet"])), "max resid", float(r["residual"].max()))
    elif f[0] == "field":
        nx, npts, lMax = int(f[1]), int(f[2]), int(f[3])
        pos = _sq(nx, 400e-9)
        ss = qpms_gb300.ScatteringSystem(pos, 60e-9, EPS_I, EPS_E, lMax)
        rng = np.random.default_rng(1)
        cv = rng.normal(size=ss.fecv_size) + 1j * rng.normal(size=ss.fecv_size)
        pts = rng.uniform(-nx * 2e-7, nx * 2e-7, size=(npts, 3))
        E = ss.scattered_E(1.6e7, cv, pts)
        print("field", nx, npts, lMax, "sum |E|", float(np.abs(E).sum()))
    elif f[0] == "axsym":
        from qpms_gb300.tmatrices import TMatrixGenerator
        L, nw = int(f[1]), int(f[2])
        g = TMatrixGenerator.cylinder(2.25, EPS_I, 50e-9, 100e-9, L)
        T = g.batch(3, np.linspace(1.6, 2.6, nw) * EV / HBAR)
        print("axsym", L, nw, "sum |T|", float(np.abs(T).sum()))
    elif f[0] == "beyn":
        nx, nodes, mode = int(f[1]), int(f[2]), int(f[3])
        ss = qpms_gb300.ScatteringSystem(_sq(nx, 400e-9), 60e-9, EPS_I, EPS_E, 2)
        r = ss.find_modes(2.1 * EV / HBAR, 0.05 * EV / HBAR, 0.005 * EV / HBAR, contour_points=nodes,
                          rank_tol=-1e-10, rank_min_sel=0, l=64, seed=12345, mode=mode)
        print("beyn", nx, nodes, "neig", r["eigval"].size, "node resid", r["node_residual_max"])
    elif f[0] == "serve":  # serve:NREQ:MODE -- the first NREQ requests of the serving trace, saturated
        from qpms_gb300.serving import Server, run_trace
        nreq, mode = int(f[1]), int(f[2])
        reqs, _ = build_trace(trace_specs(N_REQ)[:nreq])
        srv = Server(mode=mode, workers=WORKERS)
        _, summ = run_trace(srv, reqs)
        srv.close()
        print("serve", nreq, mode, "solves/s", summ["solves_per_s"], "max resid", summ["max_residual"])
    elif f[0] == "trans":  # trans:NVEC:LMAX
        from qpms_gb300.workloads import translation_vectors
        n, lm = int(f[1]), int(f[2])
        dev = torch.device("cuda:0")
        kr, th, ph = translation_vectors(n, seed=1000)
        c = qpms_gb300.trans_calculator(lm)
        ne = lm * (lm + 2)
        A = torch.empty((n, ne, ne), dtype=torch.complex128, device=dev)
        B = torch.empty_like(A)
        c.get_AB_arrays_device(*(torch.from_numpy(x).to(dev) for x in (kr, th, ph)), 3, A, B)
        print("trans", n, lm, "sum |A|", float(A.abs().sum()))
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
