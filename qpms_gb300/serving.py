"""Serving loop over the C-ABI: continuous batching of scattering solves.

``Server`` wraps qpms_gpu_server_*; ``run_trace`` replays a timed request
stream (Poisson arrivals) against it and reports latency percentiles and
throughput.  Each request is one plane-wave scattering solve of a finite
cluster or of a 2D lattice (the unit of work of the reference's
misc/finiterectlat-scatter.py / misc/infiniterectlat-scatter.py loops).
"""
import ctypes as C
import time

import numpy as np

from ._lib import QpmsGpuError, last_error, lib


class _Request(C.Structure):
    _fields_ = [("ss", C.c_void_p), ("omega", C.c_double), ("k", C.c_double * 2), ("k_dir", C.c_double * 3),
                ("E", C.c_double * 6)]


class _Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iters", C.c_int), ("batch_size", C.c_int), ("fallback", C.c_int),
                ("sigma_ext", C.c_double), ("residual", C.c_double), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double)]


def declare(L):
    vp, sz, ci, cd = C.c_void_p, C.c_size_t, C.c_int, C.c_double
    L.qpms_gpu_server_create.restype = vp
    L.qpms_gpu_server_create.argtypes = [sz, ci, ci]
    L.qpms_gpu_server_submit.restype = ci
    L.qpms_gpu_server_submit.argtypes = [vp, C.POINTER(_Request), vp, C.POINTER(C.c_uint64)]
    L.qpms_gpu_server_wait.restype = ci
    L.qpms_gpu_server_wait.argtypes = [vp, C.c_uint64, C.POINTER(_Result)]
    L.qpms_gpu_server_drain.restype = ci
    L.qpms_gpu_server_drain.argtypes = [vp]
    L.qpms_gpu_server_cancel.restype = ci
    L.qpms_gpu_server_cancel.argtypes = [vp, C.c_uint64]
    L.qpms_gpu_server_testing_fail_allocations.restype = ci
    L.qpms_gpu_server_testing_fail_allocations.argtypes = [vp, ci]
    L.qpms_gpu_testing_set_max_refine.restype = ci
    L.qpms_gpu_testing_set_max_refine.argtypes = [ci]
    L.qpms_gpu_server_clock.restype = cd
    L.qpms_gpu_server_clock.argtypes = [vp]
    L.qpms_gpu_server_stats.restype = ci
    L.qpms_gpu_server_stats.argtypes = [vp, vp, vp, vp, vp, vp]
    L.qpms_gpu_server_destroy.restype = None
    L.qpms_gpu_server_destroy.argtypes = [vp]


class Server:
    """Continuous-batching solve server on the current GPU."""

    def __init__(self, hbm_budget=0, mode=1, workers=4):
        self._L = lib()
        self.mode = mode
        self.s = self._L.qpms_gpu_server_create(int(hbm_budget), int(mode), int(workers))
        if not self.s:
            raise QpmsGpuError("qpms_gpu_server_create: " + last_error())
        self._live = {}

    def submit(self, system, omega, k=(0.0, 0.0), k_dir=(0.0, 0.0, 1.0), E=(1.0, 0.0, 0.0), want_f=True):
        """Queue one solve of ``system`` (a ScatteringSystem) at omega; returns a ticket."""
        r = _Request()
        r.ss = system.s
        r.omega = float(omega)
        r.k[0], r.k[1] = float(k[0]), float(k[1])
        for i in range(3):
            r.k_dir[i] = float(k_dir[i])
            e = complex(E[i])
            r.E[2 * i], r.E[2 * i + 1] = e.real, e.imag
        f = np.empty(system.fecv_size, dtype=np.complex128) if want_f else None
        t = C.c_uint64(0)
        rc = self._L.qpms_gpu_server_submit(self.s, C.byref(r), f.ctypes.data if f is not None else None,
                                           C.byref(t))
        if rc:
            raise QpmsGpuError("submit: " + last_error())
        self._live[t.value] = (f, system)      # keep the output buffer and the system alive
        return t.value

    def wait(self, ticket):
        res = _Result()
        rc = self._L.qpms_gpu_server_wait(self.s, ticket, C.byref(res))
        f, _ = self._live.pop(ticket)
        out = {"status": rc, "sigma_ext": res.sigma_ext, "residual": res.residual, "iters": res.iters,
               "batch_size": res.batch_size, "fallback": res.fallback, "t_submit": res.t_submit,
               "t_start": res.t_start, "t_done": res.t_done, "f": f}
        if rc:
            out["error"] = last_error()
        return out

    def cancel(self, ticket):
        """Withdraw a request that has not started (True), or False if it already
        started; a cancelled request still has to be waited for (status
        QPMS_ECANCELED)."""
        return self._L.qpms_gpu_server_cancel(self.s, ticket) == 0

    def drain(self):
        self._L.qpms_gpu_server_drain(self.s)

    def clock(self):
        return self._L.qpms_gpu_server_clock(self.s)

    def stats(self):
        v = [C.c_size_t(0), C.c_size_t(0), C.c_size_t(0), C.c_int(0), C.c_size_t(0)]
        self._L.qpms_gpu_server_stats(self.s, *[C.byref(x) for x in v])
        return {"completed": v[0].value, "batches": v[1].value, "peak_bytes": v[2].value,
                "max_concurrent": v[3].value, "budget_bytes": v[4].value}

    def close(self):
        if getattr(self, "s", None):
            self.drain()
            self._L.qpms_gpu_server_destroy(self.s)
            self.s = None

    def __del__(self):
        self.close()


def run_trace(server, requests, arrivals=None, want_f=False):
    """Submit ``requests`` (dicts with system, omega[, k, k_dir, E]) at the
    given arrival times (seconds from the start; None: all at once), wait for
    all; returns per-request results and the summary (p50/p99 latency,
    solves/s over the makespan)."""
    n = len(requests)
    arrivals = np.zeros(n) if arrivals is None else np.asarray(arrivals, dtype=float)
    tickets = []
    t0 = time.perf_counter()
    for i, rq in enumerate(requests):
        dt = arrivals[i] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(server.submit(rq["system"], rq["omega"], rq.get("k", (0.0, 0.0)),
                                     rq.get("k_dir", (0.0, 0.0, 1.0)), rq.get("E", (1.0, 0.0, 0.0)), want_f))
    results = [server.wait(t) for t in tickets]
    makespan = time.perf_counter() - t0
    lat = np.array([r["t_done"] - r["t_submit"] for r in results])
    return results, {
        "requests": n, "makespan_s": makespan, "solves_per_s": n / makespan,
        "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "mean_batch": float(np.mean([r["batch_size"] for r in results])),
        "max_residual": float(np.max([r["residual"] for r in results])),
        "failed": int(sum(1 for r in results if r["status"])),
    }
