"""Loader of the in-tree libqpms_gb300.so (the CUDA implementation).

There is no CPU fallback: if the library is missing or cannot be loaded, every
entry point raises.  ``build()`` compiles it in place (nvcc, sm_103a).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqpms_gb300.so")

_lib = None


class QpmsGpuError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise QpmsGpuError("libqpms_gb300.so is not built (run qpms_gb300.build.build())")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def last_error():
    return lib().qpms_gpu_last_error().decode(errors="replace")


def check(rc, what):
    if rc != 0:
        raise QpmsGpuError("%s failed (code %d): %s" % (what, rc, last_error()))


def _declare(L):
    vp, sz, ci, cd = C.c_void_p, C.c_size_t, C.c_int, C.c_double
    L.qpms_gpu_last_error.restype = C.c_char_p
    L.qpms_gpu_last_error.argtypes = []
    L.qpms_gpu_kernel_launch_count.restype = C.c_ulonglong
    L.qpms_gpu_kernel_launch_count.argtypes = []
    L.qpms_gpu_graph_replay_count.restype = C.c_ulonglong
    L.qpms_gpu_graph_replay_count.argtypes = []
    L.qpms_trans_calculator_init.restype = vp
    L.qpms_trans_calculator_init.argtypes = [ci, ci]
    L.qpms_trans_calculator_free.restype = None
    L.qpms_trans_calculator_free.argtypes = [vp]
    L.qpms_gpu_trans_calculator_n_multipliers.restype = sz
    L.qpms_gpu_trans_calculator_n_multipliers.argtypes = [vp, ci]
    L.qpms_gpu_trans_AB_arrays_batch.restype = ci
    L.qpms_gpu_trans_AB_arrays_batch.argtypes = [vp, sz, vp, vp, vp, vp, ci, vp, vp, vp]
    L.qpms_gpu_trans_AB_arrays_batch_host_noalloc.restype = ci
    L.qpms_gpu_trans_AB_arrays_batch_host_noalloc.argtypes = [vp, sz, vp, vp, vp, vp, ci, vp, vp]
    L.qpms_gpu_testing_set_calculator_device.restype = ci
    L.qpms_gpu_testing_set_calculator_device.argtypes = [vp, ci]
    L.qpms_gpu_trans_AB_arrays_batch_host.restype = ci
    L.qpms_gpu_trans_AB_arrays_batch_host.argtypes = [vp, sz, vp, vp, vp, vp, ci, vp, vp]
    L.qpms_gpu_trans_multipliers_export.restype = ci
    L.qpms_gpu_trans_multipliers_export.argtypes = [ci, ci, vp, vp, vp, vp]
    L.qpms_gpu_dense_solve.restype = ci
    L.qpms_gpu_dense_solve.argtypes = [ci, ci, vp, vp, vp, ci, vp, vp]
    L.qpms_gpu_ozaki_residual.restype = ci
    L.qpms_gpu_ozaki_residual.argtypes = [ci, ci, vp, sz, ci, vp, vp, vp]
    L.qpms_gpu_bf16_gemm.restype = ci
    L.qpms_gpu_bf16_gemm.argtypes = [ci, ci, ci, vp, vp, vp]
    L.qpms_gpu_kernel_timing.restype = ci
    L.qpms_gpu_kernel_timing.argtypes = [ci]
    L.qpms_gpu_kernel_timing_get.restype = ci
    L.qpms_gpu_kernel_timing_get.argtypes = [ci, vp, vp, vp]
    L.qpms_gpu_measure_fp64_peak.restype = ci
    L.qpms_gpu_measure_fp64_peak.argtypes = [vp]
    # complex by value is passed as two doubles (same registers on x86-64 and aarch64)
    L.qpms_trans_calculator_get_AB_arrays_ext.restype = ci
    L.qpms_trans_calculator_get_AB_arrays_ext.argtypes = [vp, vp, vp, sz, sz, cd, cd, cd, cd, ci, ci]
    from . import beyn, materials, scatsystem, serving, tmatrices
    scatsystem.declare(L)
    tmatrices.declare(L)
    beyn.declare(L)
    serving.declare(L)
    materials.declare(L)


KERNEL_KINDS = ("tc_gemm", "assemble", "ewald", "batch_lu", "diag_lu", "trans", "split")


def kernel_timing(enable):
    """Start (True) or stop (False) live per-kind kernel timing; clears the sums."""
    lib().qpms_gpu_kernel_timing(1 if enable else 0)


def kernel_timing_get():
    """{kind: (device ms, work, launches)} of the launches recorded since the last kernel_timing()."""
    out = {}
    for i, name in enumerate(KERNEL_KINDS):
        ms, work, n = C.c_double(0), C.c_double(0), C.c_ulonglong(0)
        lib().qpms_gpu_kernel_timing_get(i, C.byref(ms), C.byref(work), C.byref(n))
        if n.value:
            out[name] = (ms.value, work.value, n.value)
    return out
