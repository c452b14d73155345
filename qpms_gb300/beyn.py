"""Beyn contour-integral eigensolver over the C-ABI.

Python mirror of the reference's ``ScatteringSystem.find_modes``
(qpms/qpms_c.pyx:841-900) and of the C ``beyn_solve`` (qpms/beyn.h:115-125).
The quadrature (one assembly + LU + L-column solve per contour node) runs on
the GPU; see ``libqpms_gb300``.
"""
import ctypes as C

import numpy as np

from ._lib import QpmsGpuError, last_error, lib


class _BeynResult(C.Structure):
    _fields_ = [("neig", C.c_size_t), ("vlen", C.c_size_t), ("eigval", C.c_void_p), ("eigval_err", C.c_void_p),
                ("residuals", C.c_void_p), ("eigvec", C.c_void_p), ("ranktest_SV", C.c_void_p),
                ("gsl", C.c_void_p)]


# int M(qpms_complex_t *target, size_t m, qpms_complex_t z, void *params): z arrives as two doubles
M_FUNCTION = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_size_t, C.c_double, C.c_double, C.c_void_p)

DEFAULT_SEED = 0x5eedbe11


def declare(L):
    vp, sz, ci, cd, u64 = C.c_void_p, C.c_size_t, C.c_int, C.c_double, C.c_ulonglong
    R = C.POINTER(_BeynResult)
    L.beyn_contour_ellipse.restype = vp
    L.beyn_contour_ellipse.argtypes = [cd, cd, cd, cd, sz]
    L.beyn_contour_halfellipse.restype = vp
    L.beyn_contour_halfellipse.argtypes = [cd, cd, cd, cd, sz, ci]
    L.beyn_contour_kidney.restype = vp
    L.beyn_contour_kidney.argtypes = [cd, cd, cd, cd, cd, sz, ci]
    L.beyn_result_free.restype = None
    L.beyn_result_free.argtypes = [R]
    L.beyn_solve.restype = R
    L.beyn_solve.argtypes = [sz, sz, M_FUNCTION, vp, vp, vp, cd, sz, cd]
    L.qpms_gpu_beyn_solve.restype = R
    L.qpms_gpu_beyn_solve.argtypes = [sz, sz, M_FUNCTION, vp, vp, cd, sz, cd, vp, u64, ci, cd]
    L.qpms_scatsys_finite_find_eigenmodes.restype = R
    L.qpms_scatsys_finite_find_eigenmodes.argtypes = [vp, ci, cd, cd, cd, cd, sz, cd, sz, cd]
    L.qpms_scatsys_periodic_find_eigenmodes.restype = R
    L.qpms_scatsys_periodic_find_eigenmodes.argtypes = [vp, vp, cd, cd, cd, cd, sz, cd, sz, cd]
    L.qpms_gpu_scatsys_find_eigenmodes.restype = R
    L.qpms_gpu_scatsys_find_eigenmodes.argtypes = [vp, vp, cd, cd, cd, cd, sz, cd, sz, cd, sz, vp, u64, ci, cd]
    L.qpms_gpu_scatsys_find_eigenmodes_irrep.restype = R
    L.qpms_gpu_scatsys_find_eigenmodes_irrep.argtypes = [vp, ci, cd, cd, cd, cd, sz, cd, sz, cd, sz, vp, u64, ci, cd]
    L.qpms_gpu_beyn_result_stats.restype = ci
    L.qpms_gpu_beyn_result_stats.argtypes = [R, vp, vp, vp, vp]
    L.qpms_gpu_beyn_probe_matrix.restype = ci
    L.qpms_gpu_beyn_probe_matrix.argtypes = [sz, sz, u64, vp]
    L.qpms_gpu_host_svd.restype = ci
    L.qpms_gpu_host_svd.argtypes = [ci, ci, vp, vp, vp, vp]
    L.qpms_gpu_host_eig.restype = ci
    L.qpms_gpu_host_eig.argtypes = [ci, vp, vp, vp]
    L.qpms_gpu_scatsys_beyn_quadrature.restype = ci
    L.qpms_gpu_scatsys_beyn_quadrature.argtypes = [vp, vp, vp, sz, sz, sz, vp, u64, ci, cd, vp, vp, vp, vp]
    L.qpms_gpu_beyn_process.restype = R
    L.qpms_gpu_beyn_process.argtypes = [sz, sz, vp, vp, vp, vp, cd, cd, cd, sz]


def _carray(addr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    nbytes = n * np.dtype(dtype).itemsize
    buf = (C.c_char * nbytes).from_address(addr)
    return np.frombuffer(buf, dtype=dtype).copy()


def _collect(res, l, omega_centre=None, rr=None, ri=None):
    """beyn_result_t -> dict with the keys of the reference's find_modes."""
    if not res:
        raise QpmsGpuError("Beyn solve failed: %s" % last_error())
    try:
        r = res.contents
        neig, vlen = int(r.neig), int(r.vlen)
        out = {
            "eigval": _carray(r.eigval, neig, np.complex128),
            "eigval_err": _carray(r.eigval_err, neig, np.complex128),
            "residuals": _carray(r.residuals, neig, np.float64),
            "eigvec": _carray(r.eigvec, neig * vlen, np.complex128).reshape(neig, vlen),
            "ranktest_SV": _carray(r.ranktest_SV, max(l, vlen), np.float64)[:l],
        }
        st = np.zeros(3)
        it = C.c_int(0)
        lib().qpms_gpu_beyn_result_stats(res, st[0:].ctypes.data, C.addressof(it), st[1:].ctypes.data,
                                         st[2:].ctypes.data)
        out["node_residual_max"] = float(st[0])
        out["node_refine_iters_max"] = int(it.value)
        out["quadrature_s"] = float(st[1])
        out["total_s"] = float(st[2])
    finally:
        lib().beyn_result_free(res)
    if omega_centre is not None:
        zd = out["eigval"] - omega_centre
        out["eigval_inside_metric"] = np.hypot(zd.real / rr, zd.imag / ri)
    return out


def probe_matrix(m, l, seed=DEFAULT_SEED):
    """The library's seeded complex-Gaussian probe matrix (m x l)."""
    out = np.empty((m, l), dtype=np.complex128)
    if lib().qpms_gpu_beyn_probe_matrix(m, l, seed, out.ctypes.data):
        raise QpmsGpuError(last_error())
    return out


# orientations of the half-ellipse and kidney contours (beyn.h:50-55): the
# side of the straight edge's normal that the curved part lies on
HALFELLIPSE_RE_PLUS, HALFELLIPSE_RE_MINUS, HALFELLIPSE_IM_PLUS, HALFELLIPSE_IM_MINUS = 3, 1, 0, 2


def make_contour(centre, rr, ri, n, shape=None):
    """beyn_contour_t pointer (free with libc free): an ellipse (shape None),
    ("halfellipse", orientation) or ("kidney", rounding, orientation)
    (beyn.c:69-226)."""
    L = lib()
    c = complex(centre)
    if shape is None:
        p = L.beyn_contour_ellipse(c.real, c.imag, rr, ri, n)
    elif shape[0] == "halfellipse":
        p = L.beyn_contour_halfellipse(c.real, c.imag, rr, ri, n, shape[1])
    elif shape[0] == "kidney":
        p = L.beyn_contour_kidney(c.real, c.imag, rr, ri, shape[1], n, shape[2])
    else:
        raise ValueError("unknown contour shape %r" % (shape,))
    if not p:
        raise QpmsGpuError(last_error())
    return p


def contour_nodes(p):
    """(z, dz) arrays of a beyn_contour_t pointer."""
    n = C.c_size_t.from_address(p).value
    # header: n (8 bytes), centre (16), inside_test (8)
    zdz = np.frombuffer((C.c_char * (32 * n)).from_address(p + 32), dtype=np.complex128).reshape(n, 2)
    return zdz[:, 0].copy(), zdz[:, 1].copy()


def beyn_solve(M_function, m, l, omega_centre, omega_rr, omega_ri, contour_points, rank_tol=1e-4,
               rank_sel_min=1, res_tol=0.0, Vhat=None, seed=DEFAULT_SEED, mode=1, refine_tol=0.0, shape=None):
    """Eigenvalues of M(z) inside a contour; M_function(z) -> m x m complex array.

    The quadrature solves run on the GPU; M is evaluated on the host by the
    callback at every contour node (and at every candidate if res_tol > 0).
    shape: None for the ellipse, else as in make_contour."""
    L = lib()

    @M_FUNCTION
    def cb(target, mm, zr, zi, _params):
        try:
            M = np.asarray(M_function(complex(zr, zi)), dtype=np.complex128)
            dst = np.frombuffer((C.c_char * (16 * mm * mm)).from_address(target), dtype=np.complex128)
            dst[:] = M.reshape(-1)
            return 0
        except Exception:  # the error code reaches the C side, which reports it
            return 1

    c = complex(omega_centre)
    contour = make_contour(c, omega_rr, omega_ri, contour_points, shape)
    try:
        V = None
        if Vhat is not None:
            V = np.ascontiguousarray(Vhat, dtype=np.complex128)
            assert V.shape == (m, l)
        if V is None and seed == DEFAULT_SEED and mode == 1 and refine_tol == 0:
            res = L.beyn_solve(m, l, cb, None, None, contour, rank_tol, rank_sel_min, res_tol)   # the drop-in
        else:
            res = L.qpms_gpu_beyn_solve(m, l, cb, None, contour, rank_tol, rank_sel_min, res_tol,
                                        V.ctypes.data if V is not None else None, seed, mode, refine_tol)
    finally:
        C.CDLL(None).free(C.c_void_p(contour))
    if shape is not None:
        return _collect(res, l)
    return _collect(res, l, c, omega_rr, omega_ri)


def scatsys_find_modes(ss_ptr, fecv_size, omega_centre, omega_rr, omega_ri, blochvector=None, contour_points=20,
                       rank_tol=1e-4, rank_min_sel=1, res_tol=0.0, l=None, Vhat=None, seed=None, mode=None,
                       refine_tol=0.0, iri=None):
    """qpms_scatsys_{finite,periodic}_find_eigenmodes, or the extended entry
    point when l, Vhat, seed or mode is given.  With iri, fecv_size is the
    packed size of that irrep."""
    L = lib()
    c = complex(omega_centre)
    if iri is not None:
        V = None
        if Vhat is not None:
            V = np.ascontiguousarray(Vhat, dtype=np.complex128)
            l = V.shape[1]
            assert V.shape[0] == fecv_size
        l = fecv_size if l is None else int(l)
        res = L.qpms_gpu_scatsys_find_eigenmodes_irrep(ss_ptr, int(iri), c.real, c.imag, omega_rr, omega_ri,
                                                        contour_points, rank_tol, rank_min_sel, res_tol, l,
                                                        V.ctypes.data if V is not None else None,
                                                        DEFAULT_SEED if seed is None else seed,
                                                        1 if mode is None else mode, refine_tol)
        return _collect(res, l, c, omega_rr, omega_ri)
    kv = None
    if blochvector is not None:
        kv = np.zeros(3)
        kv[:len(blochvector)] = blochvector
    if l is None and Vhat is None and seed is None and mode is None:
        if kv is None:
            res = L.qpms_scatsys_finite_find_eigenmodes(ss_ptr, -1, c.real, c.imag, omega_rr, omega_ri,
                                                         contour_points, rank_tol, rank_min_sel, res_tol)
        else:
            res = L.qpms_scatsys_periodic_find_eigenmodes(ss_ptr, kv.ctypes.data, c.real, c.imag, omega_rr,
                                                           omega_ri, contour_points, rank_tol, rank_min_sel, res_tol)
        return _collect(res, fecv_size, c, omega_rr, omega_ri)
    V = None
    if Vhat is not None:
        V = np.ascontiguousarray(Vhat, dtype=np.complex128)
        l = V.shape[1]
        assert V.shape[0] == fecv_size
    l = fecv_size if l is None else int(l)
    res = L.qpms_gpu_scatsys_find_eigenmodes(ss_ptr, kv.ctypes.data if kv is not None else None, c.real, c.imag,
                                              omega_rr, omega_ri, contour_points, rank_tol, rank_min_sel, res_tol, l,
                                              V.ctypes.data if V is not None else None,
                                              DEFAULT_SEED if seed is None else seed, 1 if mode is None else mode,
                                              refine_tol)
    return _collect(res, l, c, omega_rr, omega_ri)


def host_svd(A):
    """The library's host thin SVD (for tests): A = U diag(s) V^H."""
    A = np.asfortranarray(A, dtype=np.complex128)
    m, n = A.shape
    U = np.zeros((m, n), dtype=np.complex128, order="F")
    s = np.zeros(n)
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    if lib().qpms_gpu_host_svd(m, n, A.ctypes.data, U.ctypes.data, s.ctypes.data, V.ctypes.data):
        raise QpmsGpuError("host SVD failed")
    return U, s, V


def host_eig(A):
    """The library's host eigen-decomposition (for tests): A X = X diag(w)."""
    A = np.asfortranarray(A, dtype=np.complex128)
    n = A.shape[0]
    w = np.zeros(n, dtype=np.complex128)
    X = np.zeros((n, n), dtype=np.complex128, order="F")
    if lib().qpms_gpu_host_eig(n, A.ctypes.data, w.ctypes.data, X.ctypes.data):
        raise QpmsGpuError("host eig failed")
    return w, X


# ---------------- sharding the contour (replicas with one exchange step) ----------------

def node_range(n_nodes, rank, world):
    """Contiguous share [begin, end) of n_nodes contour nodes for `rank` of `world`."""
    base, extra = divmod(n_nodes, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def scatsys_quadrature(ss_ptr, fecv_size, omega_centre, omega_rr, omega_ri, contour_points, node_begin, node_end,
                       l, blochvector=None, Vhat=None, seed=DEFAULT_SEED, mode=1, refine_tol=0.0):
    """Partial contour sums (A0, A1, A0c, A1c), each fecv_size x l, of the nodes
    [node_begin, node_end) of a scattering system's elliptic contour (GPU)."""
    L = lib()
    c = complex(omega_centre)
    contour = L.beyn_contour_ellipse(c.real, c.imag, omega_rr, omega_ri, contour_points)
    if not contour:
        raise QpmsGpuError(last_error())
    out = [np.zeros((fecv_size, l), dtype=np.complex128, order="F") for _ in range(4)]
    kv = None
    if blochvector is not None:
        kv = np.zeros(3)
        kv[:len(blochvector)] = blochvector
    V = None if Vhat is None else np.ascontiguousarray(Vhat, dtype=np.complex128)
    try:
        rc = L.qpms_gpu_scatsys_beyn_quadrature(ss_ptr, kv.ctypes.data if kv is not None else None, contour,
                                                node_begin, node_end, l, V.ctypes.data if V is not None else None,
                                                seed, mode, refine_tol, *[a.ctypes.data for a in out])
    finally:
        C.CDLL(None).free(C.c_void_p(contour))
    if rc:
        raise QpmsGpuError("Beyn quadrature: " + last_error())
    return tuple(out)


def process(A0, A1, A0c, A1c, z0, rank_tol=1e-4, rank_sel_min=1):
    """Beyn steps 3-6 on summed quadratures (host; no residual filter)."""
    arrs = [np.asfortranarray(a, dtype=np.complex128) for a in (A0, A1, A0c, A1c)]
    m, l = arrs[0].shape
    z = complex(z0)
    res = lib().qpms_gpu_beyn_process(m, l, *[a.ctypes.data for a in arrs], z.real, z.imag, rank_tol, rank_sel_min)
    return _collect(res, l)


def allreduce_sum(arrays, group=None):
    """Sum complex128 arrays over the ranks of `group` (torch.distributed),
    staged through host memory: CPU tensors on a gloo group."""
    import torch
    import torch.distributed as dist
    out = []
    for a in arrays:
        a = np.asfortranarray(a, dtype=np.complex128)
        t = torch.from_numpy(a.reshape(-1, order="F").view(np.float64).copy())
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out.append(t.numpy().view(np.complex128).reshape(a.shape, order="F"))
    return out


def sharded_find_modes(ss, omega_centre, omega_rr, omega_ri, contour_points, l, rank_tol=1e-4, rank_sel_min=1,
                       blochvector=None, Vhat=None, seed=DEFAULT_SEED, mode=1, group=None):
    """find_modes with the contour nodes split over the ranks of `group`: each
    rank sums its share on its GPU, the sums are added (host-staged), rank 0
    processes them and returns the result dict (other ranks return None)."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    b, e = node_range(contour_points, rank, world)
    parts = scatsys_quadrature(ss.s, ss.fecv_size, omega_centre, omega_rr, omega_ri, contour_points, b, e, l,
                               blochvector, Vhat, seed, mode)
    total = allreduce_sum(parts, group)
    return process(*total, omega_centre, rank_tol, rank_sel_min) if rank == 0 else None
