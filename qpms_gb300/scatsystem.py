"""Python mirror of the reference's scattering-system wrappers (qpms_c.pyx):
``ScatteringSystem`` (:390-902), ``_ScatteringSystemAtOmega`` (:1000-1082) and
``ScatteringMatrix`` (:1144-1195), over the C-ABI of libqpms_gb300.

Systems are built from spheres with constant permittivities (the Mie T-matrix
generator of the benchmark configurations); every heavy step runs on the GPU.
"""
import ctypes as C

import numpy as np

from . import _lib

QPMS_HANKEL_PLUS = 3


class _SSWK(C.Structure):
    _fields_ = [("ssw", C.c_void_p), ("k", C.c_double * 3), ("eta", C.c_double)]


class _SSW(C.Structure):
    _fields_ = [("ss", C.c_void_p), ("tm", C.c_void_p), ("omega", C.c_double * 2),
                ("medium", C.c_double * 4), ("wavenumber", C.c_double * 2)]


class _Cplx2(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class _Arc(C.Structure):
    _fields_ = [("function", C.c_void_p), ("params", C.c_void_p)]


class _Kind(C.Structure):
    """qpms_gpu_particle_kind_t"""
    _fields_ = [("type", C.c_int), ("radius", C.c_double), ("eps", _Cplx2), ("ld", C.c_void_p),
                ("eps_interp", C.c_void_p), ("tmatrix", C.c_void_p), ("shape", _Arc), ("lMax_extend", C.c_int)]


class _LU(C.Structure):
    _fields_ = [("ssw", C.c_void_p), ("sswk", C.c_void_p), ("full", C.c_bool), ("iri", C.c_int),
                ("a", C.c_void_p), ("ipiv", C.c_void_p)]


class _Cart3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class _CCart3(C.Structure):
    _fields_ = [("v", C.c_double * 6)]


def _scattered_E(L, s, wavenumber, cvf, evalpos, n, btyp):
    """qpms_c.pyx:904-927: evalpos [..., 3] -> E [..., 3] complex, one batched call."""
    evalpos = np.asarray(evalpos, dtype=np.float64)
    if evalpos.shape[-1] != 3:
        raise ValueError("Last dimension of evalpos has to be 3")
    w = np.ascontiguousarray(evalpos.reshape(-1, 3))
    cv = np.ascontiguousarray(cvf, dtype=np.complex128)
    if cv.size != n:
        raise ValueError("Length of a full coefficient vector has to be %d, not %d" % (n, cv.size))
    E = np.empty((w.shape[0], 3), dtype=np.complex128)
    k = complex(wavenumber)
    _lib.check(L.qpms_gpu_scatsys_scattered_E(s, int(btyp), k.real, k.imag, cv.ctypes.data, w.shape[0],
                                              w.ctypes.data, E.ctypes.data), "qpms_gpu_scatsys_scattered_E")
    return E.reshape(evalpos.shape)


def declare(L):
    vp, ci, cd, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    L.qpms_gpu_scatsys_create_spheres.restype = vp
    L.qpms_gpu_scatsys_create_spheres.argtypes = [ci, vp, vp, ci, vp, vp, cd, cd, ci]
    L.qpms_gpu_scatsys_create.restype = vp
    L.qpms_gpu_scatsys_create.argtypes = [ci, vp, vp, ci, vp, cd, cd, ci, vp, vp]
    L.qpms_gpu_scatsys_set_symmetry.restype = ci
    L.qpms_gpu_scatsys_set_symmetry.argtypes = [vp, C.c_char_p]
    L.qpms_gpu_scatsys_nirreps.restype = ci
    L.qpms_gpu_scatsys_nirreps.argtypes = [vp]
    L.qpms_gpu_scatsys_irrep_name.restype = C.c_char_p
    L.qpms_gpu_scatsys_irrep_name.argtypes = [vp, ci]
    L.qpms_gpu_scatsys_saecv_sizes.restype = vp
    L.qpms_gpu_scatsys_saecv_sizes.argtypes = [vp]
    for name in ("qpms_scatsys_irrep_pack_vector", "qpms_scatsys_irrep_pack_matrix"):
        getattr(L, name).restype = vp
        getattr(L, name).argtypes = [vp, vp, vp, ci]
    for name in ("qpms_scatsys_irrep_unpack_vector", "qpms_scatsys_irrep_unpack_matrix"):
        getattr(L, name).restype = vp
        getattr(L, name).argtypes = [vp, vp, vp, ci, C.c_bool]
    L.qpms_scatsys_irrep_transform_matrix.restype = vp
    L.qpms_scatsys_irrep_transform_matrix.argtypes = [vp, vp, ci]
    L.qpms_scatsysw_build_modeproblem_matrix_irrep_packed.restype = vp
    L.qpms_scatsysw_build_modeproblem_matrix_irrep_packed.argtypes = [vp, vp, ci]
    L.qpms_scatsys_build_translation_matrix_e_irrep_packed.restype = vp
    L.qpms_scatsys_build_translation_matrix_e_irrep_packed.argtypes = [vp, vp, ci, cd, cd, ci]
    L.qpms_scatsysw_build_modeproblem_matrix_irrep_packed_LU.restype = _LU
    L.qpms_scatsysw_build_modeproblem_matrix_irrep_packed_LU.argtypes = [vp, vp, vp, ci]
    L.qpms_gpu_scatsys_free.restype = None
    L.qpms_gpu_scatsys_free.argtypes = [vp]
    L.qpms_gpu_scatsys_at_omega.restype = vp
    L.qpms_gpu_scatsys_at_omega.argtypes = [vp, cd, cd]
    L.qpms_gpu_scatsys_at_omega_free.restype = None
    L.qpms_gpu_scatsys_at_omega_free.argtypes = [vp]
    L.qpms_scatsysw_build_modeproblem_matrix_full.restype = vp
    L.qpms_scatsysw_build_modeproblem_matrix_full.argtypes = [vp, vp]
    L.qpms_scatsys_build_translation_matrix_e_full.restype = vp
    L.qpms_scatsys_build_translation_matrix_e_full.argtypes = [vp, vp, cd, cd, ci]
    L.qpms_scatsysw_build_modeproblem_matrix_full_LU.restype = _LU
    L.qpms_scatsysw_build_modeproblem_matrix_full_LU.argtypes = [vp, vp, vp]
    L.qpms_scatsysw_modeproblem_matrix_full_factorise.restype = _LU
    L.qpms_scatsysw_modeproblem_matrix_full_factorise.argtypes = [vp, vp, vp, vp]
    L.qpms_scatsys_scatter_solve.restype = vp
    L.qpms_scatsys_scatter_solve.argtypes = [vp, vp, _LU]
    L.qpms_ss_LU_free.restype = None
    L.qpms_ss_LU_free.argtypes = [_LU]
    L.qpms_scatsysw_apply_Tmatrices_full.restype = vp
    L.qpms_scatsysw_apply_Tmatrices_full.argtypes = [vp, vp, vp]
    L.qpms_gpu_incident_planewave_full.restype = ci
    L.qpms_gpu_incident_planewave_full.argtypes = [vp, vp, vp, vp]
    L.qpms_gpu_scatsys_create_spheres_2d.restype = vp
    L.qpms_gpu_scatsys_create_spheres_2d.argtypes = [ci, vp, vp, ci, vp, vp, cd, cd, ci, vp, vp]
    L.qpms_ss_adjusted_eta.restype = cd
    L.qpms_ss_adjusted_eta.argtypes = [vp, cd, cd, vp]
    L.qpms_scatsyswk_build_modeproblem_matrix_full.restype = vp
    L.qpms_scatsyswk_build_modeproblem_matrix_full.argtypes = [vp, C.POINTER(_SSWK)]
    L.qpms_gpu_periodic_scan.restype = ci
    L.qpms_gpu_periodic_scan.argtypes = [vp, sz, vp, sz, vp, ci, vp, vp, vp, vp, vp]
    L.qpms_gpu_debug_cerfc.restype = ci
    L.qpms_gpu_debug_cerfc.argtypes = [cd, cd, vp]
    L.qpms_gpu_finite_planewave_scatter.restype = ci
    L.qpms_gpu_finite_planewave_scatter.argtypes = [vp, sz, vp, vp, vp, ci, vp, vp, vp, vp]
    L.qpms_gpu_finite_planewave_scatter_ext.restype = ci
    L.qpms_gpu_scatsys_scattered_E.restype = ci
    L.qpms_gpu_scatsys_scattered_E.argtypes = [vp, ci, cd, cd, vp, sz, vp, vp]
    L.qpms_gpu_scatsyswk_scattered_E.restype = ci
    L.qpms_gpu_scatsyswk_scattered_E.argtypes = [C.POINTER(_SSWK), ci, vp, sz, vp, vp]
    L.qpms_gpu_scatsys_scattered_E_device.restype = ci
    L.qpms_gpu_scatsys_scattered_E_device.argtypes = [vp, ci, cd, cd, vp, sz, vp, vp, vp]
    for name in ("qpms_scatsys_scattered_E", "qpms_scatsys_scattered_E__alt"):
        getattr(L, name).restype = _CCart3
        getattr(L, name).argtypes = [vp, ci, cd, cd, vp, _Cart3]
    for name in ("qpms_scatsysw_scattered_E", "qpms_scatsysw_scattered_E__alt"):
        getattr(L, name).restype = _CCart3
        getattr(L, name).argtypes = [vp, ci, vp, _Cart3]
    L.qpms_gpu_finite_planewave_scatter_ext.argtypes = [vp, sz, vp, vp, vp, ci, vp, vp, vp, vp, vp]


class ScatteringSystem:
    """Finite system of spheres; ``ss(omega)`` evaluates it at a frequency."""

    def __init__(self, positions, radius, eps_inside, eps_medium, lMax, kinds=None, lattice=None, sym=None):
        """lattice: None (finite system) or (b1, b2), 2D basis vectors in the xy plane.

        eps_inside: one entry per particle kind (or a single one): a constant
        permittivity, a ``materials.LorentzDrude`` model, a
        ``materials.MaterialInterpolator`` (tabulated n, k) or a
        ``tmatrices.TMatrixInterpolator`` (a tabulated T-matrix kind; its radius
        entry is ignored) or a ``tmatrices.TMatrixGenerator`` (an axially
        symmetric particle: its shape and inside medium; the outside medium is
        eps_medium).  kinds[i] selects the kind of particle i."""
        self._L = _lib.lib()
        from .materials import LorentzDrude, MaterialInterpolator
        from .tmatrices import TMatrixGenerator, TMatrixInterpolator
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        eps_list = list(eps_inside) if isinstance(eps_inside, (list, tuple)) else [eps_inside]
        nk = len(eps_list)
        radius = np.broadcast_to(np.atleast_1d(np.asarray(radius, dtype=np.float64)), (nk,))
        karr = (_Kind * nk)()
        self._keep = []  # interpolators and models referenced by the system
        for t, e in enumerate(eps_list):
            K = karr[t]
            K.radius = float(radius[t])
            if isinstance(e, TMatrixGenerator):
                K.type = 2
                K.shape = _Arc(e.shape.arc.function, e.shape.arc.params)
                K.lMax_extend = max(int(e.lMax_extend), int(lMax))
                inner = e.inside
                if isinstance(inner, LorentzDrude):
                    K.ld = inner.ptr
                elif isinstance(inner, MaterialInterpolator):
                    K.eps_interp = inner.ptr
                else:
                    c = complex(inner)
                    K.eps = _Cplx2(c.real, c.imag)
                self._keep.append(e)
            elif isinstance(e, TMatrixInterpolator):
                K.type = 1
                K.tmatrix = e.ptr
                self._keep.append(e)
            elif isinstance(e, LorentzDrude):
                K.ld = e.ptr
                self._keep.append(e)
            elif isinstance(e, MaterialInterpolator):
                K.eps_interp = e.ptr
                self._keep.append(e)
            else:
                c = complex(e)
                K.eps = _Cplx2(c.real, c.imag)
        self._models = [e if isinstance(e, LorentzDrude) else None for e in eps_list]
        if kinds is None:
            kinds = np.zeros(pos.shape[0], dtype=np.int32)
        kinds = np.ascontiguousarray(kinds, dtype=np.int32)
        em = complex(eps_medium)
        self.positions = pos
        self.lMax = int(lMax)
        self.lattice = lattice
        self.eps_medium = em
        b1 = b2 = None
        if lattice is not None:
            b1 = np.ascontiguousarray(lattice[0][:2], dtype=np.float64)
            b2 = np.ascontiguousarray(lattice[1][:2], dtype=np.float64)
        self.s = self._L.qpms_gpu_scatsys_create(
            pos.shape[0], pos.ctypes.data, kinds.ctypes.data, nk, C.addressof(karr), em.real, em.imag, self.lMax,
            b1.ctypes.data if b1 is not None else None, b2.ctypes.data if b2 is not None else None)
        if not self.s:
            raise _lib.QpmsGpuError("qpms_gpu_scatsys_create: " + _lib.last_error())
        self.sym = sym
        if sym is not None:  # a point_group_info name: "D2h", "D4h", "D3h", "C4v", ...
            _lib.check(self._L.qpms_gpu_scatsys_set_symmetry(self.s, str(sym).encode()),
                       "qpms_gpu_scatsys_set_symmetry")
        self.fecv_size = pos.shape[0] * 2 * self.lMax * (self.lMax + 2)

    def __del__(self):
        s = getattr(self, "s", None)
        if s:
            self._L.qpms_gpu_scatsys_free(s)
            self.s = None

    def __call__(self, omega):
        return _ScatteringSystemAtOmega(self, omega)

    def planewave_full(self, k_cart, E_cart):
        k = np.ascontiguousarray(k_cart, dtype=np.float64)
        E = np.ascontiguousarray(E_cart, dtype=np.complex128)
        out = np.empty(self.fecv_size, dtype=np.complex128)
        _lib.check(self._L.qpms_gpu_incident_planewave_full(out.ctypes.data, self.s, k.ctypes.data, E.ctypes.data),
                   "qpms_gpu_incident_planewave_full")
        return out

    # ---- irreps (qpms_c.pyx:541-560, 590-730, 777-786) ----
    @property
    def nirreps(self):
        return self._L.qpms_gpu_scatsys_nirreps(self.s)

    @property
    def irrep_names(self):
        return [self._L.qpms_gpu_scatsys_irrep_name(self.s, i).decode() for i in range(self.nirreps)]

    @property
    def saecv_sizes(self):
        p = C.cast(self._L.qpms_gpu_scatsys_saecv_sizes(self.s), C.POINTER(C.c_size_t))
        return [p[i] for i in range(self.nirreps)]

    def _check_iri(self, iri):
        if not 0 <= int(iri) < self.nirreps:
            raise ValueError("Invalid irrep index %s (of %d irreps)" % (iri, self.nirreps))
        return int(iri)

    def pack_vector(self, vect, iri):
        iri = self._check_iri(iri)
        v = np.ascontiguousarray(vect, dtype=np.complex128)
        if v.size != self.fecv_size:
            raise ValueError("Length of a full vector has to be %d, not %d" % (self.fecv_size, v.size))
        out = np.empty(self.saecv_sizes[iri], dtype=np.complex128)
        if not self._L.qpms_scatsys_irrep_pack_vector(out.ctypes.data, v.ctypes.data, self.s, iri):
            raise _lib.QpmsGpuError("pack_vector: " + _lib.last_error())
        return out

    def unpack_vector(self, packed, iri):
        iri = self._check_iri(iri)
        p = np.ascontiguousarray(packed, dtype=np.complex128)
        if p.size != self.saecv_sizes[iri]:
            raise ValueError("Length of %d. irrep-packed vector has to be %d, not %d"
                             % (iri, self.saecv_sizes[iri], p.size))
        out = np.empty(self.fecv_size, dtype=np.complex128)
        if not self._L.qpms_scatsys_irrep_unpack_vector(out.ctypes.data, p.ctypes.data, self.s, iri, False):
            raise _lib.QpmsGpuError("unpack_vector: " + _lib.last_error())
        return out

    def pack_matrix(self, fullmatrix, iri):
        iri = self._check_iri(iri)
        M = np.ascontiguousarray(fullmatrix, dtype=np.complex128)
        n = self.saecv_sizes[iri]
        out = np.empty((n, n), dtype=np.complex128)
        if not self._L.qpms_scatsys_irrep_pack_matrix(out.ctypes.data, M.ctypes.data, self.s, iri):
            raise _lib.QpmsGpuError("pack_matrix: " + _lib.last_error())
        return out

    def unpack_matrix(self, packedmatrix, iri):
        iri = self._check_iri(iri)
        P = np.ascontiguousarray(packedmatrix, dtype=np.complex128)
        out = np.empty((self.fecv_size, self.fecv_size), dtype=np.complex128)
        if not self._L.qpms_scatsys_irrep_unpack_matrix(out.ctypes.data, P.ctypes.data, self.s, iri, False):
            raise _lib.QpmsGpuError("unpack_matrix: " + _lib.last_error())
        return out

    def irrep_transform_matrix(self, iri):
        """U (saecv_sizes[iri] x fecv_size): packed = U full."""
        iri = self._check_iri(iri)
        out = np.empty((self.saecv_sizes[iri], self.fecv_size), dtype=np.complex128)
        if not self._L.qpms_scatsys_irrep_transform_matrix(out.ctypes.data, self.s, iri):
            raise _lib.QpmsGpuError("irrep_transform_matrix: " + _lib.last_error())
        return out

    def translation_matrix_packed(self, wavenumber, iri, J=QPMS_HANKEL_PLUS):
        iri = self._check_iri(iri)
        k = complex(wavenumber)
        n = self.saecv_sizes[iri]
        out = np.empty((n, n), dtype=np.complex128)
        if not self._L.qpms_scatsys_build_translation_matrix_e_irrep_packed(out.ctypes.data, self.s, iri, k.real,
                                                                            k.imag, int(J)):
            raise _lib.QpmsGpuError("translation_matrix_packed: " + _lib.last_error())
        return out

    def scattered_E(self, wavenumber, scatcoeffvector_full, evalpos, alt=False, btyp=QPMS_HANKEL_PLUS):
        """Field of the full coefficient vector at the points evalpos [..., 3]
        (qpms_c.pyx:904-927); ``alt`` selects the reference's alternative route,
        which evaluates the same field."""
        return _scattered_E(self._L, self.s, wavenumber, scatcoeffvector_full, evalpos, self.fecv_size, btyp)

    def scattered_E_device(self, wavenumber, cvf, evalpos, out=None, btyp=QPMS_HANKEL_PLUS, stream=None):
        """Device-tensor variant: cvf (fecv_size,) complex128, evalpos (n, 3)
        float64 and out (n, 3) complex128 CUDA tensors; runs on `stream`
        (default: torch's current stream)."""
        import torch
        if out is None:
            out = torch.empty((evalpos.shape[0], 3), dtype=torch.complex128, device=evalpos.device)
        if stream is None:
            stream = torch.cuda.current_stream(evalpos.device)
        k = complex(wavenumber)
        _lib.check(self._L.qpms_gpu_scatsys_scattered_E_device(
            self.s, int(btyp), k.real, k.imag, cvf.data_ptr(), evalpos.shape[0], evalpos.data_ptr(),
            out.data_ptr(), stream.cuda_stream), "qpms_gpu_scatsys_scattered_E_device")
        return out

    def translation_matrix_full(self, wavenumber, J=QPMS_HANKEL_PLUS):
        k = complex(wavenumber)
        out = np.empty((self.fecv_size, self.fecv_size), dtype=np.complex128)
        r = self._L.qpms_scatsys_build_translation_matrix_e_full(out.ctypes.data, self.s, k.real, k.imag, int(J))
        if not r:
            raise _lib.QpmsGpuError("translation matrix: " + _lib.last_error())
        return out

    def adjusted_eta(self, wavenumber, kvec):
        """qpms_ss_adjusted_eta (scatsystem.c:68-80)."""
        k = complex(wavenumber)
        kv = np.zeros(3)
        kv[:len(kvec)] = kvec
        return self._L.qpms_ss_adjusted_eta(self.s, k.real, k.imag, kv.ctypes.data)

    def dispersion_scan(self, omegas, kvecs, want_f=False, want_sigma=True, mode=1):
        """Batched 2D-lattice scan: log|det M(omega, k)| for all pairs, plus the
        plane-wave excitation (f, sigma_ext per cell, residual, refinement
        steps).  mode 1: complex64 LU + FP64 refinement; mode 0: complex128 LU."""
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        kv = np.ascontiguousarray(kvecs, dtype=np.float64).reshape(-1, 2)
        nw, nk = om.size, kv.shape[0]
        logdet = np.empty((nw, nk))
        sig = np.empty((nw, nk))
        res = np.empty((nw, nk))
        its = np.empty((nw, nk), dtype=np.int32)
        f = np.empty((nw, nk, self.fecv_size), dtype=np.complex128) if want_f else None
        rc = self._L.qpms_gpu_periodic_scan(self.s, nw, om.ctypes.data, nk, kv.ctypes.data, int(mode),
                                            logdet.ctypes.data, f.ctypes.data if want_f else None,
                                            sig.ctypes.data, res.ctypes.data, its.ctypes.data)
        _lib.check(rc, "qpms_gpu_periodic_scan")
        out = {"logdet": logdet, "iters": its}
        if want_sigma:
            out["sigma_ext"] = sig
            out["residual"] = res
        if want_f:
            out["f"] = f
        return out

    def planewave_scatter_batch(self, omegas, k_dir=(0.0, 0.0, 1.0), E_cart=(1.0, 0.0, 0.0), mode=1,
                                want_f=False, want_scat=False):
        """Batched loop of misc/finiterectlat-scatter.py over frequencies:
        returns dict(sigma_ext, residual, iters[, f][, sigma_scat, sigma_abs]).
        mode 0: FP64 LU; mode 1: complex64 LU + FP64 refinement."""
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        kd = np.ascontiguousarray(k_dir, dtype=np.float64)
        E = np.ascontiguousarray(E_cart, dtype=np.complex128)
        nw = om.size
        sig = np.empty(nw)
        scat = np.empty(nw) if want_scat else None
        res = np.empty(nw)
        it = np.empty(nw, dtype=np.int32)
        f = np.empty((nw, self.fecv_size), dtype=np.complex128) if want_f else None
        rc = self._L.qpms_gpu_finite_planewave_scatter_ext(self.s, nw, om.ctypes.data, kd.ctypes.data,
                                                           E.ctypes.data, int(mode),
                                                           f.ctypes.data if want_f else None, sig.ctypes.data,
                                                           scat.ctypes.data if want_scat else None,
                                                           res.ctypes.data, it.ctypes.data)
        _lib.check(rc, "qpms_gpu_finite_planewave_scatter")
        out = {"sigma_ext": sig, "residual": res, "iters": it}
        if want_scat:
            out["sigma_scat"] = scat
            out["sigma_abs"] = sig - scat
        if want_f:
            out["f"] = f
        return out


    def find_modes(self, omega_centre, omega_rr, omega_ri, iri=None, blochvector=None, contour_points=20,
                   rank_tol=1e-4, rank_min_sel=1, res_tol=0.0, l=None, Vhat=None, seed=None, mode=None,
                   refine_tol=0.0):
        """Eigenmodes inside an ellipse in the complex omega plane by Beyn's
        method (qpms_c.pyx:841-900): dict(eigval, eigval_inside_metric,
        eigvec, residuals, eigval_err, ranktest_SV, iri, blochvector).

        Extensions: l (probe columns; the reference uses fecv_size), Vhat
        (explicit probe matrix), seed, mode (0 plain FP64, 1 mixed), refine_tol."""
        from . import beyn
        if iri is not None:
            if blochvector is not None:
                raise NotImplementedError("Irreps decomposition not yet supported for periodic systems")
            iri = self._check_iri(iri)
            out = beyn.scatsys_find_modes(self.s, self.saecv_sizes[iri], omega_centre, omega_rr, omega_ri, None,
                                          contour_points, rank_tol, rank_min_sel, res_tol, l, Vhat, seed, mode,
                                          refine_tol, iri=iri)
            out["iri"] = iri
            out["blochvector"] = None
            return out
        if self.lattice is None and blochvector is not None:
            raise ValueError("a Bloch vector needs a periodic system")
        if self.lattice is not None and blochvector is None:
            raise ValueError("a periodic system needs a Bloch vector")
        out = beyn.scatsys_find_modes(self.s, self.fecv_size, omega_centre, omega_rr, omega_ri, blochvector,
                                      contour_points, rank_tol, rank_min_sel, res_tol, l, Vhat, seed, mode,
                                      refine_tol)
        out["iri"] = iri
        out["blochvector"] = blochvector
        return out


class _ScatteringSystemAtOmega:
    def __init__(self, ss, omega):
        self.ss = ss
        self._L = ss._L
        om = complex(omega)
        self.omega = om
        self.ssw = self._L.qpms_gpu_scatsys_at_omega(ss.s, om.real, om.imag)
        if not self.ssw:
            raise _lib.QpmsGpuError("qpms_gpu_scatsys_at_omega: " + _lib.last_error())

    def __del__(self):
        w = getattr(self, "ssw", None)
        if w:
            self._L.qpms_gpu_scatsys_at_omega_free(w)
            self.ssw = None

    def modeproblem_matrix_full(self, k=None, eta=0.0):
        """M = I - T S (finite) or, with a Bloch vector k, M = I - T W(k) (2D lattice)."""
        n = self.ss.fecv_size
        out = np.empty((n, n), dtype=np.complex128)
        if k is None:
            r = self._L.qpms_scatsysw_build_modeproblem_matrix_full(out.ctypes.data, self.ssw)
        else:
            wk = _SSWK()
            wk.ssw = self.ssw
            kk = list(k) + [0.0] * (3 - len(k))
            for i in range(3):
                wk.k[i] = kk[i]
            wk.eta = float(eta)
            r = self._L.qpms_scatsyswk_build_modeproblem_matrix_full(out.ctypes.data, C.byref(wk))
        if not r:
            raise _lib.QpmsGpuError("modeproblem_matrix_full: " + _lib.last_error())
        return out

    def apply_Tmatrices_full(self, a):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        out = np.empty_like(a)
        if not self._L.qpms_scatsysw_apply_Tmatrices_full(out.ctypes.data, a.ctypes.data, self.ssw):
            raise _lib.QpmsGpuError("apply_Tmatrices_full: " + _lib.last_error())
        return out

    def scatter_solver(self, iri=None):
        return ScatteringMatrix(self, iri)

    def modeproblem_matrix_packed(self, iri):
        """(I - T S) projected on irrep iri (qpms_c.pyx:1084-1098)."""
        n = self.ss.saecv_sizes[iri]
        out = np.empty((n, n), dtype=np.complex128)
        if not self._L.qpms_scatsysw_build_modeproblem_matrix_irrep_packed(out.ctypes.data, self.ssw, int(iri)):
            raise _lib.QpmsGpuError("modeproblem_matrix_packed: " + _lib.last_error())
        return out

    def wavenumber(self):
        """ssw->wavenumber of the C structure (scatsystem.h:239-249)."""
        w = C.cast(self.ssw, C.POINTER(_SSW)).contents
        return complex(w.wavenumber[0], w.wavenumber[1])

    def scattered_E(self, scatcoeffvector_full, evalpos, alt=False, btyp=QPMS_HANKEL_PLUS, k=None, eta=0.0):
        """qpms_c.pyx:1118-1141, at this frequency's wavenumber; for a 2D lattice
        give the Bloch vector k (qpms_c.pyx:974-996, points in the particles'
        plane; eta = 0 selects the adjusted Ewald parameter)."""
        if k is None:
            return self.ss.scattered_E(self.wavenumber(), scatcoeffvector_full, evalpos, alt, btyp)
        evalpos = np.asarray(evalpos, dtype=np.float64)
        if evalpos.shape[-1] != 3:
            raise ValueError("Last dimension of evalpos has to be 3")
        w = np.ascontiguousarray(evalpos.reshape(-1, 3))
        cv = np.ascontiguousarray(scatcoeffvector_full, dtype=np.complex128)
        if cv.size != self.ss.fecv_size:
            raise ValueError("Length of a full coefficient vector has to be %d, not %d" % (self.ss.fecv_size, cv.size))
        wk = _SSWK()
        wk.ssw = self.ssw
        kk = list(k) + [0.0] * (3 - len(k))
        for i in range(3):
            wk.k[i] = kk[i]
        wk.eta = float(eta)
        E = np.empty((w.shape[0], 3), dtype=np.complex128)
        _lib.check(self._L.qpms_gpu_scatsyswk_scattered_E(C.byref(wk), int(btyp), cv.ctypes.data, w.shape[0],
                                                          w.ctypes.data, E.ctypes.data),
                   "qpms_gpu_scatsyswk_scattered_E")
        return E.reshape(evalpos.shape)


class ScatteringMatrix:
    """LU-factorised (I - T S) (qpms_ss_LU), full or projected on irrep ``iri``
    (qpms_c.pyx:1144-1195); calling it solves for f (full or packed)."""

    def __init__(self, ssw, iri=None):
        self.ssw = ssw
        self._L = ssw._L
        self.iri = iri
        if iri is None:
            self.lu = self._L.qpms_scatsysw_build_modeproblem_matrix_full_LU(None, None, ssw.ssw)
        else:
            self.lu = self._L.qpms_scatsysw_build_modeproblem_matrix_irrep_packed_LU(None, None, ssw.ssw, int(iri))
        if not self.lu.a:
            raise _lib.QpmsGpuError("LU: " + _lib.last_error())

    def __del__(self):
        lu = getattr(self, "lu", None)
        if lu is not None and lu.a:
            self._L.qpms_ss_LU_free(lu)
            self.lu = None

    def __call__(self, a_inc):
        n = self.ssw.ss.fecv_size if self.iri is None else self.ssw.ss.saecv_sizes[self.iri]
        a = np.ascontiguousarray(a_inc, dtype=np.complex128)
        if a.size != n:
            raise ValueError("Length of a %s coefficient vector has to be %d, not %d"
                             % ("full" if self.iri is None else "packed", n, a.size))
        f = np.empty(n, dtype=np.complex128)
        if not self._L.qpms_scatsys_scatter_solve(f.ctypes.data, a.ctypes.data, self.lu):
            raise _lib.QpmsGpuError("scatter_solve: " + _lib.last_error())
        return f
