// LU factorisation / solve drop-ins and the batched plane-wave scattering
// pipeline (assembly -> incident field -> T a -> LU solve -> sigma_ext).
//
// Two solve modes for the batched pipeline:
//   mode 0 ("plain FP64"): complex128 LU with partial pivoting (cuBLAS
//          getrf/getrs batched) -- the plain FP64 GPU path;
//   mode 1 ("mixed"):      complex64 LU of the same matrices, then FP64
//          iterative refinement x += LU64^{-1} (b - M x) with the residual
//          formed in FP64 from the FP64 matrix, until ||b - M x|| / ||b||
//          <= 1e-13 (or stagnation); the achieved residual is reported.
#include <cublas_v2.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "qg_assembly.h"
#include "qg_batched.h"
#include "qg_batchlu.h"
#include "qg_dense.h"
#include "qg_internal.h"

namespace qg {
bool scatsys_is_own(const qpms_scatsys_t *ss);
int scatsys_lmax(const qpms_scatsys_t *ss);
bool scatsys_dense(const qpms_scatsys_t *ss);
int sym_nirreps(const qpms_scatsys_t *ss);
size_t sym_size(const qpms_scatsys_t *ss, int iri);
int sym_pack_matrix_device(const qpms_scatsys_t *ss, int iri, const qg_c *dM, size_t ldm, qg_c *dout,
                           cudaStream_t st);
int sym_pack_vectors_device(const qpms_scatsys_t *ss, int iri, const qg_c *dv, int nrhs, size_t ldv, qg_c *dout,
                            size_t ldo, cudaStream_t st);
int sym_unpack_add_vectors_device(const qpms_scatsys_t *ss, int iri, const qg_c *dp, int nrhs, size_t ldp,
                                  qg_c *dfull, size_t ldf, cudaStream_t st);
void scatsys_tdiag(const qpms_scatsys_t *ss, int t, double om_re, double om_im, std::vector<qg_c> &out);
qg_c scatsys_wavenumber(const qpms_scatsys_t *ss, double om_re, double om_im);
void planewave_direction_coeffs(int lMax, const double k_dir[3], const qpms_complex_t E_cart[3],
                                std::vector<qg_c> &coef);
int blas_handle_get(cublasHandle_t *h);
int assemble_modeproblem_device(const qpms_scatsys_t *ss, int nw, const std::vector<qg_c> &T_host, bool dense,
                                const std::vector<qg_c> &k_host, int J, qg_c *dM, cudaStream_t st);

namespace {



struct Dev {
  void *p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  template <typename T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};
int dalloc(Dev &b, size_t bytes) {
  QG_CUDA_TRY(cudaMalloc(&b.p, bytes ? bytes : 16));
  return QPMS_SUCCESS;
}

// device array of nb pointers base + i * stride_bytes
int ptr_array(Dev &arr, void *base, size_t stride_bytes, int nb) {
  std::vector<void *> h(nb);
  for (int i = 0; i < nb; ++i) h[i] = (char *)base + (size_t)i * stride_bytes;
  int e;
  if ((e = dalloc(arr, sizeof(void *) * nb))) return e;
  QG_CUDA_TRY(cudaMemcpy(arr.p, h.data(), sizeof(void *) * nb, cudaMemcpyHostToDevice));
  return QPMS_SUCCESS;
}

// Above this size the batched (one kernel per small matrix) LU is slow and
// each frequency runs through the dense solver (RBT + blocked LU) instead.
constexpr size_t kBatchedMaxN = 512;

// The finite plane-wave scatter for large systems: one frequency at a time
// (one N x N matrix resident), assembly -> incidence -> T a -> dense solve
// with FP64 refinement -> sigma_ext (and sigma_scat).
int finite_scatter_dense(const qpms_scatsys_t *ss, int W, const std::vector<qg_c> &T, const std::vector<qg_c> &k,
                         const std::vector<double> &kvec, const std::vector<qg_c> &coef, int mode, qpms_complex_t *f_out,
                         double *sigma_ext, double *sigma_scat, double *resid_out, int *iters_out) {
  const int lMax = scatsys_lmax(ss), np = ss->p_count, ntm = ss->tm_count;
  const int n = 2 * lMax * (lMax + 2);
  const size_t N = ss->fecv_size, N2 = N * N;
  const size_t tper = T.size() / W;
  cudaStream_t st = 0;
  int e;
  Dev dM, dT, dtm, dpos, dk, dkv, dcoef, da, db, dx, dr, dn, dsig;
  if ((e = dalloc(dM, N2 * 16)) || (e = dalloc(dT, tper * 16)) || (e = dalloc(dtm, np * 4)) ||
      (e = dalloc(dpos, np * 24)) || (e = dalloc(dk, 16)) || (e = dalloc(dkv, 24)) || (e = dalloc(dcoef, n * 16)) ||
      (e = dalloc(da, N * 16)) || (e = dalloc(db, N * 16)) || (e = dalloc(dx, N * 16)) || (e = dalloc(dr, N * 16)) ||
      (e = dalloc(dn, 16)) || (e = dalloc(dsig, 8)))
    return e;
  std::vector<double> pos(3 * np);
  std::vector<int> tm(np);
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
    tm[i] = ss->p[i].tmatrix_id;
  }
  QG_CUDA_TRY(cudaMemcpy(dtm.p, tm.data(), np * 4, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dpos.p, pos.data(), np * 24, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dcoef.p, coef.data(), n * 16, cudaMemcpyHostToDevice));
  // With a point symmetry the system splits into one independent system per
  // irrep (about N / |G| unknowns each: |G|^2 fewer LU flops): M and T a are
  // packed on the device, each irrep is solved, and the solutions unpacked.
  const int nir = sym_nirreps(ss);
  DenseSolver ds;
  std::vector<std::unique_ptr<DenseSolver>> dsi(nir);
  Dev dMp, dbp, dxp;
  size_t namax = 0;
  for (int i = 0; i < nir; ++i) namax = std::max(namax, sym_size(ss, i));
  if (nir == 0) {
    if ((e = ds.init((int)N, 1, mode, 0x5eedbe11))) return e;
  } else {
    if ((e = dalloc(dMp, namax * namax * 16)) || (e = dalloc(dbp, namax * 16)) || (e = dalloc(dxp, namax * 16)))
      return e;
    for (int i = 0; i < nir; ++i) {
      const size_t na = sym_size(ss, i);
      if (!na) continue;
      dsi[i].reset(new DenseSolver());
      if ((e = dsi[i]->init((int)na, 1, mode, 0x5eedbe11 + i))) return e;
    }
  }
  const bool dense = scatsys_dense(ss);
  auto assemble = [&](int J, const qg_c *Tsrc, size_t count, bool dn) -> int {
    QG_CUDA_TRY(cudaMemcpy(dT.p, Tsrc, count * 16, cudaMemcpyHostToDevice));
    AsmArgs a;
    a.nw = 1;
    a.np = np;
    a.ntm = ntm;
    a.dense = dn ? 1 : 0;
    a.J = J;
    a.pos = dpos.as<double>();
    a.tmid = dtm.as<int>();
    a.T = dT.as<qg_c>();
    a.k = dk.as<qg_c>();
    a.M = dM.as<qg_c>();
    return launch_assemble(a, priv(ss->c)->dev, st);
  };
  const std::vector<qg_c> mone((size_t)ntm * n, cmk(-1.0, 0.0));  // diagonal -1
  for (int w = 0; w < W; ++w) {
    QG_CUDA_TRY(cudaMemcpy(dk.p, &k[w], 16, cudaMemcpyHostToDevice));
    QG_CUDA_TRY(cudaMemcpy(dkv.p, &kvec[3 * w], 24, cudaMemcpyHostToDevice));
    if ((e = assemble(3, T.data() + w * tper, tper, dense))) return e;  // row-major M = I - T S
    if ((e = launch_incident(1, np, n, dcoef.as<qg_c>(), dkv.as<double>(), dpos.as<double>(), da.as<qg_c>(), st)))
      return e;
    if ((e = launch_apply_t(1, np, n, ntm, dense ? 1 : 0, dtm.as<int>(), dT.as<qg_c>(), da.as<qg_c>(),
                            db.as<qg_c>(), st)))
      return e;
    double res = 0;
    int it = 0;
    if (nir == 0) {
      if ((e = ds.factorize(dM.p, N, st, true))) return e;
      if ((e = ds.solve(dM.p, N, db.p, dx.p, 1, 1e-13, 12, &res, &it, st))) return e;
    } else {
      QG_CUDA_TRY(cudaMemsetAsync(dx.p, 0, N * 16, st));
      for (int i = 0; i < nir; ++i) {
        const size_t na = sym_size(ss, i);
        if (!na) continue;
        double ri = 0;
        int iti = 0;
        if ((e = sym_pack_matrix_device(ss, i, dM.as<qg_c>(), N, dMp.as<qg_c>(), st)) ||
            (e = sym_pack_vectors_device(ss, i, db.as<qg_c>(), 1, N, dbp.as<qg_c>(), na, st)) ||
            (e = dsi[i]->factorize(dMp.p, na, st, true)) ||
            (e = dsi[i]->solve(dMp.p, na, dbp.p, dxp.p, 1, 1e-13, 12, &ri, &iti, st)) ||
            (e = sym_unpack_add_vectors_device(ss, i, dxp.as<qg_c>(), 1, na, dx.as<qg_c>(), N, st)))
          return e;
        it = std::max(it, iti);
      }
      // the residual of the unpacked solution in the full system (FP64)
      double *rn2 = dn.as<double>(), h2[2];
      if ((e = launch_residual(1, N, dM.as<qg_c>(), dx.as<qg_c>(), db.as<qg_c>(), dr.as<qg_c>(), rn2, rn2 + 1, st)))
        return e;
      QG_CUDA_TRY(cudaMemcpy(h2, rn2, 16, cudaMemcpyDeviceToHost));
      res = sqrt(h2[0] / (h2[1] > 0 ? h2[1] : 1));
    }
    if (resid_out) resid_out[w] = res;
    if (iters_out) iters_out[w] = it;
    if ((e = launch_sigma_ext(1, N, da.as<qg_c>(), dx.as<qg_c>(), dk.as<qg_c>(), dsig.as<double>(), st))) return e;
    QG_CUDA_TRY(cudaMemcpy(sigma_ext + w, dsig.p, 8, cudaMemcpyDeviceToHost));
    if (sigma_scat) {
      if ((e = assemble(1, mone.data(), mone.size(), false))) return e;  // I + R (regular waves, zero self blocks)
      QG_CUDA_TRY(cudaMemsetAsync(db.p, 0, N * 16, st));
      double *rn2 = dn.as<double>();
      if ((e = launch_residual(1, N, dM.as<qg_c>(), dx.as<qg_c>(), db.as<qg_c>(), dr.as<qg_c>(), rn2, rn2 + 1, st)))
        return e;
      if ((e = launch_sigma_ext(1, N, dx.as<qg_c>(), dr.as<qg_c>(), dk.as<qg_c>(), dsig.as<double>(), st))) return e;
      QG_CUDA_TRY(cudaMemcpy(sigma_scat + w, dsig.p, 8, cudaMemcpyDeviceToHost));
    }
    if (f_out) QG_CUDA_TRY(cudaMemcpy(f_out + w * N, dx.p, N * 16, cudaMemcpyDeviceToHost));
  }
  return QPMS_SUCCESS;
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

static qpms_ss_LU factorise_any(qpms_complex_t *mpmatrix_full, int *target_piv, const qpms_scatsys_at_omega_t *ssw,
                                const qpms_scatsys_at_omega_k_t *sswk, int iri);

qpms_ss_LU qpms_scatsysw_modeproblem_matrix_full_factorise(qpms_complex_t *mpmatrix_full, int *target_piv,
                                                           const qpms_scatsys_at_omega_t *ssw,
                                                           const qpms_scatsys_at_omega_k_t *sswk) {
  return factorise_any(mpmatrix_full, target_piv, ssw, sswk, -1);
}

// Irrep-packed counterpart (scatsystem.h:467-473): the matrix is
// saecv_sizes[iri] squared.
qpms_ss_LU qpms_scatsysw_modeproblem_matrix_irrep_packed_factorise(qpms_complex_t *mpmatrix_packed, int *target_piv,
                                                                   const qpms_scatsys_at_omega_t *ssw, int iri) {
  return factorise_any(mpmatrix_packed, target_piv, ssw, nullptr, iri);
}

qpms_ss_LU qpms_scatsysw_build_modeproblem_matrix_irrep_packed_LU(qpms_complex_t *target, int *target_piv,
                                                                  const qpms_scatsys_at_omega_t *ssw, int iri) {
  qpms_complex_t *M = qpms_scatsysw_build_modeproblem_matrix_irrep_packed(target, ssw, iri);
  if (!M) {
    qpms_ss_LU lu;
    memset(&lu, 0, sizeof lu);
    return lu;
  }
  return factorise_any(M, target_piv, ssw, nullptr, iri);
}

static qpms_ss_LU factorise_any(qpms_complex_t *mpmatrix_full, int *target_piv, const qpms_scatsys_at_omega_t *ssw,
                                const qpms_scatsys_at_omega_k_t *sswk, int iri) {
  clear_error();
  qpms_ss_LU lu;
  memset(&lu, 0, sizeof lu);
  if (sswk && !ssw) ssw = sswk->ssw;
  lu.ssw = ssw;
  lu.sswk = sswk;
  lu.full = iri < 0;
  lu.iri = iri < 0 ? -1 : iri;
  if (!mpmatrix_full || !ssw) { set_error("NULL matrix or ssw"); return lu; }
  if (iri >= 0 && !ssw->ss->saecv_sizes) { set_error("the system has no point symmetry"); return lu; }
  const size_t N = iri < 0 ? ssw->ss->fecv_size : ssw->ss->saecv_sizes[iri];
  if (N == 0) { set_error("empty irrep"); return lu; }
  bool own_piv = false;
  if (!target_piv) {
    target_piv = (int *)malloc(sizeof(int) * N);
    own_piv = true;
  }
  cublasHandle_t h;
  Dev dA, dT, dP, dI, arr;
  int info = 0;
  auto fail = [&]() {
    if (own_piv) free(target_piv);
    lu.a = nullptr;
    lu.ipiv = nullptr;
    return lu;
  };
  if (blas_handle_get(&h) || dalloc(dA, N * N * 16) || dalloc(dT, N * N * 16) || dalloc(dP, N * 4) ||
      dalloc(dI, 4))
    return fail();
  if (cudaMemcpy(dA.p, mpmatrix_full, N * N * 16, cudaMemcpyHostToDevice) != cudaSuccess) return fail();
  if (N <= (size_t)kBatchLuMaxN) {
    // the library's batched LU on the row-major matrix; LAPACK's 1-based pivots
    std::vector<int> p0(N);
    if (batch_getrf_c128(1, (int)N, dA.p, dP.as<int>(), dI.as<int>(), 0) ||
        cudaMemcpy(mpmatrix_full, dA.p, N * N * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(p0.data(), dP.p, N * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&info, dI.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
      if (!qpms_gpu_last_error()[0]) set_error("batched LU or device to host copy failed");
      return fail();
    }
    for (size_t i = 0; i < N; ++i) target_piv[i] = p0[i] + 1;
    if (info != 0) set_error("LU: U(%d,%d) is exactly zero", info, info);
    lu.a = mpmatrix_full;
    lu.ipiv = target_piv;
    return lu;
  }
  // larger orders: row-major M -> column-major M, cuBLAS zgetrf, back to row-major storage
  if (launch_transpose(N, 1, dA.as<qg_c>(), dT.as<qg_c>(), 0)) return fail();
  if (ptr_array(arr, dT.p, 0, 1)) return fail();
  if (cublasZgetrfBatched(h, (int)N, arr.as<cuDoubleComplex *>(), (int)N, dP.as<int>(), dI.as<int>(), 1) !=
      CUBLAS_STATUS_SUCCESS) {
    set_error("cublasZgetrfBatched failed");
    return fail();
  }
  g_launches.fetch_add(1);
  if (launch_transpose(N, 1, dT.as<qg_c>(), dA.as<qg_c>(), 0)) return fail();
  if (cudaMemcpy(mpmatrix_full, dA.p, N * N * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(target_piv, dP.p, N * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(&info, dI.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    return fail();
  }
  if (info != 0) set_error("LU: U(%d,%d) is exactly zero", info, info);
  lu.a = mpmatrix_full;
  lu.ipiv = target_piv;
  return lu;
}

qpms_ss_LU qpms_scatsysw_build_modeproblem_matrix_full_LU(qpms_complex_t *target, int *target_piv,
                                                          const qpms_scatsys_at_omega_t *ssw) {
  qpms_complex_t *M = qpms_scatsysw_build_modeproblem_matrix_full(target, ssw);
  if (!M) {
    qpms_ss_LU lu;
    memset(&lu, 0, sizeof lu);
    return lu;
  }
  return qpms_scatsysw_modeproblem_matrix_full_factorise(M, target_piv, ssw, nullptr);
}

qpms_complex_t *qpms_scatsys_scatter_solve(qpms_complex_t *f, const qpms_complex_t *a_inc, qpms_ss_LU lu) {
  clear_error();
  if (!lu.a || !lu.ipiv || !lu.ssw || !a_inc) { set_error("invalid LU or a_inc"); return nullptr; }
  // full or irrep-packed vectors (scatsystem.c:2262-2273)
  const size_t N = lu.full ? lu.ssw->ss->fecv_size : lu.ssw->ss->saecv_sizes[lu.iri];
  cublasHandle_t h;
  Dev dA, dT, dP, dB, arrA, arrB;
  if (blas_handle_get(&h) || dalloc(dA, N * N * 16) || dalloc(dT, N * N * 16) || dalloc(dP, N * 4) ||
      dalloc(dB, N * 16))
    return nullptr;
  if (cudaMemcpy(dA.p, lu.a, N * N * 16, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dP.p, lu.ipiv, N * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dB.p, a_inc, N * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("host to device copy failed");
    return nullptr;
  }
  int info = 0;
  if (N <= (size_t)kBatchLuMaxN) {  // LAPACK's 1-based pivots -> the batched kernel's 0-based
    std::vector<int> p0(N);
    for (size_t i = 0; i < N; ++i) {
      p0[i] = lu.ipiv[i] - 1;
      if (p0[i] < 0 || p0[i] >= (int)N) {
        set_error("LU: pivot %d of row %zu outside 1..%zu", lu.ipiv[i], i + 1, N);
        return nullptr;
      }
    }
    if (cudaMemcpy(dP.p, p0.data(), N * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        batch_getrs_c128(1, (int)N, dA.p, dP.as<int>(), dB.p, 0))
      return nullptr;
  } else if (launch_transpose(N, 1, dA.as<qg_c>(), dT.as<qg_c>(), 0) || ptr_array(arrA, dT.p, 0, 1) ||
             ptr_array(arrB, dB.p, 0, 1)) {
    return nullptr;
  } else if (cublasZgetrsBatched(h, CUBLAS_OP_N, (int)N, 1, arrA.as<const cuDoubleComplex *>(), (int)N, dP.as<int>(),
                          arrB.as<cuDoubleComplex *>(), (int)N, &info, 1) != CUBLAS_STATUS_SUCCESS ||
      info != 0) {
    set_error("cublasZgetrsBatched failed (info %d)", info);
    return nullptr;
  }
  g_launches.fetch_add(1);
  bool own = false;
  if (!f) {
    f = (qpms_complex_t *)malloc(N * 16);
    own = true;
  }
  if (cudaMemcpy(f, dB.p, N * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    if (own) free(f);
    return nullptr;
  }
  return f;
}

void qpms_ss_LU_free(qpms_ss_LU lu) {
  free(lu.a);
  free(lu.ipiv);
}

qpms_complex_t *qpms_scatsysw_apply_Tmatrices_full(qpms_complex_t *target_full, const qpms_complex_t *inc_full,
                                                   const qpms_scatsys_at_omega_t *ssw) {
  clear_error();
  if (!ssw || !inc_full) { set_error("NULL argument"); return nullptr; }
  const qpms_scatsys_t *ss = ssw->ss;
  const size_t N = ss->fecv_size, n = ssw->tm[0]->spec->n;
  std::vector<qg_c> T;
  for (int t = 0; t < ss->tm_count; ++t)
    for (size_t i = 0; i < n * n; ++i) T.push_back(*(const qg_c *)&ssw->tm[t]->m[i]);
  std::vector<int> tm(ss->p_count);
  for (int i = 0; i < ss->p_count; ++i) tm[i] = ss->p[i].tmatrix_id;
  Dev dT, dtm, da, db;
  if (dalloc(dT, T.size() * 16) || dalloc(dtm, tm.size() * 4) || dalloc(da, N * 16) || dalloc(db, N * 16))
    return nullptr;
  if (cudaMemcpy(dT.p, T.data(), T.size() * 16, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dtm.p, tm.data(), tm.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(da.p, inc_full, N * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("host to device copy failed");
    return nullptr;
  }
  if (launch_apply_t(1, ss->p_count, (int)n, ss->tm_count, 1, dtm.as<int>(), dT.as<qg_c>(), da.as<qg_c>(),
                     db.as<qg_c>(), 0))
    return nullptr;
  bool own = false;
  if (!target_full) {
    target_full = (qpms_complex_t *)malloc(N * 16);
    own = true;
  }
  if (cudaMemcpy(target_full, db.p, N * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    if (own) free(target_full);
    return nullptr;
  }
  return target_full;
}

int qpms_gpu_incident_planewave_full(qpms_complex_t *target_full, const qpms_scatsys_t *ss, const double k_cart[3],
                                     const qpms_complex_t E_cart[3]) {
  clear_error();
  if (!ss || !target_full || !k_cart || !E_cart) { set_error("NULL argument"); return QPMS_EINVAL; }
  const int np = ss->p_count;
  const size_t N = ss->fecv_size, n = N / np;
  const int lMax = (int)(sqrt((double)n / 2 + 1) - 1 + 0.5);
  std::vector<qg_c> coef;
  planewave_direction_coeffs(lMax, k_cart, E_cart, coef);
  std::vector<double> pos(3 * np);
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
  }
  Dev dc, dk, dp, da;
  int e;
  if ((e = dalloc(dc, coef.size() * 16)) || (e = dalloc(dk, 24)) || (e = dalloc(dp, pos.size() * 8)) ||
      (e = dalloc(da, N * 16)))
    return e;
  QG_CUDA_TRY(cudaMemcpy(dc.p, coef.data(), coef.size() * 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dk.p, k_cart, 24, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dp.p, pos.data(), pos.size() * 8, cudaMemcpyHostToDevice));
  if ((e = launch_incident(1, np, (int)n, dc.as<qg_c>(), dk.as<double>(), dp.as<double>(), da.as<qg_c>(), 0)))
    return e;
  QG_CUDA_TRY(cudaMemcpy(target_full, da.p, N * 16, cudaMemcpyDeviceToHost));
  return QPMS_SUCCESS;
}

int qpms_gpu_finite_planewave_scatter(const qpms_scatsys_t *ss, size_t nw, const double *omegas,
                                      const double k_dir[3], const qpms_complex_t E_cart[3], int mode,
                                      qpms_complex_t *f_out, double *sigma_ext, double *resid_out, int *iters_out) {
  return qpms_gpu_finite_planewave_scatter_ext(ss, nw, omegas, k_dir, E_cart, mode, f_out, sigma_ext, nullptr,
                                               resid_out, iters_out);
}

int qpms_gpu_finite_planewave_scatter_ext(const qpms_scatsys_t *ss, size_t nw, const double *omegas,
                                          const double k_dir[3], const qpms_complex_t E_cart[3], int mode,
                                          qpms_complex_t *f_out, double *sigma_ext, double *sigma_scat,
                                          double *resid_out, int *iters_out) {
  clear_error();
  if (!scatsys_is_own(ss)) { set_error("system must come from qpms_gpu_scatsys_create_spheres"); return QPMS_EINVAL; }
  if (!omegas || !k_dir || !E_cart || !sigma_ext) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (mode != 0 && mode != 1) { set_error("mode must be 0 (FP64) or 1 (mixed)"); return QPMS_EINVAL; }
  if (nw == 0) return QPMS_SUCCESS;
  const int lMax = scatsys_lmax(ss), np = ss->p_count, ntm = ss->tm_count;
  const int n = 2 * lMax * (lMax + 2);
  const size_t N = ss->fecv_size, N2 = N * N;
  const int W = (int)nw;
  // host set-up: T diagonals per (omega, type), wavenumbers, incidence
  std::vector<qg_c> T, k(W), coef;
  std::vector<double> kvec(3 * W);
  const double kn = sqrt(k_dir[0] * k_dir[0] + k_dir[1] * k_dir[1] + k_dir[2] * k_dir[2]);
  for (int w = 0; w < W; ++w) {
    for (int t = 0; t < ntm; ++t) {
      std::vector<qg_c> d;
      scatsys_tdiag(ss, t, omegas[w], 0.0, d);
      T.insert(T.end(), d.begin(), d.end());
    }
    k[w] = scatsys_wavenumber(ss, omegas[w], 0.0);
    for (int c = 0; c < 3; ++c) kvec[3 * w + c] = k[w].re * k_dir[c] / kn;
  }
  planewave_direction_coeffs(lMax, k_dir, E_cart, coef);
  if (N > kBatchedMaxN)
    return finite_scatter_dense(ss, W, T, k, kvec, coef, mode, f_out, sigma_ext, sigma_scat, resid_out, iters_out);
  cudaStream_t st = 0;
  cublasHandle_t h;
  int e;
  if ((e = blas_handle_get(&h))) return e;
  QG_BLAS_TRY(cublasSetStream(h, st));
  Dev dM, dLU, dpiv, dinfo, dT, dtm, dpos, dk, dkv, dcoef, da, db, dx, dr, dn, dsig, dcb;
  if ((e = dalloc(dM, N2 * W * 16)) || (e = dalloc(dLU, N2 * W * (mode ? 8 : 16))) ||
      (e = dalloc(dpiv, N * W * 4)) || (e = dalloc(dinfo, W * 4)) || (e = dalloc(dT, T.size() * 16)) ||
      (e = dalloc(dtm, np * 4)) || (e = dalloc(dpos, np * 24)) || (e = dalloc(dk, W * 16)) ||
      (e = dalloc(dkv, W * 24)) || (e = dalloc(dcoef, n * 16)) || (e = dalloc(da, N * W * 16)) ||
      (e = dalloc(db, N * W * 16)) || (e = dalloc(dx, N * W * 16)) || (e = dalloc(dr, N * W * 16)) ||
      (e = dalloc(dn, W * 16)) || (e = dalloc(dsig, W * 8)) || (e = dalloc(dcb, N * W * 8)))
    return e;
  std::vector<double> pos(3 * np);
  std::vector<int> tm(np);
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
    tm[i] = ss->p[i].tmatrix_id;
  }
  QG_CUDA_TRY(cudaMemcpy(dT.p, T.data(), T.size() * 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dtm.p, tm.data(), np * 4, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dpos.p, pos.data(), np * 24, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dk.p, k.data(), W * 16, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dkv.p, kvec.data(), W * 24, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dcoef.p, coef.data(), n * 16, cudaMemcpyHostToDevice));
  // assemble M_w = I - T_w S_w (FP64)
  {
    AsmArgs a;
    a.nw = W;
    a.np = np;
    a.ntm = ntm;
    a.dense = scatsys_dense(ss) ? 1 : 0;
    a.J = 3;
    a.pos = dpos.as<double>();
    a.tmid = dtm.as<int>();
    a.T = dT.as<qg_c>();
    a.k = dk.as<qg_c>();
    a.M = dM.as<qg_c>();
    if ((e = launch_assemble(a, priv(ss->c)->dev, st))) return e;
  }
  if ((e = launch_incident(W, np, n, dcoef.as<qg_c>(), dkv.as<double>(), dpos.as<double>(), da.as<qg_c>(), st)))
    return e;
  if ((e = launch_apply_t(W, np, n, ntm, scatsys_dense(ss) ? 1 : 0, dtm.as<int>(), dT.as<qg_c>(), da.as<qg_c>(),
                          db.as<qg_c>(), st)))
    return e;
  double *rn2 = dn.as<double>(), *bn2 = rn2 + W;
  std::vector<double> hr(W), hb(W);
  std::vector<int> iters(W, 0);
  int info = 0;
  if (mode == 0) {
    QG_CUDA_TRY(cudaMemcpyAsync(dLU.p, dM.p, N2 * W * 16, cudaMemcpyDeviceToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dx.p, db.p, N * W * 16, cudaMemcpyDeviceToDevice, st));
    if ((e = batch_getrf_c128(W, (int)N, dLU.p, dpiv.as<int>(), dinfo.as<int>(), st))) return e;
    if ((e = batch_getrs_c128(W, (int)N, dLU.p, dpiv.as<int>(), dx.p, st))) return e;
    if ((e = launch_residual(W, N, dM.as<qg_c>(), dx.as<qg_c>(), db.as<qg_c>(), dr.as<qg_c>(), rn2, bn2, st)))
      return e;
    QG_CUDA_TRY(cudaMemcpy(hr.data(), rn2, W * 8, cudaMemcpyDeviceToHost));
    QG_CUDA_TRY(cudaMemcpy(hb.data(), bn2, W * 8, cudaMemcpyDeviceToHost));
  } else {
    if ((e = launch_c128_to_c64(N2 * W, dM.as<qg_c>(), dLU.p, st))) return e;
    if ((e = batch_getrf_c64(W, (int)N, dLU.p, dpiv.as<int>(), dinfo.as<int>(), st))) return e;
    // x0 = LU32^{-1} b, then refine: r = b - M x (FP64), x += LU32^{-1} r
    QG_CUDA_TRY(cudaMemcpyAsync(dr.p, db.p, N * W * 16, cudaMemcpyDeviceToDevice, st));
    const int kMaxIter = max_refine_steps(12);
    double prev = 1e300;
    for (int it = 0; it <= kMaxIter; ++it) {
      if ((e = launch_c128_to_c64(N * W, dr.as<qg_c>(), dcb.p, st))) return e;
      if ((e = batch_getrs_c64(W, (int)N, dLU.p, dpiv.as<int>(), dcb.p, st))) return e;
      if ((e = launch_add_c64(N * W, dcb.p, dx.as<qg_c>(), it == 0, st))) return e;
      if ((e = launch_residual(W, N, dM.as<qg_c>(), dx.as<qg_c>(), db.as<qg_c>(), dr.as<qg_c>(), rn2, bn2, st)))
        return e;
      QG_CUDA_TRY(cudaMemcpy(hr.data(), rn2, W * 8, cudaMemcpyDeviceToHost));
      QG_CUDA_TRY(cudaMemcpy(hb.data(), bn2, W * 8, cudaMemcpyDeviceToHost));
      double worst = 0;
      for (int w = 0; w < W; ++w) {
        const double rel = sqrt(hr[w] / (hb[w] > 0 ? hb[w] : 1));
        if (rel > 1e-13) iters[w] = it + 1;
        worst = fmax(worst, rel);
      }
      if (worst <= 1e-13 || worst >= 0.5 * prev) break;  // converged or stagnated
      prev = worst;
    }
    // frequencies whose refinement stalled: solved again in complex128
    std::vector<int> bad;
    for (int w = 0; w < W; ++w)
      if (sqrt(hr[w] / (hb[w] > 0 ? hb[w] : 1)) > 1e-13) bad.push_back(w);
    if (!bad.empty()) {
      if ((e = resolve_fp64(st, bad, N, dM.as<qg_c>(), db.as<qg_c>(), dx.as<qg_c>()))) return e;
      if ((e = launch_residual(W, N, dM.as<qg_c>(), dx.as<qg_c>(), db.as<qg_c>(), dr.as<qg_c>(), rn2, bn2, st)))
        return e;
      QG_CUDA_TRY(cudaMemcpy(hr.data(), rn2, W * 8, cudaMemcpyDeviceToHost));
      QG_CUDA_TRY(cudaMemcpy(hb.data(), bn2, W * 8, cudaMemcpyDeviceToHost));
    }
  }
  if ((e = launch_sigma_ext(W, N, da.as<qg_c>(), dx.as<qg_c>(), dk.as<qg_c>(), dsig.as<double>(), st))) return e;
  QG_CUDA_TRY(cudaMemcpy(sigma_ext, dsig.p, W * 8, cudaMemcpyDeviceToHost));
  if (sigma_scat) {
    // sigma_scat = Re(f^H (I + R) f) / k^2 with R the regular-wave translation
    // matrix, zero self blocks (misc/finiterectlat-scatter.py:98-111): the
    // assembly with J = 1 and T = -1 builds I + R in place of M
    std::vector<qg_c> mone((size_t)W * ntm * n, cmk(-1.0, 0.0));  // diagonal -1 (dT holds at least this)
    QG_CUDA_TRY(cudaMemcpy(dT.p, mone.data(), mone.size() * 16, cudaMemcpyHostToDevice));
    AsmArgs a;
    a.nw = W;
    a.np = np;
    a.ntm = ntm;
    a.dense = 0;
    a.J = 1;
    a.pos = dpos.as<double>();
    a.tmid = dtm.as<int>();
    a.T = dT.as<qg_c>();
    a.k = dk.as<qg_c>();
    a.M = dM.as<qg_c>();
    if ((e = launch_assemble(a, priv(ss->c)->dev, st))) return e;
    // r = 0 - (I + R) f, then -Re(f^H r) / k^2
    QG_CUDA_TRY(cudaMemsetAsync(db.p, 0, N * W * 16, st));
    if ((e = launch_residual(W, N, dM.as<qg_c>(), dx.as<qg_c>(), db.as<qg_c>(), dr.as<qg_c>(), rn2, bn2, st)))
      return e;
    if ((e = launch_sigma_ext(W, N, dx.as<qg_c>(), dr.as<qg_c>(), dk.as<qg_c>(), dsig.as<double>(), st))) return e;
    QG_CUDA_TRY(cudaMemcpy(sigma_scat, dsig.p, W * 8, cudaMemcpyDeviceToHost));
  }
  if (f_out) QG_CUDA_TRY(cudaMemcpy(f_out, dx.p, N * W * 16, cudaMemcpyDeviceToHost));
  for (int w = 0; w < W; ++w) {
    if (resid_out) resid_out[w] = sqrt(hr[w] / (hb[w] > 0 ? hb[w] : 1));
    if (iters_out) iters_out[w] = mode ? iters[w] + 1 : 0;
  }
  std::vector<int> hinfo(W);
  QG_CUDA_TRY(cudaMemcpy(hinfo.data(), dinfo.p, W * 4, cudaMemcpyDeviceToHost));
  for (int w = 0; w < W; ++w)
    if (hinfo[w] != 0) {
      set_error("singular matrix at frequency %d (info %d)", w, hinfo[w]);
      return QPMS_ERROR;
    }
  return QPMS_SUCCESS;
}

}  // extern "C"
