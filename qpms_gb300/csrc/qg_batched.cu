// Batched solve of many small mode-problem systems (the (omega, k) points of a
// dispersion scan, serving batches of lattice solves): one batched LU launch
// for all systems (qg_batchlu.cu, partial pivoting on the row-major matrices),
// then the right-hand sides.  The mixed mode factorises in
// complex64 and recovers FP64 accuracy by iterative refinement with an FP64
// residual (residual_kernel, one warp per row), as qg_solve.cu does for the
// finite plane-wave scatter.  The reference factorises each matrix with
// LAPACKE_zgetrf and solves with zgetrs (scatsystem.c:2202-2273).
#include <math.h>

#include <atomic>
#include <vector>

#include "qg_assembly.h"
#include "qg_batched.h"
#include "qg_batchlu.h"

namespace qg {

namespace {

size_t al(size_t b) { return (b + 255) / 256 * 256; }

template <typename T>
__global__ void logabsdet_kernel(int nm, size_t N, const T *LU, double *out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nm) return;
  const T *A = LU + (size_t)b * N * N;
  double s = 0;
  for (size_t i = 0; i < N; ++i) s += log(hypot((double)A[i * N + i].x, (double)A[i * N + i].y));
  out[b] = s;
}

}  // namespace

size_t batched_solve_bytes(int nm, size_t N, int mode) {
  const size_t m = (size_t)nm;
  return al(m * N * N * (mode ? 8 : 16)) + al(m * N * 4) + al(m * 4) + al(m * N * 8) + al(m * N * 16) +
         al(2 * m * 8);
}

namespace {
std::atomic<int> g_max_refine{-1};
}  // namespace

int max_refine_steps(int dflt) {
  const int v = g_max_refine.load();
  return v >= 0 ? v : dflt;
}

// Re-solve the systems listed in idx (of a contiguous batch) with complex128
// LU and partial pivoting: the fallback of a stalled complex64 refinement.
int resolve_fp64(cudaStream_t st, const std::vector<int> &idx, size_t N, const qg_c *dM, const qg_c *db, qg_c *dx) {
  if (idx.empty()) return QPMS_SUCCESS;
  const size_t nb = idx.size(), N2 = N * N;
  void *LU = nullptr, *piv = nullptr;
  QG_CUDA_TRY(cudaMallocAsync(&LU, nb * N2 * 16, st));
  QG_CUDA_TRY(cudaMallocAsync(&piv, nb * N * 4, st));
  int e = QPMS_SUCCESS;
  for (size_t i = 0; i < nb && !e; ++i) {
    if (cudaMemcpyAsync((char *)LU + i * N2 * 16, dM + (size_t)idx[i] * N2, N2 * 16, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(dx + (size_t)idx[i] * N, db + (size_t)idx[i] * N, N * 16, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess) {
      set_error("batched solve: fallback copy failed");
      e = QPMS_ERROR;
    }
  }
  if (!e) e = batch_getrf_c128((int)nb, (int)N, LU, (int *)piv, nullptr, st);
  // the right-hand sides were copied into dx in place; solve them where they lie
  for (size_t i = 0; i < nb && !e; ++i)
    e = batch_getrs_c128(1, (int)N, (char *)LU + i * N2 * 16, (int *)piv + i * N, dx + (size_t)idx[i] * N, st);
  cudaFreeAsync(LU, st);
  cudaFreeAsync(piv, st);
  return e;
}

int batched_solve(cublasHandle_t h, cudaStream_t st, int nm, size_t N, const qg_c *dM, const qg_c *db, qg_c *dx,
                  int mode, double tol, int max_iter, void *scratch, double *resid_host, int *iters_host,
                  int *info_host, double *logabsdet, int *fallback_host) {
  if (nm <= 0) return QPMS_SUCCESS;
  max_iter = max_refine_steps(max_iter);
  const size_t m = (size_t)nm, N2 = N * N;
  char *p = (char *)scratch;
  void *LU = p;
  p += al(m * N2 * (mode ? 8 : 16));
  int *piv = (int *)p;
  p += al(m * N * 4);
  int *info = (int *)p;
  p += al(m * 4);
  void *cb = p;
  p += al(m * N * 8);
  qg_c *r = (qg_c *)p;
  p += al(m * N * 16);
  double *rn2 = (double *)p, *bn2 = rn2 + m;
  (void)h;
  std::vector<double> hr(m), hb(m);
  std::vector<int> its(m, 0);
  int e;
  if (N > (size_t)kBatchLuMaxN) {
    set_error("batched solve: N = %zu above %d", N, kBatchLuMaxN);
    return QPMS_EINVAL;
  }
  // log|det| wanted: the complex128 factors it needs also solve the systems
  // (these small LUs are not the cost of a scan), so the mixed mode takes the
  // complex128 path outright, with factors in buffers of their own (the
  // scratch holds complex64 factors in mixed mode)
  void *LU64 = nullptr, *piv64 = nullptr;
  if (mode == 1 && logabsdet) {
    QG_CUDA_TRY(cudaMallocAsync(&LU64, m * N2 * 16, st));
    if (cudaMallocAsync(&piv64, m * N * 4, st) != cudaSuccess) {
      cudaFreeAsync(LU64, st);
      set_error("batched solve: out of device memory");
      return QPMS_ENOMEM;
    }
  }
  struct Free64 {
    void *a, *b;
    cudaStream_t s;
    ~Free64() {
      if (a) cudaFreeAsync(a, s);
      if (b) cudaFreeAsync(b, s);
    }
  } free64{LU64, piv64, st};
  if (mode == 0 || LU64) {
    void *LUd = LU64 ? LU64 : LU;
    int *pivd = LU64 ? (int *)piv64 : piv;
    QG_CUDA_TRY(cudaMemcpyAsync(LUd, dM, m * N2 * 16, cudaMemcpyDeviceToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(dx, db, m * N * 16, cudaMemcpyDeviceToDevice, st));
    if ((e = batch_getrf_c128(nm, (int)N, LUd, pivd, info, st))) return e;
    if ((e = batch_getrs_c128(nm, (int)N, LUd, pivd, dx, st))) return e;
    if ((e = launch_residual(nm, N, dM, dx, db, r, rn2, bn2, st))) return e;
    QG_CUDA_TRY(cudaMemcpyAsync(hr.data(), rn2, m * 8, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaMemcpyAsync(hb.data(), bn2, m * 8, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
  } else {
    if ((e = launch_c128_to_c64(m * N2, dM, LU, st))) return e;
    if ((e = batch_getrf_c64(nm, (int)N, LU, piv, info, st))) return e;
    QG_CUDA_TRY(cudaMemcpyAsync(r, db, m * N * 16, cudaMemcpyDeviceToDevice, st));
    double prev = 1e300;
    for (int it = 0; it <= max_iter; ++it) {
      if ((e = launch_c128_to_c64(m * N, r, cb, st))) return e;
      if ((e = batch_getrs_c64(nm, (int)N, LU, piv, cb, st))) return e;
      if ((e = launch_add_c64(m * N, cb, dx, it == 0, st))) return e;
      if ((e = launch_residual(nm, N, dM, dx, db, r, rn2, bn2, st))) return e;
      QG_CUDA_TRY(cudaMemcpyAsync(hr.data(), rn2, m * 8, cudaMemcpyDeviceToHost, st));
      QG_CUDA_TRY(cudaMemcpyAsync(hb.data(), bn2, m * 8, cudaMemcpyDeviceToHost, st));
      QG_CUDA_TRY(cudaStreamSynchronize(st));
      double worst = 0;
      for (size_t i = 0; i < m; ++i) {
        const double rel = sqrt(hr[i] / (hb[i] > 0 ? hb[i] : 1));
        if (rel > tol) its[i] = it + 1;
        worst = fmax(worst, rel);
      }
      if (worst <= tol || worst >= 0.5 * prev) break;  // converged or stagnated
      prev = worst;
    }
    // systems whose refinement stalled above tol: solved again in complex128
    std::vector<int> bad;
    for (size_t i = 0; i < m; ++i)
      if (sqrt(hr[i] / (hb[i] > 0 ? hb[i] : 1)) > tol) bad.push_back((int)i);
    if (!bad.empty()) {
      if ((e = resolve_fp64(st, bad, N, dM, db, dx))) return e;
      if ((e = launch_residual(nm, N, dM, dx, db, r, rn2, bn2, st))) return e;
      QG_CUDA_TRY(cudaMemcpyAsync(hr.data(), rn2, m * 8, cudaMemcpyDeviceToHost, st));
      QG_CUDA_TRY(cudaMemcpyAsync(hb.data(), bn2, m * 8, cudaMemcpyDeviceToHost, st));
      QG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (fallback_host) {
      for (size_t i = 0; i < m; ++i) fallback_host[i] = 0;
      for (int i : bad) fallback_host[i] = 1;
    }
  }
  if ((mode == 0 || LU64) && fallback_host)
    for (size_t i = 0; i < m; ++i) fallback_host[i] = 0;
  if (logabsdet) {
    if (LU64) {
      logabsdet_kernel<double2><<<(nm + 127) / 128, 128, 0, st>>>(nm, N, (const double2 *)LU64, logabsdet);
      QG_CUDA_TRY(cudaGetLastError());
      g_launches.fetch_add(1);
    } else {
      logabsdet_kernel<double2><<<(nm + 127) / 128, 128, 0, st>>>(nm, N, (const double2 *)LU, logabsdet);
      QG_CUDA_TRY(cudaGetLastError());
      g_launches.fetch_add(1);
    }
  }
  if (info_host) {
    QG_CUDA_TRY(cudaMemcpyAsync(info_host, info, m * 4, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  for (size_t i = 0; i < m; ++i) {
    if (resid_host) resid_host[i] = sqrt(hr[i] / (hb[i] > 0 ? hb[i] : 1));
    if (iters_host) iters_host[i] = mode ? its[i] + 1 : 0;
  }
  return QPMS_SUCCESS;
}

}  // namespace qg

extern "C" int qpms_gpu_testing_set_max_refine(int max_steps) {
  qg::g_max_refine.store(max_steps < 0 ? -1 : max_steps);
  return QPMS_SUCCESS;
}
