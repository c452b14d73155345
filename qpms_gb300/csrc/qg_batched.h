// Batched solve of many small mode-problem systems (qg_batched.cu).
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include "qg_internal.h"

namespace qg {

// Device scratch bytes batched_solve needs for nm systems of size N.
size_t batched_solve_bytes(int nm, size_t N, int mode);

// Solves M_i x_i = b_i for nm row-major complex128 N x N matrices (contiguous,
// the reference's layout), one right-hand side each, on stream st:
//   mode 0 - complex128 LU with partial pivoting (cuBLAS getrfBatched/getrsBatched);
//   mode 1 - complex64 LU of the same matrices, FP64 iterative refinement with
//            the residual b - M x formed in FP64, until every system reaches
//            tol (relative) or the worst stagnates, at most max_iter steps.
// scratch: batched_solve_bytes(nm, N, mode) device bytes.  Host outputs per
// system (each may be NULL): relative FP64 residual, refinement steps, LU info.
// logabsdet (device, may be NULL): log|det M_i| from the LU diagonal.
int batched_solve(cublasHandle_t h, cudaStream_t st, int nm, size_t N, const qg_c *dM, const qg_c *db, qg_c *dx,
                  int mode, double tol, int max_iter, void *scratch, double *resid_host, int *iters_host,
                  int *info_host, double *logabsdet);

}  // namespace qg
