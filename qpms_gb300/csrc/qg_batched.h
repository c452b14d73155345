// Batched solve of many small mode-problem systems (qg_batched.cu).
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <vector>

#include "qg_internal.h"

namespace qg {

// Device scratch bytes batched_solve needs for nm systems of size N.
size_t batched_solve_bytes(int nm, size_t N, int mode);

// Solves M_i x_i = b_i for nm row-major complex128 N x N matrices (contiguous,
// the reference's layout), one right-hand side each, on stream st:
//   mode 0 - complex128 LU with partial pivoting (qg_batchlu.cu);
//   mode 1 - complex64 LU of the same matrices, FP64 iterative refinement with
//            the residual b - M x formed in FP64, until every system reaches
//            tol (relative) or the worst stagnates, at most max_iter steps;
//            systems still above tol are then solved again in complex128
//            (fallback_host[i] = 1 for those).
// scratch: batched_solve_bytes(nm, N, mode) device bytes.  Host outputs per
// system (each may be NULL): relative FP64 residual, refinement steps, LU info.
// logabsdet (device, may be NULL): log|det M_i| from the diagonal of complex128
// factors; with it, mode 1 solves through those complex128 factors as mode 0
// does (the factors it needs solve the systems too).
int batched_solve(cublasHandle_t h, cudaStream_t st, int nm, size_t N, const qg_c *dM, const qg_c *db, qg_c *dx,
                  int mode, double tol, int max_iter, void *scratch, double *resid_host, int *iters_host,
                  int *info_host, double *logabsdet, int *fallback_host = nullptr);

// Systems idx of a contiguous batch solved again in complex128 (partial
// pivoting), x overwritten: the fallback of a stalled complex64 refinement.
int resolve_fp64(cudaStream_t st, const std::vector<int> &idx, size_t N, const qg_c *dM, const qg_c *db, qg_c *dx);

// The refinement step cap of the mixed-precision solves: dflt unless the test
// hook qpms_gpu_testing_set_max_refine set one.
int max_refine_steps(int dflt);

}  // namespace qg
