// Batched LU with partial pivoting of small row-major complex matrices and the
// matching one-right-hand-side substitutions (qg_batchlu.cu).
#pragma once
#include <cuda_runtime.h>

namespace qg {

// Largest order the batched kernels take (shared-memory panel of N rows).
constexpr int kBatchLuMaxN = 512;

// nm contiguous row-major N x N matrices factored in place: P M = L U (unit
// lower L below the diagonal, U on and above); piv[b * N + i] (0-based) is the
// row exchanged with row i at step i, info[b] the first zero pivot (1-based)
// or 0.  info may be NULL.
int batch_getrf_c64(int nm, int N, void *A, int *piv, int *info, cudaStream_t st);
int batch_getrf_c128(int nm, int N, void *A, int *piv, int *info, cudaStream_t st);
// b (nm x N, contiguous) <- M^-1 b from the factors.
int batch_getrs_c64(int nm, int N, const void *LU, const int *piv, void *b, cudaStream_t st);
int batch_getrs_c128(int nm, int N, const void *LU, const int *piv, void *b, cudaStream_t st);

}  // namespace qg
