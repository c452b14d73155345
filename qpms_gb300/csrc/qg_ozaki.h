// FP64-accurate complex matrix products on the bf16 tensor cores (Ozaki
// splitting), for the refinement residual R = B - M X of the dense solver.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace qg {

// Slices of the real matrix [Re M; Im M] (2N x N): row R is scaled by a
// power of two sigma_R (its largest |entry| over sigma_R lies in [1/2, 1)) and
// written as p digits of s bits, A_R,k = sigma_R sum_i d_i[R, k] 2^{-s (i+1)},
// d_i integers with |d_0| <= 2^s, |d_i| <= 2^{s-1}, stored exactly in bf16.
struct OzakiMatrix {
  int N = 0, s = 0, p = 0;
  bool row_major = false;  // layout of the source M
  size_t ld = 0;           // slice row length: N rounded up to a multiple of 8
  void *slices = nullptr;  // p x 2N x ld bf16, rows of [Re M; Im M] contiguous
  double *scale = nullptr; // 2N row scales sigma_R
  unsigned long long *rowmax = nullptr;  // 2N, bits of max |entry|
};

// Digit width s for inner dimension K: every partial sum of a product of
// digits, K 2^{2s} at most, is an integer below 2^24 and so exact in the FP32
// accumulators; p = ceil(55 / s) digits keep 55 bits.
void ozaki_digits(int K, int *s, int *p);

// Device bytes of the matrix slices and of the per-product workspace for
// nrhs right-hand sides.
size_t ozaki_matrix_bytes(int N);
size_t ozaki_work_bytes(int N, int nrhs);

// Slices M (complex128 N x N, leading dimension ldm, column-major or
// row-major).  om.slices / om.scale / om.rowmax point into `buf`
// (ozaki_matrix_bytes(N) bytes).
int ozaki_split_matrix(const void *M, size_t ldm, bool row_major, int N, void *buf, OzakiMatrix *om,
                       cudaStream_t st);

// R = B - M X for complex128 X, B, R (N x nrhs, leading dimension N) with the
// slices of M; work: ozaki_work_bytes(N, nrhs).  The products of digits run as
// bf16 GEMMs with FP32 accumulation (exact), their sums in FP64.
int ozaki_residual(const OzakiMatrix &om, const void *X, const void *B, void *R, int nrhs, void *work,
                   cudaStream_t st);

}  // namespace qg
