// Complex64 GEMM on the sm_103a tensor cores (tcgen05 + TMA), split-bf16
// operands with FP32 accumulation in tensor memory (qg_tcgemm.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>

namespace qg {

// Operand planes of a complex product C (m x n) +-= A (m x k) B (k x n):
//   A as its real embedding E(A) (2m x 2k rows (2i+p), columns (2l+q):
//   [[Re, -Im], [Im, Re]]), B as its real view (2k x n: column j holds
//   Re B(l, j), Im B(l, j) at rows 2l, 2l+1), each cut into nsplit bf16 digit
//   planes (x = x_0 + x_1 + ... with x_s = bf16(x - x_0 - ... - x_{s-1})),
//   stored K-major: A planes [s][2m][2k], B planes [s][n][2k].
struct TcPlanes {
  __nv_bfloat16 *a = nullptr, *b = nullptr;
  int m = 0, n = 0, k = 0, nsplit = 0;
  // Distance between digit planes in elements; 0: that of planes filled for
  // exactly (m, n, k) (2m rows of A, n rows of B).  Set to use a block of
  // rows of larger planes (a / b then point at the first row of the block).
  size_t a_plane = 0, b_plane = 0;
  // Row length of the A planes in elements; 0: tc_planes_row(k).  Set to use
  // a block of columns of planes cut for a larger k (a then points at the
  // block's first element; its column offset a multiple of 8 elements).
  size_t a_rs = 0;
};

// Row length (elements) of the digit planes for inner dimension k.
size_t tc_planes_row(int k);

// Bytes of the A and B planes for (m, n, k, nsplit).
size_t tc_planes_bytes_a(int m, int k, int nsplit);
size_t tc_planes_bytes_b(int n, int k, int nsplit);

// Fill the A planes from complex64 A (m x k, column-major, lda) -- or from
// A^T when trans_a: A(i, l) = Asrc(l, i).
int tc_split_a(const float2 *A, size_t lda, int m, int k, int nsplit, __nv_bfloat16 *planes, cudaStream_t st,
               bool trans_a = false);
// Fill the B planes from complex64 B (k x n, column-major, ldb).
int tc_split_b(const float2 *B, size_t ldb, int k, int n, int nsplit, __nv_bfloat16 *planes, cudaStream_t st);
// Both operands of one product A (m x k) B (k x n) in one launch.
int tc_split_ab(const float2 *A, size_t lda, int m, int k, const float2 *B, size_t ldb, int n, int nsplit,
                __nv_bfloat16 *a_planes, __nv_bfloat16 *b_planes, cudaStream_t st);

// D = beta C + alpha A B on complex64 column-major C, D (leading dimensions in
// complex elements; C == D allowed, C unused when beta == 0) from the planes.
// Digit products with s_a + s_b < nsplit are accumulated (1, 3 or 6
// products for nsplit 1, 2, 3).  alpha, beta real.
int tc_cgemm_planes(const TcPlanes &P, float alpha, float beta, const float2 *C, size_t ldc, float2 *D, size_t ldd,
                    cudaStream_t st);

// Same GEMM on real bf16 operands given K-major (A: [m][k], B: [n][k], row
// strides in elements, multiples of 8) with FP32 output D (m x n column-major,
// leading dimension ldd): D = beta C + alpha A B^T.  For the digit products of
// the FP64 residual (exact integer sums below 2^24).
int tc_gemm_bf16(const __nv_bfloat16 *A, size_t lda, const __nv_bfloat16 *B, size_t ldb, int m, int n, int k,
                 float alpha, float beta, const float *C, size_t ldc, float *D, size_t ldd, cudaStream_t st);

// Device-wide error flag of the tensor-core kernels (a wait that ran out of
// time); returns QPMS_ERROR with a message if set and clears it.
int tc_check_error(cudaStream_t st);

}  // namespace qg
