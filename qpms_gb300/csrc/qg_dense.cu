// Dense LU solver for large mode-problem matrices (Beyn contour nodes,
// 14,400-unknown systems and up) on sm_103a.
//
// The reference factorises with LAPACKE_zgetrf (partial pivoting) and solves
// with zgetrs (scatsystem.c:2202-2273; beyn.c:552-564).  Partial pivoting
// serialises a global pivot search per column, the latency bound of GPU LU;
// this solver instead
//   1. applies a depth-2 random butterfly transform (RBT) to both sides,
//      A' = W_u^T M W_v (Parker's randomisation, as in Baboulin, Dongarra,
//      Herrmann, Tomov, "Accelerating linear system solutions using
//      randomization techniques", ACM TOMS 39 (2013)), after which Gaussian
//      elimination without pivoting is stable with high probability;
//   2. factorises A' = L U without pivoting by blocks: an nb x nb diagonal
//      block is factored and its triangular factors inverted in shared memory
//      by one CTA; the panels below and to the right and the trailing update are
//      then GEMMs (cuBLAS, tensor cores);
//   3. solves by blocked forward/back substitution (GEMMs with the inverted
//      diagonal blocks);
//   4. in the mixed mode, the factorisation and substitutions run in complex64
//      (GEMMs with FP32-accurate BF16x9 emulation on the tensor cores) and the
//      FP64 solution is recovered by iterative refinement against the FP64
//      matrix: x += W_v (LU)^-1 W_u^T (b - M x), residual in FP64.
// The plain mode runs steps 1-3 in complex128 (FP64 GEMMs).
// All matrices are column-major (LAPACK order).  The butterflies halve the
// system twice, so it is padded internally to a multiple of 4 with identity.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <random>
#include <vector>

#include "qg_assembly.h"
#include "qg_batched.h"
#include "qg_dense.h"
#include "qg_internal.h"
#include "qg_ktimer.h"
#include "qg_tcgemm.h"

namespace qg {
int blas_handle_get(cublasHandle_t *h);

namespace {

template <typename T>
struct CTraits;
template <>
struct CTraits<float2> {
  typedef float real;
  static constexpr cudaDataType_t dt = CUDA_C_32F;
};
template <>
struct CTraits<double2> {
  typedef double real;
  static constexpr cudaDataType_t dt = CUDA_C_64F;
};

template <typename T>
__device__ __forceinline__ T mk(typename CTraits<T>::real r, typename CTraits<T>::real i) {
  T z;
  z.x = r;
  z.y = i;
  return z;
}
template <typename T>
__device__ __forceinline__ T mul(T a, T b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ T sub(T a, T b) {
  return mk<T>(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ T rcp(T b) {
  typedef typename CTraits<T>::real R;
  const R d = b.x * b.x + b.y * b.y;
  return mk<T>(b.x / d, -b.y / d);
}

// ---------------- diagonal block: LU without pivoting + triangular inverses ----------------
// D (kb x kb, kb <= 128 and a multiple of 32 except for the last block,
// column-major in global, leading dimension lda) is factored in place
// (unit-lower L below the diagonal, U on and above); L^-1 and U^-1 are written
// to Linv and Uinv (column-major kb x kb each).  info is set to 1 on an
// exactly zero pivot.  One CTA of 1024 threads with the block in shared
// memory:
//   1. right-looking elimination, a 32 x 32 thread tile sweeping the trailing
//      matrix of each step (no index division);
//   2. the inverses by recursive doubling: each 32 x 32 diagonal block is
//      inverted by one warp (substitution with warp barriers only), then
//      adjacent blocks are combined level by level,
//        [L11 0; L21 L22]^-1 = [X11 0; -X22 L21 X11  X22],
//        [U11 U12; 0 U22]^-1 = [Y11 -Y11 U12 Y22; 0 Y22],
//      as two small products per level through a shared-memory temporary.
// The unit diagonal of L^-1 is implicit in shared memory (the slot holds U^-1).
// Capacity of each doubling temporary: npair * h^2 <= 4096 for every block size
// kb <= 128 the solver uses (h = 32: at most 2 pairs; h = 64: one pair).
constexpr int kDiagTmp = 4096;

template <typename T>
__device__ __forceinline__ T fma_c(T acc, T a, T b) {  // acc + a b
  return mk<T>(acc.x + a.x * b.x - a.y * b.y, acc.y + a.x * b.y + a.y * b.x);
}

template <typename T>
__global__ void __launch_bounds__(1024) diag_lu_inv_kernel(T *D, size_t lda, int kb, T *Linv, T *Uinv, int *info) {
  extern __shared__ __align__(16) unsigned char sm[];
  T *S = reinterpret_cast<T *>(sm);  // [kb][kb] column-major: S[c * kb + r]
  T *TL = S + kb * kb;               // temporaries of the doubling products (kDiagTmp entries each)
  T *TU = TL + kDiagTmp;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  for (int t = tid; t < kb * kb; t += nt) {
    const int c = t / kb, r = t - c * kb;
    S[t] = D[(size_t)c * lda + r];
  }
  __syncthreads();
  // ---- 1. elimination ----
  for (int j = 0; j < kb; ++j) {
    const T d = S[j * kb + j];
    const bool zero = (d.x == 0 && d.y == 0);
    if (zero && tid == 0) atomicOr(info, 1);
    const T inv = zero ? mk<T>(0, 0) : rcp(d);
    if (tid > j && tid < kb) S[j * kb + tid] = mul(S[j * kb + tid], inv);
    __syncthreads();
    for (int c = j + 1 + warp; c < kb; c += 32) {
      const T u = S[c * kb + j];
      for (int r = j + 1 + lane; r < kb; r += 32) S[c * kb + r] = sub(S[c * kb + r], mul(S[j * kb + r], u));
    }
    __syncthreads();
  }
  for (int t = tid; t < kb * kb; t += nt) {
    const int c = t / kb, r = t - c * kb;
    D[(size_t)c * lda + r] = S[t];
  }
  // ---- 2a. 32 x 32 diagonal blocks, one warp each: warps [0, nblk) L, [16, 16 + nblk) U ----
  const int nb32 = (kb + 31) / 32;
  if (warp < nb32 || (warp >= 16 && warp < 16 + nb32)) {
    const bool isL = warp < 16;
    const int o = (isL ? warp : warp - 16) * 32;
    const int s = min(32, kb - o);  // block size (the last block may be short)
    const int i = lane;
    if (isL) {
      // X(i, j) = -(L(i, j) + sum_{j<k<i} X(i, k) L(k, j)), columns from the right
      for (int j = s - 2; j >= 0; --j) {
        T acc = mk<T>(0, 0);
        if (i > j && i < s) {
          acc = S[(o + j) * kb + o + i];
          for (int k = j + 1; k < i; ++k) acc = fma_c(acc, S[(o + k) * kb + o + i], S[(o + j) * kb + o + k]);
        }
        __syncwarp();
        if (i > j && i < s) S[(o + j) * kb + o + i] = mk<T>(-acc.x, -acc.y);
        __syncwarp();
      }
    } else {
      // Y(j, j) = 1 / U(j, j); Y(i, j) = -(sum_{i<=k<j} Y(i, k) U(k, j)) Y(j, j), columns from the left
      for (int j = 0; j < s; ++j) {
        const T u = S[(o + j) * kb + o + j];
        const T dj = (u.x == 0 && u.y == 0) ? mk<T>(0, 0) : rcp(u);
        T acc = mk<T>(0, 0);
        if (i < j) {
          for (int k = i; k < j; ++k) {
            const T yik = (k == i) ? S[(o + i) * kb + o + i] : S[(o + k) * kb + o + i];
            acc = fma_c(acc, yik, S[(o + j) * kb + o + k]);
          }
        }
        __syncwarp();
        if (i < j) S[(o + j) * kb + o + i] = mk<T>(-(acc.x * dj.x - acc.y * dj.y), -(acc.x * dj.y + acc.y * dj.x));
        if (i == j) S[(o + j) * kb + o + j] = dj;
        __syncwarp();
      }
    }
  }
  __syncthreads();
  // ---- 2b. doubling: blocks of size h are combined into blocks of size 2h ----
  for (int h = 32; h < kb; h *= 2) {
    const int npair = kb / (2 * h) + ((kb % (2 * h)) > h ? 1 : 0);
    // products 1: TL = L21 X11, TU = U12 Y22 (h2 = rows / cols of the second block)
    for (int t = tid; t < 2 * npair * h * h; t += nt) {
      const bool isL = t < npair * h * h;
      const int tt = isL ? t : t - npair * h * h;
      const int p = tt / (h * h), e = tt - p * h * h, r = e % h, c = e / h;
      const int o = p * 2 * h, h2 = min(h, kb - o - h);
      if (r >= h2 && isL) continue;   // rows of L21 beyond the short block
      if (c >= h2 && !isL) continue;  // columns of U12 beyond the short block
      T acc = mk<T>(0, 0);
      if (isL) {  // T(r, c) = sum_{k >= c} L21(r, k) X11(k, c), X11(c, c) = 1
        acc = S[(o + c) * kb + o + h + r];
        for (int k = c + 1; k < h; ++k) acc = fma_c(acc, S[(o + k) * kb + o + h + r], S[(o + c) * kb + o + k]);
        TL[p * h * h + c * h + r] = acc;
      } else {    // T(r, c) = sum_{k <= c} U12(r, k) Y22(k, c)
        for (int k = 0; k <= c; ++k) acc = fma_c(acc, S[(o + h + k) * kb + o + r], S[(o + h + c) * kb + o + h + k]);
        TU[p * h * h + c * h + r] = acc;
      }
    }
    __syncthreads();
    // products 2: X21 = -X22 TL, Y12 = -Y11 TU, written over L21 / U12
    for (int t = tid; t < 2 * npair * h * h; t += nt) {
      const bool isL = t < npair * h * h;
      const int tt = isL ? t : t - npair * h * h;
      const int p = tt / (h * h), e = tt - p * h * h, r = e % h, c = e / h;
      const int o = p * 2 * h, h2 = min(h, kb - o - h);
      T acc = mk<T>(0, 0);
      if (isL) {  // X21(r, c) = -(T(r, c) + sum_{k < r} X22(r, k) T(k, c)), X22 unit lower
        if (r >= h2) continue;
        acc = TL[p * h * h + c * h + r];
        for (int k = 0; k < r; ++k) acc = fma_c(acc, S[(o + h + k) * kb + o + h + r], TL[p * h * h + c * h + k]);
        S[(o + c) * kb + o + h + r] = mk<T>(-acc.x, -acc.y);
      } else {    // Y12(r, c) = -sum_{k >= r} Y11(r, k) T(k, c)
        if (c >= h2) continue;
        for (int k = r; k < h; ++k) acc = fma_c(acc, S[(o + k) * kb + o + r], TU[p * h * h + c * h + k]);
        S[(o + h + c) * kb + o + r] = mk<T>(-acc.x, -acc.y);
      }
    }
    __syncthreads();
  }
  for (int t = tid; t < kb * kb; t += nt) {
    const int c = t / kb, r = t - c * kb;
    const T v = S[t];
    Linv[t] = r > c ? v : (r == c ? mk<T>(1, 0) : mk<T>(0, 0));
    Uinv[t] = r <= c ? v : mk<T>(0, 0);
  }
}

// shared memory of diag_lu_inv_kernel for block size kb
template <typename T>
size_t diag_smem(int kb) {
  return ((size_t)kb * kb + 2 * (size_t)kDiagTmp) * sizeof(T);
}

// ---------------- random butterfly transforms (FP64) ----------------
// Row pass: within each block of size h2 = 2h along the rows (block b covers
// rows [b*2h, (b+1)*2h)), for i < h: top = A[i], bot = A[i + h]:
//   transposed butterfly (left, W^T):  top' = R_i (top + bot)/sqrt2, bot' = S_i (top - bot)/sqrt2
//   butterfly (right or solution, W):   column form uses the same pairing.
// R and S are stored per level in d[level][N]: R at d[b*2h + i], S at d[b*2h + h + i].
__global__ void rbt_rows_kernel(size_t N, size_t ncols, size_t ld, double2 *A, int h, const double *rs,
                                int transposed) {
  const double is2 = 0.70710678118654752440;
  const size_t pairs = N / 2;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs * ncols;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t col = t / pairs, p = t - col * pairs;
    const size_t b = p / h, i = p - b * h;
    const size_t r0 = b * 2 * h + i, r1 = r0 + h;
    double2 *x = A + col * ld;
    const double2 top = x[r0], bot = x[r1];
    const double R = rs[b * 2 * h + i], S = rs[b * 2 * h + h + i];
    if (transposed) {  // W^T: [R R; S -S] / sqrt2
      x[r0] = make_double2(R * (top.x + bot.x) * is2, R * (top.y + bot.y) * is2);
      x[r1] = make_double2(S * (top.x - bot.x) * is2, S * (top.y - bot.y) * is2);
    } else {  // W: [R S; R -S] / sqrt2
      x[r0] = make_double2((R * top.x + S * bot.x) * is2, (R * top.y + S * bot.y) * is2);
      x[r1] = make_double2((R * top.x - S * bot.x) * is2, (R * top.y - S * bot.y) * is2);
    }
  }
}

// Column pass of A W (right multiplication): columns j and j + h within blocks of 2h:
//   (A W)[:, j] = R_j (A_j + A_{j+h}) / sqrt2,  (A W)[:, j+h] = S_j (A_j - A_{j+h}) / sqrt2
__global__ void rbt_cols_kernel(size_t N, size_t ld, double2 *A, int h, const double *rs) {
  const double is2 = 0.70710678118654752440;
  const size_t pairs = N / 2;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs * N;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t p = t / N, row = t - p * N;  // consecutive threads walk rows (coalesced)
    const size_t b = p / h, j = p - b * h;
    const size_t c0 = b * 2 * h + j, c1 = c0 + h;
    const double2 a0 = A[c0 * ld + row], a1 = A[c1 * ld + row];
    const double R = rs[b * 2 * h + j], S = rs[b * 2 * h + h + j];
    A[c0 * ld + row] = make_double2(R * (a0.x + a1.x) * is2, R * (a0.y + a1.y) * is2);
    A[c1 * ld + row] = make_double2(S * (a0.x - a1.x) * is2, S * (a0.y - a1.y) * is2);
  }
}

__global__ void d2f_kernel(size_t n, const double2 *src, float2 *dst) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    dst[t] = make_float2((float)src[t].x, (float)src[t].y);
}
__global__ void f2d_add_kernel(size_t n, const float2 *src, double2 *dst, int init) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const float2 v = src[t];
    dst[t] = init ? make_double2(v.x, v.y) : make_double2(dst[t].x + v.x, dst[t].y + v.y);
  }
}
__global__ void add_kernel(size_t n, const double2 *src, double2 *dst, int init) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    dst[t] = init ? src[t] : make_double2(dst[t].x + src[t].x, dst[t].y + src[t].y);
}
// sum of |x|^2 over n entries into out[0] (atomic)
__global__ void norm2_kernel(size_t n, const double2 *x, double *out) {
  double s = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    s += x[t].x * x[t].x + x[t].y * x[t].y;
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

unsigned grid1(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (unsigned)(g ? g : 1);
}

template <typename T>
int gemm(cublasHandle_t h, int m, int n, int k, T alpha, const T *A, size_t lda, const T *B, size_t ldb, T beta,
         T *C, size_t ldc, cublasComputeType_t ct) {
  const cudaDataType_t dt = CTraits<T>::dt;
  if (ct == CUBLAS_COMPUTE_32F_EMULATED_16BFX9) cublasSetEmulationStrategy(h, CUBLAS_EMULATION_STRATEGY_EAGER);
  cublasStatus_t s = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &alpha, A, dt, (int)lda, B, dt, (int)ldb,
                                  &beta, C, dt, (int)ldc, ct, CUBLAS_GEMM_DEFAULT);
  if (s == CUBLAS_STATUS_NOT_SUPPORTED && ct != CUBLAS_COMPUTE_32F && ct != CUBLAS_COMPUTE_64F) {
    ct = (dt == CUDA_C_32F) ? CUBLAS_COMPUTE_32F : CUBLAS_COMPUTE_64F;
    s = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &alpha, A, dt, (int)lda, B, dt, (int)ldb, &beta, C, dt,
                     (int)ldc, ct, CUBLAS_GEMM_DEFAULT);
  }
  if (s != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasGemmEx(%d, %d, %d) failed: status %d", m, n, k, (int)s);
    return QPMS_ERROR;
  }
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

template <typename T>
T cone() {
  T z;
  z.x = 1;
  z.y = 0;
  return z;
}
template <typename T>
T cval(double r) {
  T z;
  z.x = (typename CTraits<T>::real)r;
  z.y = 0;
  return z;
}

// LU without pivoting, blocked (see the header comment).
template <typename T>
int lu_nopiv(cublasHandle_t h, int N, int nb, T *A, size_t lda, T *Dinv, T *work, int *dinfo,
             cublasComputeType_t ct, cudaStream_t st) {
  const size_t smem = diag_smem<T>(nb);
  QG_CUDA_TRY(cudaFuncSetAttribute(diag_lu_inv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for (int k = 0, blk = 0; k < N; k += nb, ++blk) {
    const int kb = (N - k < nb) ? N - k : nb;
    T *Lk = Dinv + (size_t)blk * 2 * nb * nb, *Uk = Lk + (size_t)nb * nb;
    diag_lu_inv_kernel<T><<<1, 1024, diag_smem<T>(kb), st>>>(A + (size_t)k * lda + k, lda, kb, Lk, Uk, dinfo);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
    const int m2 = N - k - kb;
    if (m2 <= 0) break;
    T *A21 = A + (size_t)k * lda + k + kb, *A12 = A + (size_t)(k + kb) * lda + k, *A22 = A21 + (size_t)kb * lda;
    int e;
    // L21 = A21 Uinv   (m2 x kb)
    const cublasComputeType_t cp = (sizeof(T) == 8) ? CUBLAS_COMPUTE_32F : CUBLAS_COMPUTE_64F;  // panels
    if ((e = gemm<T>(h, m2, kb, kb, cone<T>(), A21, lda, Uk, kb, cval<T>(0), work, m2, cp))) return e;
    QG_CUDA_TRY(cudaMemcpy2DAsync(A21, lda * sizeof(T), work, (size_t)m2 * sizeof(T), (size_t)m2 * sizeof(T), kb,
                                  cudaMemcpyDeviceToDevice, st));
    // U12 = Linv A12   (kb x m2)
    if ((e = gemm<T>(h, kb, m2, kb, cone<T>(), Lk, kb, A12, lda, cval<T>(0), work, kb, cp))) return e;
    QG_CUDA_TRY(cudaMemcpy2DAsync(A12, lda * sizeof(T), work, (size_t)kb * sizeof(T), (size_t)kb * sizeof(T), m2,
                                  cudaMemcpyDeviceToDevice, st));
    // A22 -= L21 U12
    if ((e = gemm<T>(h, m2, m2, kb, cval<T>(-1), A21, lda, A12, lda, cone<T>(), A22, lda, ct))) return e;
  }
  return QPMS_SUCCESS;
}

// Solve (L U) X = B in place (B: N x nrhs, column-major, ldb).
template <typename T>
int lu_solve(cublasHandle_t h, int N, int nb, const T *A, size_t lda, const T *Dinv, T *B, size_t ldb, int nrhs,
             T *work, cublasComputeType_t ct, cudaStream_t st) {
  int e;
  const int nblk = (N + nb - 1) / nb;
  for (int blk = 0; blk < nblk; ++blk) {  // forward: L y = b
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    const T *Lk = Dinv + (size_t)blk * 2 * nb * nb;
    if ((e = gemm<T>(h, kb, nrhs, kb, cone<T>(), Lk, kb, B + k, ldb, cval<T>(0), work, kb, ct))) return e;
    QG_CUDA_TRY(cudaMemcpy2DAsync(B + k, ldb * sizeof(T), work, (size_t)kb * sizeof(T), (size_t)kb * sizeof(T), nrhs,
                                  cudaMemcpyDeviceToDevice, st));
    const int m2 = N - k - kb;
    if (m2 > 0)
      if ((e = gemm<T>(h, m2, nrhs, kb, cval<T>(-1), A + (size_t)k * lda + k + kb, lda, B + k, ldb, cone<T>(),
                       B + k + kb, ldb, ct)))
        return e;
  }
  for (int blk = nblk - 1; blk >= 0; --blk) {  // backward: U x = y
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    const T *Uk = Dinv + (size_t)blk * 2 * nb * nb + (size_t)nb * nb;
    if ((e = gemm<T>(h, kb, nrhs, kb, cone<T>(), Uk, kb, B + k, ldb, cval<T>(0), work, kb, ct))) return e;
    QG_CUDA_TRY(cudaMemcpy2DAsync(B + k, ldb * sizeof(T), work, (size_t)kb * sizeof(T), (size_t)kb * sizeof(T), nrhs,
                                  cudaMemcpyDeviceToDevice, st));
    if (k > 0)
      if ((e = gemm<T>(h, k, nrhs, kb, cval<T>(-1), A + (size_t)k * lda, lda, B + k, ldb, cone<T>(), B, ldb, ct)))
        return e;
  }
  return QPMS_SUCCESS;
}

// ---------------- complex64 LU and substitutions on the tensor cores ----------------
// The same blocked algorithm as lu_nopiv / lu_solve with every product a
// tcgen05 GEMM of split-bf16 digits (qg_tcgemm.cu): operands are cut into
// digit planes first, so each GEMM may write its result over an operand it
// read (the panels L21 = A21 U^-1, U12 = L^-1 A12 and the right-hand-side
// blocks are formed in place).
int lu_nopiv_tc(int N, int nb, float2 *A, size_t lda, float2 *Dinv, int *dinfo, int nsplit, __nv_bfloat16 *pa,
                __nv_bfloat16 *pb, cudaStream_t st) {
  const size_t smem = diag_smem<float2>(nb);
  QG_CUDA_TRY(
      cudaFuncSetAttribute(diag_lu_inv_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  TcPlanes P;
  P.a = pa;
  P.b = pb;
  P.nsplit = nsplit;
  int e;
  for (int k = 0, blk = 0; k < N; k += nb, ++blk) {
    const int kb = (N - k < nb) ? N - k : nb;
    float2 *Lk = Dinv + (size_t)blk * 2 * nb * nb, *Uk = Lk + (size_t)nb * nb;
    {
      KtScope kt(KT_DIAGLU, st, 8.0 * kb * (double)kb * kb / 3.0);
      diag_lu_inv_kernel<float2><<<1, 1024, diag_smem<float2>(kb), st>>>(A + (size_t)k * lda + k, lda, kb, Lk,
                                                                         Uk, dinfo);
    }
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
    const int m2 = N - k - kb;
    if (m2 <= 0) break;
    float2 *A21 = A + (size_t)k * lda + k + kb, *A12 = A + (size_t)(k + kb) * lda + k, *A22 = A21 + (size_t)kb * lda;
    // L21 = A21 U^-1
    if ((e = tc_split_ab(A21, lda, m2, kb, Uk, kb, kb, nsplit, pa, pb, st))) return e;
    P.m = m2, P.n = kb, P.k = kb;
    if ((e = tc_cgemm_planes(P, 1.f, 0.f, nullptr, 0, A21, lda, st))) return e;
    // U12 = L^-1 A12
    if ((e = tc_split_ab(Lk, kb, kb, kb, A12, lda, m2, nsplit, pa, pb, st))) return e;
    P.m = kb, P.n = m2, P.k = kb;
    if ((e = tc_cgemm_planes(P, 1.f, 0.f, nullptr, 0, A12, lda, st))) return e;
    // A22 -= L21 U12
    if ((e = tc_split_ab(A21, lda, m2, kb, A12, lda, m2, nsplit, pa, pb, st))) return e;
    P.m = m2, P.n = m2, P.k = kb;
    if ((e = tc_cgemm_planes(P, -1.f, 1.f, A22, lda, A22, lda, st))) return e;
  }
  return QPMS_SUCCESS;
}

// (L U) X = B in place, B: N x nrhs (ldb), products on the tensor cores.
int lu_solve_tc(int N, int nb, const float2 *A, size_t lda, const float2 *Dinv, float2 *B, size_t ldb, int nrhs,
                int nsplit, __nv_bfloat16 *pa, __nv_bfloat16 *pb, cudaStream_t st) {
  TcPlanes P;
  P.a = pa;
  P.b = pb;
  P.nsplit = nsplit;
  int e;
  const int nblk = (N + nb - 1) / nb;
  for (int blk = 0; blk < nblk; ++blk) {  // forward: L y = b
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    const float2 *Lk = Dinv + (size_t)blk * 2 * nb * nb;
    if ((e = tc_split_ab(Lk, kb, kb, kb, B + k, ldb, nrhs, nsplit, pa, pb, st))) return e;
    P.m = kb, P.n = nrhs, P.k = kb;
    if ((e = tc_cgemm_planes(P, 1.f, 0.f, nullptr, 0, B + k, ldb, st))) return e;
    const int m2 = N - k - kb;
    if (m2 <= 0) continue;
    if ((e = tc_split_ab(A + (size_t)k * lda + k + kb, lda, m2, kb, B + k, ldb, nrhs, nsplit, pa, pb, st))) return e;
    P.m = m2, P.n = nrhs, P.k = kb;
    if ((e = tc_cgemm_planes(P, -1.f, 1.f, B + k + kb, ldb, B + k + kb, ldb, st))) return e;
  }
  for (int blk = nblk - 1; blk >= 0; --blk) {  // backward: U x = y
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    const float2 *Uk = Dinv + (size_t)blk * 2 * nb * nb + (size_t)nb * nb;
    if ((e = tc_split_ab(Uk, kb, kb, kb, B + k, ldb, nrhs, nsplit, pa, pb, st))) return e;
    P.m = kb, P.n = nrhs, P.k = kb;
    if ((e = tc_cgemm_planes(P, 1.f, 0.f, nullptr, 0, B + k, ldb, st))) return e;
    if (k == 0) continue;
    if ((e = tc_split_ab(A + (size_t)k * lda, lda, k, kb, B + k, ldb, nrhs, nsplit, pa, pb, st))) return e;
    P.m = k, P.n = nrhs, P.k = kb;
    if ((e = tc_cgemm_planes(P, -1.f, 1.f, B, ldb, B, ldb, st))) return e;
  }
  return QPMS_SUCCESS;
}

// ---------------- substitutions for a few right-hand sides (bandwidth-bound) ----------------
constexpr int kSmallRhs = 8;

// Bk (kb x nrhs, ldb) <- Tri (kb x kb, leading dimension kb) Bk; one CTA.
template <typename T>
__global__ void __launch_bounds__(256) blk_apply_kernel(const T *__restrict__ Tri, int kb, T *Bk, size_t ldb,
                                                        int nrhs) {
  __shared__ T sB[128 * kSmallRhs];
  for (int t = threadIdx.x; t < kb * nrhs; t += blockDim.x) {
    const int c = t / kb, r = t - c * kb;
    sB[c * kb + r] = Bk[(size_t)c * ldb + r];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kb * nrhs; t += blockDim.x) {
    const int c = t / kb, r = t - c * kb;
    T acc = mk<T>(0, 0);
    for (int l = 0; l < kb; ++l) acc = fma_c(acc, Tri[(size_t)l * kb + r], sB[c * kb + l]);
    Bk[(size_t)c * ldb + r] = acc;
  }
}

// Bdst (m2 x nrhs) -= Pn (m2 x kb, leading dimension lda) Bk (kb x nrhs); a
// thread per row, the panel read once and coalesced.
template <typename T>
__global__ void __launch_bounds__(256) panel_sub_kernel(const T *__restrict__ Pn, size_t lda, int m2, int kb,
                                                        const T *Bk, size_t ldb, T *Bdst, int nrhs) {
  __shared__ T sB[128 * kSmallRhs];
  for (int t = threadIdx.x; t < kb * nrhs; t += blockDim.x) {
    const int c = t / kb, r = t - c * kb;
    sB[c * kb + r] = Bk[(size_t)c * ldb + r];
  }
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m2) return;
  T acc[kSmallRhs];
#pragma unroll
  for (int c = 0; c < kSmallRhs; ++c) acc[c] = mk<T>(0, 0);
  for (int l = 0; l < kb; ++l) {
    const T p = Pn[(size_t)l * lda + r];
#pragma unroll
    for (int c = 0; c < kSmallRhs; ++c)
      if (c < nrhs) acc[c] = fma_c(acc[c], p, sB[c * kb + l]);
  }
#pragma unroll
  for (int c = 0; c < kSmallRhs; ++c)
    if (c < nrhs) Bdst[(size_t)c * ldb + r] = sub(Bdst[(size_t)c * ldb + r], acc[c]);
}

template <typename T>
int lu_solve_small(int N, int nb, const T *A, size_t lda, const T *Dinv, T *B, size_t ldb, int nrhs, cudaStream_t st) {
  const int nblk = (N + nb - 1) / nb;
  for (int blk = 0; blk < nblk; ++blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    blk_apply_kernel<T><<<1, 256, 0, st>>>(Dinv + (size_t)blk * 2 * nb * nb, kb, B + k, ldb, nrhs);
    const int m2 = N - k - kb;
    if (m2 > 0)
      panel_sub_kernel<T><<<(m2 + 255) / 256, 256, 0, st>>>(A + (size_t)k * lda + k + kb, lda, m2, kb, B + k, ldb,
                                                            B + k + kb, nrhs);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(m2 > 0 ? 2 : 1);
  }
  for (int blk = nblk - 1; blk >= 0; --blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    blk_apply_kernel<T><<<1, 256, 0, st>>>(Dinv + (size_t)blk * 2 * nb * nb + (size_t)nb * nb, kb, B + k, ldb, nrhs);
    if (k > 0)
      panel_sub_kernel<T><<<(k + 255) / 256, 256, 0, st>>>(A + (size_t)k * lda, lda, k, kb, B + k, ldb, B, nrhs);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(k > 0 ? 2 : 1);
  }
  return QPMS_SUCCESS;
}

}  // namespace

// ---------------- solver object ----------------

namespace {
// identity on the padding rows/columns N..Np-1 of an Np x Np matrix
__global__ void pad_identity_kernel(double2 *A, size_t Np, size_t N) {
  for (size_t i = N + threadIdx.x; i < Np; i += blockDim.x) A[i * Np + i] = make_double2(1, 0);
}
// dst (column-major, leading dimension ldd) = M for M given row-major N x N
// with leading dimension lds: dst[i + j ldd] = src[i lds + j]; 32 x 32 tiles.
__global__ void rowmajor_to_colmajor_kernel(size_t N, const double2 *src, size_t lds, double2 *dst, size_t ldd) {
  __shared__ double2 tile[32][33];
  const size_t i0 = (size_t)blockIdx.y * 32, j0 = (size_t)blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {  // read rows i0 + r, columns j0 + threadIdx.x
    const size_t i = i0 + r, j = j0 + threadIdx.x;
    if (i < N && j < N) tile[r][threadIdx.x] = src[i * lds + j];
  }
  __syncthreads();
  for (int c = threadIdx.y; c < 32; c += blockDim.y) {  // write column j0 + c, rows i0 + threadIdx.x
    const size_t i = i0 + threadIdx.x, j = j0 + c;
    if (i < N && j < N) dst[i + j * ldd] = tile[threadIdx.x][c];
  }
}
// Compute type of the complex64 trailing updates (the bulk of the LU flops).
// Measured on the LU's shrinking sequence of strided rank-128 updates at
// N = 8192: FP32 SIMT 57-59 TF/s, BF16x9 emulation 33 TF/s (slower here than
// on packed beta = 0 products), TF32 tensor cores 166-183 TF/s with ~3e-4
// relative product error.  With one or a few right-hand sides the FP64
// refinement steps are cheap, so the TF32 factors are used and refinement
// recovers FP64 accuracy (falling back to FP32 factors if it stalls); with
// many right-hand sides each refinement step costs an FP64 GEMM, so FP32
// factors (fewer steps) are used.  QPMS_GB300_LU_COMPUTE = 32F / TF32 / BF16X9
// overrides the choice.
cublasComputeType_t trailing_compute(int nrhs_max) {
  const char *ev = getenv("QPMS_GB300_LU_COMPUTE");
  if (ev && !strcmp(ev, "32F")) return CUBLAS_COMPUTE_32F;
  if (ev && !strcmp(ev, "TF32")) return CUBLAS_COMPUTE_32F_FAST_TF32;
  if (ev && !strcmp(ev, "BF16X9")) return CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
  return nrhs_max <= 4 ? CUBLAS_COMPUTE_32F_FAST_TF32 : CUBLAS_COMPUTE_32F;
}
// bf16 digits per operand of the tensor-core LU (0: the cuBLAS path chosen by
// QPMS_GB300_LU_COMPUTE).  Two digits (three digit products, ~1e-5 relative
// product error) by default; a refinement that stalls refactors with three
// digits (six products, FP32-like), then in complex128.
int tc_digits(int nrhs_max) {
  (void)nrhs_max;
  const char *ev = getenv("QPMS_GB300_LU_COMPUTE");
  if (ev && !strcmp(ev, "TC3")) return 3;
  if (ev && !strcmp(ev, "TC2")) return 2;
  if (ev && (!strcmp(ev, "32F") || !strcmp(ev, "TF32") || !strcmp(ev, "BF16X9"))) return 0;
  return 2;
}
size_t tc_plane_bytes(int Np, int nrhs_max, int nb) {
  return tc_planes_bytes_a(Np, nb, 3) + tc_planes_bytes_b(std::max(Np, nrhs_max), nb, 3) + 512;
}
}  // namespace

int DenseSolver::init(int N_, int nrhs_max_, int mode_, unsigned long long seed, cudaMemPool_t pool_,
                      cudaStream_t alloc_stream) {
  release();
  pool = pool_;
  ast = alloc_stream;
  if (N_ <= 0 || nrhs_max_ <= 0 || (mode_ != 0 && mode_ != 1)) {
    set_error("dense solver: invalid size N = %d, nrhs = %d or mode %d", N_, nrhs_max_, mode_);
    return QPMS_EINVAL;
  }
  N = N_;
  Np = (N + 3) / 4 * 4;
  nrhs_max = nrhs_max_;
  mode = mode_;
  trail_ct = (int)trailing_compute(nrhs_max);
  tc_split = mode ? tc_digits(nrhs_max) : 0;
  refactors = 0;
  base_mode = mode;
  base_trail = trail_ct;
  base_tc = tc_split;
  nb = mode ? 128 : 64;
  const size_t esz = mode ? 8 : 16;
  const size_t NN = (size_t)Np * Np;
  const int nblk = (Np + nb - 1) / nb;
  size_t wsz = std::max<size_t>((size_t)Np * nb, (size_t)nb * std::max(Np, nrhs_max)) * esz;
  if (mode) QG_CUDA_TRY(dev_alloc(&A, NN * esz));
  QG_CUDA_TRY(dev_alloc(&T64, NN * 16));
  QG_CUDA_TRY(dev_alloc(&Dinv, (size_t)nblk * 2 * nb * nb * esz));
  QG_CUDA_TRY(dev_alloc(&work, wsz));
  QG_CUDA_TRY(dev_alloc(&rhs_lo, (size_t)Np * nrhs_max * 8));
  QG_CUDA_TRY(dev_alloc(&rp, (size_t)Np * nrhs_max * 16));
  QG_CUDA_TRY(dev_alloc(&r64, (size_t)N * nrhs_max * 16));
  QG_CUDA_TRY(dev_alloc(&y64, (size_t)N * nrhs_max * 16));
  QG_CUDA_TRY(dev_alloc(&dinfo, 16));
  QG_CUDA_TRY(dev_alloc(&rs, (size_t)4 * Np * sizeof(double)));
  QG_CUDA_TRY(dev_alloc(&res_nrm, (size_t)2 * kOzakiMinRhs * sizeof(double)));
  if (tc_split) {
    QG_CUDA_TRY(dev_alloc(&tc_pa, tc_planes_bytes_a(Np, nb, 3)));
    QG_CUDA_TRY(dev_alloc(&tc_pb, tc_planes_bytes_b(std::max(Np, nrhs_max), nb, 3)));
  }
  use_ozaki = ozaki_wanted(nrhs_max);
  if (use_ozaki && (dev_alloc(&oz_mat, ozaki_matrix_bytes(N)) != cudaSuccess ||
                    dev_alloc(&oz_work, ozaki_work_bytes(N, nrhs_max)) != cudaSuccess)) {
    cudaGetLastError();  // no room for the slices: keep the complex128 residual
    for (void **q : {&oz_mat, &oz_work})
      if (*q) {
        if (pool)
          cudaFreeAsync(*q, ast);
        else
          cudaFree(*q);
        *q = nullptr;
      }
    use_ozaki = false;
  }
  // random butterfly diagonals exp(r/10), r ~ U(-1/2, 1/2): [u level1][u level2][v level1][v level2]
  std::mt19937_64 gen(seed);
  std::uniform_real_distribution<double> U(-0.5, 0.5);
  std::vector<double> h(4 * (size_t)Np);
  for (auto &v : h) v = exp(U(gen) / 10);
  QG_CUDA_TRY(cudaMemcpyAsync(rs, h.data(), h.size() * 8, cudaMemcpyHostToDevice, ast));
  QG_CUDA_TRY(cudaStreamSynchronize(ast));  // h is a local buffer
  return QPMS_SUCCESS;
}

size_t DenseSolver::footprint(int N, int nrhs, int mode) {
  const size_t Np = (size_t)(N + 3) / 4 * 4, nb = mode ? 128 : 64, esz = mode ? 8 : 16;
  const size_t nblk = (Np + nb - 1) / nb;
  size_t b = (mode ? Np * Np * esz : 0) + Np * Np * 16 + nblk * 2 * nb * nb * esz;
  b += std::max<size_t>(Np * nb, nb * std::max<size_t>(Np, nrhs)) * esz;
  b += Np * nrhs * (8 + 16) + (size_t)N * nrhs * 32 + 16 + 4 * Np * 8 + 2 * kOzakiMinRhs * 8;
  if (ozaki_wanted(nrhs)) b += ozaki_matrix_bytes(N) + ozaki_work_bytes(N, nrhs);
  if (mode && tc_digits(nrhs)) b += tc_plane_bytes((int)Np, nrhs, (int)nb);
  return b + 12 * 512;  // allocation rounding
}

bool ozaki_wanted(int nrhs_max) {
  if (nrhs_max < kOzakiMinRhs) return false;
  const char *e = getenv("QPMS_GB300_RESIDUAL");
  return !(e && !strcmp(e, "ZGEMM"));
}

cudaError_t DenseSolver::dev_alloc(void *ptr, size_t bytes) {
  void **pp = (void **)ptr;
  return pool ? cudaMallocFromPoolAsync(pp, bytes, pool, ast) : cudaMalloc(pp, bytes);
}

void DenseSolver::release() {
  for (void *p : {(void *)A, (void *)T64, (void *)Dinv, (void *)work, (void *)rhs_lo, (void *)rp, (void *)r64,
                  (void *)y64, (void *)dinfo, (void *)rs, (void *)res_nrm, oz_mat, oz_work, tc_pa, tc_pb})
    if (p) {
      if (pool)
        cudaFreeAsync(p, ast);
      else
        cudaFree(p);
    }
  A = T64 = Dinv = work = rhs_lo = rp = nullptr;
  r64 = y64 = nullptr;
  dinfo = nullptr;
  rs = nullptr;
  res_nrm = nullptr;
  oz_mat = oz_work = nullptr;
  tc_pa = tc_pb = nullptr;
  use_ozaki = false;
}

// W_u^T (rows) of an Np x ncols FP64 block
static int rbt_left(const DenseSolver &s, double2 *X, size_t ld, size_t ncols, cudaStream_t st) {
  // level 2 (blocks of Np/2, halves Np/4) then level 1 (halves Np/2)
  rbt_rows_kernel<<<grid1((size_t)s.Np / 2 * ncols), 256, 0, st>>>(s.Np, ncols, ld, X, s.Np / 4, s.rs + s.Np, 1);
  rbt_rows_kernel<<<grid1((size_t)s.Np / 2 * ncols), 256, 0, st>>>(s.Np, ncols, ld, X, s.Np / 2, s.rs, 1);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(2);
  return QPMS_SUCCESS;
}
// W_v y (rows, non-transposed): level 1 first, then level 2 (W = L2 L1)
static int rbt_right_solution(const DenseSolver &s, double2 *X, size_t ld, size_t ncols, cudaStream_t st) {
  rbt_rows_kernel<<<grid1((size_t)s.Np / 2 * ncols), 256, 0, st>>>(s.Np, ncols, ld, X, s.Np / 2, s.rs + 2 * s.Np,
                                                                   0);
  rbt_rows_kernel<<<grid1((size_t)s.Np / 2 * ncols), 256, 0, st>>>(s.Np, ncols, ld, X, s.Np / 4, s.rs + 3 * s.Np,
                                                                   0);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(2);
  return QPMS_SUCCESS;
}

int DenseSolver::factorize(const void *M64, size_t ldm, cudaStream_t st, bool rowmaj) {
  row_major = rowmaj;
  mode = base_mode;
  trail_ct = base_trail;
  tc_split = base_tc;
  nb = mode ? 128 : 64;
  if (use_ozaki) {
    int e;
    if ((e = ozaki_split_matrix(M64, ldm, rowmaj, N, oz_mat, &oz, st))) return e;
  }
  return factorize_current(M64, ldm, st);
}

int DenseSolver::factorize_current(const void *M64, size_t ldm, cudaStream_t st) {
  const bool rowmaj = row_major;
  const size_t NN = (size_t)Np * Np;
  cublasHandle_t h;
  int e;
  if ((e = blas_handle_get(&h))) return e;
  QG_BLAS_TRY(cublasSetStream(h, st));
  QG_CUDA_TRY(cudaMemsetAsync(dinfo, 0, 4, st));
  // T64 = W_u^T diag(M, I) W_v   (M W = column pass with level 2 first: M L2 L1)
  if (Np != N) QG_CUDA_TRY(cudaMemsetAsync(T64, 0, NN * 16, st));
  if (rowmaj) {
    const dim3 g((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32)), b(32, 8);
    rowmajor_to_colmajor_kernel<<<g, b, 0, st>>>(N, (const double2 *)M64, ldm, (double2 *)T64, Np);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  } else {
    QG_CUDA_TRY(cudaMemcpy2DAsync(T64, (size_t)Np * 16, M64, ldm * 16, (size_t)N * 16, N,
                                  cudaMemcpyDeviceToDevice, st));
  }
  if (Np != N) {
    pad_identity_kernel<<<1, 32, 0, st>>>((double2 *)T64, Np, N);
    g_launches.fetch_add(1);
  }
  if ((e = rbt_left(*this, (double2 *)T64, Np, Np, st))) return e;
  rbt_cols_kernel<<<grid1(NN / 2), 256, 0, st>>>(Np, Np, (double2 *)T64, Np / 4, rs + 3 * Np);
  rbt_cols_kernel<<<grid1(NN / 2), 256, 0, st>>>(Np, Np, (double2 *)T64, Np / 2, rs + 2 * Np);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(2);
  if (mode) {
    d2f_kernel<<<grid1(NN), 256, 0, st>>>(NN, (const double2 *)T64, (float2 *)A);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
    if (tc_split) {
      e = lu_nopiv_tc(Np, nb, (float2 *)A, Np, (float2 *)Dinv, dinfo, tc_split, (__nv_bfloat16 *)tc_pa,
                      (__nv_bfloat16 *)tc_pb, st);
    } else {
      e = lu_nopiv<float2>(h, Np, nb, (float2 *)A, Np, (float2 *)Dinv, (float2 *)work, dinfo,
                           (cublasComputeType_t)trail_ct, st);
    }
  } else {
    e = lu_nopiv<double2>(h, Np, nb, (double2 *)T64, Np, (double2 *)Dinv, (double2 *)work, dinfo,
                          CUBLAS_COMPUTE_64F, st);
  }
  if (e) return e;
  int info = 0;
  QG_CUDA_TRY(cudaMemcpyAsync(&info, dinfo, 4, cudaMemcpyDeviceToHost, st));
  QG_CUDA_TRY(cudaStreamSynchronize(st));
  if (info) {
    set_error("dense LU: zero pivot");
    return QPMS_ERROR;
  }
  return QPMS_SUCCESS;
}

// One application of the factorised inverse: Y = W_v (LU)^-1 W_u^T R  (FP64 in and out)
int DenseSolver::apply_inverse(const void *R, size_t ldr, void *Y, size_t ldy, int nrhs, cudaStream_t st) {
  cublasHandle_t h;
  int e;
  if ((e = blas_handle_get(&h))) return e;
  QG_BLAS_TRY(cublasSetStream(h, st));
  const size_t n = (size_t)Np * nrhs;
  if (Np != N) QG_CUDA_TRY(cudaMemsetAsync(rp, 0, n * 16, st));
  QG_CUDA_TRY(cudaMemcpy2DAsync(rp, (size_t)Np * 16, R, ldr * 16, (size_t)N * 16, nrhs, cudaMemcpyDeviceToDevice,
                                st));
  if ((e = rbt_left(*this, (double2 *)rp, Np, nrhs, st))) return e;
  if (mode) {
    d2f_kernel<<<grid1(n), 256, 0, st>>>(n, (const double2 *)rp, (float2 *)rhs_lo);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
    if (nrhs <= kSmallRhs)
      e = lu_solve_small<float2>(Np, nb, (const float2 *)A, Np, (const float2 *)Dinv, (float2 *)rhs_lo, Np, nrhs, st);
    else if (tc_split)
      e = lu_solve_tc(Np, nb, (const float2 *)A, Np, (const float2 *)Dinv, (float2 *)rhs_lo, Np, nrhs, 3,
                      (__nv_bfloat16 *)tc_pa, (__nv_bfloat16 *)tc_pb, st);
    else
      e = lu_solve<float2>(h, Np, nb, (const float2 *)A, Np, (const float2 *)Dinv, (float2 *)rhs_lo, Np, nrhs,
                           (float2 *)work, CUBLAS_COMPUTE_32F, st);
    if (e) return e;
    f2d_add_kernel<<<grid1(n), 256, 0, st>>>(n, (const float2 *)rhs_lo, (double2 *)rp, 1);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  } else {
    if (nrhs <= kSmallRhs)
      e = lu_solve_small<double2>(Np, nb, (const double2 *)T64, Np, (const double2 *)Dinv, (double2 *)rp, Np, nrhs,
                                  st);
    else
      e = lu_solve<double2>(h, Np, nb, (const double2 *)T64, Np, (const double2 *)Dinv, (double2 *)rp, Np, nrhs,
                            (double2 *)work, CUBLAS_COMPUTE_64F, st);
    if (e) return e;
  }
  if ((e = rbt_right_solution(*this, (double2 *)rp, Np, nrhs, st))) return e;
  QG_CUDA_TRY(cudaMemcpy2DAsync(Y, ldy * 16, rp, (size_t)Np * 16, (size_t)N * 16, nrhs, cudaMemcpyDeviceToDevice,
                                st));
  return QPMS_SUCCESS;
}

// X = M^-1 B with FP64 iterative refinement: in mode 1 it recovers FP64
// accuracy from the complex64 factors; in mode 0 it usually stops after the
// first solve and otherwise removes the growth of pivot-free elimination.
// M64 (ldm), B, X (ld N): device FP64.
int DenseSolver::solve(const void *M64, size_t ldm, const void *B, void *X, int nrhs, double tol, int max_iter,
                       double *resid_out, int *iters_out, cudaStream_t st) {
  if (nrhs > nrhs_max || nrhs <= 0) {
    set_error("dense solver: nrhs %d outside 1..%d", nrhs, nrhs_max);
    return QPMS_EINVAL;
  }
  max_iter = max_refine_steps(max_iter);
  cublasHandle_t h;
  int e;
  if ((e = blas_handle_get(&h))) return e;
  QG_BLAS_TRY(cublasSetStream(h, st));
  const size_t n = (size_t)N * nrhs;
  double *nrm = (double *)dinfo + 1;  // two doubles after the info word
  double hb = 0, hr = 0;
  QG_CUDA_TRY(cudaMemsetAsync(nrm, 0, 8, st));
  norm2_kernel<<<grid1(n), 256, 0, st>>>(n, (const double2 *)B, nrm);
  QG_CUDA_TRY(cudaMemcpyAsync(&hb, nrm, 8, cudaMemcpyDeviceToHost, st));
  QG_CUDA_TRY(cudaMemcpyAsync(r64, B, n * 16, cudaMemcpyDeviceToDevice, st));
  double prev = 1e300, rel = 0;
  int it = 0;
  const cuDoubleComplex one = make_cuDoubleComplex(1, 0), mone = make_cuDoubleComplex(-1, 0);
  bool first = true;
  int extra = 0;  // iterations granted again after a refactorisation
  for (it = 0; it <= max_iter + extra; ++it) {
    if ((e = apply_inverse(r64, N, y64, N, nrhs, st))) return e;
    add_kernel<<<grid1(n), 256, 0, st>>>(n, (const double2 *)y64, (double2 *)X, first);
    first = false;
    // r = B - M X (FP64 accuracy)
    if (use_ozaki && nrhs >= kOzakiMinRhs) {
      if ((e = ozaki_residual(oz, X, B, r64, nrhs, oz_work, st))) return e;
    } else if (row_major && ldm == (size_t)N && nrhs <= kOzakiMinRhs) {
      // few right-hand sides: one warp per row of the row-major M, FP64 (a pass over M per column)
      for (int c = 0; c < nrhs; ++c)
        if ((e = launch_residual(1, N, (const qg_c *)M64, (const qg_c *)X + (size_t)c * N,
                                 (const qg_c *)B + (size_t)c * N, (qg_c *)r64 + (size_t)c * N, res_nrm + 2 * c,
                                 res_nrm + 2 * c + 1, st)))
          return e;
    } else {
      QG_CUDA_TRY(cudaMemcpyAsync(r64, B, n * 16, cudaMemcpyDeviceToDevice, st));
      // a row-major M read column-major is M^T: multiply with OP_T
      QG_BLAS_TRY(cublasZgemm(h, row_major ? CUBLAS_OP_T : CUBLAS_OP_N, CUBLAS_OP_N, N, nrhs, N, &mone,
                              (const cuDoubleComplex *)M64, (int)ldm, (const cuDoubleComplex *)X, N, &one,
                              (cuDoubleComplex *)r64, N));
      g_launches.fetch_add(2);
    }
    QG_CUDA_TRY(cudaMemsetAsync(nrm, 0, 8, st));
    norm2_kernel<<<grid1(n), 256, 0, st>>>(n, (const double2 *)r64, nrm);
    QG_CUDA_TRY(cudaMemcpyAsync(&hr, nrm, 8, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
    g_launches.fetch_add(1);
    rel = sqrt(hr / (hb > 0 ? hb : 1));
    if (rel <= tol) break;
    if (rel >= 0.5 * prev || it == max_iter + extra) {  // stagnated
      if (mode) {
        // factors too coarse for this matrix (the refinement contracts by about
        // cond x the factors' error): TF32 -> FP32 -> FP64 factors, continue from x.
        // mode 0 reuses the same buffers: T64 is factored in place, Dinv and
        // work hold 2 x (64 x 64 x 16 B) per 64 rows as 2 x (128 x 128 x 8 B) per 128
        if (tc_split == 2) {
          tc_split = 3;
        } else if (!tc_split && trail_ct != (int)CUBLAS_COMPUTE_32F) {
          trail_ct = (int)CUBLAS_COMPUTE_32F;
        } else {
          mode = 0;
          nb = 64;
        }
        ++refactors;
        if ((e = factorize_current(M64, ldm, st))) return e;
        if ((e = blas_handle_get(&h))) return e;
        QG_BLAS_TRY(cublasSetStream(h, st));
        prev = 1e300;
        extra = it + 1;
        continue;
      }
      break;
    }
    prev = rel;
  }
  if (resid_out) *resid_out = rel;
  if (iters_out) *iters_out = it + 1;  // applications of the factors
  return QPMS_SUCCESS;
}

}  // namespace qg

using namespace qg;

extern "C" int qpms_gpu_dense_solve(int N, int nrhs, const qpms_complex_t *M, const qpms_complex_t *B,
                                    qpms_complex_t *X, int mode, double *resid, int *iters) {
  clear_error();
  if (!M || !B || !X || N <= 0 || nrhs <= 0 || (mode != 0 && mode != 1)) {
    set_error("invalid arguments");
    return QPMS_EINVAL;
  }
  DenseSolver s;
  int e;
  if ((e = s.init(N, nrhs, mode, 0x5eed))) return e;
  if ((e = s.factorize(M, N, 0))) return e;
  return s.solve(M, N, B, X, nrhs, 1e-13, 12, resid, iters, 0);
}
