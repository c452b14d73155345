// Batched LU with partial pivoting of small row-major complex matrices, and
// the matching substitutions, for the mode problems of dispersion scans,
// serving batches and the finite plane-wave scatter (N <= 512).  The
// reference factorises each matrix with LAPACKE_zgetrf and solves with
// LAPACKE_zgetrs (scatsystem.c:2202-2273); the factors here have the same
// meaning (P M = L U, unit-lower L below the diagonal, U on and above, ipiv[i]
// the row exchanged with row i at step i, 0-based) on the row-major matrix
// as the reference stores it.
//
// getrf: one CTA per matrix, right-looking by panels of PW columns.  The
// panel (rows k..N-1) is factored in shared memory by the whole CTA (block
// argmax for the pivot, row exchange, scaling, rank-1 update of the panel),
// written back; the CTA then applies the panel's exchanges to the other
// columns, forms U12 = L11^-1 A12 (a thread per column) and updates
// A22 -= L21 U12 with U12 staged in shared memory in chunks of 128 columns.
// The matrix itself stays in global memory (L2-resident for these sizes).
// getrs: one warp per system, dot-product substitutions over the contiguous
// rows (exchange, L y = P b, U x = y).
#include <cuda_runtime.h>
#include <math.h>

#include "qg_batchlu.h"
#include "qg_internal.h"
#include "qg_ktimer.h"

namespace qg {
namespace {

template <typename T>
struct BL;
template <>
struct BL<float2> {
  typedef float R;
  static constexpr int PW = 32;
};
template <>
struct BL<double2> {
  typedef double R;
  static constexpr int PW = 16;
};

template <typename T>
__device__ __forceinline__ T cmk(typename BL<T>::R r, typename BL<T>::R i) {
  T z;
  z.x = r;
  z.y = i;
  return z;
}
template <typename T>
__device__ __forceinline__ T cfma(T acc, T a, T b) {
  return cmk<T>(acc.x + a.x * b.x - a.y * b.y, acc.y + a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ T cfms(T acc, T a, T b) {  // acc - a b
  return cmk<T>(acc.x - a.x * b.x + a.y * b.y, acc.y - a.x * b.y - a.y * b.x);
}
template <typename T>
__device__ __forceinline__ T cdiv(T a, T b) {
  typedef typename BL<T>::R R;
  const R d = b.x * b.x + b.y * b.y;
  return cmk<T>((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
template <typename T>
__device__ __forceinline__ double cabs1(T a) {  // |Re| + |Im|, LAPACK's izamax measure
  return fabs((double)a.x) + fabs((double)a.y);
}

constexpr int kThreads = 256;
constexpr int kChunk = 128;  // trailing-update columns staged per pass

template <typename T>
__global__ void __launch_bounds__(kThreads) getrf_kernel(int N, T *A_all, int *piv_all, int *info_all) {
  constexpr int PW = BL<T>::PW;
  extern __shared__ __align__(16) unsigned char sm[];
  T *P = reinterpret_cast<T *>(sm);  // panel [N][PW] (rows k..N-1 used, row r at P[(r - k) * PW])
  T *U = P + (size_t)N * PW;         // U12 chunk [PW][kChunk]
  __shared__ double red_v[kThreads / 32];
  __shared__ int red_i[kThreads / 32];
  __shared__ int s_piv;
  T *A = A_all + (size_t)blockIdx.x * N * N;
  int *piv = piv_all + (size_t)blockIdx.x * N;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int info = 0;
  for (int k = 0; k < N; k += PW) {
    const int pw = min(PW, N - k), rows = N - k;
    // load the panel
    for (int t = tid; t < rows * pw; t += kThreads) {
      const int r = t / pw, c = t - r * pw;
      P[r * PW + c] = A[(size_t)(k + r) * N + k + c];
    }
    __syncthreads();
    for (int c = 0; c < pw; ++c) {
      // pivot: argmax |Re| + |Im| over panel rows c..rows-1 of column c (first of equals)
      double bv = -1;
      int bi = c;
      for (int r = c + tid; r < rows; r += kThreads) {
        const double v = cabs1(P[r * PW + c]);
        if (v > bv) {
          bv = v;
          bi = r;
        }
      }
      for (int o = 16; o; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) {
          bv = ov;
          bi = oi;
        }
      }
      if (lane == 0) {
        red_v[warp] = bv;
        red_i[warp] = bi;
      }
      __syncthreads();
      if (tid == 0) {
        double v = red_v[0];
        int i = red_i[0];
        for (int w = 1; w < kThreads / 32; ++w)
          if (red_v[w] > v || (red_v[w] == v && red_i[w] < i)) {
            v = red_v[w];
            i = red_i[w];
          }
        s_piv = i;
        piv[k + c] = k + i;
      }
      __syncthreads();
      const int p = s_piv;
      if (p != c && tid < pw) {  // exchange panel rows c and p
        const T a = P[c * PW + tid];
        P[c * PW + tid] = P[p * PW + tid];
        P[p * PW + tid] = a;
      }
      __syncthreads();
      const T d = P[c * PW + c];
      const bool zero = (d.x == 0 && d.y == 0);
      if (zero && info == 0) info = k + c + 1;
      // scale the column below the diagonal, then the rank-1 update of the panel
      if (!zero)
        for (int r = c + 1 + tid; r < rows; r += kThreads) P[r * PW + c] = cdiv(P[r * PW + c], d);
      __syncthreads();
      const int nc = pw - c - 1;
      if (nc > 0 && !zero)
        for (int t = tid; t < (rows - c - 1) * nc; t += kThreads) {
          const int r = c + 1 + t / nc, j = c + 1 + t % nc;
          P[r * PW + j] = cfms(P[r * PW + j], P[r * PW + c], P[c * PW + j]);
        }
      __syncthreads();
    }
    // write the panel back
    for (int t = tid; t < rows * pw; t += kThreads) {
      const int r = t / pw, c = t - r * pw;
      A[(size_t)(k + r) * N + k + c] = P[r * PW + c];
    }
    // the panel's row exchanges on the columns outside it, in order, a thread per column
    for (int j = tid; j < N - pw; j += kThreads) {
      const int col = j < k ? j : j + pw;
      for (int c = 0; c < pw; ++c) {
        const int p = piv[k + c];
        if (p != k + c) {
          const T a = A[(size_t)(k + c) * N + col];
          A[(size_t)(k + c) * N + col] = A[(size_t)p * N + col];
          A[(size_t)p * N + col] = a;
        }
      }
    }
    __syncthreads();
    const int k2 = k + pw;
    if (k2 >= N) break;
    // U12 = L11^-1 A12 (unit lower), a thread per column
    for (int col = k2 + tid; col < N; col += kThreads) {
      T x[PW];
#pragma unroll
      for (int r = 0; r < PW; ++r)
        if (r < pw) x[r] = A[(size_t)(k + r) * N + col];
#pragma unroll
      for (int r = 1; r < PW; ++r)
        if (r < pw)
#pragma unroll
          for (int s = 0; s < PW; ++s)
            if (s < r) x[r] = cfms(x[r], P[r * PW + s], x[s]);
#pragma unroll
      for (int r = 0; r < PW; ++r)
        if (r < pw) A[(size_t)(k + r) * N + col] = x[r];
    }
    __syncthreads();
    // A22 -= L21 U12, U12 staged by column chunks
    for (int c0 = k2; c0 < N; c0 += kChunk) {
      const int cw = min(kChunk, N - c0);
      for (int t = tid; t < pw * cw; t += kThreads) {
        const int r = t / cw, j = t - r * cw;
        U[r * kChunk + j] = A[(size_t)(k + r) * N + c0 + j];
      }
      __syncthreads();
      const int nr = N - k2;
      for (int t = tid; t < nr * cw; t += kThreads) {
        const int i = t / cw, j = t - i * cw;
        const T *l = P + (size_t)(pw + i) * PW;
        T acc = A[(size_t)(k2 + i) * N + c0 + j];
#pragma unroll 8
        for (int s = 0; s < pw; ++s) acc = cfms(acc, l[s], U[s * kChunk + j]);
        A[(size_t)(k2 + i) * N + c0 + j] = acc;
      }
      __syncthreads();
    }
  }
  if (tid == 0 && info_all) info_all[blockIdx.x] = info;
}

// One warp per system: x = (P M)^-1 b in place on b (one right-hand side).
template <typename T>
__global__ void getrs_kernel(int nm, int N, const T *LU_all, const int *piv_all, T *b_all) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nm) return;
  const T *A = LU_all + (size_t)w * N * N;
  const int *piv = piv_all + (size_t)w * N;
  T *b = b_all + (size_t)w * N;
  if (lane == 0)
    for (int i = 0; i < N; ++i) {
      const int p = piv[i];
      if (p != i) {
        const T a = b[i];
        b[i] = b[p];
        b[p] = a;
      }
    }
  __syncwarp();
  for (int i = 1; i < N; ++i) {  // L y = P b, unit lower
    T acc = cmk<T>(0, 0);
    for (int j = lane; j < i; j += 32) acc = cfma(acc, A[(size_t)i * N + j], b[j]);
    for (int o = 16; o; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) b[i] = cmk<T>(b[i].x - acc.x, b[i].y - acc.y);
    __syncwarp();
  }
  for (int i = N - 1; i >= 0; --i) {  // U x = y
    T acc = cmk<T>(0, 0);
    for (int j = i + 1 + lane; j < N; j += 32) acc = cfma(acc, A[(size_t)i * N + j], b[j]);
    for (int o = 16; o; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) b[i] = cdiv(cmk<T>(b[i].x - acc.x, b[i].y - acc.y), A[(size_t)i * N + i]);
    __syncwarp();
  }
}

template <typename T>
size_t getrf_smem(int N) {
  return ((size_t)N * BL<T>::PW + (size_t)BL<T>::PW * kChunk) * sizeof(T);
}

template <typename T>
int getrf_launch(int nm, int N, T *A, int *piv, int *info, cudaStream_t st) {
  const size_t smem = getrf_smem<T>(N);
  if (N > kBatchLuMaxN) {
    set_error("batched LU: N = %d above %d", N, kBatchLuMaxN);
    return QPMS_EINVAL;
  }
  QG_CUDA_TRY(cudaFuncSetAttribute(getrf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  KtScope kt(KT_BATCHLU, st, nm * 8.0 * N * (double)N * N / 3.0);
  getrf_kernel<T><<<nm, kThreads, smem, st>>>(N, A, piv, info);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

template <typename T>
int getrs_launch(int nm, int N, const T *LU, const int *piv, T *b, cudaStream_t st) {
  const int wpb = 4;
  getrs_kernel<T><<<(nm + wpb - 1) / wpb, 32 * wpb, 0, st>>>(nm, N, LU, piv, b);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

}  // namespace

int batch_getrf_c64(int nm, int N, void *A, int *piv, int *info, cudaStream_t st) {
  if (nm <= 0 || N <= 0) return QPMS_SUCCESS;
  return getrf_launch<float2>(nm, N, (float2 *)A, piv, info, st);
}
int batch_getrf_c128(int nm, int N, void *A, int *piv, int *info, cudaStream_t st) {
  if (nm <= 0 || N <= 0) return QPMS_SUCCESS;
  return getrf_launch<double2>(nm, N, (double2 *)A, piv, info, st);
}
int batch_getrs_c64(int nm, int N, const void *LU, const int *piv, void *b, cudaStream_t st) {
  if (nm <= 0 || N <= 0) return QPMS_SUCCESS;
  return getrs_launch<float2>(nm, N, (const float2 *)LU, piv, (float2 *)b, st);
}
int batch_getrs_c128(int nm, int N, const void *LU, const int *piv, void *b, cudaStream_t st) {
  if (nm <= 0 || N <= 0) return QPMS_SUCCESS;
  return getrs_launch<double2>(nm, N, (const double2 *)LU, piv, (double2 *)b, st);
}

}  // namespace qg
