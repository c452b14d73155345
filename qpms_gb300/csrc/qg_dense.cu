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
//   2. factorises A' without pivoting by blocks in Schur-complement form: at
//      step k the nb x nb diagonal block D is inverted by one CTA
//      (Gauss-Jordan in registers), the whole column block k is multiplied
//      by D^-1 (below the block this is P = A21 D^-1, above it
//      Q = A_0:k,k D^-1, the block itself becomes I - D^-1) and the trailing
//      matrix is updated, A22 -= P A12, with the row panel A12 kept as it is;
//      A' = L U with L = [I 0; P I] (per level) and U = [D A12; 0 S];
//   3. solves with two sweeps of one product per block: forward
//      b_below -= P_k b_k, backward b_0:k+kb -= [Q_k; I - D_k^-1] b_k (which
//      leaves D_k^-1 b_k, the block's solution, in b_k);
//   4. in the mixed mode, the factorisation and substitutions run in complex64
//      (products on the tensor cores, qg_tcgemm.cu) and the FP64 solution is
//      recovered by iterative refinement against the FP64 matrix:
//      x += W_v (LU)^-1 W_u^T (b - M x), residual in FP64.
// The plain mode runs steps 1-3 in complex128 (FP64 GEMMs).
// All matrices are column-major (LAPACK order).  The butterflies halve the
// system twice, so it is padded internally to a multiple of 4 with identity.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <random>
#include <vector>

#include "qg_assembly.h"
#include "qg_batched.h"
#include "qg_dense.h"
#include "qg_internal.h"
#include "qg_ktimer.h"
#include "qg_tcgemm.h"
#include "qg_tuned.h"

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

// ---------------- diagonal block: inverse by Gauss-Jordan ----------------
// D (kb x kb, kb even and <= 32 NB, column-major in global, leading
// dimension lda): Ainv (column-major kb x kb, leading dimension kb) receives
// D^-1, and D is overwritten with D - I (the column-block product that follows
// turns it into I - D^-1, the slot the back substitution reads).  info is set
// to 1 on a singular pivot block.  Gauss-Jordan elimination without pivoting
// (the random butterflies make it safe with high probability, as for the
// whole LU), two columns per step: with J = {j, j + 1} and the 2 x 2 pivot
// block P,
//   A_JJ <- P^-1,  A_Jc <- P^-1 A_Jc,  A_rJ <- -A_rJ P^-1,
//   A_rc <- A_rc - A_rJ P^-1 A_Jc        (r, c not in J).
// One CTA of 512 threads with the block in registers: thread t holds the
// NA x NB elements (t % 16 + 16 i, t / 16 + 32 j), rows-heavy so that the
// per-column factors u = P^-1 A_Jc (the costly part of a step besides the
// update) are formed for NB = 4 columns only.  Row r lives in the threads with
// t % 16 == r % 16, column c in those with t / 16 == c % 32.  At each step the
// two pivot rows and columns are published through two alternating
// shared-memory slots (one barrier per step); every thread then forms P^-1
// itself, updates all its elements and overwrites the pivot rows and columns.
constexpr int kDiagMaxNb = 128, kDiagThreads = 512;

// Complex multiply-add as four fused multiply-adds (no separate product and
// sum: fewer instructions in the update loops, one rounding per term).
__device__ __forceinline__ float fmar(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmar(double a, double b, double c) { return fma(a, b, c); }
template <typename T>
__device__ __forceinline__ T fma_c(T acc, T a, T b) {  // acc + a b
  return mk<T>(fmar(-a.y, b.y, fmar(a.x, b.x, acc.x)), fmar(a.y, b.x, fmar(a.x, b.y, acc.y)));
}
template <typename T>
__device__ __forceinline__ T fms_c(T acc, T a, T b) {  // acc - a b
  return mk<T>(fmar(a.y, b.y, fmar(-a.x, b.x, acc.x)), fmar(-a.y, b.x, fmar(-a.x, b.y, acc.y)));
}

template <typename T, int NB>
__global__ void __launch_bounds__(kDiagThreads, 1) diag_inv_kernel(T *D, size_t lda, int kb, T *Ainv, int *info) {
  constexpr int NA = 2 * NB;  // row tiles per thread: 16 rows x NA, 32 columns x NB
  __shared__ T sc[2][2][kDiagMaxNb];  // [slot][e][r] = a_(r, j+e)
  __shared__ T sr[2][2][kDiagMaxNb];  // [slot][e][c] = a_(j+e, c)
  const int lr = threadIdx.x & 15, lc = threadIdx.x >> 4;
  T a[NA][NB];
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      const int r = lr + 16 * i, c = lc + 32 * j;
      a[i][j] = mk<T>(0, 0);
      if (r < kb && c < kb) {
        T v = D[(size_t)c * lda + r];
        a[i][j] = v;
        if (r == c) v.x -= 1;
        D[(size_t)c * lda + r] = v;
      }
    }
  bool zero = false;
  // Step (j, j + 1), j = 32 ct + 16 h + q, q even: rows j, j + 1 are tile row
  // 2 ct + h of the threads with lr = q, q + 1; columns j, j + 1 are tile
  // column ct of the threads with lc = 16 h + q, 16 h + q + 1.  ct and h are
  // unrolled, so every register index is static.
#pragma unroll
  for (int ct = 0; ct < NB; ++ct) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int rt = 2 * ct + h;
      for (int q = 0; q < 16; q += 2) {
        const int j = 32 * ct + 16 * h + q;
        if (j >= kb) break;  // uniform
        const int slot = (j >> 1) & 1, cl = 16 * h + q;
        if (lr == q || lr == q + 1) {
          const int e = lr - q;
#pragma unroll
          for (int jj = 0; jj < NB; ++jj) {
            const int c = lc + 32 * jj;
            if (c < kb) sr[slot][e][c] = a[rt][jj];
          }
        }
        if (lc == cl || lc == cl + 1) {
          const int e = lc - cl;
#pragma unroll
          for (int i = 0; i < NA; ++i) {
            const int r = lr + 16 * i;
            if (r < kb) sc[slot][e][r] = a[i][ct];
          }
        }
        __syncthreads();
        // P = [p00 p01; p10 p11], P^-1 = [q00 q01; q10 q11]
        const T p00 = sc[slot][0][j], p10 = sc[slot][0][j + 1], p01 = sc[slot][1][j], p11 = sc[slot][1][j + 1];
        const T det = sub(mul(p00, p11), mul(p01, p10));
        const bool z = (det.x == 0 && det.y == 0);
        zero |= z;
        const T dinv = z ? mk<T>(0, 0) : rcp(det);
        const T q00 = mul(p11, dinv), q11 = mul(p00, dinv);
        const T q01 = mk<T>(-(p01.x * dinv.x - p01.y * dinv.y), -(p01.x * dinv.y + p01.y * dinv.x));
        const T q10 = mk<T>(-(p10.x * dinv.x - p10.y * dinv.y), -(p10.x * dinv.y + p10.y * dinv.x));
        // u = P^-1 A_Jc for this thread's NB columns
        T u0[NB], u1[NB];
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) {
          const int c = min(lc + 32 * jj, kb - 1);  // columns >= kb are padding, never stored
          const T x0 = sr[slot][0][c], x1 = sr[slot][1][c];
          u0[jj] = fma_c(mul(q00, x0), q01, x1);
          u1[jj] = fma_c(mul(q10, x0), q11, x1);
        }
        // every element: a_rc -= a_rj u0_c + a_r,j+1 u1_c; the pivot rows and
        // columns are overwritten right after
#pragma unroll
        for (int i = 0; i < NA; ++i) {
          if (16 * i >= kb) continue;  // uniform
          const int r = min(lr + 16 * i, kb - 1);  // rows >= kb are padding, never stored
          const T f0 = sc[slot][0][r], f1 = sc[slot][1][r];
#pragma unroll
          for (int jj = 0; jj < NB; ++jj) a[i][jj] = fms_c(fms_c(a[i][jj], f0, u0[jj]), f1, u1[jj]);
          if (i == rt) {  // static: the pivot rows' tile row
            if (lr == q)
#pragma unroll
              for (int jj = 0; jj < NB; ++jj) a[i][jj] = u0[jj];
            if (lr == q + 1)
#pragma unroll
              for (int jj = 0; jj < NB; ++jj) a[i][jj] = u1[jj];
          }
        }
        if (lc == cl || lc == cl + 1) {  // columns j + e: -A_rJ P^-1, the pivot block P^-1
          const bool e0 = lc == cl;
          const T qa = e0 ? q00 : q01, qb = e0 ? q10 : q11;
#pragma unroll
          for (int i = 0; i < NA; ++i) {
            const int r = min(lr + 16 * i, kb - 1);
            const T g = fma_c(mul(sc[slot][0][r], qa), sc[slot][1][r], qb);
            a[i][ct] = mk<T>(-g.x, -g.y);
          }
          if (lr == q) a[rt][ct] = qa;
          if (lr == q + 1) a[rt][ct] = qb;
        }
      }
    }
  }
  if (zero && threadIdx.x == 0) atomicOr(info, 1);
#pragma unroll
  for (int j = 0; j < NB; ++j)
#pragma unroll
    for (int i = 0; i < NA; ++i) {
      const int r = lr + 16 * i, c = lc + 32 * j;
      if (r < kb && c < kb) Ainv[c * kb + r] = a[i][j];
    }
}

// Invert one diagonal block (kb <= 128; complex128 blocks up to 64).
template <typename T>
int launch_diag(T *D, size_t lda, int kb, T *Ainv, int *info, cudaStream_t st) {
  constexpr int kMaxNb = sizeof(T) == 16 ? 2 : 4;  // complex128 blocks: nb <= 64
  if (kb <= 0 || kb > 32 * kMaxNb || (kb & 1)) {
    set_error("diagonal block of size %d not supported", kb);
    return QPMS_EINVAL;
  }
  KtScope kt(KT_DIAGLU, st, 8.0 * kb * (double)kb * kb);
  if (kb <= 64)
    diag_inv_kernel<T, 2><<<1, kDiagThreads, 0, st>>>(D, lda, kb, Ainv, info);
  else
    diag_inv_kernel<T, kMaxNb><<<1, kDiagThreads, 0, st>>>(D, lda, kb, Ainv, info);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
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

// A = W_u^T diag(M, I) W_v in complex64 (Np x Np, column-major): the depth-2
// butterflies of rbt_rows_kernel / rbt_cols_kernel fused with the FP64 ->
// complex64 conversion, one pass over M.  Entry (r, c) of the result depends
// only on the 4 x 4 entries of diag(M, I) in the rows r mod Np/4 + q Np/4 and
// the columns c mod Np/4 + p Np/4 (q, p = 0..3).  A CTA takes kRbtT x kRbtT
// such row / column orbits: it stages their 4 kRbtT x 4 kRbtT entries in
// shared memory (reads coalesced in M's own layout, row- or column-major),
// each thread transforms one orbit pair in registers (rows level 2 then 1,
// columns level 2 then 1, in the order of the separate passes), and the
// results leave coalesced down A's columns.  The entries are rounded to
// complex64 as they are read and the butterflies run in FP32: the factors are
// complex64 anyway, and GB300's FP64 rate (1/64 of FP32) would make this pass
// arithmetic-bound; the FP64 refinement works against the exact transform.
constexpr int kRbtT = 16, kRbtS = 4 * kRbtT;  // orbits per CTA side, staged entries per side

__device__ __forceinline__ void rbt_pair(float2 &top, float2 &bot, float R, float S) {
  const float is2 = 0.70710678118654752440f;
  const float2 t = top, b = bot;
  top = make_float2(R * is2 * (t.x + b.x), R * is2 * (t.y + b.y));
  bot = make_float2(S * is2 * (t.x - b.x), S * is2 * (t.y - b.y));
}

__global__ void __launch_bounds__(256) rbt_convert_kernel(const double2 *__restrict__ M, size_t ldm, int rowmaj,
                                                          int N, int Np, const double *__restrict__ rs,
                                                          float2 *__restrict__ A) {
  constexpr int LD = kRbtS + 1;
  __shared__ float2 S[kRbtS * LD];  // S[lc * LD + lr]
  const int Q = Np / 4;
  const int I0 = blockIdx.x * kRbtT, J0 = blockIdx.y * kRbtT;
  const int tid = threadIdx.x;
  // global index of local row / column l: (l / kRbtT) Q + base + l % kRbtT
  for (int t = tid; t < kRbtS * kRbtS; t += blockDim.x) {
    const int la = t % kRbtS, lb = t / kRbtS;  // la walks the source's contiguous dimension
    const int lr = rowmaj ? lb : la, lc = rowmaj ? la : lb;
    const int ir = I0 + lr % kRbtT, jc = J0 + lc % kRbtT;
    if (ir >= Q || jc >= Q) continue;
    const int R = (lr / kRbtT) * Q + ir, C = (lc / kRbtT) * Q + jc;
    float2 v;
    if (R < N && C < N) {
      const double2 d = rowmaj ? M[(size_t)R * ldm + C] : M[(size_t)C * ldm + R];
      v = make_float2((float)d.x, (float)d.y);
    } else {
      v = make_float2(R == C ? 1.f : 0.f, 0.f);
    }
    S[lc * LD + lr] = v;
  }
  __syncthreads();
  {
    const int i = tid % kRbtT, j = tid / kRbtT;
    const int i0 = I0 + i, j0 = J0 + j;
    if (i0 < Q && j0 < Q) {
      float2 x[4][4];  // x[q][p]: row q Q + i0, column p Q + j0
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) x[q][p] = S[(p * kRbtT + j) * LD + q * kRbtT + i];
      const double *r2 = rs + Np, *r1 = rs, *c2 = rs + 3 * (size_t)Np, *c1 = rs + 2 * (size_t)Np;
      // rows, level 2 (halves Q within blocks of 2Q): pairs (0, 1), (2, 3)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const float R = (float)r2[b * 2 * Q + i0], Sv = (float)r2[b * 2 * Q + Q + i0];
#pragma unroll
        for (int p = 0; p < 4; ++p) rbt_pair(x[2 * b][p], x[2 * b + 1][p], R, Sv);
      }
      // rows, level 1 (halves 2Q): pairs (0, 2), (1, 3)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const float R = (float)r1[q * Q + i0], Sv = (float)r1[2 * Q + q * Q + i0];
#pragma unroll
        for (int p = 0; p < 4; ++p) rbt_pair(x[q][p], x[q + 2][p], R, Sv);
      }
      // columns, level 2 then level 1
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const float R = (float)c2[b * 2 * Q + j0], Sv = (float)c2[b * 2 * Q + Q + j0];
#pragma unroll
        for (int q = 0; q < 4; ++q) rbt_pair(x[q][2 * b], x[q][2 * b + 1], R, Sv);
      }
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const float R = (float)c1[p * Q + j0], Sv = (float)c1[2 * Q + p * Q + j0];
#pragma unroll
        for (int q = 0; q < 4; ++q) rbt_pair(x[q][p], x[q][p + 2], R, Sv);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) S[(p * kRbtT + j) * LD + q * kRbtT + i] = x[q][p];
    }
  }
  __syncthreads();
  for (int t = tid; t < kRbtS * kRbtS; t += blockDim.x) {
    const int lr = t % kRbtS, lc = t / kRbtS;
    const int ir = I0 + lr % kRbtT, jc = J0 + lc % kRbtT;
    if (ir >= Q || jc >= Q) continue;
    const int R = (lr / kRbtT) * Q + ir, C = (lc / kRbtT) * Q + jc;
    A[(size_t)C * Np + R] = S[lc * LD + lr];
  }
}

// exp(r / 10) with r uniform in [-1/2, 1/2) from a counter-based generator
// (splitmix64 of seed + i): the random butterfly diagonals.
__global__ void rbt_diag_kernel(double *rs, size_t n, unsigned long long seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long z = seed + (i + 1) * 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    const double r = (double)(z >> 11) * 0x1.0p-53 - 0.5;
    rs[i] = exp(r / 10);
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

// Blocked LU without pivoting in Schur-complement form (see the header
// comment).  Step k with the diagonal block D = A_kk, kb columns:
//   Ainv = D^-1 (diag_inv_kernel, which also leaves D - I in the slot);
//   column block k (all N rows) <- column block k x Ainv: the rows below the
//     block become P_k = A21 D^-1, the block itself I - D^-1, the rows above
//     Q_k = A_0:k,k D^-1;
//   A22 -= P_k A12 (A12: the row panel right of the block, kept as it is).
template <typename T>
int lu_nopiv(cublasHandle_t h, int N, int nb, T *A, size_t lda, T *Dinv, T *work, int *dinfo,
             cublasComputeType_t ct, cudaStream_t st) {
  int e;
  const cublasComputeType_t cp = (sizeof(T) == 8) ? CUBLAS_COMPUTE_32F : CUBLAS_COMPUTE_64F;  // column blocks
  for (int k = 0, blk = 0; k < N; k += nb, ++blk) {
    const int kb = (N - k < nb) ? N - k : nb;
    T *Ainv = Dinv + (size_t)blk * nb * nb, *Ck = A + (size_t)k * lda;
    if ((e = launch_diag<T>(Ck + k, lda, kb, Ainv, dinfo, st))) return e;
    if ((e = gemm<T>(h, N, kb, kb, cone<T>(), Ck, lda, Ainv, kb, cval<T>(0), work, N, cp))) return e;
    QG_CUDA_TRY(cudaMemcpy2DAsync(Ck, lda * sizeof(T), work, (size_t)N * sizeof(T), (size_t)N * sizeof(T), kb,
                                  cudaMemcpyDeviceToDevice, st));
    const int m2 = N - k - kb;
    if (m2 <= 0) break;
    T *P = Ck + k + kb, *A12 = A + (size_t)(k + kb) * lda + k, *A22 = P + (size_t)kb * lda;
    if ((e = gemm<T>(h, m2, m2, kb, cval<T>(-1), P, lda, A12, lda, cone<T>(), A22, lda, ct))) return e;
  }
  return QPMS_SUCCESS;
}

// Solve with the factors of lu_nopiv (B: N x nrhs, column-major, ldb, in place):
//   forward, k ascending:   B_k+kb:N -= P_k B_k
//   backward, k descending: B_0:k+kb -= [Q_k; I - D_k^-1] B_k
// (the block rows of the second product leave D_k^-1 B_k in B_k).  B_k is
// copied to `work` first where the product writes over it.
template <typename T>
int lu_solve(cublasHandle_t h, int N, int nb, const T *A, size_t lda, T *B, size_t ldb, int nrhs, T *work,
             cublasComputeType_t ct, cudaStream_t st) {
  int e;
  const int nblk = (N + nb - 1) / nb;
  for (int blk = 0; blk < nblk; ++blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb, m2 = N - k - kb;
    if (m2 > 0)
      if ((e = gemm<T>(h, m2, nrhs, kb, cval<T>(-1), A + (size_t)k * lda + k + kb, lda, B + k, ldb, cone<T>(),
                       B + k + kb, ldb, ct)))
        return e;
  }
  for (int blk = nblk - 1; blk >= 0; --blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    QG_CUDA_TRY(cudaMemcpy2DAsync(work, (size_t)kb * sizeof(T), B + k, ldb * sizeof(T), (size_t)kb * sizeof(T), nrhs,
                                  cudaMemcpyDeviceToDevice, st));
    if ((e = gemm<T>(h, k + kb, nrhs, kb, cval<T>(-1), A + (size_t)k * lda, lda, work, kb, cone<T>(), B, ldb, ct)))
      return e;
  }
  return QPMS_SUCCESS;
}

// ---------------- complex64 LU and substitutions on the tensor cores ----------------
// The same blocked algorithm as lu_nopiv / lu_solve with every product a
// tcgen05 GEMM of split-bf16 digits (qg_tcgemm.cu): operands are cut into
// digit planes first, so each GEMM may write its result over an operand it
// read (the column blocks and the right-hand-side blocks are formed in place).
int lu_nopiv_tc(int N, int nb, float2 *A, size_t lda, float2 *Dinv, int *dinfo, int nsplit, __nv_bfloat16 *pa,
                __nv_bfloat16 *pb, cudaStream_t st, cudaStream_t side, cudaEvent_t ev_a, cudaEvent_t ev_d,
                int group) {
  // Lookahead (side != nullptr): the trailing update first updates the next
  // block column, then the next diagonal block is inverted on the side stream
  // while the rest of the update runs; the next step waits for it before its
  // column-block product.  The update GEMMs leave SMs free for the single-CTA
  // inversion.
  // Groups: blocks are taken `group` at a time.  Within a group, block i's
  // update is applied at once only to the group's later block columns (every
  // row below block i) and to the group's later block rows (the columns past
  // the group): two narrow products.  The rest of the group's updates runs as
  // one product with K = the group's width past its last block:
  //   A33 -= [P_0 ... P_g-1] [A12_0; ...; A12_g-1].
  // The same sums as g updates in sequence, with 1/g of the passes over the
  // trailing matrix (its complex64 read and write bound a K = nb update on HBM).
  const bool la = side != nullptr;
  if (group < 1) group = 1;
  TcPlanes P;
  P.a = pa;
  P.b = pb;
  P.nsplit = nsplit;
  int e;
  // column block k <- column block k x D^-1 (all N rows)
  auto colprod = [&](int k, int kb, const float2 *Ainv) -> int {
    float2 *Ck = A + (size_t)k * lda;
    int e2;
    if ((e2 = tc_split_ab(Ck, lda, N, kb, Ainv, kb, kb, nsplit, pa, pb, st))) return e2;
    TcPlanes Q = P;
    Q.m = N, Q.n = kb, Q.k = kb;
    return tc_cgemm_planes(Q, 1.f, 0.f, nullptr, 0, Ck, lda, st);
  };
  // rows and columns r0.. (m of each) -= A(r0.., c0..c0+kk) A(c0..c0+kk, r0..);
  // with lookahead the first block column first, then the inversion of that
  // diagonal block (slot next_blk of Dinv) on the side stream
  auto trailing = [&](int r0, int c0, int kk, int m, int next_blk) -> int {
    float2 *C = A + (size_t)r0 * lda + r0;
    int e2;
    if ((e2 = tc_split_ab(A + (size_t)c0 * lda + r0, lda, m, kk, A + (size_t)r0 * lda + c0, lda, m, nsplit, pa, pb,
                          st)))
      return e2;
    TcPlanes Q = P;
    Q.m = m, Q.k = kk;
    if (!la) {
      Q.n = m;
      return tc_cgemm_planes(Q, -1.f, 1.f, C, lda, C, lda, st);
    }
    const int kb1 = m < nb ? m : nb;
    const size_t rs = tc_planes_row(kk);
    Q.n = kb1;
    Q.b_plane = (size_t)m * rs;
    if ((e2 = tc_cgemm_planes(Q, -1.f, 1.f, C, lda, C, lda, st))) return e2;
    QG_CUDA_TRY(cudaEventRecord(ev_a, st));
    QG_CUDA_TRY(cudaStreamWaitEvent(side, ev_a, 0));
    if ((e2 = launch_diag<float2>(C, lda, kb1, Dinv + (size_t)next_blk * nb * nb, dinfo, side))) return e2;
    QG_CUDA_TRY(cudaEventRecord(ev_d, side));
    if (m > kb1) {
      Q.b = pb + (size_t)kb1 * rs;
      Q.n = m - kb1;
      if ((e2 = tc_cgemm_planes(Q, -1.f, 1.f, C + (size_t)kb1 * lda, lda, C + (size_t)kb1 * lda, lda, st)))
        return e2;
    }
    return QPMS_SUCCESS;
  };
  for (int k = 0, blk = 0; k < N;) {  // one group per pass: blocks blk.., columns k..ge
    const int ge = std::min<long>((long)k + (long)group * nb, (long)N);
    for (int ki = k, b = blk; ki < ge; ki += nb, ++b) {
      const int kbi = (N - ki < nb) ? N - ki : nb, ke = ki + kbi, mi = N - ke;
      float2 *Ainv = Dinv + (size_t)b * nb * nb;
      if (ki > k || !la || blk == 0) {
        if ((e = launch_diag<float2>(A + (size_t)ki * lda + ki, lda, kbi, Ainv, dinfo, st))) return e;
      } else {
        QG_CUDA_TRY(cudaStreamWaitEvent(st, ev_d, 0));
      }
      if ((e = colprod(ki, kbi, Ainv))) return e;
      if (mi <= 0) return QPMS_SUCCESS;
      if (ke == ge) {  // the group's last block: everything past the group at once
        if ((e = trailing(ge, k, ge - k, mi, b + 1))) return e;
        break;
      }
      // block i's update of the group's later block columns and rows
      const int wi = ge - ke;
      if ((e = tc_split_ab(A + (size_t)ki * lda + ke, lda, mi, kbi, A + (size_t)ke * lda + ki, lda, mi, nsplit, pa,
                           pb, st)))
        return e;
      const size_t rs = tc_planes_row(kbi);
      float2 *C = A + (size_t)ke * lda + ke;
      TcPlanes Q = P;
      Q.k = kbi;
      Q.m = mi, Q.n = wi;  // the later block columns of the group, every row below block i
      Q.b_plane = (size_t)mi * rs;
      if ((e = tc_cgemm_planes(Q, -1.f, 1.f, C, lda, C, lda, st))) return e;
      if (mi > wi) {  // the later block rows of the group, past the group: the first wi rows of the A planes
        Q.m = wi, Q.a_plane = (size_t)2 * mi * rs;
        Q.b = pb + (size_t)wi * rs, Q.n = mi - wi;
        if ((e = tc_cgemm_planes(Q, -1.f, 1.f, C + (size_t)wi * lda, lda, C + (size_t)wi * lda, lda, st))) return e;
      }
    }
    blk += (ge - k + nb - 1) / nb;
    k = ge;
  }
  return QPMS_SUCCESS;
}

// lu_solve's substitutions with the products on the tensor cores (in place).
// fp: nsplit digit planes of the whole factored matrix (tc_split_a of the
// N x N factors), or null.  With them each step cuts only its right-hand-side
// block into digits and reads its panel's planes in place (row length
// tc_planes_row(N)); without them each step cuts its panel too.
int lu_solve_tc(int N, int nb, const float2 *A, size_t lda, float2 *B, size_t ldb, int nrhs, int nsplit,
                __nv_bfloat16 *pa, __nv_bfloat16 *pb, const __nv_bfloat16 *fp, cudaStream_t st) {
  TcPlanes P;
  P.a = pa;
  P.b = pb;
  P.nsplit = nsplit;
  const size_t frs = tc_planes_row(N);
  if (fp) {
    P.a_rs = frs;
    P.a_plane = (size_t)2 * N * frs;
  }
  int e;
  const int nblk = (N + nb - 1) / nb;
  for (int blk = 0; blk < nblk; ++blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb, m2 = N - k - kb;
    if (m2 <= 0) continue;
    if (fp) {
      if ((e = tc_split_b(B + k, ldb, kb, nrhs, nsplit, pb, st))) return e;
      P.a = const_cast<__nv_bfloat16 *>(fp) + (size_t)2 * (k + kb) * frs + 2 * (size_t)k;
    } else if ((e = tc_split_ab(A + (size_t)k * lda + k + kb, lda, m2, kb, B + k, ldb, nrhs, nsplit, pa, pb, st))) {
      return e;
    }
    P.m = m2, P.n = nrhs, P.k = kb;
    if ((e = tc_cgemm_planes(P, -1.f, 1.f, B + k + kb, ldb, B + k + kb, ldb, st))) return e;
  }
  for (int blk = nblk - 1; blk >= 0; --blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    if (fp) {
      if ((e = tc_split_b(B + k, ldb, kb, nrhs, nsplit, pb, st))) return e;
      P.a = const_cast<__nv_bfloat16 *>(fp) + 2 * (size_t)k;
    } else if ((e = tc_split_ab(A + (size_t)k * lda, lda, k + kb, kb, B + k, ldb, nrhs, nsplit, pa, pb, st))) {
      return e;
    }
    P.m = k + kb, P.n = nrhs, P.k = kb;
    if ((e = tc_cgemm_planes(P, -1.f, 1.f, B, ldb, B, ldb, st))) return e;
  }
  return QPMS_SUCCESS;
}

// ---------------- substitutions for a few right-hand sides (bandwidth-bound) ----------------
constexpr int kSmallRhs = 8;

// One block step of lu_solve's substitutions for nrhs <= kSmallRhs:
//   rows r < msub:              Bsub_r -= Pn_r V
//   rows msub <= r < msub+mout: Xout_(r-msub) = V_(r-msub) - Pn_r V
// with Pn (msub + mout) x kb (leading dimension lda) and V kb x nrhs (ldv).
// V is staged in shared memory by every CTA; it is only read in this launch
// (Bsub and Xout never overlap it), so the CTAs need no ordering.  Each CTA
// takes kSubRows rows: thread (r, s) sums the columns l = s, s + kSubSlices,
// ... of row r (coalesced loads down the columns); the kSubSlices partial sums
// meet in shared memory.
constexpr int kSubRows = 32, kSubSlices = 8;

template <typename T>
__global__ void __launch_bounds__(256) panel_apply_kernel(const T *__restrict__ Pn, size_t lda, int msub, int mout,
                                                          int kb, const T *V, size_t ldv, T *Bsub, size_t ldb,
                                                          T *Xout, size_t ldx, int nrhs) {
  constexpr int kPer = 128 / kSubSlices;               // panel entries per thread (kb <= 128)
  __shared__ T sV[128 * kSmallRhs];                  // [c][l]
  __shared__ T sP[kSubSlices * kSmallRhs * kSubRows];  // [slice][c][r]
  const int tid = threadIdx.x;
  const int m = msub + mout;
  const int r = tid % kSubRows, sl = tid / kSubRows;
  const int row = blockIdx.x * kSubRows + r;
  // the panel entries are requested first, so their latency overlaps the
  // staging of V (one round trip to memory per step, not two)
  T pv[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int l = sl + q * kSubSlices;
    pv[q] = (row < m && l < kb) ? Pn[(size_t)l * lda + row] : mk<T>(0, 0);
  }
  for (int t = tid; t < kb * nrhs; t += blockDim.x) {
    const int c = t / kb, l = t - c * kb;
    sV[c * kb + l] = V[(size_t)c * ldv + l];
  }
  __syncthreads();
  T acc[kSmallRhs];
#pragma unroll
  for (int c = 0; c < kSmallRhs; ++c) acc[c] = mk<T>(0, 0);
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int l = sl + q * kSubSlices;
    if (l < kb) {
#pragma unroll
      for (int c = 0; c < kSmallRhs; ++c)
        if (c < nrhs) acc[c] = fma_c(acc[c], pv[q], sV[c * kb + l]);
    }
  }
#pragma unroll
  for (int c = 0; c < kSmallRhs; ++c)
    if (c < nrhs) sP[(sl * kSmallRhs + c) * kSubRows + r] = acc[c];
  __syncthreads();
  for (int t = tid; t < kSubRows * nrhs; t += blockDim.x) {
    const int c = t / kSubRows, rr = t - c * kSubRows, rw = blockIdx.x * kSubRows + rr;
    if (rw >= m) continue;
    T s = sP[c * kSubRows + rr];
#pragma unroll
    for (int q = 1; q < kSubSlices; ++q) {
      const T v = sP[(q * kSmallRhs + c) * kSubRows + rr];
      s = mk<T>(s.x + v.x, s.y + v.y);
    }
    if (rw < msub) {
      T *d = Bsub + (size_t)c * ldb + rw;
      *d = sub(*d, s);
    } else {
      const int i = rw - msub;
      Xout[(size_t)c * ldx + i] = sub(sV[c * kb + i], s);
    }
  }
}

// lu_solve for nrhs <= kSmallRhs: one launch per block and sweep.  The
// forward sweep works in place in B; the backward sweep updates the rows
// above each block in B and writes the block's solution to X (N x nrhs, ld
// ldb; X must not overlap B).
template <typename T>
int lu_solve_small(int N, int nb, const T *A, size_t lda, T *B, size_t ldb, int nrhs, T *X, cudaStream_t st) {
  const int nblk = (N + nb - 1) / nb;
  for (int blk = 0; blk < nblk; ++blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb, m2 = N - k - kb;
    if (m2 <= 0) continue;
    panel_apply_kernel<T><<<(m2 + kSubRows - 1) / kSubRows, 256, 0, st>>>(A + (size_t)k * lda + k + kb, lda, m2, 0,
                                                                          kb, B + k, ldb, B + k + kb, ldb, nullptr,
                                                                          0, nrhs);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  }
  for (int blk = nblk - 1; blk >= 0; --blk) {
    const int k = blk * nb, kb = (N - k < nb) ? N - k : nb;
    panel_apply_kernel<T><<<(k + kb + kSubRows - 1) / kSubRows, 256, 0, st>>>(A + (size_t)k * lda, lda, k, kb, kb,
                                                                               B + k, ldb, B, ldb, X + k, ldb, nrhs);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  }
  return QPMS_SUCCESS;
}

// ---------------- the same sweeps in one launch each ----------------
// The two substitutions of lu_solve_small as one launch per sweep, over tiles
// of kSweepRows rows, one warp per tile (nb a multiple of kSweepRows, at most
// 128):
//   forward, tile rows r of block j:  b_r <- b_r - sum_{k<j} P_k(r, :) b_k
//   backward:                          b_r <- b_r - sum_{k>j} Q_k(r, :) b_k,
// then a third launch writes every block's solution x_j = b_j - (I - D_j^-1)
// b_j (no dependencies left).  b_k is final once every tile of block k has
// written its rows (per-block completion counters, released after a fence,
// read with acquire loads; b_k itself is read through L2).  A tile keeps its
// sums over all k in registers and writes its rows once; the panel entries of
// step k + 1 are requested before step k's wait.
// Tiles are handed out in dependency order by an atomic ticket (ascending
// rows forward, descending backward): a tile only waits for tiles with earlier
// tickets, which warps already running hold, so the waits end whatever number
// of CTAs is resident (the argument of single-pass decoupled look-back scans).
// Blocks also finish in sweep order (block k's tiles wait for block k - 1
// forward, k + 1 backward), so a warp that has seen block k final knows the
// earlier ones are.  Every wait is bounded (kSweepWaitNs); a wait that runs
// out sets the error word, which makes the other warps leave too.  Warps are
// independent (no CTA barrier), and a CTA of 4 warps at about 100 registers
// fits on an SM beside a tensor-core GEMM CTA.
// Sync words of one pair of sweeps (sweep_words): [0] error, [1] forward
// ticket, [2] backward ticket, [3, 3 + nblk) forward block counters,
// [3 + nblk, 3 + 2 nblk) backward block counters.
// Lane 8 r + s of a warp handles row r of the tile and the columns
// l = s + 8 q of each block: the eight partial sums of a row sit in eight
// adjacent lanes and meet by shuffles; a column's four rows are one 32-byte
// sector (complex64).
constexpr int kSweepRows = 4, kSweepThreads = 128;
// complex64: at most 102 registers, so that a sweep CTA fits on an SM beside a
// tensor-core GEMM CTA (320 threads x 160 registers)
template <typename T>
struct SweepMinCtas {
  static constexpr int v = sizeof(T) == 8 ? 5 : 2;
};
constexpr unsigned long long kSweepWaitNs = 2000000000ull;  // 2 s
size_t sweep_words(int nblk) { return 3 + 2 * (size_t)nblk; }

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long sweep_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait until *cnt >= need; false if the error word is set or the wait ran out
// (which sets it).
__device__ bool sweep_wait(const unsigned *cnt, unsigned need, unsigned *err) {
  if (ld_acquire(cnt) >= need) return true;
  const unsigned long long t0 = sweep_clock();
  for (;;) {
    __nanosleep(32);
    if (ld_acquire(cnt) >= need) return true;
    if (ld_acquire(err)) return false;
    if (sweep_clock() - t0 > kSweepWaitNs) {
      atomicExch(err, 1u);
      return false;
    }
  }
}
// lane 0 waits, the warp follows (the barrier orders the other lanes' loads
// after lane 0's acquire)
__device__ __forceinline__ bool warp_wait(const unsigned *cnt, unsigned need, unsigned *err, int lane) {
  int ok = 1;
  if (lane == 0) ok = sweep_wait(cnt, need, err) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}
// lane 0 looks once (no wait): is *cnt >= need?
__device__ __forceinline__ bool warp_peek(const unsigned *cnt, unsigned need, int lane) {
  int ok = 0;
  if (lane == 0) ok = ld_acquire(cnt) >= need ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}
__device__ __forceinline__ int warp_ticket(unsigned *ticket, int lane) {
  int t = 0;
  if (lane == 0) t = (int)atomicAdd(ticket, 1u);
  return __shfl_sync(0xffffffffu, t, 0);
}

// the 16 entries l = sl + 8 q < kb of one row of a block column (col0: its
// first column at that row)
template <typename T>
__device__ __forceinline__ void sweep_load(const T *col0, size_t lda, int kb, bool rowok, int sl, T (&pv)[16]) {
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int l = sl + 8 * q;
    pv[q] = (rowok && l < kb) ? col0[(size_t)l * lda] : mk<T>(0, 0);
  }
}
// acc[c] += sum_l pv[l] b_k(l, c), b_k (kb x nrhs from Bk) read through L2
template <typename T>
__device__ __forceinline__ void sweep_fma(const T (&pv)[16], const T *Bk, size_t ldb, int kb, int nrhs, int sl,
                                          T (&acc)[kSmallRhs]) {
#pragma unroll
  for (int c = 0; c < kSmallRhs; ++c)
    if (c < nrhs) {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int l = sl + 8 * q;
        if (l < kb) acc[c] = fma_c(acc[c], pv[q], __ldcg(Bk + (size_t)c * ldb + l));
      }
    }
}
// sums over the eight lanes of a row (every lane gets the total)
template <typename T>
__device__ __forceinline__ void sweep_reduce(T (&acc)[kSmallRhs], int nrhs) {
#pragma unroll
  for (int c = 0; c < kSmallRhs; ++c)
    if (c < nrhs) {
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        acc[c].x += __shfl_xor_sync(0xffffffffu, acc[c].x, o);
        acc[c].y += __shfl_xor_sync(0xffffffffu, acc[c].y, o);
      }
    }
}
// the tile's rows: b_r <- b_r - acc, then the tile is counted in its block
template <typename T>
__device__ __forceinline__ void sweep_finish(T *B, size_t ldb, int row, bool rowok, int sl, int nrhs,
                                             const T (&acc)[kSmallRhs], unsigned *cnt, int lane) {
  if (sl == 0 && rowok) {
#pragma unroll
    for (int c = 0; c < kSmallRhs; ++c)
      if (c < nrhs) {
        T *d = B + (size_t)c * ldb + row;
        *d = sub(__ldcg(d), acc[c]);
      }
    __threadfence();
  }
  __syncwarp();
  if (lane == 0) atomicAdd(cnt, 1u);
}

template <typename T>
__global__ void __launch_bounds__(kSweepThreads, SweepMinCtas<T>::v) sweep_fwd_kernel(const T *__restrict__ A, size_t lda, int N, int nb,
                                                                  T *B, size_t ldb, int nrhs, unsigned *sync) {
  const int lane = threadIdx.x & 31, sl = lane & 7, rr = lane >> 3;
  const int ntiles = (N + kSweepRows - 1) / kSweepRows;
  const unsigned need = (unsigned)(nb / kSweepRows);  // tiles of a full block
  unsigned *err = sync, *ticket = sync + 1, *cnt = sync + 3;
  int known = -1;  // blocks 0..known are final
  for (;;) {
    const int t = warp_ticket(ticket, lane);
    if (t >= ntiles) return;
    const int row0 = t * kSweepRows, j = row0 / nb, row = row0 + rr;
    const bool rowok = row < N;
    T acc[kSmallRhs];
#pragma unroll
    for (int c = 0; c < kSmallRhs; ++c) acc[c] = mk<T>(0, 0);
    if (j - 1 > known && warp_peek(cnt + j - 1, need, lane)) known = j - 1;
    T pv[16];
    if (j > 0) sweep_load(A + row, lda, nb, rowok, sl, pv);
    for (int k = 0; k < j; ++k) {  // the blocks above are full: kb = nb
      T pn[16];
      if (k + 1 < j) sweep_load(A + (size_t)(k + 1) * nb * lda + row, lda, nb, rowok, sl, pn);
      if (k > known) {
        if (!warp_wait(cnt + k, need, err, lane)) return;
        known = k;
      }
      sweep_fma(pv, B + (size_t)k * nb, ldb, nb, nrhs, sl, acc);
      if (k + 1 < j) {
#pragma unroll
        for (int q = 0; q < 16; ++q) pv[q] = pn[q];
      }
    }
    sweep_reduce(acc, nrhs);
    sweep_finish(B, ldb, row, rowok, sl, nrhs, acc, cnt + j, lane);
  }
}

template <typename T>
__global__ void __launch_bounds__(kSweepThreads, SweepMinCtas<T>::v) sweep_bwd_kernel(const T *__restrict__ A, size_t lda, int N, int nb,
                                                                  T *B, size_t ldb, int nrhs, unsigned *sync) {
  const int lane = threadIdx.x & 31, sl = lane & 7, rr = lane >> 3;
  const int ntiles = (N + kSweepRows - 1) / kSweepRows, nblk = (N + nb - 1) / nb;
  unsigned *err = sync, *ticket = sync + 2, *cnt = sync + 3 + nblk;
  auto need = [&](int k) { return (unsigned)((min(nb, N - k * nb) + kSweepRows - 1) / kSweepRows); };
  int known = nblk;  // blocks known..nblk-1 are final
  for (;;) {
    const int tk = warp_ticket(ticket, lane);
    if (tk >= ntiles) return;
    const int t = ntiles - 1 - tk, row0 = t * kSweepRows, j = row0 / nb, row = row0 + rr;
    const bool rowok = row < N;
    T acc[kSmallRhs];
#pragma unroll
    for (int c = 0; c < kSmallRhs; ++c) acc[c] = mk<T>(0, 0);
    if (j + 1 < known && j + 1 < nblk && warp_peek(cnt + j + 1, need(j + 1), lane)) known = j + 1;
    T pv[16];
    if (j < nblk - 1) sweep_load(A + (size_t)(nblk - 1) * nb * lda + row, lda, N - (nblk - 1) * nb, rowok, sl, pv);
    for (int k = nblk - 1; k > j; --k) {
      const int k0 = k * nb, kb = min(nb, N - k0);
      T pn[16];
      if (k - 1 > j) sweep_load(A + (size_t)(k0 - nb) * lda + row, lda, nb, rowok, sl, pn);  // block k - 1 is full
      if (k < known) {
        if (!warp_wait(cnt + k, need(k), err, lane)) return;
        known = k;
      }
      sweep_fma(pv, B + k0, ldb, kb, nrhs, sl, acc);
      if (k - 1 > j) {
#pragma unroll
        for (int q = 0; q < 16; ++q) pv[q] = pn[q];
      }
    }
    sweep_reduce(acc, nrhs);
    sweep_finish(B, ldb, row, rowok, sl, nrhs, acc, cnt + j, lane);
  }
}

// x_j = b_j - (I - D_j^-1) b_j for every block, one warp per tile of rows
template <typename T>
__global__ void __launch_bounds__(kSweepThreads) sweep_diag_kernel(const T *__restrict__ A, size_t lda, int N, int nb,
                                                                   const T *B, size_t ldb, T *X, size_t ldx,
                                                                   int nrhs) {
  const int lane = threadIdx.x & 31, sl = lane & 7, rr = lane >> 3;
  const int ntiles = (N + kSweepRows - 1) / kSweepRows;
  const int nwarps = (int)(gridDim.x * blockDim.x) >> 5;
  for (int t = (int)(blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nwarps) {
    const int row0 = t * kSweepRows, j0 = row0 / nb * nb, kbj = min(nb, N - j0), row = row0 + rr;
    const bool rowok = row < N;
    T pv[16], acc[kSmallRhs];
#pragma unroll
    for (int c = 0; c < kSmallRhs; ++c) acc[c] = mk<T>(0, 0);
    sweep_load(A + (size_t)j0 * lda + row, lda, kbj, rowok, sl, pv);
    sweep_fma(pv, B + j0, ldb, kbj, nrhs, sl, acc);
    sweep_reduce(acc, nrhs);
    if (sl == 0 && rowok) {
#pragma unroll
      for (int c = 0; c < kSmallRhs; ++c)
        if (c < nrhs) X[(size_t)c * ldx + row] = sub(B[(size_t)c * ldb + row], acc[c]);
    }
  }
}

// lu_solve_small's result in three launches.  sync: sweep_words(nblk) words
// whose error word is zero; the others are cleared here.
template <typename T>
int lu_solve_sweep(int N, int nb, const T *A, size_t lda, T *B, size_t ldb, int nrhs, T *X, unsigned *sync,
                   cudaStream_t st) {
  if (nb % kSweepRows || nb > 128) return lu_solve_small<T>(N, nb, A, lda, B, ldb, nrhs, X, st);
  const int nblk = (N + nb - 1) / nb, ntiles = (N + kSweepRows - 1) / kSweepRows;
  const int wpc = kSweepThreads / 32, ctas = (ntiles + wpc - 1) / wpc;
  int dev = 0, sms = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  QG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  sms = std::max(sms, 1);
  QG_CUDA_TRY(cudaMemsetAsync(sync + 1, 0, (sweep_words(nblk) - 1) * sizeof(unsigned), st));
  // two CTAs (8 warps) per SM: at 8,192 unknowns 345 us per forward sweep,
  // against 398 us with a warp for every tile (512 CTAs), whose extra waiting
  // warps only add polls of the block counters
  const int grid = std::min(ctas, 2 * sms);
  sweep_fwd_kernel<T><<<grid, kSweepThreads, 0, st>>>(A, lda, N, nb, B, ldb, nrhs, sync);
  QG_CUDA_TRY(cudaGetLastError());
  sweep_bwd_kernel<T><<<grid, kSweepThreads, 0, st>>>(A, lda, N, nb, B, ldb, nrhs, sync);
  QG_CUDA_TRY(cudaGetLastError());
  sweep_diag_kernel<T><<<std::min(ctas, 8 * sms), kSweepThreads, 0, st>>>(A, lda, N, nb, B, ldb, X, ldb, nrhs);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(3);
  return QPMS_SUCCESS;
}

// Environment override of a solver's boolean choice: 1 / 0 when the variable
// holds one of the two words, else -1 (the solver's own setting).
int env_choice(const char *name, const char *yes, const char *no) {
  const char *e = getenv(name);
  if (e && !strcmp(e, yes)) return 1;
  if (e && !strcmp(e, no)) return 0;
  return -1;
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

// Block size of the LU: complex128 factors use 64; complex64 factors use 128
// for large systems (the trailing updates carry the time) and 64 below the
// tuned size kTunedNb64Below (the chain of diagonal-block inversions carries
// it there: an inversion costs nb^3).  QPMS_GB300_LU_NB = 64 / 128 overrides.
int lu_block_size(int N, int mode) {
  if (!mode) return 64;
  const char *ev = getenv("QPMS_GB300_LU_NB");
  if (ev && (!strcmp(ev, "64") || !strcmp(ev, "128"))) return atoi(ev);
  return N < kTunedNb64Below ? 64 : 128;
}

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
  nb = (mode && (nb_pref == 64 || nb_pref == 128)) ? nb_pref : lu_block_size(N, mode);
  const size_t esz = mode ? 8 : 16;
  const size_t NN = (size_t)Np * Np;
  const int nblk = (Np + nb - 1) / nb;
  size_t wsz = std::max<size_t>((size_t)Np * nb, (size_t)nb * std::max(Np, nrhs_max)) * esz;
  // a mixed solver that falls back to complex128 factors uses the same work
  // buffer for nb = 64 complex128 column blocks (N x 64 x 16 bytes)
  if (mode) wsz = std::max<size_t>(wsz, (size_t)std::max(Np, nrhs_max) * 64 * 16);
  if (mode)
    QG_CUDA_TRY(dev_alloc(&A, NN * esz));  // complex64 factors; the FP64 transform is fused into their fill
  else
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
  // sized for 64-wide blocks (the complex128 fallback's), the larger count
  const size_t sweep_bytes = sweep_words((Np + 63) / 64) * sizeof(unsigned);
  QG_CUDA_TRY(dev_alloc(&sweep, sweep_bytes));
  QG_CUDA_TRY(cudaMemsetAsync(sweep, 0, sweep_bytes, ast));
  if (tc_split) {
    // K up to group x nb: the combined update of a group of blocks
    const int kmax = lu_group() * nb;
    QG_CUDA_TRY(dev_alloc(&tc_pa, tc_planes_bytes_a(Np, kmax, 3)));
    QG_CUDA_TRY(dev_alloc(&tc_pb, tc_planes_bytes_b(std::max(Np, nrhs_max), kmax, 3)));
    const char *la = getenv("QPMS_GB300_LOOKAHEAD");
    if (lookahead && !(la && !strcmp(la, "0")) && Np > nb) {
      int lo = 0, hi = 0;
      QG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      QG_CUDA_TRY(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi));
      QG_CUDA_TRY(cudaEventCreateWithFlags(&ev_a, cudaEventDisableTiming));
      QG_CUDA_TRY(cudaEventCreateWithFlags(&ev_d, cudaEventDisableTiming));
    }
  }
  // many right-hand sides on the tensor cores: the factors' digit planes, cut
  // once per factorisation instead of per substitution step (skipped when
  // they do not fit: the steps then cut their panels themselves)
  if (tc_split && nrhs_max > kSmallRhs && fac_planes_wanted()) {
    if (dev_alloc(&fac_planes, tc_planes_bytes_a(Np, Np, 3)) != cudaSuccess) {
      cudaGetLastError();
      fac_planes = nullptr;
    }
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
  // random butterfly diagonals exp(r/10), r ~ U(-1/2, 1/2): [u level1][u level2][v level1][v level2],
  // drawn on the device in allocation order (no host work, no synchronisation)
  rbt_diag_kernel<<<grid1(4 * (size_t)Np), 256, 0, ast>>>(rs, 4 * (size_t)Np, seed);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

size_t DenseSolver::footprint(int N, int nrhs, int mode) {
  // mode 1: sized for 128-wide blocks, the larger of the two block sizes
  const size_t Np = (size_t)(N + 3) / 4 * 4, nb = mode ? 128 : 64, esz = mode ? 8 : 16;
  const size_t nblk = (Np + nb - 1) / nb;
  size_t b = (mode ? Np * Np * esz : Np * Np * 16) + nblk * 2 * nb * nb * esz;
  b += std::max<size_t>(std::max<size_t>(Np * nb, nb * std::max<size_t>(Np, nrhs)) * esz,
                        mode ? std::max<size_t>(Np, nrhs) * 64 * 16 : 0);
  b += Np * nrhs * (8 + 16) + (size_t)N * nrhs * 32 + 16 + 4 * Np * 8 + 2 * kOzakiMinRhs * 8;
  b += sweep_words((int)((Np + 63) / 64)) * sizeof(unsigned);
  if (ozaki_wanted(nrhs)) b += ozaki_matrix_bytes(N) + ozaki_work_bytes(N, nrhs);
  if (mode && tc_digits(nrhs)) b += tc_plane_bytes((int)Np, nrhs, kMaxLuGroup * (int)nb);
  if (mode && tc_digits(nrhs) && nrhs > kSmallRhs && fac_planes_wanted()) b += tc_planes_bytes_a((int)Np, (int)Np, 3);
  return b + 13 * 512;  // allocation rounding
}

bool fac_planes_wanted() {
  static const int v = env_choice("QPMS_GB300_FACTOR_PLANES", "1", "0");
  return v != 0;
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
  if (side) cudaStreamSynchronize(side);  // its last inversion reads buffers freed below
  for (void *p : {(void *)A, (void *)T64, (void *)Dinv, (void *)work, (void *)rhs_lo, (void *)rp, (void *)r64,
                  (void *)y64, (void *)dinfo, (void *)rs, (void *)res_nrm, (void *)sweep, oz_mat, oz_work, tc_pa,
                  tc_pb, fac_planes})
    if (p) {
      if (pool)
        cudaFreeAsync(p, ast);
      else
        cudaFree(p);
    }
  for (Graph *g : {&gf, &gs}) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    *g = Graph();
  }
  if (side) cudaStreamDestroy(side);
  if (ev_a) cudaEventDestroy(ev_a);
  if (ev_d) cudaEventDestroy(ev_d);
  side = nullptr;
  ev_a = ev_d = nullptr;
  A = T64 = Dinv = work = rhs_lo = rp = nullptr;
  r64 = y64 = nullptr;
  dinfo = nullptr;
  rs = nullptr;
  res_nrm = nullptr;
  sweep = nullptr;
  oz_mat = oz_work = nullptr;
  tc_pa = tc_pb = nullptr;
  fac_planes = nullptr;
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

template <class F>
int DenseSolver::run_graph(Graph &g, const unsigned long long (&key)[6], bool capturable, cudaStream_t st, F body) {
  const char *ev = getenv("QPMS_GB300_GRAPHS");
  const bool env_off = ev && !strcmp(ev, "0");
  if (!graphs || env_off || !capturable || st == 0 || kt_on()) return body();
  bool same = g.keyed;
  for (int i = 0; i < 6 && same; ++i) same = g.key[i] == key[i];
  if (same && g.exec) {
    QG_CUDA_TRY(cudaGraphLaunch(g.exec, st));
    g_launches.fetch_add(g.launches);
    g_graph_replays.fetch_add(1);
    ++graph_replays;
    return QPMS_SUCCESS;
  }
  if (!same) {  // first call with these buffers: eager
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    for (int i = 0; i < 6; ++i) g.key[i] = key[i];
    g.keyed = true;
    return body();
  }
  // second call with the same buffers: capture, then launch the graph
  cudaGraph_t graph = nullptr;
  const unsigned long long l0 = g_launches.load();
  QG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int e = body();
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (e || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    g.keyed = false;
    if (e) return e;
    set_error("stream capture failed: %s", cudaGetErrorString(ce));
    return QPMS_ERROR;
  }
  g.launches = g_launches.load() - l0;
  const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    g.exec = nullptr;
    g.keyed = false;
    set_error("graph instantiation failed: %s", cudaGetErrorString(ie));
    return QPMS_ERROR;
  }
  QG_CUDA_TRY(cudaGraphLaunch(g.exec, st));
  return QPMS_SUCCESS;
}

int DenseSolver::factorize(const void *M64, size_t ldm, cudaStream_t st, bool rowmaj) {
  row_major = rowmaj;
  mode = base_mode;
  trail_ct = base_trail;
  tc_split = base_tc;
  nb = (mode && (nb_pref == 64 || nb_pref == 128)) ? nb_pref : lu_block_size(N, mode);
  const unsigned long long key[6] = {(unsigned long long)(uintptr_t)M64, ldm, rowmaj ? 1ull : 0ull,
                                     (unsigned long long)mode, (unsigned long long)tc_split,
                                     use_ozaki ? 1ull : 0ull};
  int e = run_graph(gf, key, mode == 1 && tc_split != 0, st, [&]() -> int {
    int e2;
    if (use_ozaki && (e2 = ozaki_split_matrix(M64, ldm, row_major, N, oz_mat, &oz, st))) return e2;
    return factor_launch(M64, ldm, st);
  });
  if (e) return e;
  return check_info(st);
}

int DenseSolver::factorize_current(const void *M64, size_t ldm, cudaStream_t st) {
  int e;
  if ((e = factor_launch(M64, ldm, st))) return e;
  return check_info(st);
}

int DenseSolver::factor_launch(const void *M64, size_t ldm, cudaStream_t st) {
  const bool rowmaj = row_major;
  const size_t NN = (size_t)Np * Np;
  cublasHandle_t h;
  int e;
  if ((e = blas_handle_get(&h))) return e;
  QG_BLAS_TRY(cublasSetStream(h, st));
  QG_CUDA_TRY(cudaMemsetAsync(dinfo, 0, 4, st));
  if (mode) {
    // complex64 A = W_u^T diag(M, I) W_v in one pass over M
    const unsigned g = (unsigned)((Np / 4 + kRbtT - 1) / kRbtT);
    rbt_convert_kernel<<<dim3(g, g), 256, 0, st>>>((const double2 *)M64, ldm, rowmaj ? 1 : 0, N, Np, rs,
                                                   (float2 *)A);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
    if (tc_split) {
      e = lu_nopiv_tc(Np, nb, (float2 *)A, Np, (float2 *)Dinv, dinfo, tc_split, (__nv_bfloat16 *)tc_pa,
                      (__nv_bfloat16 *)tc_pb, st, side, ev_a, ev_d, lu_group());
      // the substitutions' panels as 3-digit planes, cut once per factorisation
      if (!e && fac_planes) e = tc_split_a((const float2 *)A, Np, Np, Np, 3, (__nv_bfloat16 *)fac_planes, st);
    } else {
      e = lu_nopiv<float2>(h, Np, nb, (float2 *)A, Np, (float2 *)Dinv, (float2 *)work, dinfo,
                           (cublasComputeType_t)trail_ct, st);
    }
    return e;
  }
  // complex128: T64 = W_u^T diag(M, I) W_v   (M W = column pass with level 2 first: M L2 L1)
  if (!T64) {  // mixed-mode solvers allocate it at their first fallback to complex128
    QG_CUDA_TRY(dev_alloc(&T64, NN * 16));
    if (pool) QG_CUDA_TRY(cudaStreamSynchronize(ast));  // allocated in ast's order, used in st's
  }
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
  return lu_nopiv<double2>(h, Np, nb, (double2 *)T64, Np, (double2 *)Dinv, (double2 *)work, dinfo,
                           CUBLAS_COMPUTE_64F, st);
}

bool DenseSolver::use_sweeps() const {
  static const int v = env_choice("QPMS_GB300_SUBST", "sweep", "steps");
  return v < 0 ? sweeps : v == 1;
}
int DenseSolver::lu_group() const {
  static const int v = [] {
    const char *e = getenv("QPMS_GB300_LU_GROUP");
    const int g = e ? atoi(e) : 0;
    return g >= 1 && g <= kMaxLuGroup ? g : 0;
  }();
  return v ? v : std::max(1, std::min(group, kMaxLuGroup));
}

int DenseSolver::check_info(cudaStream_t st) {
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
  const unsigned long long key[6] = {(unsigned long long)(uintptr_t)R, ldr, (unsigned long long)(uintptr_t)Y, ldy,
                                     (unsigned long long)nrhs,
                                     (unsigned long long)mode | ((unsigned long long)tc_split << 8)};
  const bool capturable = mode == 1 && (nrhs <= kSmallRhs || tc_split != 0);
  return run_graph(gs, key, capturable, st, [&]() { return apply_launch(R, ldr, Y, ldy, nrhs, st); });
}

int DenseSolver::apply_launch(const void *R, size_t ldr, void *Y, size_t ldy, int nrhs, cudaStream_t st) {
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
    const float2 *sol = (const float2 *)rhs_lo;
    if (nrhs <= kSmallRhs) {
      e = !use_sweeps() ? lu_solve_small<float2>(Np, nb, (const float2 *)A, Np, (float2 *)rhs_lo, Np, nrhs,
                                                 (float2 *)work, st)
                        : lu_solve_sweep<float2>(Np, nb, (const float2 *)A, Np, (float2 *)rhs_lo, Np, nrhs,
                                                 (float2 *)work, sweep, st);
      sol = (const float2 *)work;
    } else if (tc_split) {
      e = lu_solve_tc(Np, nb, (const float2 *)A, Np, (float2 *)rhs_lo, Np, nrhs, 3, (__nv_bfloat16 *)tc_pa,
                      (__nv_bfloat16 *)tc_pb, (const __nv_bfloat16 *)fac_planes, st);
    } else {
      e = lu_solve<float2>(h, Np, nb, (const float2 *)A, Np, (float2 *)rhs_lo, Np, nrhs, (float2 *)work,
                           CUBLAS_COMPUTE_32F, st);
    }
    if (e) return e;
    f2d_add_kernel<<<grid1(n), 256, 0, st>>>(n, sol, (double2 *)rp, 1);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  } else {
    if (nrhs <= kSmallRhs) {
      e = !use_sweeps() ? lu_solve_small<double2>(Np, nb, (const double2 *)T64, Np, (double2 *)rp, Np, nrhs,
                                                  (double2 *)work, st)
                        : lu_solve_sweep<double2>(Np, nb, (const double2 *)T64, Np, (double2 *)rp, Np, nrhs,
                                                  (double2 *)work, sweep, st);
      if (!e)
        QG_CUDA_TRY(cudaMemcpyAsync(rp, work, n * 16, cudaMemcpyDeviceToDevice, st));
    } else {
      e = lu_solve<double2>(h, Np, nb, (const double2 *)T64, Np, (double2 *)rp, Np, nrhs, (double2 *)work,
                            CUBLAS_COMPUTE_64F, st);
    }
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
    unsigned sweep_err = 0;
    if (nrhs <= kSmallRhs) QG_CUDA_TRY(cudaMemcpyAsync(&sweep_err, sweep, 4, cudaMemcpyDeviceToHost, st));
    QG_CUDA_TRY(cudaStreamSynchronize(st));
    g_launches.fetch_add(1);
    if (sweep_err) {
      QG_CUDA_TRY(cudaMemsetAsync(sweep, 0, 4, st));
      set_error("dense solver: a substitution sweep waited more than 2 s for a block");
      return QPMS_ERROR;
    }
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
