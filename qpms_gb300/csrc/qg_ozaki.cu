// FP64-accurate residual R = B - M X on the bf16 tensor cores (error-free
// splitting after Ozaki, Ogita, Oishi and Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012) 95-118).
//
// GB300 runs FP64 at about 1.2 TFLOP/s (DMMA) but bf16 at about 2 PFLOP/s.
// The refinement residual of the dense solver is a complex128 GEMM of the
// N x N matrix with the N x nrhs iterate: at N = 14400, nrhs = 64 it is
// about 1e11 FP64 flops, 0.1 s per application on the FP64 pipe.  Here the
// real matrix [Re M; Im M] (2N x N) is cut row by row into p digits of s bits
// (integers, exact in bf16), the iterate [Re X, Im X] (N x 2 nrhs) column by
// column likewise, and every product of digits D_i E_j is formed by a bf16
// GEMM with FP32 accumulation.  s is chosen so that every partial sum is an
// integer below 2^24 (ozaki_digits): the GEMMs are exact whatever their
// summation order or split-K.  The products with i + j <= p - 1 are summed in
// FP64, scaled back by the powers of two of the rows and columns; the result
// carries the normwise error of an FP64 GEMM (55 bits of digits).
//
// One GEMM per row digit i multiplies D_i with the concatenation
// [E_0 | ... | E_{p-1-i}] (the column digits are stored contiguously, so
// that concatenation is a prefix): p GEMMs of 2N x 2 nrhs (p - i) x N, on the
// library's tcgen05 GEMM (qg_tcgemm.cu).  Both digit sets are stored K-major
// (rows of M, columns of X contiguous) with the row length padded to a
// multiple of 8 (N8), the alignment the tensor-memory-access loads need.
#include <cuda_bf16.h>
#include <math.h>

#include "qg_internal.h"
#include "qg_ozaki.h"
#include "qg_tcgemm.h"

namespace qg {

namespace {

size_t al256(size_t b) { return (b + 255) / 256 * 256; }
unsigned grid1(size_t n) { return (unsigned)((n + 255) / 256); }

__device__ __forceinline__ void umax(unsigned long long *a, double v) {
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// max |Re|, |Im| per row of a row-major M: one block per row.
__global__ void rowmax_rowmajor_kernel(const double2 *__restrict__ M, size_t ldm, int N,
                                       unsigned long long *rowmax) {
  const int r = blockIdx.x;
  double mr = 0, mi = 0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const double2 v = M[(size_t)r * ldm + k];
    mr = fmax(mr, fabs(v.x));
    mi = fmax(mi, fabs(v.y));
  }
  for (int o = 16; o; o >>= 1) {
    mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    mi = fmax(mi, __shfl_xor_sync(0xffffffffu, mi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    umax(rowmax + r, mr);
    umax(rowmax + N + r, mi);
  }
}

// The same for a column-major M: a thread per row, columns split over grid.y.
__global__ void rowmax_colmajor_kernel(const double2 *__restrict__ M, size_t ldm, int N, int kchunk,
                                       unsigned long long *rowmax) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  const int k0 = blockIdx.y * kchunk, k1 = min(N, k0 + kchunk);
  double mr = 0, mi = 0;
  for (int k = k0; k < k1; ++k) {
    const double2 v = M[(size_t)k * ldm + r];
    mr = fmax(mr, fabs(v.x));
    mi = fmax(mi, fabs(v.y));
  }
  umax(rowmax + r, mr);
  umax(rowmax + N + r, mi);
}

// sigma = 2^e with max / sigma in [1/2, 1) (1 for a zero row).
__global__ void scale_kernel(const unsigned long long *rowmax, int n, double *scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double m = __longlong_as_double((long long)rowmax[i]);
  int e = 0;
  if (m > 0) frexp(m, &e);
  scale[i] = ldexp(1.0, e);
}

// p digits of x = v / 2^e, |x| < 1, in integer arithmetic (GB300's FP64 rate
// is 1/64 of its FP32 rate, and this runs over every entry of M): the 64-bit
// fixed-point integer X = round(x 2^(s p)) (round half to even, exact from the
// double's mantissa and exponent) is cut into base-2^s digits from the least
// significant one, each balanced into [-2^(s-1), 2^(s-1)); the carry left over
// goes to the leading digit, |d_0| <= 2^s.  x = sum_i d_i 2^(-s (i+1)) up to
// the rounding of X, 2^(-s p - 1) <= 2^-56.  Every digit is an integer of at
// most 9 bits (s <= 8), exact in bf16.
__device__ __forceinline__ long long fixed_point(double v, int shift) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7ff);
  if (ex == 0) return 0;  // zero or subnormal: below 2^-1022, nothing at these shifts
  const unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);  // v = mant 2^(ex - 1075)
  const int e = ex - 1075 + shift;
  unsigned long long q;
  if (e >= 0) {
    q = e < 10 ? mant << e : 0;  // |x| < 1 keeps |X| < 2^(s p) <= 2^62: e <= 9
  } else if (e < -53) {
    q = 0;  // below 1/2
  } else {
    const int sh = -e;
    q = mant >> sh;
    const unsigned long long rem = mant & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) ++q;
  }
  return (bits >> 63) ? -(long long)q : (long long)q;
}

template <typename Store>
__device__ __forceinline__ void digits(double v, int e, int s, int p, Store st) {
  long long X = fixed_point(v, s * p - e);
  const long long mask = (1ll << s) - 1, halfd = 1ll << (s - 1);
  for (int i = p - 1; i >= 1; --i) {
    long long d = X & mask;
    if (d >= halfd) d -= (1ll << s);
    X = (X - d) >> s;
    st(i, __int2bfloat16_rn((int)d));
  }
  st(0, __int2bfloat16_rn((int)X));
}

// exponent e of a power of two 2^e (the row and column scales)
__device__ __forceinline__ int pow2_exp(double x) {
  return (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}

// Slices of [Re M; Im M]; element (R, k) of digit i at sl[i 2N N8 + R N8 + k]
// (rows of M contiguous, K-major for the GEMM), from M row-major or column-major.
__global__ void split_matrix_kernel(const double2 *__restrict__ M, size_t ldm, int N, size_t N8, bool row_major,
                                    const double *__restrict__ scale, int s, int p, __nv_bfloat16 *sl) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t NN = (size_t)N * N;
  if (idx >= NN) return;
  int r, k;
  if (row_major) {
    r = (int)(idx / N);
    k = (int)(idx % N);
  } else {
    k = (int)(idx / N);
    r = (int)(idx % N);
  }
  const double2 v = row_major ? M[(size_t)r * ldm + k] : M[(size_t)k * ldm + r];
  const size_t slab = 2 * (size_t)N * N8;
  const size_t oR = (size_t)r * N8 + k;
  const size_t oI = (size_t)(N + r) * N8 + k;
  digits(v.x, pow2_exp(scale[r]), s, p, [&](int i, __nv_bfloat16 d) { sl[i * slab + oR] = d; });
  digits(v.y, pow2_exp(scale[N + r]), s, p, [&](int i, __nv_bfloat16 d) { sl[i * slab + oI] = d; });
}

// The same for a row-major M, four consecutive columns k per thread: each
// digit plane then takes one 8-byte store per thread for Re and one for Im
// instead of four 2-byte ones (the narrow stores throttled the load/store
// unit).  Columns N..N8-1 of the planes receive zeros.
__device__ __forceinline__ unsigned short next_digit(long long &X, int s, bool last) {
  long long d;
  if (last) {
    d = X;
  } else {
    d = X & ((1ll << s) - 1);
    if (d >= (1ll << (s - 1))) d -= (1ll << s);
    X = (X - d) >> s;
  }
  return __bfloat16_as_ushort(__int2bfloat16_rn((int)d));
}

__global__ void split_matrix_rows4_kernel(const double2 *__restrict__ M, size_t ldm, int N, size_t N8,
                                          const double *__restrict__ scale, int s, int p, __nv_bfloat16 *sl) {
  const size_t q = N8 / 4;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)N * q) return;
  const int r = (int)(idx / q), k0 = 4 * (int)(idx % q);
  const int er = pow2_exp(scale[r]), ei = pow2_exp(scale[N + r]);
  long long XR[4], XI[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int k = k0 + j;
    const double2 v = k < N ? M[(size_t)r * ldm + k] : make_double2(0.0, 0.0);
    XR[j] = fixed_point(v.x, s * p - er);
    XI[j] = fixed_point(v.y, s * p - ei);
  }
  const size_t slab = 2 * (size_t)N * N8;
  uint2 *oR = reinterpret_cast<uint2 *>(sl + (size_t)r * N8 + k0);
  uint2 *oI = reinterpret_cast<uint2 *>(sl + (size_t)(N + r) * N8 + k0);
  for (int i = p - 1; i >= 0; --i) {
    unsigned short hr[4], hi[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      hr[j] = next_digit(XR[j], s, i == 0);
      hi[j] = next_digit(XI[j], s, i == 0);
    }
    const size_t o = (size_t)i * slab / 4;  // in uint2 (4 bf16) units
    oR[o] = make_uint2((unsigned)hr[0] | ((unsigned)hr[1] << 16), (unsigned)hr[2] | ((unsigned)hr[3] << 16));
    oI[o] = make_uint2((unsigned)hi[0] | ((unsigned)hi[1] << 16), (unsigned)hi[2] | ((unsigned)hi[3] << 16));
  }
}

// max |entry| per column of [Re X, Im X] (N x 2 nrhs): one block per column.
__global__ void colmax_kernel(const double2 *__restrict__ X, int N, int nrhs, double *tau) {
  const int C = blockIdx.x;
  const int c = C % nrhs;
  const bool im = C >= nrhs;
  double m = 0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const double2 v = X[(size_t)c * N + k];
    m = fmax(m, fabs(im ? v.y : v.x));
  }
  __shared__ double red[32];
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    int e = 0;
    if (m > 0) frexp(m, &e);
    tau[C] = ldexp(1.0, e);
  }
}

// Column digits: element (k, C) of digit j at bsl[(j 2nrhs + C) N8 + k].
__global__ void split_rhs_kernel(const double2 *__restrict__ X, int N, size_t N8, int nrhs,
                                 const double *__restrict__ tau, int s, int p, __nv_bfloat16 *bsl) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)N * nrhs) return;
  const int c = (int)(idx / N), k = (int)(idx % N);
  const double2 v = X[idx];
  const size_t w = (size_t)2 * nrhs * N8;
  digits(v.x, pow2_exp(tau[c]), s, p, [&](int j, __nv_bfloat16 d) { bsl[j * w + (size_t)c * N8 + k] = d; });
  digits(v.y, pow2_exp(tau[nrhs + c]), s, p,
         [&](int j, __nv_bfloat16 d) { bsl[j * w + (size_t)(nrhs + c) * N8 + k] = d; });
}

// Digit products of equal total weight summed exactly: for the products of
// digit i of M with digits j = 0..p-1-i of X (G = D_i [E_0 | ... ], exact
// integers in FP32, |G| < 2^24), H[t][e] (+)= G[j][e] with t = i + j.  A
// weight t gets at most p terms, so |H| < p 2^24 fits int32 exactly.  The
// calls run i = p-1 .. 0, so weight t is first reached at i = t (j = 0),
// which writes instead of adding (no clearing pass).  cnt = 2N x 2nrhs.
__global__ void accumulate_kernel(const float *__restrict__ G, size_t cnt, int i, int p, int *__restrict__ H) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt) return;
  H[(size_t)i * cnt + e] = __float2int_rn(G[e]);
  for (int j = 1; j <= p - 1 - i; ++j) H[(size_t)(i + j) * cnt + e] += __float2int_rn(G[(size_t)j * cnt + e]);
}

// sum_t H[t][e] 2^{-s (t + 2)}, smallest weights first (exact powers of two
// built from their exponent bits)
__device__ __forceinline__ double digit_sum(const int *__restrict__ H, size_t cnt, size_t e, int s, int p) {
  double acc = 0;
  for (int t = p - 1; t >= 0; --t)
    acc = fma((double)H[(size_t)t * cnt + e], __hiloint2double((1023 - s * (t + 2)) << 20, 0), acc);
  return acc;
}

// R = B - M X from H, the digit sums of [Re M; Im M] [Re X, Im X] (unscaled).
__global__ void combine_kernel(const int *__restrict__ H, int s, int p, const double *__restrict__ sigma,
                               const double *__restrict__ tau, int N, int nrhs, const double2 *__restrict__ B,
                               double2 *__restrict__ Rout) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)N * nrhs) return;
  const int c = (int)(idx / N), r = (int)(idx % N);
  const size_t twoN = 2 * (size_t)N, cnt = twoN * 2 * nrhs;
  const double sr = sigma[r], si = sigma[N + r], tr = tau[c], ti = tau[nrhs + c];
  const double pRR = digit_sum(H, cnt, (size_t)c * twoN + r, s, p) * sr * tr;
  const double pII = digit_sum(H, cnt, (size_t)(nrhs + c) * twoN + N + r, s, p) * si * ti;
  const double pRI = digit_sum(H, cnt, (size_t)(nrhs + c) * twoN + r, s, p) * sr * ti;
  const double pIR = digit_sum(H, cnt, (size_t)c * twoN + N + r, s, p) * si * tr;
  const double2 b = B[idx];
  Rout[idx] = make_double2(b.x - (pRR - pII), b.y - (pRI + pIR));
}

}  // namespace

void ozaki_digits(int K, int *s, int *p) {
  int lk = 0;
  while ((1LL << lk) < (long long)K) ++lk;  // ceil(log2 K)
  int ss = (24 - lk) / 2;
  if (ss > 8) ss = 8;  // bf16 holds integers up to 2^8 exactly
  if (ss < 1) ss = 1;
  *s = ss;
  *p = (55 + ss - 1) / ss;
}

size_t n8(int N) { return ((size_t)N + 7) / 8 * 8; }

size_t ozaki_matrix_bytes(int N) {
  int s, p;
  ozaki_digits(N, &s, &p);
  return al256((size_t)p * 2 * N * n8(N) * 2) + 2 * al256((size_t)2 * N * 8);
}

size_t ozaki_work_bytes(int N, int nrhs) {
  int s, p;
  ozaki_digits(N, &s, &p);
  const size_t tn = 2 * (size_t)nrhs;
  return al256((size_t)p * n8(N) * tn * 2) + al256(tn * 8) + 2 * al256((size_t)2 * N * tn * p * 4);
}

int ozaki_split_matrix(const void *M, size_t ldm, bool row_major, int N, void *buf, OzakiMatrix *om,
                       cudaStream_t st) {
  int s, p;
  ozaki_digits(N, &s, &p);
  char *b = (char *)buf;
  om->N = N;
  om->s = s;
  om->p = p;
  om->row_major = row_major;
  om->slices = b;
  om->ld = n8(N);
  b += al256((size_t)p * 2 * N * om->ld * 2);
  om->scale = (double *)b;
  b += al256((size_t)2 * N * 8);
  om->rowmax = (unsigned long long *)b;
  const double2 *Md = (const double2 *)M;
  QG_CUDA_TRY(cudaMemsetAsync(om->rowmax, 0, (size_t)2 * N * 8, st));
  if (row_major) {
    rowmax_rowmajor_kernel<<<N, 256, 0, st>>>(Md, ldm, N, om->rowmax);
  } else {
    const int kchunk = 256;
    rowmax_colmajor_kernel<<<dim3((N + 255) / 256, (N + kchunk - 1) / kchunk), 256, 0, st>>>(Md, ldm, N, kchunk,
                                                                                           om->rowmax);
  }
  QG_CUDA_TRY(cudaGetLastError());
  scale_kernel<<<grid1(2 * (size_t)N), 256, 0, st>>>(om->rowmax, 2 * N, om->scale);
  QG_CUDA_TRY(cudaGetLastError());
  if (row_major)
    split_matrix_rows4_kernel<<<grid1((size_t)N * (om->ld / 4)), 256, 0, st>>>(Md, ldm, N, om->ld, om->scale, s, p,
                                                                              (__nv_bfloat16 *)om->slices);
  else
    split_matrix_kernel<<<grid1((size_t)N * N), 256, 0, st>>>(Md, ldm, N, om->ld, row_major, om->scale, s, p,
                                                              (__nv_bfloat16 *)om->slices);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(3);
  return QPMS_SUCCESS;
}

int ozaki_residual(const OzakiMatrix &om, const void *X, const void *B, void *R, int nrhs, void *work,
                   cudaStream_t st) {
  const int N = om.N, s = om.s, p = om.p, tn = 2 * nrhs, twoN = 2 * N;
  const size_t ld = om.ld;
  char *w = (char *)work;
  __nv_bfloat16 *bsl = (__nv_bfloat16 *)w;
  w += al256((size_t)p * ld * tn * 2);
  double *tau = (double *)w;
  w += al256((size_t)tn * 8);
  float *G = (float *)w;
  w += al256((size_t)twoN * tn * p * 4);
  int *H = (int *)w;  // [p][2N x 2nrhs]
  colmax_kernel<<<tn, 256, 0, st>>>((const double2 *)X, N, nrhs, tau);
  QG_CUDA_TRY(cudaGetLastError());
  split_rhs_kernel<<<grid1((size_t)N * nrhs), 256, 0, st>>>((const double2 *)X, N, ld, nrhs, tau, s, p, bsl);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(2);
  int e;
  for (int i = p - 1; i >= 0; --i) {  // smallest contributions first
    const int n = tn * (p - i);
    const __nv_bfloat16 *Ai = (const __nv_bfloat16 *)om.slices + (size_t)i * twoN * ld;
    if ((e = tc_gemm_bf16(Ai, ld, bsl, ld, twoN, n, N, 1.f, 0.f, nullptr, 0, G, twoN, st))) return e;
    accumulate_kernel<<<grid1((size_t)twoN * tn), 256, 0, st>>>(G, (size_t)twoN * tn, i, p, H);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  }
  combine_kernel<<<grid1((size_t)N * nrhs), 256, 0, st>>>(H, s, p, om.scale, tau, N, nrhs, (const double2 *)B,
                                                          (double2 *)R);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

}  // namespace qg

using namespace qg;

// Test entry: R = B - M X (device complex128; M column-major or row-major
// N x N with leading dimension ldm; X, B, R N x nrhs, leading dimension N)
// through the digit GEMMs.  Allocates its own buffers.
extern "C" int qpms_gpu_ozaki_residual(int N, int nrhs, const qpms_complex_t *M, size_t ldm, int row_major,
                                       const qpms_complex_t *X, const qpms_complex_t *B, qpms_complex_t *R) {
  clear_error();
  if (N <= 0 || nrhs <= 0 || !M || !X || !B || !R || ldm < (size_t)N) {
    set_error("invalid arguments");
    return QPMS_EINVAL;
  }
  int e;
  void *mb = nullptr, *wb = nullptr;
  QG_CUDA_TRY(cudaMalloc(&mb, ozaki_matrix_bytes(N)));
  if (cudaMalloc(&wb, ozaki_work_bytes(N, nrhs)) != cudaSuccess) {
    cudaFree(mb);
    set_error("ozaki workspace: out of memory");
    return QPMS_ERROR;
  }
  OzakiMatrix om;
  e = ozaki_split_matrix(M, ldm, row_major != 0, N, mb, &om, 0);
  if (!e) e = ozaki_residual(om, X, B, R, nrhs, wb, 0);
  cudaError_t se = cudaDeviceSynchronize();
  cudaFree(mb);
  cudaFree(wb);
  if (e) return e;
  QG_CUDA_TRY(se);
  return QPMS_SUCCESS;
}

namespace qg {
namespace {
// dst [m][k] (row stride ld) = src (m x k column-major)
__global__ void bf16_to_kmajor_kernel(int m, int k, const __nv_bfloat16 *__restrict__ src, size_t ld,
                                      __nv_bfloat16 *__restrict__ dst) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)m * k) return;
  const int c = (int)(idx / m), r = (int)(idx % m);
  dst[(size_t)r * ld + c] = src[idx];
}
}  // namespace
}  // namespace qg

// Test entry: C = A B for bf16 A (m x k), B (k x n) column-major, FP32 C,
// through the tensor-core GEMM of the digit products (checks that integer
// products with partial sums below 2^24 come out exact).  A is first copied
// K-major (the GEMM's operand layout).
extern "C" int qpms_gpu_bf16_gemm(int m, int n, int k, const void *A, const void *B, float *C) {
  clear_error();
  if (m <= 0 || n <= 0 || k <= 0 || !A || !B || !C) {
    set_error("invalid arguments");
    return QPMS_EINVAL;
  }
  const size_t ld = n8(k);
  __nv_bfloat16 *Ak = nullptr, *Bk = nullptr;
  QG_CUDA_TRY(cudaMalloc(&Ak, (size_t)m * ld * 2));
  if (cudaMalloc(&Bk, (size_t)n * ld * 2) != cudaSuccess) {
    cudaFree(Ak);
    set_error("out of device memory");
    return QPMS_ENOMEM;
  }
  bf16_to_kmajor_kernel<<<grid1((size_t)m * k), 256>>>(m, k, (const __nv_bfloat16 *)A, ld, Ak);
  // B (k x n column-major) is K-major already: row stride k, copied to stride ld
  cudaError_t ce = cudaMemcpy2D(Bk, ld * 2, B, (size_t)k * 2, (size_t)k * 2, n, cudaMemcpyDeviceToDevice);
  int e = ce == cudaSuccess ? tc_gemm_bf16(Ak, ld, Bk, ld, m, n, k, 1.f, 0.f, nullptr, 0, C, m, 0) : QPMS_ERROR;
  if (ce != cudaSuccess) set_error("copy failed: %s", cudaGetErrorString(ce));
  cudaError_t se = cudaDeviceSynchronize();
  cudaFree(Ak);
  cudaFree(Bk);
  if (e) return e;
  QG_CUDA_TRY(se);
  return tc_check_error(0);
}
