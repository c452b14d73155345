// Mode-problem assembly and the small-system solve pipeline on sm_103a.
//
// assemble_kernel: for every (frequency w, particle pair R, C) unit of a batch
// it writes the fecv x fecv block M_w[R, C] = delta_RC I - T_R S_w(R <- C)
// straight into the row-major complex128 matrix M_w (the reference's
// qpms_scatsysw_build_modeproblem_matrix_full, scatsystem.c:1283-1343, with
// the finite semantics S(R <- R) = 0).  S comes from the translation tables
// of the calculator: the per-pair factor table w (Hankel+ Bessel, Legendre,
// azimuthal phases) is built in shared memory, every (y, yu) element of A and
// B is one short FP64 dot product, and each A/B value lands in two blocks of
// the 2x2 (electric, magnetic) type structure (translations_inlines.h:213-240).
// Diagonal T (Mie spheres) scales rows; a dense T is applied from shared memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qg_internal.h"
#include "qg_ktimer.h"
#include "qg_specfunc.cuh"
#include "qg_assembly.h"

namespace qg {
namespace {

constexpr int kAThreads = 256;

template <int LMAX>
struct AsmShape {
  static constexpr int L = 2 * LMAX + 1;
  static constexpr int S = (L + 1) * (L + 1);
  static constexpr int NL = (L + 1) * (L + 2) / 2;
  static constexpr int NE = LMAX * (LMAX + 2);
  static constexpr int NE2 = NE * NE;
  static constexpr int NB = 2 * NE;  // block side
  static constexpr int V = LMAX <= 2 ? 16 : (LMAX <= 4 ? 8 : 4);
};

template <int LMAX>
constexpr size_t asm_smem_bytes(bool dense) {
  using Sh = AsmShape<LMAX>;
  return (size_t)Sh::V * Sh::S * 16 + (size_t)Sh::V * (Sh::L + 1) * 16 * 2 + (size_t)Sh::V * Sh::NL * 8 +
         (size_t)Sh::V * 32 + (dense ? (size_t)Sh::NB * Sh::NB * 16 : 0);
}

struct __align__(16) PairInfo {
  double ct;
  int diag;   // R == C: identity block, no translation
  int valid;
  int w, R, C, pad;
};

template <int LMAX, bool DENSE>
__global__ void __launch_bounds__(kAThreads) assemble_kernel(AsmArgs a, TransDevTables T) {
  using Sh = AsmShape<LMAX>;
  constexpr int L = Sh::L, S = Sh::S, NL = Sh::NL, NE = Sh::NE, NE2 = Sh::NE2, NB = Sh::NB, V = Sh::V;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  qg_c *w = reinterpret_cast<qg_c *>(smem_raw);
  qg_c *zb = w + V * S;
  qg_c *eph = zb + V * (L + 1);
  double *leg = reinterpret_cast<double *>(eph + V * (L + 1));
  PairInfo *info = reinterpret_cast<PairInfo *>(leg + V * NL);
  qg_c *sblk = reinterpret_cast<qg_c *>(info + V);  // [NB][NB] if DENSE

  const int tid = threadIdx.x;
  const size_t np = (size_t)a.np, units = (size_t)a.nw * np * np;
  const size_t N = np * NB;
  const size_t nchunks = (units + V - 1) / V;
  for (size_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
    const size_t base = chunk * V;
    if (tid < V) {
      const size_t u = base + tid;
      PairInfo inf;
      inf.valid = u < units;
      inf.diag = 1;
      inf.ct = 1.0;
      inf.w = inf.R = inf.C = 0;
      qg_c z[L + 1];
#pragma unroll
      for (int l = 0; l <= L; ++l) z[l] = cmk(0.0, 0.0);
      if (inf.valid) {
        const int wi = (int)(u / (np * np));
        const size_t pr = u - (size_t)wi * np * np;
        inf.w = wi;
        inf.R = (int)(pr / np);
        inf.C = (int)(pr - (size_t)inf.R * np);
        inf.diag = inf.R == inf.C;
        if (!inf.diag) {
          const double dx = a.pos[3 * inf.R] - a.pos[3 * inf.C];
          const double dy = a.pos[3 * inf.R + 1] - a.pos[3 * inf.C + 1];
          const double dz = a.pos[3 * inf.R + 2] - a.pos[3 * inf.C + 2];
          const double r = sqrt(dx * dx + dy * dy + dz * dz);
          // cart2sph (vectors.h:134-140), then kd.r *= k (translations.c:808-809)
          const double th = r > 0 ? acos(dz / r) : 1.5707963267948966;
          const double ph = atan2(dy, dx);
          const qg_c k = a.k[wi];
          sph_bessel<L>(a.J, cmk(k.re * r, k.im * r), z);
          inf.ct = cos(th);
          double s1, c1;
          sincos(ph, &s1, &c1);
          qg_c e1 = cmk(c1, s1), e = cmk(1.0, 0.0);
#pragma unroll
          for (int d = 0; d <= L; ++d) {
            eph[tid * (L + 1) + d] = e;
            e = cmul(e, e1);
          }
        }
      }
#pragma unroll
      for (int l = 0; l <= L; ++l) zb[tid * (L + 1) + l] = z[l];
      info[tid] = inf;
    }
    __syncthreads();
    for (int t = tid; t < V * (L + 1); t += kAThreads) {
      const int v = t / (L + 1), m = t - v * (L + 1);
      if (!info[v].diag) legendre_column_rt(L, m, info[v].ct, leg + v * NL);
    }
    __syncthreads();
    for (int t = tid; t < V * NL; t += kAThreads) {
      const int v = t / NL, i = t - v * NL;
      if (info[v].diag) continue;
      int p = (int)((sqrtf(8.0f * i + 1.0f) - 1.0f) * 0.5f);
      if ((p + 1) * (p + 2) / 2 <= i) ++p;
      if (p * (p + 1) / 2 > i) --p;
      const int ad = i - p * (p + 1) / 2;
      const qg_c uu = cscale(zb[v * (L + 1) + p], leg[v * NL + i]);
      const qg_c ph = eph[v * (L + 1) + ad];
      qg_c *wv = w + v * S + p * p + p;
      wv[ad] = cmul(uu, ph);
      if (ad) wv[-ad] = cmul(uu, cconj(ph));
    }
    __syncthreads();

    for (int v = 0; v < V; ++v) {
      const PairInfo inf = info[v];
      if (!inf.valid) break;
      qg_c *M = a.M + (size_t)inf.w * N * N;
      const size_t row0 = (size_t)inf.R * NB, col0 = (size_t)inf.C * NB;
      if (inf.diag) {
        for (int t = tid; t < NB * NB; t += kAThreads) {
          const int i = t / NB, j = t - i * NB;
          M[(row0 + i) * N + col0 + j] = cmk(i == j ? 1.0 : 0.0, 0.0);
        }
        continue;
      }
      const qg_c *wv = w + v * S;
      const int tmR = a.tmid[inf.R];
      const qg_c *TR = a.T + ((size_t)inf.w * a.ntm + tmR) * (DENSE ? NB * NB : NB);
      // A and B each in their own term-count order; each value lands in two
      // blocks of the (electric, magnetic) type structure
#pragma unroll 1
      for (int which = 0; which < 2; ++which) {
        const uint8_t *cnt = which ? T.cntB : T.cntA;
        const double *coef = which ? T.coefB : T.coefA;
        const uint16_t *slot = which ? T.slotB : T.slotA;
        const int32_t *perm = which ? T.permB : T.perm;
        for (int k = tid; k < NE2; k += kAThreads) {
          const int c = cnt[k];
          double sr = 0, si = 0;
          for (int q = 0; q < c; ++q) {
            const double cf = __ldg(coef + q * NE2 + k);
            const qg_c x = wv[__ldg(slot + q * NE2 + k)];
            sr = fma(cf, x.re, sr);
            si = fma(cf, x.im, si);
          }
          const qg_c v = which ? cmk(-si, sr) : cmk(sr, si);  // B multipliers are imaginary
          const int e = __ldg(perm + k);
          const int yi = e / NE, yj = e - yi * NE;
          // A: (E <- E) and (M <- M) blocks; B: (E <- M) and (M <- E) blocks
          const int r1 = yi, c1 = which ? NE + yj : yj;
          const int r2 = NE + yi, c2 = which ? yj : NE + yj;
          if (DENSE) {
            sblk[r1 * NB + c1] = v;
            sblk[r2 * NB + c2] = v;
          } else {
            M[(row0 + r1) * N + col0 + c1] = cscale(cmul(TR[r1], v), -1.0);
            M[(row0 + r2) * N + col0 + c2] = cscale(cmul(TR[r2], v), -1.0);
          }
        }
      }
      if (DENSE) {
        __syncthreads();
        for (int t = tid; t < NB * NB; t += kAThreads) {
          const int i = t / NB, j = t - i * NB;
          double sr = 0, si = 0;
          for (int q = 0; q < NB; ++q) {
            const qg_c tq = TR[i * NB + q], sq = sblk[q * NB + j];
            sr = fma(tq.re, sq.re, fma(-tq.im, sq.im, sr));
            si = fma(tq.re, sq.im, fma(tq.im, sq.re, si));
          }
          M[(row0 + i) * N + col0 + j] = cmk(-sr, -si);
        }
        __syncthreads();
      }
    }
    __syncthreads();
  }
}

template <int LMAX>
int launch_asm(const AsmArgs &a, const TransDevTables &T, cudaStream_t st) {
  using Sh = AsmShape<LMAX>;
  int dev = 0, nsm = 0, per_sm = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  QG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t units = (size_t)a.nw * a.np * a.np;
  const size_t nchunks = (units + Sh::V - 1) / Sh::V;
  if (nchunks == 0) return QPMS_SUCCESS;
  const double nrow = (double)a.np * 2 * LMAX * (LMAX + 2);
  KtScope kt(KT_ASSEMBLE, st, 16.0 * a.nw * nrow * nrow);
  if (a.dense) {
    auto k = assemble_kernel<LMAX, true>;
    const size_t smem = asm_smem_bytes<LMAX>(true);
    QG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    QG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kAThreads, smem));
    size_t grid = std::min<size_t>((size_t)nsm * std::max(per_sm, 1), nchunks);
    k<<<(unsigned)grid, kAThreads, smem, st>>>(a, T);
  } else {
    auto k = assemble_kernel<LMAX, false>;
    const size_t smem = asm_smem_bytes<LMAX>(false);
    QG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    QG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kAThreads, smem));
    size_t grid = std::min<size_t>((size_t)nsm * std::max(per_sm, 1), nchunks);
    k<<<(unsigned)grid, kAThreads, smem, st>>>(a, T);
  }
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

// ---------------- small pipeline kernels ----------------

// a[w][p*n + i] = coef[i] * exp(i kvec_w . r_p)
__global__ void incident_kernel(int nw, int np, int n, const qg_c *coef, size_t coef_stride, const double *kvec,
                                const double *pos, qg_c *a) {
  const size_t N = (size_t)np * n, tot = (size_t)nw * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
    const int w = (int)(t / N);
    const size_t r = t - (size_t)w * N;
    const int p = (int)(r / n), i = (int)(r - (size_t)p * n);
    const double ph = kvec[3 * w] * pos[3 * p] + kvec[3 * w + 1] * pos[3 * p + 1] + kvec[3 * w + 2] * pos[3 * p + 2];
    double s, c;
    sincos(ph, &s, &c);
    a[t] = cmul(coef[(size_t)w * coef_stride + i], cmk(c, s));
  }
}

// b[w][p*n + i] = sum_j T_w,tm(p)[i][j] a[w][p*n + j]  (diag: T[i] a[i])
__global__ void apply_t_kernel(int nw, int np, int n, int ntm, int dense, const int *tmid, const qg_c *T,
                               const qg_c *a, qg_c *b) {
  const size_t N = (size_t)np * n, tot = (size_t)nw * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
    const int w = (int)(t / N);
    const size_t r = t - (size_t)w * N;
    const int p = (int)(r / n), i = (int)(r - (size_t)p * n);
    const qg_c *Tp = T + ((size_t)w * ntm + tmid[p]) * (dense ? (size_t)n * n : n);
    if (!dense) {
      b[t] = cmul(Tp[i], a[t]);
    } else {
      const qg_c *ap = a + (size_t)w * N + (size_t)p * n;
      qg_c s = cmk(0, 0);
      for (int j = 0; j < n; ++j) s = cadd(s, cmul(Tp[i * n + j], ap[j]));
      b[t] = s;
    }
  }
}

// r = b - M x for nw row-major N x N systems; one warp per row.  Also
// accumulates ||r||^2 and ||b||^2 per system (atomics on doubles).
__global__ void residual_kernel(int nw, size_t N, const qg_c *M, const qg_c *x, const qg_c *b, qg_c *r,
                                double *rn2, double *bn2) {
  const int lane = threadIdx.x & 31;
  const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t row = warp; row < (size_t)nw * N; row += nwarps) {
    const size_t w = row / N, i = row - w * N;
    const qg_c *Mi = M + w * N * N + i * N;
    const qg_c *xw = x + w * N;
    double sr = 0, si = 0;
    for (size_t j = lane; j < N; j += 32) {
      const qg_c m = Mi[j], xv = xw[j];
      sr = fma(m.re, xv.re, fma(-m.im, xv.im, sr));
      si = fma(m.re, xv.im, fma(m.im, xv.re, si));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
      const qg_c bv = b[row];
      const qg_c rv = cmk(bv.re - sr, bv.im - si);
      r[row] = rv;
      atomicAdd(rn2 + w, cabs2(rv));
      atomicAdd(bn2 + w, cabs2(bv));
    }
  }
}

__global__ void c128_to_c64_kernel(size_t n, const qg_c *src, float2 *dst) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const qg_c v = src[t];
    dst[t] = make_float2((float)v.re, (float)v.im);
  }
}

// x += dx (complex64 correction), optionally x = dx when init
__global__ void add_c64_kernel(size_t n, const float2 *dx, qg_c *x, int init) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const float2 d = dx[t];
    if (init)
      x[t] = cmk(d.x, d.y);
    else
      x[t] = cmk(x[t].re + d.x, x[t].im + d.y);
  }
}

// sigma_w = -Re(a_w^H f_w) / Re(k_w)^2 ; one block per system
__global__ void sigma_ext_kernel(int nw, size_t N, const qg_c *a, const qg_c *f, const qg_c *k, double *sig) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  if (w >= nw) return;
  double s = 0;
  for (size_t i = threadIdx.x; i < N; i += blockDim.x) {
    const qg_c av = a[(size_t)w * N + i], fv = f[(size_t)w * N + i];
    s += av.re * fv.re + av.im * fv.im;  // Re(conj(a) f)
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = (threadIdx.x < blockDim.x / 32) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) {
      const double kr = k[w].re;
      sig[w] = -s / (kr * kr);
    }
  }
}

// out-of-place transpose of nb square n x n complex128 matrices
__global__ void transpose_kernel(size_t n, int nb, const qg_c *src, qg_c *dst) {
  __shared__ qg_c tile[32][33];
  const int b = blockIdx.z;
  const size_t bx = blockIdx.x * 32, by = blockIdx.y * 32;
  const qg_c *s = src + (size_t)b * n * n;
  qg_c *d = dst + (size_t)b * n * n;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const size_t r = by + j, c = bx + threadIdx.x;
    if (r < n && c < n) tile[j][threadIdx.x] = s[r * n + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const size_t r = bx + j, c = by + threadIdx.x;
    if (r < n && c < n) d[r * n + c] = tile[threadIdx.x][j];
  }
}

unsigned grid_for(size_t n, int threads) {
  size_t g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  if (g == 0) g = 1;
  return (unsigned)g;
}

}  // namespace

int launch_assemble(const AsmArgs &a, const TransDevTables &T, cudaStream_t st) {
  switch (T.lMax) {
#define QG_CASE(LM) \
  case LM: return launch_asm<LM>(a, T, st);
    QG_CASE(1) QG_CASE(2) QG_CASE(3) QG_CASE(4) QG_CASE(5) QG_CASE(6)
#undef QG_CASE
    default: set_error("assembly kernel: lMax %d not compiled (1..6)", T.lMax); return QPMS_EINVAL;
  }
}

int launch_incident(int nw, int np, int n, const qg_c *coef, const double *kvec, const double *pos, qg_c *a,
                    cudaStream_t st, size_t coef_stride) {
  incident_kernel<<<grid_for((size_t)nw * np * n, 256), 256, 0, st>>>(nw, np, n, coef, coef_stride, kvec, pos, a);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int launch_apply_t(int nw, int np, int n, int ntm, int dense, const int *tmid, const qg_c *T, const qg_c *a,
                   qg_c *b, cudaStream_t st) {
  apply_t_kernel<<<grid_for((size_t)nw * np * n, 256), 256, 0, st>>>(nw, np, n, ntm, dense, tmid, T, a, b);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int launch_residual(int nw, size_t N, const qg_c *M, const qg_c *x, const qg_c *b, qg_c *r, double *rn2,
                    double *bn2, cudaStream_t st) {
  QG_CUDA_TRY(cudaMemsetAsync(rn2, 0, sizeof(double) * nw, st));
  QG_CUDA_TRY(cudaMemsetAsync(bn2, 0, sizeof(double) * nw, st));
  residual_kernel<<<grid_for((size_t)nw * N * 32, 256), 256, 0, st>>>(nw, N, M, x, b, r, rn2, bn2);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int launch_c128_to_c64(size_t n, const qg_c *src, void *dst, cudaStream_t st) {
  c128_to_c64_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, src, (float2 *)dst);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int launch_add_c64(size_t n, const void *dx, qg_c *x, int init, cudaStream_t st) {
  add_c64_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, (const float2 *)dx, x, init);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int launch_sigma_ext(int nw, size_t N, const qg_c *a, const qg_c *f, const qg_c *k, double *sig, cudaStream_t st) {
  sigma_ext_kernel<<<nw, 256, 0, st>>>(nw, N, a, f, k, sig);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int launch_transpose(size_t n, int nb, const qg_c *src, qg_c *dst, cudaStream_t st) {
  dim3 grid((unsigned)((n + 31) / 32), (unsigned)((n + 31) / 32), (unsigned)nb), block(32, 8);
  transpose_kernel<<<grid, block, 0, st>>>(n, nb, src, dst);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

}  // namespace qg
