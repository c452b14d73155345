// Batched VSWF translation coefficients A, B on sm_103a.
//
// Computes, for every translation i of a batch, the reference's
// qpms_trans_calculator_get_AB_arrays (qpms/translations.c:610-698):
//   A[y,yu] = e^{i d phi} sum_q a_q P_p^{|d|}(cos th) z_p(kr),      p = n+nu-2q
//   B[y,yu] = e^{i d phi} sum_q b_q P_{p+1}^{|d|}(cos th) z_{p+1}(kr)
// with d = mu - m.  The per-translation factor table
//   w[p^2+p+d] = P_p^{|d|}(cos th) z_p(kr) e^{i d phi},  0 <= p <= 2 lMax + 1,
// is built once per translation in shared memory; every output element is
// then a short real-coefficient dot product over w (A multipliers are real,
// B multipliers purely imaginary), i.e. two FP64 FMAs per term.
//
// Work layout: a persistent CTA of 256 threads owns a chunk of V
// translations.  Phase 1 (setup): one thread per translation runs the Bessel
// recurrence, one thread per (translation, m) a Legendre column, all threads
// fill w.  Phase 2 (contraction): threads walk the elements in term-count
// order (uniform trip counts per warp) and write each output row (one A or B
// matrix, nelem^2 complex128, contiguous in HBM) to a shared-memory stage;
// one elected thread then writes the row to HBM with a TMA bulk copy
// (cp.async.bulk.global.shared::cta), double-buffered so the copy overlaps
// the next row's arithmetic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qg_internal.h"
#include "qg_specfunc.cuh"

namespace qg {
namespace {

constexpr int kThreads = 256;
// Output-row stage buffers: 2 overlaps the TMA store of one row with the next
// row's arithmetic; 1 frees shared memory for the L1 that caches the
// multiplier tables.
#ifndef QG_TRANS_STAGES
#define QG_TRANS_STAGES 2
#endif
constexpr int kStages = QG_TRANS_STAGES;

template <int LMAX>
struct TransShape {
  static constexpr int L = 2 * LMAX + 1;            // highest Bessel / Legendre order
  static constexpr int S = (L + 1) * (L + 1);       // w-table slots
  static constexpr int NL = (L + 1) * (L + 2) / 2;  // Legendre entries
  static constexpr int NE = LMAX * (LMAX + 2);
  static constexpr int NE2 = NE * NE;
  // translations per chunk: keep the w tables ~25-40 KB
  static constexpr int V = LMAX <= 3 ? 32 : (LMAX <= 5 ? 16 : (LMAX <= 7 ? 8 : 4));
  static constexpr bool kStaged = (kStages * NE2 * 16 + V * (S * 16 + 2 * (L + 1) * 16 + NL * 8 + 16)) <= 200 * 1024;
};

struct __align__(16) VecInfo {
  double ct;
  int nan_out;
  int valid;
};

template <int LMAX>
constexpr size_t trans_smem_bytes(bool staged) {
  using Sh = TransShape<LMAX>;
  return (size_t)Sh::V * Sh::S * 16 + (size_t)Sh::V * (Sh::L + 1) * 16 * 2 + (size_t)Sh::V * Sh::NL * 8 +
         (size_t)Sh::V * sizeof(VecInfo) + (staged ? (size_t)kStages * Sh::NE2 * 16 : 0);
}

__device__ __forceinline__ void bulk_store_row(void *gdst, const void *ssrc, uint32_t bytes) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(ssrc);
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(gdst), "r"(s), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read_le0() {
  asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read_le1() {
  asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

template <int LMAX, bool STAGED>
__global__ void __launch_bounds__(kThreads) trans_ab_kernel(TransDevTables T, size_t n, const qg_c *__restrict__ kr,
                                                            const double *__restrict__ theta,
                                                            const double *__restrict__ phi,
                                                            const unsigned char *__restrict__ r_ge_d, int J,
                                                            qg_c *__restrict__ A, qg_c *__restrict__ B) {
  using Sh = TransShape<LMAX>;
  constexpr int L = Sh::L, S = Sh::S, NL = Sh::NL, NE2 = Sh::NE2, V = Sh::V;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  qg_c *w = reinterpret_cast<qg_c *>(smem_raw);  // [V][S]
  qg_c *zb = w + V * S;                           // [V][L+1]
  qg_c *eph = zb + V * (L + 1);                   // [V][L+1]
  double *leg = reinterpret_cast<double *>(eph + V * (L + 1));  // [V][NL]
  VecInfo *info = reinterpret_cast<VecInfo *>(leg + V * NL);    // [V]
  qg_c *stage = reinterpret_cast<qg_c *>(info + V);             // [kStages][NE2] if STAGED

  const int tid = threadIdx.x;
  const size_t nchunks = (n + V - 1) / V;
  int row_counter = 0;  // rows issued by this CTA (selects the stage buffer)

  for (size_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
    const size_t base = chunk * V;
    // ---------------- phase 1: per-translation factors ----------------
    if (tid < V) {
      const size_t i = base + tid;
      VecInfo inf;
      inf.valid = (i < n);
      inf.nan_out = 0;
      inf.ct = 1.0;
      qg_c z[L + 1];
      if (inf.valid) {
        const qg_c x = kr[i];
        const double th = theta[i], ph = phi[i];
        const int Jeff = (r_ge_d && r_ge_d[i]) ? 1 : J;
        if (x.re == 0.0 && x.im == 0.0 && Jeff != 1) inf.nan_out = 1;  // translations.c:641-649
        sph_bessel<L>(Jeff, x, z);
        inf.ct = cos(th);
        double s1, c1;
        sincos(ph, &s1, &c1);
        qg_c e1 = cmk(c1, s1), e = cmk(1.0, 0.0);
#pragma unroll
        for (int d = 0; d <= L; ++d) {
          eph[tid * (L + 1) + d] = e;
          e = cmul(e, e1);
        }
      } else {
#pragma unroll
        for (int l = 0; l <= L; ++l) z[l] = cmk(0.0, 0.0);
      }
#pragma unroll
      for (int l = 0; l <= L; ++l) zb[tid * (L + 1) + l] = z[l];
      info[tid] = inf;
    }
    __syncthreads();
    for (int t = tid; t < V * (L + 1); t += kThreads) {
      const int v = t / (L + 1), m = t - v * (L + 1);
      legendre_column_rt(L, m, info[v].ct, leg + v * NL);
    }
    __syncthreads();
    // w[p^2+p+d] and w[p^2+p-d] share P_p^{|d|} z_p; the phases are conjugate
    constexpr int NPD = (L + 1) * (L + 2) / 2;  // (p, |d|) pairs
    for (int t = tid; t < V * NPD; t += kThreads) {
      const int v = t / NPD, i = t - v * NPD;
      int p = (int)((sqrtf(8.0f * i + 1.0f) - 1.0f) * 0.5f);
      if ((p + 1) * (p + 2) / 2 <= i) ++p;
      if (p * (p + 1) / 2 > i) --p;
      const int ad = i - p * (p + 1) / 2;
      const qg_c u = cscale(zb[v * (L + 1) + p], leg[v * NL + i]);
      const qg_c ph = eph[v * (L + 1) + ad];
      qg_c wp = cmul(u, ph), wm = cmul(u, cconj(ph));
      if (info[v].nan_out) {
        const double nan = __longlong_as_double(0x7ff8000000000000ULL);
        wp = wm = cmk(nan, nan);
      }
      qg_c *wv = w + v * S + p * p + p;
      wv[ad] = wp;
      if (ad) wv[-ad] = wm;
    }
    __syncthreads();

    // ---------------- phase 2: contraction ----------------
    const int vmax = (int)((n - base) < (size_t)V ? (n - base) : (size_t)V);
    for (int v = 0; v < vmax; ++v) {
      const qg_c *wv = w + v * S;
#pragma unroll 1
      for (int which = 0; which < 2; ++which) {
        const uint8_t *cnt = which ? T.cntB : T.cntA;
        const double *coef = which ? T.coefB : T.coefA;
        const uint16_t *slot = which ? T.slotB : T.slotA;
        const int32_t *perm = which ? T.permB : T.perm;
        qg_c *out = (which ? B : A) + (base + v) * (size_t)NE2;
        qg_c *buf = nullptr;
        if (STAGED) {
          buf = stage + (row_counter % kStages) * NE2;
          if (tid == 0) {  // the copy that last read this buffer is done
            if (kStages == 2)
              bulk_wait_read_le1();
            else
              bulk_wait_read_le0();
          }
          __syncthreads();
        }
        for (int k = tid; k < NE2; k += kThreads) {
          // term counts are sorted, so the trip count is (nearly) warp-uniform
          const int c = cnt[k];
          double sr = 0.0, si = 0.0;
          const double *cq = coef + k;
          const uint16_t *sq = slot + k;
#pragma unroll 2
          for (int q = 0; q < c; ++q) {
            const double a = __ldg(cq + q * NE2);
            const qg_c x = wv[__ldg(sq + q * NE2)];
            sr = fma(a, x.re, sr);
            si = fma(a, x.im, si);
          }
          const qg_c r = which ? cmk(-si, sr) : cmk(sr, si);
          const int e = __ldg(perm + k);
          if (STAGED)
            buf[e] = r;
          else
            out[e] = r;
        }
        if (STAGED) {
          fence_proxy_async_smem();
          __syncthreads();
          if (tid == 0) bulk_store_row(out, buf, (uint32_t)(NE2 * 16));
          ++row_counter;
        }
      }
    }
    __syncthreads();  // w / zb / leg are rewritten by the next chunk
  }
  if (STAGED && tid == 0) bulk_wait_all();
}

template <int LMAX>
int launch_lmax(const TransDevTables &T, size_t n, const qg_c *kr, const double *th, const double *ph,
                const unsigned char *rgd, int J, qg_c *A, qg_c *B, cudaStream_t st, int variant) {
  using Sh = TransShape<LMAX>;
  const bool staged = Sh::kStaged && variant == 0;
  const size_t smem = trans_smem_bytes<LMAX>(staged);
  int dev = 0, nsm = 0, per_sm = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  QG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t nchunks = (n + Sh::V - 1) / Sh::V;
  if (staged) {
    auto k = trans_ab_kernel<LMAX, Sh::kStaged>;
    QG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    QG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem));
    if (per_sm < 1) per_sm = 1;
    size_t grid = (size_t)nsm * per_sm;
    if (grid > nchunks) grid = nchunks;
    k<<<(unsigned)grid, kThreads, smem, st>>>(T, n, kr, th, ph, rgd, J, A, B);
  } else {
    auto k = trans_ab_kernel<LMAX, false>;
    QG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    QG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem));
    if (per_sm < 1) per_sm = 1;
    size_t grid = (size_t)nsm * per_sm;
    if (grid > nchunks) grid = nchunks;
    k<<<(unsigned)grid, kThreads, smem, st>>>(T, n, kr, th, ph, rgd, J, A, B);
  }
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

}  // namespace

int launch_trans_ab(const TransDevTables &T, size_t n, const qg_c *kr, const double *theta, const double *phi,
                    const unsigned char *r_ge_d, int J, qg_c *A, qg_c *B, cudaStream_t st, int variant) {
  if (n == 0) return QPMS_SUCCESS;
  switch (T.lMax) {
#define QG_CASE(LM) \
  case LM: return launch_lmax<LM>(T, n, kr, theta, phi, r_ge_d, J, A, B, st, variant);
    QG_CASE(1) QG_CASE(2) QG_CASE(3) QG_CASE(4) QG_CASE(5) QG_CASE(6) QG_CASE(7) QG_CASE(8) QG_CASE(9) QG_CASE(10)
#undef QG_CASE
    default: set_error("translation kernel: lMax %d not compiled (1..%d)", T.lMax, kTransLmaxMax); return QPMS_EINVAL;
  }
}

}  // namespace qg
