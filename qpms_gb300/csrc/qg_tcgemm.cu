// GEMMs on the sm_103a tensor cores: tcgen05.mma (bf16 x bf16 -> FP32 in
// tensor memory), operands staged by TMA (cp.async.bulk.tensor, 128-byte
// swizzle), one persistent warp-specialised kernel.
//
// Uses in this library: the complex64 trailing updates, panels and
// many-right-hand-side substitutions of the mixed-precision dense LU
// (qg_dense.cu) -- the LAPACKE_zgetrf / zgetrs work of the reference
// (scatsystem.c:2202-2273, beyn.c:552-564) -- and the digit products of the
// FP64-accurate refinement residual (qg_ozaki.cu).
//
// Complex products run on the real embedding: with E(A) the 2m x 2k real
// matrix [[Re A, -Im A], [Im A, Re A]] interleaved by rows (2i + p) and
// columns (2l + q), and B viewed as the 2k x n real matrix of its interleaved
// parts, E(A) B is C = A B viewed as a 2m x n real matrix -- exactly the memory
// of a column-major complex64 matrix read as floats.  FP32 accuracy comes from
// splitting each operand into bf16 digits x = x_0 + x_1 (+ x_2) and summing
// the digit products x_s y_t with s + t < nsplit in the same FP32 accumulator
// (3 products give about 2^-16 relative error, 6 products about FP32's 2^-24).
//
// Kernel layout (one CTA per SM, 320 threads):
//   warp 0  TMA producer: A tile 128 x 64 and B tile BN x 64 (bf16, K-major,
//           128-byte swizzle) per pipeline stage, STAGES stages;
//   warp 1  allocates 2 x BN tensor-memory columns (two accumulators), and its
//           lane 0 issues tcgen05.mma (M 128, N BN, K 16; four per stage),
//           committing each stage back to the producer and each finished tile
//           to the epilogue;
//   warps 2-9  epilogue: tcgen05.ld of the accumulator (a warp reads its
//           32-lane quarter, two warps per quarter with half the columns
//           each), D = beta C + alpha acc, stores coalesced along the rows,
//           while the MMA warp fills the other accumulator.
// Every wait on an mbarrier is bounded (kTimeoutNs); a wait that runs out
// sets a device error flag (tc_check_error) and the kernel winds down.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "qg_internal.h"
#include "qg_ktimer.h"
#include "qg_tcgemm.h"
#include "qg_tuned.h"

namespace qg {
namespace {

constexpr int BM = 128;  // accumulator rows = tensor-memory lanes
constexpr int BK = 64;   // bf16 per 128-byte swizzled row
constexpr unsigned long long kTimeoutNs = 4000000000ull;  // 4 s per wait
constexpr int kReservedSms = 8;
constexpr int kEpiWarps = 8;  // warps 2..9: two per tensor-memory lane quarter, half the columns each

__device__ int g_tc_error;

// ---------------- PTX wrappers ----------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of the given parity; false (and the error flag
// set) if it did not complete within kTimeoutNs.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer() - t0 > kTimeoutNs) {
      atomicExch(&g_tc_error, code);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y,
                                            int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand tile in shared memory, 128-byte rows, 128-byte swizzle:
// 8-row groups 1024 bytes apart (stride byte offset); the leading byte
// offset is not used by this layout.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;  // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, M = 128, N = bn.
__host__ __device__ constexpr uint32_t idesc_bf16(int bn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 32 consecutive accumulator columns of this thread's lane, load and wait in
// one statement.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}
// 64 consecutive accumulator columns of this thread's lane: two loads and one
// wait in a single statement, so no use of r can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%64];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%65];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr), "r"(taddr + 32u)
      : "memory");
}

// ---------------- the GEMM kernel ----------------
constexpr int kMaxPairs = 6;

struct GemmArgs {
  int Md, Nd;         // output rows (real) and columns
  int kblocks;        // ceil(K / 64) per digit product
  int npairs;
  uint32_t pa, pb;  // digit planes of product i in bits [4i, 4i + 4)
  float alpha, beta;
  const float *C;
  float *D;
  size_t ldc, ldd;  // in floats
};

template <int BN, int STAGES>
struct Smem {
  static constexpr int kA = BM * BK * 2, kB = BN * BK * 2, kStage = kA + kB;
  static constexpr int kBytes = STAGES * kStage + 1024 /* align */ + 256 /* barriers */;
};

template <int BN, int STAGES, int NACC>
__global__ void __launch_bounds__(64 + 32 * kEpiWarps, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const GemmArgs g) {
  using S = Smem<BN, STAGES>;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  unsigned char *base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(base + STAGES * S::kStage);
  uint64_t *empty = full + STAGES;
  uint64_t *tfull = empty + STAGES;  // [NACC]
  uint64_t *tempty = tfull + NACC;   // [NACC]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tempty + NACC);
  // tensor-memory columns: NACC accumulators of BN, allocated as a power of two
  constexpr uint32_t kTmemCols = (NACC * BN <= 32) ? 32 : (NACC * BN <= 64) ? 64 : (NACC * BN <= 128) ? 128
                                 : (NACC * BN <= 256) ? 256 : 512;
  static_assert(NACC * BN <= 512, "accumulators exceed tensor memory");

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = (g.Md + BM - 1) / BM, nt = (g.Nd + BN - 1) / BN;
  const int ntiles = mt * nt;
  const int nkb = g.kblocks * g.npairs;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    for (int b = 0; b < NACC; ++b) {
      mbar_init(tfull + b, 1);
      mbar_init(tempty + b, 32 * kEpiWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer ----
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mapB) : "memory");
    uint32_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int m0 = (tile % mt) * BM, n0 = (tile / mt) * BN;
      for (int kb = 0; kb < nkb; ++kb, ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!(ok = mbar_wait(empty + s, ph ^ 1, 1))) break;
        const int pr = kb / g.kblocks, kk = kb - pr * g.kblocks;
        unsigned char *sa = base + s * S::kStage, *sb = sa + S::kA;
        mbar_expect_tx(full + s, S::kStage);
        tma_load_3d(sa, &mapA, full + s, kk * BK, m0, (int)((g.pa >> (4 * pr)) & 15u));
        tma_load_3d(sb, &mapB, full + s, kk * BK, n0, (int)((g.pb >> (4 * pr)) & 15u));
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer ----
    constexpr uint32_t idesc = idesc_bf16(BN);
    uint32_t it = 0, t = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++t) {
      const uint32_t b = t % NACC, tph = (t / NACC) & 1;
      if (!(ok = mbar_wait(tempty + b, tph ^ 1, 2))) break;
      tc_fence_after();
      const uint32_t dt = tmem + b * BN;
      for (int kb = 0; kb < nkb; ++kb, ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!(ok = mbar_wait(full + s, ph, 3))) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(base + s * S::kStage), sb = sa + S::kA;
        const uint64_t da = sw128_desc(sa), db = sw128_desc(sb);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k)  // 16 bf16 = 32 bytes = 2 descriptor units per step
          mma_bf16(dt, da + 2 * k, db + 2 * k, idesc, (kb | k) ? 1u : 0u);
        mma_commit(empty + s);
      }
      if (ok) mma_commit(tfull + b);
    }
  } else if (warp >= 2) {
    // ---- epilogue ----
    // Each thread owns one accumulator row (its tensor-memory lane) of the
    // tile.  Its BN values of C are loaded into registers before the wait for
    // the accumulator, so the HBM reads of this tile overlap its MMAs; D is
    // then stored column by column (a warp writes 32 consecutive floats).
    const int quad = warp & 3;  // tensor-memory lane quarter this warp may read
    constexpr int CW = BN / 2;  // columns per epilogue warp: two warps share each lane quarter
    constexpr int CH = CW < 64 ? CW : 64;  // columns per chunk (registers: C and accumulator of one chunk)
    constexpr int NCH = CW / CH;
    const int c0 = ((warp - 2) >> 2) * CW;
    const bool has_c = g.beta != 0.f;
    uint32_t t = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++t) {
      const uint32_t b = t % NACC, tph = (t / NACC) & 1;
      const int m0 = (tile % mt) * BM, n0 = (tile / mt) * BN + c0;
      const int r = m0 + quad * 32 + lane;
      const bool rok = r < g.Md;
      float cv[CH];
      auto load_c = [&](int nc) {
        if (has_c && rok) {
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            const int j = nc + c;
            cv[c] = (j < g.Nd) ? g.C[(size_t)j * g.ldc + r] : 0.f;
          }
        }
      };
      load_c(n0);  // the first chunk's C before the wait: its reads overlap the tile's MMAs
      if (!(ok = mbar_wait(tfull + b, tph, 4))) break;
      tc_fence_after();
#pragma unroll
      for (int h = 0; h < NCH; ++h) {
        const int nc = n0 + h * CH;
        uint32_t v[CH];
        if constexpr (CH == 64)
          tmem_ld64(tmem + ((uint32_t)(quad * 32) << 16) + b * BN + c0 + h * CH, v);
        else
          tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + b * BN + c0 + h * CH, v);
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          float x = g.alpha * __uint_as_float(v[c]);
          if (has_c) x += g.beta * cv[c];
          v[c] = __float_as_uint(x);
        }
        if (h + 1 < NCH) load_c(nc + CH);  // the next chunk's C, in flight during these stores
        if (h + 1 == NCH) {                 // the accumulator is read out: free it for the MMAs
          tc_fence_before();
          mbar_arrive(tempty + b);
        }
        if (rok) {
          float *drow = g.D + (size_t)nc * g.ldd + r;
          if (nc + CH <= g.Nd) {
#pragma unroll
            for (int c = 0; c < CH; ++c) drow[(size_t)c * g.ldd] = __uint_as_float(v[c]);
          } else {
#pragma unroll
            for (int c = 0; c < CH; ++c)
              if (nc + c < g.Nd) drow[(size_t)c * g.ldd] = __uint_as_float(v[c]);
          }
        }
      }
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// ---------------- operand splitting ----------------
__device__ __forceinline__ void digits(float x, int ns, __nv_bfloat16 *d) {
  float r = x;
  for (int s = 0; s < ns; ++s) {
    d[s] = __float2bfloat16_rn(r);
    r -= __bfloat162float(d[s]);
  }
}

// A planes [s][2m][rs]: rows 2i, 2i+1 of E(A) at columns 2l, 2l+1.
// 32 x 32 complex tiles through shared memory, 256 threads (tx 0..31, ty 0..7).
struct SplitA {
  const float2 *A;
  size_t lda, rs, plane;
  int m, k, trans;
  __nv_bfloat16 *P;
};
__device__ __forceinline__ void split_a_tile(const SplitA &a, int ns, int bx, int by, int tx, int ty,
                                             float2 (*tile)[33]) {
  const int i0 = bx * 32, l0 = by * 32;
  for (int q = ty; q < 32; q += 8) {
    if (!a.trans) {  // A(i, l) at A[l lda + i]: threads along i
      const int i = i0 + tx, l = l0 + q;
      tile[q][tx] = (i < a.m && l < a.k) ? a.A[(size_t)l * a.lda + i] : make_float2(0.f, 0.f);
    } else {  // A(i, l) = Asrc(l, i) at A[i lda + l]: threads along l
      const int i = i0 + q, l = l0 + tx;
      tile[tx][q] = (i < a.m && l < a.k) ? a.A[(size_t)i * a.lda + l] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {  // write: threads along l
    const int i = i0 + q, l = l0 + tx;
    if (i >= a.m || l >= a.k) continue;
    const float2 v = tile[tx][q];
    __nv_bfloat16 dr[3], di[3];
    digits(v.x, ns, dr);
    digits(v.y, ns, di);
    for (int s = 0; s < ns; ++s) {
      __nv_bfloat16 *p = a.P + s * a.plane;
      __nv_bfloat162 top, bot;  // row 2i: (Re, -Im); row 2i+1: (Im, Re)
      top.x = dr[s];
      top.y = __hneg(di[s]);
      bot.x = di[s];
      bot.y = dr[s];
      *reinterpret_cast<__nv_bfloat162 *>(p + (size_t)(2 * i) * a.rs + 2 * l) = top;
      *reinterpret_cast<__nv_bfloat162 *>(p + (size_t)(2 * i + 1) * a.rs + 2 * l) = bot;
    }
  }
}

// B planes [s][n][rs]: column j, entries 2l (Re) and 2l+1 (Im).
struct SplitB {
  const float2 *B;
  size_t ldb, rs, plane;
  int k, n;
  __nv_bfloat16 *P;
};
__device__ __forceinline__ void split_b_range(const SplitB &b, int ns, size_t start, size_t stride) {
  const size_t total = (size_t)b.k * b.n;
  for (size_t t = start; t < total; t += stride) {
    const int j = (int)(t / b.k), l = (int)(t - (size_t)j * b.k);
    const float2 v = b.B[(size_t)j * b.ldb + l];
    __nv_bfloat16 dr[3], di[3];
    digits(v.x, ns, dr);
    digits(v.y, ns, di);
    for (int s = 0; s < ns; ++s) {
      __nv_bfloat162 w;
      w.x = dr[s];
      w.y = di[s];
      *reinterpret_cast<__nv_bfloat162 *>(b.P + s * b.plane + (size_t)j * b.rs + 2 * l) = w;
    }
  }
}

__global__ void __launch_bounds__(256) split_a_kernel(SplitA a, int ns) {
  __shared__ float2 tile[32][33];  // [l][i]
  split_a_tile(a, ns, blockIdx.x, blockIdx.y, threadIdx.x & 31, threadIdx.x >> 5, tile);
}

__global__ void __launch_bounds__(256) split_b_kernel(SplitB b, int ns) {
  split_b_range(b, ns, blockIdx.x * (size_t)blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}

// Both operands of one GEMM in one launch: blocks [0, na_x * na_y) make the A
// planes (tile by tile), the rest the B planes.
__global__ void __launch_bounds__(256) split_ab_kernel(SplitA a, int na_x, int na_y, SplitB b, int nb_blocks,
                                                      int ns) {
  __shared__ float2 tile[32][33];
  const int na = na_x * na_y;
  if ((int)blockIdx.x < na) {
    split_a_tile(a, ns, blockIdx.x % na_x, blockIdx.x / na_x, threadIdx.x & 31, threadIdx.x >> 5, tile);
  } else {
    const size_t bb = blockIdx.x - na;
    split_b_range(b, ns, bb * blockDim.x + threadIdx.x, (size_t)nb_blocks * blockDim.x);
  }
}

// ---------------- host side ----------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
int g_num_sms = 0;

int encode_fn(PFN_cuTensorMapEncodeTiled_v12000 *out) {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  });
  if (!g_encode) {
    set_error("cuTensorMapEncodeTiled is not available from the CUDA driver API");
    return QPMS_ERROR;
  }
  *out = g_encode;
  return QPMS_SUCCESS;
}

// 3-D K-major bf16 operand: [planes][rows][rs], box 64 x box_rows x 1.
int make_map(CUtensorMap *map, const __nv_bfloat16 *p, int kdim, int rows, int planes, size_t rs, size_t plane,
             int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc;
  int e = encode_fn(&enc);
  if (e) return e;
  if (((uintptr_t)p & 15) || (rs * 2) % 16 || (plane * 2) % 16) {
    set_error("tensor-core GEMM operand not 16-byte aligned (row stride %zu)", rs);
    return QPMS_EINVAL;
  }
  cuuint64_t dims[3] = {(cuuint64_t)kdim, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)(rs * 2), (cuuint64_t)(plane * 2)};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)p, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d): dims %d x %d x %d, row stride %zu", (int)r, kdim, rows, planes,
              rs);
    return QPMS_ERROR;
  }
  return QPMS_SUCCESS;
}

template <int BN, int STAGES, int NACC>
int launch_gemm(const CUtensorMap &ma, const CUtensorMap &mb, const GemmArgs &g, cudaStream_t st) {
  using S = Smem<BN, STAGES>;
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(tc_gemm_kernel<BN, STAGES, NACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    S::kBytes);
  });
  QG_CUDA_TRY(attr_err);
  // Persistent CTAs on all but kReservedSms SMs: the single-CTA kernels of the
  // dense LU (diagonal blocks) and the small launches of concurrent solves on
  // other streams always find an SM instead of waiting for a whole GEMM.
  const int ntiles = ((g.Md + BM - 1) / BM) * ((g.Nd + BN - 1) / BN);
  const int slots = g_num_sms > 2 * kReservedSms ? g_num_sms - kReservedSms : g_num_sms;
  const int grid = ntiles < slots ? ntiles : slots;
  if (grid <= 0) return QPMS_SUCCESS;
  KtScope kt(KT_TCGEMM, st, 2.0 * g.Md * (double)g.Nd * (double)g.kblocks * BK * g.npairs);
  tc_gemm_kernel<BN, STAGES, NACC><<<grid, 64 + 32 * kEpiWarps, S::kBytes, st>>>(ma, mb, g);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

// Pipeline depth and accumulator count of the wide-tile kernel (tuning knob
// QPMS_GB300_GEMM_PIPE = "SxA": S operand stages, A tensor-memory
// accumulators; 6x2, 6x3, 7x2 or 7x3).
int gemm_pipe() {
  static int v = [] {
    const char *e = getenv("QPMS_GB300_GEMM_PIPE");
    if (e && !strcmp(e, "6x2")) return 62;
    if (e && !strcmp(e, "6x3")) return 63;
    if (e && !strcmp(e, "7x2")) return 72;
    if (e && !strcmp(e, "7x3")) return 73;
    return kTunedGemmPipe;
  }();
  return v;
}

// 256-wide tiles for wide outputs (QPMS_GB300_GEMM_WIDE=0 turns them off).
bool gemm_wide() {
  static bool v = [] {
    const char *e = getenv("QPMS_GB300_GEMM_WIDE");
    return !(e && !strcmp(e, "0")) && kTunedGemmWide;
  }();
  return v;
}

// N tile by the output width: narrow outputs (right-hand-side blocks) waste
// fewer columns with a 64-wide tile.
int dispatch(const __nv_bfloat16 *a, int kdim, int arows, int aplanes, size_t ars, size_t aplane,
             const __nv_bfloat16 *b, int brows, int bplanes, size_t brs, size_t bplane, GemmArgs &g,
             cudaStream_t st) {
  CUtensorMap ma, mb;
  int e;
  if ((e = make_map(&ma, a, kdim, arows, aplanes, ars, aplane, BM))) return e;
  if (g.Nd <= 64) {
    if ((e = make_map(&mb, b, kdim, brows, bplanes, brs, bplane, 64))) return e;
    return launch_gemm<64, 6, 2>(ma, mb, g, st);
  }
  // wide outputs: 256-wide tiles (A tiles reloaded half as often, twice the
  // MMA work per staged byte), when they still fill the SMs twice over
  const long tiles256 = (long)((g.Md + BM - 1) / BM) * ((g.Nd + 255) / 256);
  if (g.Nd >= 256 && tiles256 >= 2L * g_num_sms && gemm_wide()) {
    if ((e = make_map(&mb, b, kdim, brows, bplanes, brs, bplane, 256))) return e;
    return launch_gemm<256, 4, 2>(ma, mb, g, st);
  }
  if ((e = make_map(&mb, b, kdim, brows, bplanes, brs, bplane, 128))) return e;
  switch (gemm_pipe()) {
    case 63: return launch_gemm<128, 6, 3>(ma, mb, g, st);
    case 72: return launch_gemm<128, 7, 2>(ma, mb, g, st);
    case 73: return launch_gemm<128, 7, 3>(ma, mb, g, st);
    default: return launch_gemm<128, 6, 2>(ma, mb, g, st);
  }
}

size_t rs_of(int k) { return ((size_t)2 * k + 7) / 8 * 8; }

}  // namespace

size_t tc_planes_row(int k) { return rs_of(k); }
size_t tc_planes_bytes_a(int m, int k, int nsplit) { return (size_t)nsplit * 2 * m * rs_of(k) * 2; }
size_t tc_planes_bytes_b(int n, int k, int nsplit) { return (size_t)nsplit * n * rs_of(k) * 2; }

namespace {
SplitA split_a_args(const float2 *A, size_t lda, int m, int k, __nv_bfloat16 *planes, bool trans_a) {
  SplitA a;
  a.A = A;
  a.lda = lda;
  a.m = m;
  a.k = k;
  a.trans = trans_a ? 1 : 0;
  a.rs = rs_of(k);
  a.plane = (size_t)2 * m * a.rs;
  a.P = planes;
  return a;
}
SplitB split_b_args(const float2 *B, size_t ldb, int k, int n, __nv_bfloat16 *planes) {
  SplitB b;
  b.B = B;
  b.ldb = ldb;
  b.k = k;
  b.n = n;
  b.rs = rs_of(k);
  b.plane = (size_t)n * b.rs;
  b.P = planes;
  return b;
}
int split_b_blocks(int k, int n) {
  size_t blocks = ((size_t)k * n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  return (int)(blocks ? blocks : 1);
}
int check_ns(int nsplit) {
  if (nsplit < 1 || nsplit > 3) {
    set_error("nsplit %d not in 1..3", nsplit);
    return QPMS_EINVAL;
  }
  return QPMS_SUCCESS;
}
}  // namespace

int tc_split_a(const float2 *A, size_t lda, int m, int k, int nsplit, __nv_bfloat16 *planes, cudaStream_t st,
               bool trans_a) {
  if (m <= 0 || k <= 0) return QPMS_SUCCESS;
  int e;
  if ((e = check_ns(nsplit))) return e;
  dim3 grid((m + 31) / 32, (k + 31) / 32);
  KtScope kt(KT_SPLIT, st, 8.0 * nsplit * m * (double)k);
  split_a_kernel<<<grid, 256, 0, st>>>(split_a_args(A, lda, m, k, planes, trans_a), nsplit);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int tc_split_b(const float2 *B, size_t ldb, int k, int n, int nsplit, __nv_bfloat16 *planes, cudaStream_t st) {
  if (n <= 0 || k <= 0) return QPMS_SUCCESS;
  int e;
  if ((e = check_ns(nsplit))) return e;
  KtScope kt(KT_SPLIT, st, 4.0 * nsplit * n * (double)k);
  split_b_kernel<<<split_b_blocks(k, n), 256, 0, st>>>(split_b_args(B, ldb, k, n, planes), nsplit);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int tc_split_ab(const float2 *A, size_t lda, int m, int k, const float2 *B, size_t ldb, int n, int nsplit,
                __nv_bfloat16 *a_planes, __nv_bfloat16 *b_planes, cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0) return QPMS_SUCCESS;
  int e;
  if ((e = check_ns(nsplit))) return e;
  const int na_x = (m + 31) / 32, na_y = (k + 31) / 32, nb = split_b_blocks(k, n);
  KtScope kt(KT_SPLIT, st, 8.0 * nsplit * m * (double)k + 4.0 * nsplit * n * (double)k);
  split_ab_kernel<<<na_x * na_y + nb, 256, 0, st>>>(split_a_args(A, lda, m, k, a_planes, false), na_x, na_y,
                                                    split_b_args(B, ldb, k, n, b_planes), nb, nsplit);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

int tc_cgemm_planes(const TcPlanes &P, float alpha, float beta, const float2 *C, size_t ldc, float2 *D, size_t ldd,
                    cudaStream_t st) {
  if (P.m <= 0 || P.n <= 0) return QPMS_SUCCESS;
  if (P.nsplit < 1 || P.nsplit > 3) {
    set_error("nsplit %d not in 1..3", P.nsplit);
    return QPMS_EINVAL;
  }
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  g.Md = 2 * P.m;
  g.Nd = P.n;
  g.kblocks = (2 * P.k + BK - 1) / BK;
  // digit products with s + t < nsplit, smallest first
  int np = 0;
  for (int sum = P.nsplit - 1; sum >= 0; --sum)
    for (int s = 0; s <= sum && np < kMaxPairs; ++s) {
      g.pa |= (uint32_t)s << (4 * np);
      g.pb |= (uint32_t)(sum - s) << (4 * np);
      ++np;
    }
  g.npairs = np;
  g.alpha = alpha;
  g.beta = beta;
  g.C = reinterpret_cast<const float *>(C);
  g.D = reinterpret_cast<float *>(D);
  g.ldc = 2 * ldc;
  g.ldd = 2 * ldd;
  if (P.k <= 0) {  // empty product: D = beta C
    g.alpha = 0.f;
  }
  const size_t rs = rs_of(P.k), ars = P.a_rs ? P.a_rs : rs;
  return dispatch(P.a, 2 * P.k, 2 * P.m, P.nsplit, ars, P.a_plane ? P.a_plane : (size_t)2 * P.m * ars, P.b, P.n,
                  P.nsplit, rs, P.b_plane ? P.b_plane : (size_t)P.n * rs, g, st);
}

int tc_gemm_bf16(const __nv_bfloat16 *A, size_t lda, const __nv_bfloat16 *B, size_t ldb, int m, int n, int k,
                 float alpha, float beta, const float *C, size_t ldc, float *D, size_t ldd, cudaStream_t st) {
  if (m <= 0 || n <= 0) return QPMS_SUCCESS;
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  g.Md = m;
  g.Nd = n;
  g.kblocks = (k + BK - 1) / BK;
  g.npairs = 1;
  g.alpha = alpha;
  g.beta = beta;
  g.C = C;
  g.D = D;
  g.ldc = ldc;
  g.ldd = ldd;
  return dispatch(A, k, m, 1, lda, (size_t)m * lda, B, n, 1, ldb, (size_t)n * ldb, g, st);
}

int tc_check_error(cudaStream_t st) {
  int h = 0;
  QG_CUDA_TRY(cudaStreamSynchronize(st));
  QG_CUDA_TRY(cudaMemcpyFromSymbol(&h, g_tc_error, sizeof(int)));
  if (h) {
    const int z = 0;
    cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
    set_error("tensor-core GEMM: a pipeline wait ran out of time (role %d)", h);
    return QPMS_ERROR;
  }
  return QPMS_SUCCESS;
}

}  // namespace qg

// ---------------- C-ABI (library utilities, device pointers) ----------------
using namespace qg;

extern "C" int qpms_gpu_tc_cgemm(int m, int n, int k, const void *A, size_t lda,
                                 const void *B, size_t ldb, float alpha, float beta,
                                 const void *C, size_t ldc, void *D, size_t ldd,
                                 int nsplit, void *stream) {
  clear_error();
  if (m < 0 || n < 0 || k < 0 || nsplit < 1 || nsplit > 3 || !D || (m && k && !A) || (n && k && !B) ||
      (beta != 0.f && !C) || lda < (size_t)(m > 0 ? m : 1) || ldb < (size_t)(k > 0 ? k : 1) ||
      ldd < (size_t)(m > 0 ? m : 1) || (beta != 0.f && ldc < (size_t)(m > 0 ? m : 1))) {
    set_error("qpms_gpu_tc_cgemm: invalid arguments");
    return QPMS_EINVAL;
  }
  if (m == 0 || n == 0) return QPMS_SUCCESS;
  cudaStream_t st = (cudaStream_t)stream;
  const int kk = k > 0 ? k : 1;
  __nv_bfloat16 *pa = nullptr, *pb = nullptr;
  QG_CUDA_TRY(cudaMallocAsync((void **)&pa, tc_planes_bytes_a(m, kk, nsplit), st));
  QG_CUDA_TRY(cudaMallocAsync((void **)&pb, tc_planes_bytes_b(n, kk, nsplit), st));
  int e = QPMS_SUCCESS;
  TcPlanes P;
  P.a = pa;
  P.b = pb;
  P.m = m;
  P.n = n;
  P.k = k;
  P.nsplit = nsplit;
  if (k > 0) {
    if (!e) e = tc_split_a((const float2 *)A, lda, m, k, nsplit, pa, st);
    if (!e) e = tc_split_b((const float2 *)B, ldb, k, n, nsplit, pb, st);
  }
  if (!e) e = tc_cgemm_planes(P, alpha, beta, (const float2 *)C, ldc, (float2 *)D, ldd, st);
  cudaFreeAsync(pa, st);
  cudaFreeAsync(pb, st);
  return e;
}

extern "C" int qpms_gpu_tc_gemm_bf16(int m, int n, int k, const void *A, size_t lda, const void *B, size_t ldb,
                                     float alpha, float beta, const float *C, size_t ldc, float *D, size_t ldd,
                                     void *stream) {
  clear_error();
  if (m < 0 || n < 0 || k <= 0 || !A || !B || !D || lda < (size_t)k || ldb < (size_t)k || lda % 8 || ldb % 8 ||
      ldd < (size_t)(m > 0 ? m : 1) || (beta != 0.f && (!C || ldc < (size_t)(m > 0 ? m : 1)))) {
    set_error("qpms_gpu_tc_gemm_bf16: invalid arguments (row strides must be multiples of 8)");
    return QPMS_EINVAL;
  }
  return tc_gemm_bf16((const __nv_bfloat16 *)A, lda, (const __nv_bfloat16 *)B, ldb, m, n, k, alpha, beta, C, ldc,
                      D, ldd, (cudaStream_t)stream);
}

extern "C" int qpms_gpu_tc_check_error(void *stream) {
  clear_error();
  return tc_check_error((cudaStream_t)stream);
}
