// Internal declarations shared by the libqpms_gb300 translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <atomic>
#include <string>
#include <vector>

#include "../../include/qpms_gb300.h"
#include "qg_complex.cuh"

namespace qg {

// thread-local last-error message (qpms_gpu_last_error)
void set_error(const char *fmt, ...);
void clear_error();
extern std::atomic<unsigned long long> g_launches;
extern std::atomic<unsigned long long> g_graph_replays;

#define QG_CUDA_TRY(expr)                                                            \
  do {                                                                               \
    cudaError_t _e = (expr);                                                         \
    if (_e != cudaSuccess) {                                                         \
      qg::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return QPMS_ERROR;                                                             \
    }                                                                                \
  } while (0)

// cuBLAS calls (CUBLAS_STATUS_SUCCESS == 0)
#define QG_BLAS_TRY(expr)                                                                \
  do {                                                                                   \
    int _s = (int)(expr);                                                                \
    if (_s != 0) {                                                                       \
      qg::set_error("%s:%d: %s: cublas status %d", __FILE__, __LINE__, #expr, _s);      \
      return QPMS_ERROR;                                                                 \
    }                                                                                    \
  } while (0)

// ---- translation tables (qg_tables.cu) ----

// Largest lMax with a compiled translation kernel.
constexpr int kTransLmaxMax = 10;

struct TransHostTables {
  int lMax = 0, nelem = 0, tq = 0;  // tq = max terms per element (lMax + 1)
  // reference-layout ragged multipliers (complex), row-major over (y, yu)
  std::vector<qg_c> A_mult, B_mult;
  std::vector<size_t> A_off, B_off;  // nelem^2 + 1 offsets
  // kernel tables, element e = y * nelem + yu; A and B each in their own
  // term-count order k (permA / permB: k -> e)
  std::vector<int32_t> perm, permB;
  std::vector<uint8_t> cntA, cntB;   // per k
  std::vector<uint8_t> cntBe;        // B order: min(cntB, cntA of the same element), the
                                     // q <= qmax_A bound of the lattice-sum contraction
  std::vector<double> coefA, coefB;  // [q][k]: A real part, B imaginary part
  std::vector<uint16_t> slotA, slotB;  // [q][k]: w-table slot p^2 + p + d
};

// Builds the tables for (lMax, normalisation); returns false on bad input.
bool build_trans_tables(int lMax, int normalisation, TransHostTables *t);

// Device copy of the kernel tables.
struct TransDevTables {
  int lMax, nelem, ne2, tq;
  const int32_t *perm, *permB;
  const uint8_t *cntA, *cntB, *cntBe;
  const double *coefA, *coefB;
  const uint16_t *slotA, *slotB;
};

// Private extension that follows the public qpms_trans_calculator.
struct TransCalcPriv {
  qpms_trans_calculator pub;
  TransHostTables host;
  TransDevTables dev;
  void *dev_block = nullptr;  // one cudaMalloc holding all device tables
  int device = 0;
  // host-API staging (lazily allocated)
  void *pin_in = nullptr, *pin_out = nullptr;
  void *dev_in = nullptr, *dev_out = nullptr;
  size_t stage_vecs = 0;
  cudaStream_t streams[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

inline TransCalcPriv *priv(const qpms_trans_calculator *c) {
  return reinterpret_cast<TransCalcPriv *>(const_cast<qpms_trans_calculator *>(c));
}

// QPMS_EINVAL (with a message) unless the current device is the one that holds
// the calculator's device tables (qg_trans_api.cu).
int check_calc_device(const qpms_trans_calculator *c);

// Kernel launcher (qg_trans_kernel.cu).  variant 0 = sorted + TMA-staged
// stores (default), 1 = natural order with direct stores.
int launch_trans_ab(const TransDevTables &T, size_t n, const qg_c *kr, const double *theta,
                    const double *phi, const unsigned char *r_ge_d, int J, qg_c *A, qg_c *B,
                    cudaStream_t stream, int variant);

}  // namespace qg
