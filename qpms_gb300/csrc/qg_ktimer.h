// Live per-kind kernel timing (qg_ktimer.cu).
#pragma once
#include <cuda_runtime.h>

namespace qg {

enum KtKind {
  KT_TCGEMM = 0,    // tensor-core GEMM (work: executed bf16 flops)
  KT_ASSEMBLE = 1,  // finite I - T S assembly (work: matrix bytes written)
  KT_EWALD = 2,     // lattice-sum assembly (work: matrix bytes written)
  KT_BATCHLU = 3,   // batched small LU (work: complex flops 8 N^3 / 3 per matrix)
  KT_DIAGLU = 4,    // diagonal-block inverse of the dense solver (work: 8 nb^3 real flops)
  KT_TRANS = 5,     // batched translation coefficients (work: output bytes)
  KT_SPLIT = 6,     // bf16 digit splitting of tensor-core operands (work: bytes written)
  KT_KINDS = 7
};

// Whether per-launch timing is on (launches are then not captured into graphs:
// the timing events belong to the eager launches).
bool kt_on();

// Records an event pair around the launches made during its lifetime, when
// timing is on.
class KtScope {
 public:
  KtScope(int kind, cudaStream_t st, double work);
  ~KtScope();
  KtScope(const KtScope &) = delete;
  KtScope &operator=(const KtScope &) = delete;

 private:
  int kind_;
  cudaStream_t st_;
  double work_;
  bool active_ = false;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
};

}  // namespace qg
