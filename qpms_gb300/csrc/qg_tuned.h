// Tuned constants of the library, written by qpms_gb300/tune.py from
// measurements on the target GPU (the measurements it used are in
// qpms_gb300/tuning.json).  Rerun it after changing the kernels:
//   python -m qpms_gb300.tune
#pragma once

namespace qg {

// The mixed dense LU uses 64-wide diagonal blocks below this many unknowns
// and 128-wide ones from it on.
constexpr int kTunedNb64Below = 6144;

// Operand stages and tensor-memory accumulators of the 128-wide GEMM tile,
// as 10 x stages + accumulators.
constexpr int kTunedGemmPipe = 62;

// 256-wide GEMM tiles for outputs wide enough to fill the GPU twice.
constexpr bool kTunedGemmWide = true;

}  // namespace qg
