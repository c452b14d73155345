// Tuned constants of the library, written by qpms_gb300/tune.py from
// measurements on the target GPU (the measurements it used are in
// qpms_gb300/tuning.json).  Rerun it after changing the kernels:
//   python -m qpms_gb300.tune
#pragma once

namespace qg {

// The mixed dense LU uses 64-wide diagonal blocks below this many unknowns
// and 128-wide ones from it on.
constexpr int kTunedNb64Below = 6144;

}  // namespace qg
