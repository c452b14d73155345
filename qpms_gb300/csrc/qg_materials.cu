// Lorentz-Drude parameter sets of metals (the reference's drudeparam_data.c,
// exported through materials.h:73-77): the published fits of A. D. Rakic,
// A. B. Djurisic, J. M. Elazar, M. L. Majewski, "Optical properties of metallic
// films for vertical-cavity optoelectronic devices", Appl. Opt. 37, 5271
// (1998) (drudelorentz.com), frequencies in eV converted with the electron
// volt and hbar of GSL's constant tables (CODATA 2006), as the reference does.
#include <stddef.h>

#include "qpms_gb300.h"

namespace {

constexpr double kEH = 1.602176487e-19 / 1.05457162825e-34;  // eV / hbar, rad/s

// Layout-compatible with qpms_ldparams_t (flexible array of n triples).
template <int N>
struct LdBlock {
  qpms_complex_t eps_inf;
  double omega_p;
  size_t n;
  qpms_ldparams_triple_t data[N];
};

const LdBlock<6> kAu = {{1, 0}, 9.03 * kEH, 6,
                        {{0.76, 0.0 * kEH, 0.053 * kEH},
                         {0.024, 0.415 * kEH, 0.241 * kEH},
                         {0.01, 0.83 * kEH, 0.345 * kEH},
                         {0.071, 2.969 * kEH, 0.87 * kEH},
                         {0.601, 4.304 * kEH, 2.494 * kEH},
                         {4.384, 13.32 * kEH, 2.214 * kEH}}};
const LdBlock<6> kAg = {{1, 0}, 9.01 * kEH, 6,
                        {{0.84, 0.0 * kEH, 0.053 * kEH},
                         {0.065, 0.816 * kEH, 3.886 * kEH},
                         {0.124, 4.481 * kEH, 0.452 * kEH},
                         {0.111, 8.185 * kEH, 0.065 * kEH},
                         {0.84, 9.083 * kEH, 0.916 * kEH},
                         {5.646, 20.29 * kEH, 2.419 * kEH}}};
const LdBlock<5> kCu = {{1, 0}, 10.83 * kEH, 5,
                        {{0.575, 0.0 * kEH, 0.03 * kEH},
                         {0.061, 0.291 * kEH, 0.378 * kEH},
                         {0.104, 2.957 * kEH, 1.056 * kEH},
                         {0.723, 5.3 * kEH, 3.213 * kEH},
                         {0.638, 11.18 * kEH, 4.305 * kEH}}};
const LdBlock<5> kAl = {{1, 0}, 14.98 * kEH, 5,
                        {{0.523, 0.0 * kEH, 0.047 * kEH},
                         {0.227, 0.162 * kEH, 0.333 * kEH},
                         {0.05, 1.544 * kEH, 0.312 * kEH},
                         {0.166, 1.808 * kEH, 1.251 * kEH},
                         {0.03, 3.473 * kEH, 3.382 * kEH}}};
const LdBlock<5> kCr = {{1, 0}, 10.75 * kEH, 5,
                        {{0.168, 0.0 * kEH, 0.047 * kEH},
                         {0.151, 0.121 * kEH, 3.175 * kEH},
                         {0.15, 0.543 * kEH, 1.305 * kEH},
                         {1.149, 1.97 * kEH, 2.676 * kEH},
                         {0.825, 8.775 * kEH, 1.335 * kEH}}};

}  // namespace

extern "C" {
const qpms_ldparams_t *const QPMS_LDPARAMS_AU = reinterpret_cast<const qpms_ldparams_t *>(&kAu);
const qpms_ldparams_t *const QPMS_LDPARAMS_AG = reinterpret_cast<const qpms_ldparams_t *>(&kAg);
const qpms_ldparams_t *const QPMS_LDPARAMS_CU = reinterpret_cast<const qpms_ldparams_t *>(&kCu);
const qpms_ldparams_t *const QPMS_LDPARAMS_AL = reinterpret_cast<const qpms_ldparams_t *>(&kAl);
const qpms_ldparams_t *const QPMS_LDPARAMS_CR = reinterpret_cast<const qpms_ldparams_t *>(&kCr);
}
