/* Plain-argument entry points into the reference's own translations.c /
 * ewald.c compiled in oracle/_ref (complex numbers and small structs passed as
 * doubles), for the pinning tests and fixture scripts.  Test infrastructure:
 * the library never links this. */
#include <complex.h>
#include <stdbool.h>
#include <stddef.h>

#include "qpms_types.h"
#include "translations.h"

void *refpin_trans_calculator_init(int lMax, int normalisation) {
  return qpms_trans_calculator_init(lMax, (qpms_normalisation_t)normalisation);
}
void refpin_trans_calculator_free(void *c) { qpms_trans_calculator_free((qpms_trans_calculator *)c); }

/* A, B: nelem x nelem row-major (deststride nelem, srcstride 1) */
int refpin_get_AB_arrays(const void *c, double complex *A, double complex *B, size_t nelem, double kr_re,
                         double kr_im, double theta, double phi, int r_ge_d, int J) {
  csph_t kd;
  kd.r = kr_re + I * kr_im;
  kd.theta = theta;
  kd.phi = phi;
  return qpms_trans_calculator_get_AB_arrays((const qpms_trans_calculator *)c, A, B, nelem, 1, kd, r_ge_d != 0,
                                             (qpms_bessel_t)J);
}

/* Lattice-summed A, B (and their error estimates) for a 2D lattice b1, b2,
 * Bloch vector beta, particle shift, at wavenumber k, Ewald parameter eta,
 * direct/reciprocal cut-offs maxR/maxK; full sums. */
int refpin_get_AB_arrays_e32(const void *c, double complex *A, double *Aerr, double complex *B, double *Berr,
                             size_t nelem, double eta, double k_re, double k_im, double b1x, double b1y, double b2x,
                             double b2y, double betax, double betay, double sx, double sy, double sz, double maxR,
                             double maxK) {
  cart2_t b1 = {b1x, b1y}, b2 = {b2x, b2y}, beta = {betax, betay};
  cart3_t sh = {sx, sy, sz};
  return qpms_trans_calculator_get_AB_arrays_e32((const qpms_trans_calculator *)c, A, Aerr, B, Berr,
                                                 (ptrdiff_t)nelem, 1, eta, k_re + I * k_im, b1, b2, beta, sh, maxR,
                                                 maxK);
}
