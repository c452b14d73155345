/* Minimal stand-in for GSL's gsl_sf_bessel.h: nothing of it is called by the
 * reference sources compiled for the oracle (its Bessel fill is supplied). */
#ifndef QG_REFSHIM_GSL_SF_BESSEL_H
#define QG_REFSHIM_GSL_SF_BESSEL_H
#endif
