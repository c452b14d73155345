/* Minimal stand-in for GSL's gsl_sf_legendre.h: the associated Legendre array
 * API the reference calls, implemented over the oracle's recurrences
 * (oracle test infrastructure). */
#ifndef QG_REFSHIM_GSL_SF_LEGENDRE_H
#define QG_REFSHIM_GSL_SF_LEGENDRE_H
#include <stddef.h>
typedef enum { GSL_SF_LEGENDRE_SCHMIDT, GSL_SF_LEGENDRE_SPHARM, GSL_SF_LEGENDRE_FULL, GSL_SF_LEGENDRE_NONE } gsl_sf_legendre_t;
int gsl_sf_legendre_array_e(const gsl_sf_legendre_t norm, const size_t lmax, const double x, const double csphase,
                            double result_array[]);
size_t gsl_sf_legendre_array_n(const size_t lmax);
size_t gsl_sf_legendre_array_index(const size_t l, const size_t m);
#endif
