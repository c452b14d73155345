/* Minimal stand-in for GSL's gsl_sf_gamma.h (oracle test infrastructure). */
#ifndef QG_REFSHIM_GSL_SF_GAMMA_H
#define QG_REFSHIM_GSL_SF_GAMMA_H
#include "gsl_sf_result.h"
#define GSL_SF_GAMMA_XMAX 171.0
int gsl_sf_gamma_e(const double x, gsl_sf_result *result);
int gsl_sf_gamma_inc_e(const double a, const double x, gsl_sf_result *result);
#endif
