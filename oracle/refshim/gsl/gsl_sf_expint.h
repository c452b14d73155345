/* Minimal stand-in for GSL's gsl_sf_expint.h (oracle test infrastructure). */
#ifndef QG_REFSHIM_GSL_SF_EXPINT_H
#define QG_REFSHIM_GSL_SF_EXPINT_H
#include "gsl_sf_result.h"
int gsl_sf_expint_En_e(const int n, const double x, gsl_sf_result *result);
#endif
