/* Minimal stand-in for GSL's gsl_sf_exp.h (oracle test infrastructure). */
#ifndef QG_REFSHIM_GSL_SF_EXP_H
#define QG_REFSHIM_GSL_SF_EXP_H
#include "gsl_sf_result.h"
int gsl_sf_exp_err_e(const double x, const double dx, gsl_sf_result *result);
#endif
