/* Minimal stand-in for GSL's gsl_sf_result.h: the result type the reference's
 * headers name (oracle test infrastructure; the values come from oracle/). */
#ifndef QG_REFSHIM_GSL_SF_RESULT_H
#define QG_REFSHIM_GSL_SF_RESULT_H
typedef struct {
  double val;
  double err;
} gsl_sf_result;
#endif
