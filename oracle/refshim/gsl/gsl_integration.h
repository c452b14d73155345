/* Minimal stand-in for GSL's gsl_integration.h: semi-infinite adaptive
 * quadrature over the oracle's QUADPACK-style integrator (oracle test
 * infrastructure). */
#ifndef QG_REFSHIM_GSL_INTEGRATION_H
#define QG_REFSHIM_GSL_INTEGRATION_H
#include <float.h>
#include <math.h>
#include <stddef.h>
typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;
typedef struct gsl_integration_workspace_s {
  size_t limit;
} gsl_integration_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(const size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace *workspace, double *result, double *abserr);
#endif
