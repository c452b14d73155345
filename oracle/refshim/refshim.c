/* The few GSL, AMOS-backed and Faddeeva functions that the reference's own
 * translations.c, ewald.c and ewaldsf.c call, implemented over the oracle's
 * restatements (orc_specfunc.c, orc_ewald.c), so that those reference files
 * compile and run here unchanged (oracle/_ref).  Test infrastructure only: the
 * library never links this.
 *
 *   gsl_sf_legendre_array_e (NONE)  -> orc_legendre_array
 *   gsl_sf_coupling_3j              -> orc_wigner3j (integer momenta only)
 *   qpms_sph_bessel_fill (bessel.c, AMOS) -> orc_sph_bessel_fill
 *   gsl_sf_gamma_inc_e, gsl_sf_expint_En_e -> orc_complex_gamma_inc on the real axis
 *   gsl_integration_qagiu           -> orc_qagiu (QUADPACK-style QAGI)
 *   gsl_sf_gamma_e, gsl_sf_exp_err_e -> C99 tgamma / exp
 *   Faddeeva_w                      -> NaN (used only by the shifted-layer sums)
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "../orc.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_machine.h"
#include "gsl/gsl_sf_coupling.h"
#include "gsl/gsl_sf_exp.h"
#include "gsl/gsl_sf_expint.h"
#include "gsl/gsl_sf_gamma.h"
#include "gsl/gsl_sf_legendre.h"
#include "cblas.h"
#include "Faddeeva.h"

/* ---- errors ---- */
static gsl_error_handler_t *g_handler = NULL;

gsl_error_handler_t *gsl_set_error_handler(gsl_error_handler_t *h) {
  gsl_error_handler_t *old = g_handler;
  g_handler = h;
  return old;
}
gsl_error_handler_t *gsl_set_error_handler_off(void) { return gsl_set_error_handler(NULL); }
void gsl_error(const char *reason, const char *file, int line, int gsl_errno) {
  if (g_handler) g_handler(reason, file, line, gsl_errno);
}
void gsl_stream_printf(const char *label, const char *file, int line, const char *reason) {
  fprintf(stderr, "%s:%d: %s: %s\n", file, line, label, reason);
}
const char *gsl_strerror(const int gsl_errno) {
  (void)gsl_errno;
  return "gsl error (oracle stand-in)";
}

/* ---- Legendre ---- */
size_t gsl_sf_legendre_array_n(const size_t lmax) { return (lmax + 1) * (lmax + 2) / 2; }
size_t gsl_sf_legendre_array_index(const size_t l, const size_t m) { return l * (l + 1) / 2 + m; }
int gsl_sf_legendre_array_e(const gsl_sf_legendre_t norm, const size_t lmax, const double x, const double csphase,
                            double result_array[]) {
  if (norm != GSL_SF_LEGENDRE_NONE || x < -1 || x > 1) return GSL_EDOM;
  orc_legendre_array((int)lmax, x, csphase, result_array);
  return GSL_SUCCESS;
}

/* ---- 3j ---- */
double gsl_sf_coupling_3j(int two_ja, int two_jb, int two_jc, int two_ma, int two_mb, int two_mc) {
  if ((two_ja | two_jb | two_jc | two_ma | two_mb | two_mc) & 1) return NAN;  /* half-integers: not needed */
  return orc_wigner3j(two_ja / 2, two_jb / 2, two_jc / 2, two_ma / 2, two_mb / 2, two_mc / 2);
}

/* ---- spherical Bessel functions (the reference's bessel.c needs AMOS) ---- */
int qpms_sph_bessel_fill(int typ, int lmax, double complex x, double complex *result_array) {
  return orc_sph_bessel_fill(typ, lmax, x, result_array);
}

/* ---- gamma, incomplete gamma, E_n, exp ---- */
int gsl_sf_gamma_e(const double x, gsl_sf_result *result) {
  if (x <= 0 && x == floor(x)) {
    result->val = NAN;
    result->err = NAN;
    return GSL_EDOM;
  }
  if (x > GSL_SF_GAMMA_XMAX) {
    result->val = INFINITY;
    result->err = INFINITY;
    return GSL_EOVRFLW;
  }
  result->val = tgamma(x);
  result->err = 2 * GSL_DBL_EPSILON * fabs(result->val);
  return GSL_SUCCESS;
}
int gsl_sf_gamma_inc_e(const double a, const double x, gsl_sf_result *result) {
  if (x < 0) return GSL_EDOM;
  result->val = creal(orc_complex_gamma_inc(a, x + 0.0 * I, 0));
  result->err = 4 * GSL_DBL_EPSILON * fabs(result->val);
  return GSL_SUCCESS;
}
int gsl_sf_expint_En_e(const int n, const double x, gsl_sf_result *result) {
  /* E_n(x) = x^(n-1) Gamma(1 - n, x) */
  if (x <= 0 && n <= 1) return GSL_EDOM;
  result->val = pow(x, n - 1) * creal(orc_complex_gamma_inc(1.0 - n, x + 0.0 * I, 0));
  result->err = 4 * GSL_DBL_EPSILON * fabs(result->val);
  return GSL_SUCCESS;
}
int gsl_sf_exp_err_e(const double x, const double dx, gsl_sf_result *result) {
  result->val = exp(x);
  result->err = result->val * (dx + 2 * GSL_DBL_EPSILON);
  return isfinite(result->val) ? GSL_SUCCESS : GSL_EOVRFLW;
}

/* ---- quadrature ---- */
gsl_integration_workspace *gsl_integration_workspace_alloc(const size_t n) {
  gsl_integration_workspace *w = malloc(sizeof *w);
  if (w) w->limit = n;
  return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

static double qagiu_trampoline(double x, const void *p) {
  const gsl_function *f = (const gsl_function *)p;
  return f->function(x, f->params);
}
int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace *workspace, double *result, double *abserr) {
  (void)limit;
  (void)workspace;
  *result = orc_qagiu(qagiu_trampoline, f, a, epsabs, epsrel, abserr);
  return isfinite(*result) ? GSL_SUCCESS : GSL_EFAILED;
}

/* ---- Faddeeva ---- */
double complex Faddeeva_w(double complex z, double relerr) {
  (void)z;
  (void)relerr;
  return NAN;
}

/* ---- the three level-1 BLAS loops of the reference's lll.c ---- */
void cblas_daxpy(const int n, const double alpha, const double *x, const int incx, double *y, const int incy) {
  for (int i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}
double cblas_ddot(const int n, const double *x, const int incx, const double *y, const int incy) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
  return s;
}
void cblas_dswap(const int n, double *x, const int incx, double *y, const int incy) {
  for (int i = 0; i < n; ++i) {
    const double t = x[(size_t)i * incx];
    x[(size_t)i * incx] = y[(size_t)i * incy];
    y[(size_t)i * incy] = t;
  }
}
