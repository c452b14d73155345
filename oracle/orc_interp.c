/*
 * Oracle interpolation (test infrastructure only; see orc.h).
 *
 * The reference interpolates tabulated permittivities and T-matrices with
 * GSL (materials.c:11-30, 120-129; tmatrices.c:287-350), gsl_interp_cspline
 * from its Python layer (cymaterials.pyx:259, cytmatrices.pyx:38-39) and
 * gsl_interp_linear declared beside it.  GSL (2.x) is absent here; restated
 * from the published definitions:
 *   linear  y = y_i + (x - x_i) (y_{i+1} - y_i) / (x_{i+1} - x_i)
 *   cspline natural cubic spline: second derivatives M_i from
 *           h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1}
 *             = 6 ((y_{i+1} - y_i)/h_i - (y_i - y_{i-1})/h_{i-1}),  M_0 = M_{n-1} = 0,
 *           evaluated in the A/B form y = A y_i + B y_{i+1}
 *             + ((A^3 - A) M_i + (B^3 - B) M_{i+1}) h_i^2 / 6.
 * Outside [x_0, x_{n-1}]: NaN (gsl_interp_eval's GSL_EDOM).
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>

void orc_spline_eval(int kind, int n, const double *x, const double *y, int nq, const double *xq, double *out) {
  double *M = calloc(n, sizeof(double));
  if (kind == 1 && n >= 3) {
    /* Gaussian elimination of the tridiagonal system (unknowns M_1..M_{n-2}) */
    int m = n - 2;
    double *a = malloc(m * sizeof(double)), *b = malloc(m * sizeof(double)), *c = malloc(m * sizeof(double)),
           *r = malloc(m * sizeof(double));
    for (int j = 0; j < m; ++j) {
      int i = j + 1;
      double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
      a[j] = h0;
      b[j] = 2 * (h0 + h1);
      c[j] = h1;
      r[j] = 6 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
    }
    for (int j = 1; j < m; ++j) {
      double f = a[j] / b[j - 1];
      b[j] -= f * c[j - 1];
      r[j] -= f * r[j - 1];
    }
    for (int j = m - 1; j >= 0; --j) M[j + 1] = (r[j] - (j + 1 < m ? c[j] * M[j + 2] : 0)) / b[j];
    free(a);
    free(b);
    free(c);
    free(r);
  }
  for (int q = 0; q < nq; ++q) {
    double v = xq[q];
    if (!(v >= x[0] && v <= x[n - 1])) {
      out[q] = NAN;
      continue;
    }
    int i = 0;
    while (i < n - 2 && x[i + 1] <= v) ++i; /* linear scan: x_i <= v */
    double h = x[i + 1] - x[i];
    double A = (x[i + 1] - v) / h, B = (v - x[i]) / h;
    double s = A * y[i] + B * y[i + 1];
    if (kind == 1) s += ((A * A * A - A) * M[i] + (B * B * B - B) * M[i + 1]) * h * h / 6;
    out[q] = s;
  }
  free(M);
}
