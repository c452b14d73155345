/*
 * Oracle special functions (test infrastructure only; see orc.h).
 *
 * Replaces the reference's third-party numerics on the translation path:
 *   - gsl_sf_coupling_3j            -> orc_wigner3j      (Racah formula)
 *   - gaunt_xu (gaunt.c:396-1179)   -> orc_gaunt         (Gaunt via two 3j symbols)
 *   - gsl_sf_legendre_array_e NONE  -> orc_legendre_array (three-term recurrences, DLMF 14.10.3/14.10.6)
 *   - GSL jl_steed/yl_array, AMOS zbesj/zbesy/zbesh
 *                                   -> orc_sph_bessel_fill (Miller backward recurrence
 *                                      for j, forward recurrence for y and h; DLMF 10.51.1)
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXFACT 400
static long double orc_fact_tab[ORC_MAXFACT + 1];
static int orc_fact_ready = 0;

static long double F(int n) {
  if (!orc_fact_ready) {
    orc_fact_tab[0] = 1.0L;
    for (int i = 1; i <= ORC_MAXFACT; ++i) orc_fact_tab[i] = orc_fact_tab[i - 1] * (long double)i;
    orc_fact_ready = 1;
  }
  if (n < 0 || n > ORC_MAXFACT) abort();
  return orc_fact_tab[n];
}

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }
static int m1pow(int p) { return (p % 2) ? -1 : 1; }

double orc_wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0;
  if (j1 < 0 || j2 < 0 || j3 < 0) return 0;
  if (j3 < abs(j1 - j2) || j3 > j1 + j2) return 0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0;
  long double tri = F(j1 + j2 - j3) * F(j1 - j2 + j3) * F(-j1 + j2 + j3) / F(j1 + j2 + j3 + 1);
  long double pre = sqrtl(tri * F(j1 + m1) * F(j1 - m1) * F(j2 + m2) * F(j2 - m2)
                          * F(j3 + m3) * F(j3 - m3));
  int kmin = imax(0, imax(j2 - j3 - m1, j1 - j3 + m2));
  int kmax = imin(j1 + j2 - j3, imin(j1 - m1, j2 + m2));
  long double s = 0;
  for (int k = kmin; k <= kmax; ++k) {
    long double den = F(k) * F(j3 - j2 + k + m1) * F(j3 - j1 + k - m2) * F(j1 + j2 - j3 - k)
                      * F(j1 - k - m1) * F(j2 - k + m2);
    s += (k % 2 ? -1.0L : 1.0L) / den;
  }
  return (double)(m1pow(j1 - j2 - m3) * pre * s);
}

/* gaunt.h:6-8 */
int orc_gaunt_q_max(int m, int n, int mu, int nu) {
  return imin(n, imin(nu, (n + nu - abs(m + mu)) / 2));
}

/* Gaunt coefficient of P_n^m P_nu^mu -> P_p^{m+mu}.  Only the ratios a_q/a_0
 * enter the translation multipliers (translations.c:321-343). */
int orc_gaunt(int m, int n, int mu, int nu, double *aq) {
  int qmax = orc_gaunt_q_max(m, n, mu, nu);
  int M = m + mu;
  for (int q = 0; q <= qmax; ++q) {
    int p = n + nu - 2 * q;
    long double w0 = orc_wigner3j(n, nu, p, 0, 0, 0);
    long double wm = orc_wigner3j(n, nu, p, m, mu, -M);
    long double r = sqrtl(F(n + m) * F(nu + mu) * F(p - M) / (F(n - m) * F(nu - mu) * F(p + M)));
    aq[q] = (double)(m1pow(M) * (2 * p + 1) * r * w0 * wm);
  }
  return qmax;
}

/* GSL_SF_LEGENDRE_NONE array, index l(l+1)/2 + m. */
void orc_legendre_array(int L, double x, double csphase, double *out) {
  const double u = sqrt((1.0 - x) * (1.0 + x));
  double pmm = 1.0; /* P_m^m */
  for (int m = 0; m <= L; ++m) {
    if (m > 0) pmm *= csphase * (2 * m - 1) * u;
    out[m * (m + 1) / 2 + m] = pmm;
    if (m + 1 <= L) {
      double pm1 = x * (2 * m + 1) * pmm;
      out[(m + 1) * (m + 2) / 2 + m] = pm1;
      double pl2 = pmm, pl1 = pm1;
      for (int l = m + 2; l <= L; ++l) {
        double pl = ((2 * l - 1) * x * pl1 - (l + m - 1) * pl2) / (l - m);
        out[l * (l + 1) / 2 + m] = pl;
        pl2 = pl1;
        pl1 = pl;
      }
    }
  }
}

/* Regular spherical Bessel j_l(x), l=0..lmax, by Miller's backward recurrence
 * normalised with j_0 = sin x / x or j_1 (whichever is larger). */
static void orc_sph_j_miller(int lmax, double complex x, double complex *res) {
  if (x == 0) {
    res[0] = 1;
    for (int l = 1; l <= lmax; ++l) res[l] = 0;
    return;
  }
  double ax = cabs(x);
  int N = lmax + 30 + (int)(1.5 * ax);
  double complex *f = malloc(sizeof(double complex) * (N + 2));
  f[N + 1] = 0;
  f[N] = 1e-300;
  for (int l = N; l >= 1; --l) {
    f[l - 1] = (2 * l + 1) / x * f[l] - f[l + 1];
    if (cabs(f[l - 1]) > 1e250) { /* rescale everything computed so far */
      for (int k = l - 1; k <= N + 1; ++k) f[k] *= 1e-250;
    }
  }
  double complex j0 = csin(x) / x;
  double complex j1 = csin(x) / (x * x) - ccos(x) / x;
  double complex scale = (cabs(j0) >= cabs(j1)) ? j0 / f[0] : j1 / f[1];
  for (int l = 0; l <= lmax; ++l) res[l] = f[l] * scale;
  free(f);
}

/* Forward recurrence z_{l+1} = (2l+1)/x z_l - z_{l-1} (DLMF 10.51.1); stable
 * for the dominant solutions y, h+ and h-. */
static void orc_sph_forward(int lmax, double complex x, double complex z0, double complex z1,
                            double complex *res) {
  res[0] = z0;
  if (lmax >= 1) res[1] = z1;
  for (int l = 1; l < lmax; ++l) res[l + 1] = (2 * l + 1) / x * res[l] - res[l - 1];
}

int orc_sph_bessel_fill(int J, int lmax, double complex x, double complex *res) {
  if (lmax < 0) return 1;
  if (isnan(creal(x)) || isnan(cimag(x))) {
    for (int l = 0; l <= lmax; ++l) res[l] = NAN + I * NAN;
    return 0;
  }
  double complex *jb = malloc(sizeof(double complex) * (lmax + 1));
  double complex *yb = malloc(sizeof(double complex) * (lmax + 1));
  int ret = 0;
  switch (J) {
    case 1:
      orc_sph_j_miller(lmax, x, res);
      break;
    case 2:
      orc_sph_forward(lmax, x, -ccos(x) / x, -ccos(x) / (x * x) - csin(x) / x, res);
      break;
    case 3:
    case 4:
      if (cimag(x) == 0) {
        /* real x: j (Steed in GSL) and y (forward) separately, bessel.c:52-83 */
        orc_sph_j_miller(lmax, x, jb);
        orc_sph_forward(lmax, x, -ccos(x) / x, -ccos(x) / (x * x) - csin(x) / x, yb);
        double s = (J == 3) ? 1.0 : -1.0;
        for (int l = 0; l <= lmax; ++l) res[l] = jb[l] + s * I * yb[l];
      } else {
        /* complex x: h directly (AMOS zbesh in the reference, bessel.c:121-127) */
        if (J == 3) {
          double complex e = cexp(I * x);
          orc_sph_forward(lmax, x, -I * e / x, -e * (x + I) / (x * x), res);
        } else {
          double complex e = cexp(-I * x);
          orc_sph_forward(lmax, x, I * e / x, -e * (x - I) / (x * x), res);
        }
      }
      break;
    default:
      ret = 1;
  }
  free(jb);
  free(yb);
  return ret;
}
