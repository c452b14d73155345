/*
 * Oracle VSWF translation operator (test infrastructure only; see orc.h).
 *
 * Restates qpms/translations.c of the reference:
 *   multipliers_A        translations.c:313-368   (Xu (61) form, AN1 phase default, :29-32)
 *   cruzan_bfactor       translations.c:372-379
 *   multipliers_B        translations.c:382-437   (BN1 phase default, :37-40)
 *   calculator_init      translations.c:439-508
 *   get_A/B_precalcbuf   translations.c:510-527, 550-567 (Kahan sums, kahansum.h)
 *   get_AB_arrays_buf    translations.c:610-658 (r == 0 && J != 1 -> NaN fill)
 *   trans_single_A/B     translations.c:135-286
 * with the normalisation factors of normalisation.h:17-90 and the index maps
 * of indexing.h:13-27.
 */
#include "orc.h"
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdlib.h>
#include <string.h>

/* qpms_normalisation_t bits, qpms_types.h:104-168 */
#define N_INVERSE 1
#define N_REVERSE_AZ 2
#define N_SPHARM_REAL 4
#define N_CSPHASE 8
#define N_M_I 16
#define N_M_MINUS 32
#define N_N_I 64
#define N_N_MINUS 128
#define N_BITSTART 65536
#define N_NORM_POWER (N_BITSTART * 1)
#define N_NORM_NONE (N_BITSTART * 2)
#define N_NORM_SPHARM (N_BITSTART * 3)
#define N_NORM_BITS (N_NORM_POWER | N_NORM_NONE | N_NORM_SPHARM)

static int m1pow(int p) { return (p % 2) ? -1 : 1; }
static double complex ipow(int x) {
  x = ((x % 4) + 4) % 4;
  switch (x) {
    case 0: return 1;
    case 1: return I;
    case 2: return -1;
    default: return -I;
  }
}
static int imin(int a, int b) { return a < b ? a : b; }
static int isq(int x) { return x * x; }

static int y2n(int y) { return (int)sqrt((double)y + 1); }
static void y2mn(int y, int *m, int *n) { *n = y2n(y); *m = y - ((*n) * ((*n) + 1) - 1); }
static int mn2y(int m, int n) { return n * (n + 1) + m - 1; }

static int csphase_of(int norm) { return (norm & N_CSPHASE) ? -1 : 1; }

/* normalisation.h:17-31 */
static double normfactor(int norm, int l, int m) {
  switch (norm & N_NORM_BITS) {
    case N_NORM_POWER: return 1;
    case N_NORM_SPHARM: return sqrt(l * (l + 1));
    case N_NORM_NONE:
      return sqrt(l * (l + 1) * 4 * M_PI / (2 * l + 1)) * exp(0.5 * (lgamma(l + m + 1) - lgamma(l - m + 1)));
    default: abort();
  }
}
/* normalisation.h:39-46 */
static double complex factor_M_noCS(int norm, int l, int m) {
  double complex f = normfactor(norm, l, m);
  if (norm & N_M_MINUS) f *= -1;
  if (norm & N_M_I) f *= I;
  if (norm & N_INVERSE) f = 1 / f;
  return f;
}
/* normalisation.h:66-73 */
static double complex factor_N_noCS(int norm, int l, int m) {
  double complex f = normfactor(norm, l, m);
  if (norm & N_N_MINUS) f *= -1;
  if (norm & N_N_I) f *= I;
  if (norm & N_INVERSE) f = 1 / f;
  return f;
}

/* translations.c:112-114 */
static int gauntB_Q_max(int M, int n, int mu, int nu) {
  return imin(n, imin(nu, (n + nu + 1 - abs(M + mu)) / 2));
}
/* translations.c:116-119 */
static double trans_normlogfac(int m, int n, int mu, int nu) {
  return -0.5 * (lgamma(n + m + 1) - lgamma(n - m + 1) + lgamma(nu - mu + 1) - lgamma(nu + mu + 1));
}
/* translations.c:121-133 */
static double trans_normfac(int norm, int m, int n, int mu, int nu) {
  int csphase = csphase_of(norm);
  double normfac = (1 == csphase) ? m1pow(m - mu) : 1.;
  normfac *= sqrt((n * (n + 1.)) / (nu * (nu + 1.)));
  normfac *= sqrt((2. * n + 1) / (2. * nu + 1));
  return normfac;
}

/* translations.c:313-368.  `normfac` is a double there, so the complex ratio
 * of normalisation factors is reduced to its real part on assignment. */
static void multipliers_A(int norm, double complex *dest, int m, int n, int mu, int nu, int qmax) {
  double a1q[qmax + 1];
  int qm = orc_gaunt(-m, n, mu, nu, a1q);
  (void)qm;
  double a1q0 = a1q[0];
  double normlogfac = trans_normlogfac(m, n, mu, nu);
  double normfac = trans_normfac(norm, m, n, mu, nu);
  normfac *= creal(factor_N_noCS(norm, nu, mu) / factor_N_noCS(norm, n, m));
  normfac *= m1pow(m);
  double exponent = (lgamma(2 * n + 1) - lgamma(n + 2) + lgamma(2 * nu + 3) - lgamma(nu + 2)
                     + lgamma(n + nu + m - mu + 1) - lgamma(n - m + 1) - lgamma(nu + mu + 1)
                     + lgamma(n + nu + 1) - lgamma(2 * (n + nu) + 1))
                    + normlogfac;
  double complex presum = exp(exponent);
  presum *= normfac / (4. * n);
  presum *= ipow(n + nu);
  for (int q = 0; q <= qmax; q++) {
    int p = n + nu - 2 * q;
    int Pp_order = mu - m;
    double a1q_n = a1q[q] / a1q0;
    double Ppfac = (Pp_order >= 0) ? 1 : m1pow(mu - m) * exp(lgamma(1 + p + Pp_order) - lgamma(1 + p - Pp_order));
    double summandfac = (n * (n + 1) + nu * (nu + 1) - p * (p + 1)) * m1pow(q) * a1q_n;
    dest[q] = presum * summandfac * Ppfac * ipow(n - nu);
  }
}

/* translations.c:372-379, Xu (61) */
static double cruzan_bfactor(int M, int n, int mu, int nu, int p) {
  double logprefac = lgamma(n + M + 1) - lgamma(n - M + 1) + lgamma(nu + mu + 1) - lgamma(nu - mu + 1)
                     + lgamma(p - M - mu + 2) - lgamma(p + M + mu + 2);
  logprefac *= 0.5;
  return m1pow(mu + M) * (2 * p + 3) * exp(logprefac)
         * orc_wigner3j(n, nu, p + 1, M, mu, -M - mu) * orc_wigner3j(n, nu, p, 0, 0, 0);
}

/* translations.c:382-437 */
static void multipliers_B(int norm, double complex *dest, int m, int n, int mu, int nu, int Qmax) {
  double normlogfac = trans_normlogfac(m, n, mu, nu);
  double normfac = trans_normfac(norm, m, n, mu, nu);
  normfac *= creal(factor_M_noCS(norm, nu, mu) / factor_N_noCS(norm, n, m));
  double presum = m1pow(1 - m) * (2 * nu + 1) / (2. * (n * (n + 1)))
                  * exp(lgamma(n + m + 1) - lgamma(n - m + 1) + lgamma(nu - mu + 1) - lgamma(nu + mu + 1) + normlogfac)
                  * normfac;
  for (int q = 0; q <= Qmax; ++q) {
    int p = n + nu - 2 * q;
    int Pp_order = mu - m;
    double Ppfac_ = (Pp_order >= 0) ? 1 : m1pow(mu - m) * exp(lgamma(1 + 1 + p + Pp_order) - lgamma(1 + 1 + p - Pp_order));
    double t = sqrt((double)(isq(p + 1) - isq(n - nu)) * (double)(isq(n + nu + 1) - isq(p + 1)));
    dest[q] = presum * t * Ppfac_ * cruzan_bfactor(-m, n, mu, nu, p) * ipow(p + 1) * ipow(n - nu);
  }
}

orc_trans_calculator *orc_trans_calculator_init(int lMax, int normalisation) {
  if (lMax <= 0) return NULL;
  orc_trans_calculator *c = malloc(sizeof(*c));
  c->lMax = lMax;
  c->nelem = lMax * (lMax + 2);
  c->normalisation = normalisation;
  const int ne = c->nelem;
  c->A_multipliers = malloc((1 + (size_t)ne * ne) * sizeof(double complex *));
  c->B_multipliers = malloc((1 + (size_t)ne * ne) * sizeof(double complex *));
  int *qmA = malloc(sizeof(int) * ne * ne), *qmB = malloc(sizeof(int) * ne * ne);
  size_t sumA = 0, sumB = 0;
  for (int y = 0; y < ne; ++y)
    for (int yu = 0; yu < ne; ++yu) {
      int m, n, mu, nu;
      y2mn(y, &m, &n);
      y2mn(yu, &mu, &nu);
      qmA[y * ne + yu] = orc_gaunt_q_max(-m, n, mu, nu);
      qmB[y * ne + yu] = gauntB_Q_max(-m, n, mu, nu);
      sumA += 1 + qmA[y * ne + yu];
      sumB += 1 + qmB[y * ne + yu];
    }
  c->A_multipliers[0] = malloc(sumA * sizeof(double complex));
  c->B_multipliers[0] = malloc(sumB * sizeof(double complex));
  for (int i = 0; i < ne * ne; ++i) {
    c->A_multipliers[i + 1] = c->A_multipliers[i] + qmA[i] + 1;
    c->B_multipliers[i + 1] = c->B_multipliers[i] + qmB[i] + 1;
  }
  for (int y = 0; y < ne; ++y)
    for (int yu = 0; yu < ne; ++yu) {
      int m, n, mu, nu, i = y * ne + yu;
      y2mn(y, &m, &n);
      y2mn(yu, &mu, &nu);
      multipliers_A(normalisation, c->A_multipliers[i], m, n, mu, nu, qmA[i]);
      multipliers_B(normalisation, c->B_multipliers[i], m, n, mu, nu, qmB[i]);
    }
  free(qmA);
  free(qmB);
  return c;
}

void orc_trans_calculator_free(orc_trans_calculator *c) {
  if (!c) return;
  free(c->A_multipliers[0]);
  free(c->B_multipliers[0]);
  free(c->A_multipliers);
  free(c->B_multipliers);
  free(c);
}

size_t orc_trans_calculator_nA(const orc_trans_calculator *c) {
  return (size_t)(c->A_multipliers[(size_t)c->nelem * c->nelem] - c->A_multipliers[0]);
}
size_t orc_trans_calculator_nB(const orc_trans_calculator *c) {
  return (size_t)(c->B_multipliers[(size_t)c->nelem * c->nelem] - c->B_multipliers[0]);
}

/* kahansum.h:25-31 */
static void ckahanadd(double complex *sum, double complex *comp, double complex input) {
  double complex ci = input - *comp;
  double complex ns = *sum + ci;
  *comp = (ns - *sum) - ci;
  *sum = ns;
}

static inline int leg_idx(int l, int m) { return l * (l + 1) / 2 + m; }

/* translations.c:510-527 */
static double complex get_A_precalc(const orc_trans_calculator *c, int m, int n, int mu, int nu,
                                    double phi, const double complex *bes, const double *leg) {
  size_t i = (size_t)c->nelem * mn2y(m, n) + mn2y(mu, nu);
  size_t qmax = c->A_multipliers[i + 1] - c->A_multipliers[i] - 1;
  double complex sum = 0, kc = 0;
  for (size_t q = 0; q <= qmax; ++q) {
    int p = n + nu - 2 * (int)q;
    double Pp = leg[leg_idx(p, abs(mu - m))];
    ckahanadd(&sum, &kc, Pp * bes[p] * c->A_multipliers[i][q]);
  }
  return sum * cexp(I * (mu - m) * phi);
}

/* translations.c:550-567 */
static double complex get_B_precalc(const orc_trans_calculator *c, int m, int n, int mu, int nu,
                                    double phi, const double complex *bes, const double *leg) {
  size_t i = (size_t)c->nelem * mn2y(m, n) + mn2y(mu, nu);
  size_t qmax = c->B_multipliers[i + 1] - c->B_multipliers[i] - 1;
  double complex sum = 0, kc = 0;
  for (size_t q = 0; q <= qmax; ++q) {
    int p = n + nu - 2 * (int)q;
    double Pp_ = leg[leg_idx(p + 1, abs(mu - m))];
    ckahanadd(&sum, &kc, Pp_ * bes[p + 1] * c->B_multipliers[i][q]);
  }
  return sum * cexp(I * (mu - m) * phi);
}

/* translations.c:610-658, 1124-1132 */
int orc_trans_calculator_get_AB_arrays_ext(const orc_trans_calculator *c,
    double complex *Adest, double complex *Bdest, size_t deststride, size_t srcstride,
    double complex kdlj_r, double kdlj_theta, double kdlj_phi, int r_ge_d, int J) {
  if (r_ge_d) J = 1;
  const int ne = c->nelem;
  if (0 == kdlj_r && J != 1) {
    for (int i = 0; i < ne; ++i)
      for (int j = 0; j < ne; ++j) {
        Adest[i * srcstride + j * deststride] = NAN + I * NAN;
        Bdest[i * srcstride + j * deststride] = NAN + I * NAN;
      }
    return 0;
  }
  const int L = 2 * c->lMax + 1;
  double leg[(L + 1) * (L + 2) / 2];
  double complex bes[L + 1];
  orc_legendre_array(L, cos(kdlj_theta), -1, leg);
  if (orc_sph_bessel_fill(J, L, kdlj_r, bes)) return 1;
  size_t desti = 0, srci = 0;
  for (int n = 1; n <= c->lMax; ++n)
    for (int m = -n; m <= n; ++m) {
      for (int nu = 1; nu <= c->lMax; ++nu)
        for (int mu = -nu; mu <= nu; ++mu) {
          Adest[deststride * desti + srcstride * srci] = get_A_precalc(c, m, n, mu, nu, kdlj_phi, bes, leg);
          Bdest[deststride * desti + srcstride * srci] = get_B_precalc(c, m, n, mu, nu, kdlj_phi, bes, leg);
          ++srci;
        }
      ++desti;
      srci = 0;
    }
  return 0;
}

/* Parallel over translations with OpenMP (the reference's loop is serial,
 * translations_python.c:76; its OMP pragmas are commented out at :68-75). */
int orc_trans_AB_batch(const orc_trans_calculator *c, size_t n, const double complex *kr,
                       const double *theta, const double *phi, int J, double complex *A, double complex *B) {
  const size_t ne2 = (size_t)c->nelem * c->nelem;
  int err = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(| : err)
  for (size_t i = 0; i < n; ++i)
    err |= orc_trans_calculator_get_AB_arrays_ext(c, A + i * ne2, B + i * ne2, c->nelem, 1,
                                                  kr[i], theta[i], phi[i], 0, J);
  return err;
}

/* translations.c:135-199 */
double complex orc_trans_single_A(int norm, int m, int n, int mu, int nu, double complex kr,
                                  double theta, double phi, int r_ge_d, int J) {
  if (r_ge_d) J = 1;
  double costheta = cos(theta);
  int qmax = orc_gaunt_q_max(-m, n, mu, nu);
  double a1q[qmax + 1];
  orc_gaunt(-m, n, mu, nu, a1q);
  double a1q0 = a1q[0];
  double leg[(n + nu + 1) * (n + nu + 2) / 2];
  orc_legendre_array(n + nu, costheta, -1, leg);
  double complex bes[n + nu + 1];
  orc_sph_bessel_fill(J, n + nu, kr, bes);
  double complex sum = 0;
  for (int q = 0; q <= qmax; ++q) {
    int p = n + nu - 2 * q;
    int Pp_order = mu - m;
    double a1q_n = a1q[q] / a1q0;
    double Pp = leg[leg_idx(p, abs(Pp_order))];
    if (Pp_order < 0) Pp *= m1pow(mu - m) * exp(lgamma(1 + p + Pp_order) - lgamma(1 + p - Pp_order));
    sum += (n * (n + 1) + nu * (nu + 1) - p * (p + 1)) * m1pow(q) * a1q_n * bes[p] * Pp;
  }
  double exponent = (lgamma(2 * n + 1) - lgamma(n + 2) + lgamma(2 * nu + 3) - lgamma(nu + 2)
                     + lgamma(n + nu + m - mu + 1) - lgamma(n - m + 1) - lgamma(nu + mu + 1)
                     + lgamma(n + nu + 1) - lgamma(2 * (n + nu) + 1));
  double complex presum = exp(exponent);
  presum *= cexp(I * (mu - m) * phi) * m1pow(m) * ipow(nu + n) / (4 * n);
  double normlogfac = trans_normlogfac(m, n, mu, nu);
  double normfac = trans_normfac(norm, m, n, mu, nu);
  normfac *= creal(factor_N_noCS(norm, nu, mu) / factor_N_noCS(norm, n, m));
  presum *= (normfac * exp(normlogfac)) * ipow(n - nu);
  return presum * sum;
}

/* translations.c:202-273 */
double complex orc_trans_single_B(int norm, int m, int n, int mu, int nu, double complex kr,
                                  double theta, double phi, int r_ge_d, int J) {
  if (r_ge_d) J = 1;
  double costheta = cos(theta);
  int q2max = orc_gaunt_q_max(-m - 1, n + 1, mu + 1, nu);
  int Qmax = orc_gaunt_q_max(-m, n + 1, mu, nu);
  int realQmax = gauntB_Q_max(-m, n, mu, nu);
  double a2q[q2max + 2], a3q[Qmax + 2], a2q0, a3q0;
  if (mu == nu) {
    for (int q = 0; q <= q2max; ++q) a2q[q] = 0;
    a2q0 = 1;
  } else {
    orc_gaunt(-m - 1, n + 1, mu + 1, nu, a2q);
    a2q0 = a2q[0];
  }
  orc_gaunt(-m, n + 1, mu, nu, a3q);
  a3q0 = a3q[0];
  double leg[(n + nu + 2) * (n + nu + 3) / 2];
  orc_legendre_array(n + nu + 1, costheta, -1, leg);
  double complex bes[n + nu + 2];
  orc_sph_bessel_fill(J, n + nu + 1, kr, bes);
  double complex sum = 0;
  for (int q = 0; q <= realQmax; ++q) {
    int p = n + nu - 2 * q;
    double a2q_n = (q <= q2max) ? a2q[q] / a2q0 : 0;
    double a3q_n = (q <= Qmax) ? a3q[q] / a3q0 : 0;
    int Pp_order_ = mu - m;
    double Pp_ = leg[leg_idx(p + 1, abs(Pp_order_))];
    if (Pp_order_ < 0) Pp_ *= m1pow(mu - m) * exp(lgamma(1 + 1 + p + Pp_order_) - lgamma(1 + 1 + p - Pp_order_));
    sum += ((2 * (n + 1) * (nu - mu) * a2q_n - (-nu * (nu + 1) - n * (n + 3) - 2 * mu * (n + 1) + p * (p + 3)) * a3q_n)
            * m1pow(q) * bes[p + 1] * Pp_);
  }
  double exponent = (lgamma(2 * n + 3) - lgamma(n + 2) + lgamma(2 * nu + 3) - lgamma(nu + 2)
                     + lgamma(n + nu + m - mu + 2) - lgamma(n - m + 1) - lgamma(nu + mu + 1)
                     + lgamma(n + nu + 2) - lgamma(2 * (n + nu) + 3));
  double complex presum = exp(exponent);
  presum *= cexp(I * (mu - m) * phi) * m1pow(m) * ipow(nu + n + 1) / ((4 * n) * (n + 1) * (n + m + 1));
  double normlogfac = trans_normlogfac(m, n, mu, nu);
  double normfac = trans_normfac(norm, m, n, mu, nu);
  normfac *= creal(factor_M_noCS(norm, nu, mu) / factor_N_noCS(norm, n, m));
  presum *= (exp(normlogfac) * normfac) * ipow(n - nu);
  return presum * sum;
}

/* ---- plain-argument shims for ctypes (complex passed as re/im pairs) ---- */
int orc_sph_bessel_fill_ri(int J, int lmax, double xr, double xi, double complex *res) {
  return orc_sph_bessel_fill(J, lmax, xr + I * xi, res);
}
int orc_trans_calculator_get_AB_arrays_ri(const orc_trans_calculator *c, double complex *A,
    double complex *B, size_t deststride, size_t srcstride, double krr, double kri,
    double theta, double phi, int r_ge_d, int J) {
  return orc_trans_calculator_get_AB_arrays_ext(c, A, B, deststride, srcstride, krr + I * kri,
                                                theta, phi, r_ge_d, J);
}
void orc_trans_single_A_out(int norm, int m, int n, int mu, int nu, double krr, double kri,
                            double theta, double phi, int r_ge_d, int J, double complex *out) {
  *out = orc_trans_single_A(norm, m, n, mu, nu, krr + I * kri, theta, phi, r_ge_d, J);
}
void orc_trans_single_B_out(int norm, int m, int n, int mu, int nu, double krr, double kri,
                            double theta, double phi, int r_ge_d, int J, double complex *out) {
  *out = orc_trans_single_B(norm, m, n, mu, nu, krr + I * kri, theta, phi, r_ge_d, J);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
