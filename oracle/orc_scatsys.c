/*
 * Oracle finite scattering system (test infrastructure only; see orc.h).
 *
 * Restates, on the host, the reference's finite mode problem:
 *   Mie T-matrix        tmatrices.c:500-561 (qpms_mie_coefficients_reflection,
 *                       J_ext = regular, J_scat = Hankel+), :564-591 (diagonal fill)
 *   bspec order         vswf.c:76-92 (electric block n=1..lMax, m=-n..n, then magnetic)
 *   pi/tau              legendre.c:65-117 (incl. the |cos theta| = 1 branch)
 *   dual harmonics      vswf.c:338-379 with qpms_normalisation_dual (normalisation.h:128-133)
 *   plane wave -> VSWF  vswf.c:445-467, 480-530 (phase e^{i k.r} per particle)
 *   S blocks            translations.c:701-722, 796-812 (lc3p: kd = cart2csph(dest - src) * k)
 *                       and translations_inlines.h:213-240 (A for same type, B for cross type)
 *   M = I - T S         scatsystem.c:1283-1343 with the intended finite semantics
 *                       (self blocks S_RR = 0, as the serial packed builder, :1429-1444)
 *   LU / solve          LAPACKE_zgetrf / zgetrs row-major, scatsystem.c:2202-2273;
 *                       pivot = first max |re| + |im| (LAPACK izamax)
 *   sigma_ext           -Re(a^H f) / k^2, misc/finiterectlat-scatter.py:104-110
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_C0 299792458.0 /* materials.h:11 */

static int m1pow(int p) { return (p % 2) ? -1 : 1; }

/* tmatrices.c:500-561 */
void orc_mie_coefficients(int lMax, double a, double complex k_i, double complex k_e,
                          double complex mu_i, double complex mu_e, int J_ext, int J_scat,
                          double complex *RV, double complex *RH) {
  double complex x_i = k_i * a, x_e = k_e * a;
  double complex eta_inv_i = k_i / mu_i, eta_inv_e = k_e / mu_e;
  double complex zi[lMax + 2], ze[lMax + 2], zs[lMax + 2];
  orc_sph_bessel_fill(1, lMax + 1, x_i, zi);
  orc_sph_bessel_fill(J_ext, lMax + 1, x_e, ze);
  orc_sph_bessel_fill(J_scat, lMax + 1, x_e, zs);
  for (int l = 0; l <= lMax; ++l) {
    double complex dzi = -zi[l + 1] + l / x_i * zi[l];
    double complex dze = -ze[l + 1] + l / x_e * ze[l];
    double complex dzs = -zs[l + 1] + l / x_e * zs[l];
    double complex fi = zi[l] / x_i + dzi;
    double complex fs = zs[l] / x_e + dzs;
    double complex fe = ze[l] / x_e + dze;
    RV[l] = (-eta_inv_i * fe * zi[l] + eta_inv_e * ze[l] * fi) / (-eta_inv_e * fi * zs[l] + eta_inv_i * zi[l] * fs);
    RH[l] = (-eta_inv_e * fe * zi[l] + eta_inv_i * ze[l] * fi) / (-eta_inv_i * fi * zs[l] + eta_inv_e * zi[l] * fs);
  }
}

/* Diagonal of the sphere T-matrix in bspec order (tmatrices.c:564-606 with mu = 1). */
void orc_tmatrix_sphere_diag(int lMax, double radius, double complex omega, double complex eps_i,
                             double complex eps_e, double complex *Tdiag) {
  double complex k_i = csqrt(eps_i) * omega / ORC_C0, k_e = csqrt(eps_e) * omega / ORC_C0;
  double complex RV[lMax + 1], RH[lMax + 1];
  orc_mie_coefficients(lMax, radius, k_i, k_e, 1, 1, 1, 3, RV, RH);
  const int ne = lMax * (lMax + 2);
  for (int it = 0; it < 2; ++it)
    for (int n = 1, i = 0; n <= lMax; ++n)
      for (int m = -n; m <= n; ++m, ++i) Tdiag[it * ne + i] = it ? RH[n] : RV[n];
}

/* legendre.c:65-117: leg, pi, tau in y = n(n+1)+m-1 layout. */
static void orc_pitau(double theta, int lMax, double csphase, double *leg, double *pi, double *tau) {
  const int ne = lMax * (lMax + 2);
  double ct = cos(theta), st = sin(theta);
  if (1 == fabs(ct)) {
    memset(pi, 0, ne * sizeof(double));
    memset(tau, 0, ne * sizeof(double));
    memset(leg, 0, ne * sizeof(double));
    for (int l = 1; l <= lMax; ++l) {
      leg[l * (l + 1) - 1] = ((l % 2) ? ct : 1.) * sqrt((2 * l + 1) / (4 * M_PI * l * (l + 1)));
      double fl = 0.25 * sqrt((2 * l + 1) * M_1_PI);
      int lpar = (l % 2) ? -1 : 1;
      pi[l * (l + 1) + 1 - 1] = -((ct > 0) ? -1 : lpar) * fl * csphase;
      pi[l * (l + 1) - 1 - 1] = -((ct > 0) ? -1 : lpar) * fl * csphase;
      tau[l * (l + 1) + 1 - 1] = ((ct > 0) ? +1 : lpar) * fl * csphase;
      tau[l * (l + 1) - 1 - 1] = -((ct > 0) ? +1 : lpar) * fl * csphase;
    }
    return;
  }
  /* GSL_SF_LEGENDRE_SPHARM normalised P and dP/dx (csphase), negative m by (-1)^m
   * (legendre.c:11-41), then the power-normalisation factor 1/sqrt(l(l+1)). */
  double P[(lMax + 2) * (lMax + 3) / 2];
  orc_legendre_array(lMax + 1, ct, csphase, P);
  for (int l = 1; l <= lMax; ++l) {
    for (int m = 0; m <= l; ++m) {
      double plm = P[l * (l + 1) / 2 + m];
      double plm1 = (l - 1 >= m) ? P[(l - 1) * l / 2 + m] : 0.0;
      /* (x^2 - 1) dP_l^m/dx = l x P_l^m - (l + m) P_{l-1}^m */
      double dplm = (l * ct * plm - (l + m) * plm1) / (ct * ct - 1);
      double nf = sqrt((2 * l + 1) / (4 * M_PI) * exp(lgamma(l - m + 1) - lgamma(l + m + 1)));
      double pref = 1. / sqrt(l * (l + 1.));
      double Lv = nf * plm * pref, Dv = nf * dplm * pref;
      int yp = l * (l + 1) + m - 1, ym = l * (l + 1) - m - 1;
      leg[yp] = Lv;
      pi[yp] = m / st * Lv;
      tau[yp] = -st * Dv;
      if (m > 0) {
        double f = m1pow(m);
        leg[ym] = f * Lv;
        pi[ym] = -m / st * f * Lv;
        tau[ym] = -st * f * Dv;
      }
    }
  }
}

/* Plane wave (k real, unit direction given by k_cart) -> electric/magnetic
 * coefficients for QPMS_NORMALISATION_DEFAULT (vswf.c:338-379, 445-467).
 * E_sph: amplitude in the local (r, theta, phi) basis at the k direction. */
static void orc_planewave2vswf(double theta, double phi, const double complex E_sph[3], int lMax,
                               double complex *mg, double complex *el) {
  const int ne = lMax * (lMax + 2);
  double leg[ne], pi[ne], tau[ne];
  /* dual normalisation of the default: INVERSE and REVERSE_AZIMUTHAL_PHASE set,
   * norm factors 1, csphase -1, azimuthal part e^{-im phi}, derivative/m = -i e^{-im phi} */
  orc_pitau(theta, lMax, -1.0, leg, pi, tau);
  for (int l = 1, y = 0; l <= lMax; ++l) {
    double complex i_l = cpow(I, l), i_l1 = cpow(I, l + 1);
    /* exact powers of i, as ipowl (vswf.c:430-443) */
    switch (l % 4) { case 0: i_l = 1; break; case 1: i_l = I; break; case 2: i_l = -1; break; default: i_l = -I; }
    switch ((l + 1) % 4) { case 0: i_l1 = 1; break; case 1: i_l1 = I; break; case 2: i_l1 = -1; break; default: i_l1 = -I; }
    double complex prefac1 = 4 * M_PI * i_l, prefac23 = -4 * M_PI * i_l1;
    for (int m = -l; m <= l; ++m, ++y) {
      double complex eimf = cexp(-I * m * phi);
      double complex deimf = (m == 0) ? 0 : -I * cexp(-I * m * phi);
      /* A1 (M dual): (0, pi deimf, -tau eimf);  A2 (N dual): (0, tau eimf, pi deimf) */
      double complex a1t = pi[y] * deimf, a1p = -tau[y] * eimf;
      double complex a2t = tau[y] * eimf, a2p = pi[y] * deimf;
      mg[y] = prefac1 * (a1t * E_sph[1] + a1p * E_sph[2]);
      el[y] = prefac23 * (a2t * E_sph[1] + a2p * E_sph[2]);
    }
  }
}

/* qpms_scatsys_incident_field_vector_full with qpms_incfield_planewave
 * (scatsystem.c:1970-1983, vswf.c:480-530): per particle 2*nelem coefficients
 * in bspec order (electric, then magnetic). */
void orc_planewave_full(int lMax, int np, const double *pos, const double k_cart[3],
                        const double complex E_cart[3], double complex *out) {
  const int ne = lMax * (lMax + 2);
  double kn = sqrt(k_cart[0] * k_cart[0] + k_cart[1] * k_cart[1] + k_cart[2] * k_cart[2]);
  double th = kn ? acos(k_cart[2] / kn) : M_PI_2, ph = atan2(k_cart[1], k_cart[0]);
  double st = sin(th), ct = cos(th), sf = sin(ph), cf = cos(ph);
  double complex Es[3];
  Es[0] = E_cart[0] * st * cf + E_cart[1] * st * sf + E_cart[2] * ct;
  Es[1] = E_cart[0] * ct * cf + E_cart[1] * ct * sf - E_cart[2] * st;
  Es[2] = -E_cart[0] * sf + E_cart[1] * cf;
  double complex mg[ne], el[ne];
  orc_planewave2vswf(th, ph, Es, lMax, mg, el);
  for (int p = 0; p < np; ++p) {
    const double *r = pos + 3 * p;
    double complex phase = cexp(I * (k_cart[0] * r[0] + k_cart[1] * r[1] + k_cart[2] * r[2]));
    for (int y = 0; y < ne; ++y) {
      out[p * 2 * ne + y] = phase * el[y];
      out[p * 2 * ne + ne + y] = phase * mg[y];
    }
  }
}

/* Full M = I - T S for a finite system of np particles with a common bspec
 * (lMax) and per-particle dense T (n x n, row-major, T + p*n*n).
 * Row-major N x N output, N = np * n, n = 2 nelem. */
int orc_finite_modeproblem(const orc_trans_calculator *c, int np, const double *pos,
                           const double complex *T, double complex k, double complex *M) {
  const int ne = c->nelem, n = 2 * ne;
  const size_t N = (size_t)np * n;
  memset(M, 0, N * N * sizeof(double complex));
  double complex *A = malloc(sizeof(double complex) * ne * ne), *B = malloc(sizeof(double complex) * ne * ne);
  double complex *S = malloc(sizeof(double complex) * n * n);
  for (int R = 0; R < np; ++R) {
    for (int Cc = 0; Cc < np; ++Cc) {
      if (R == Cc) continue;
      double d[3] = {pos[3 * R] - pos[3 * Cc], pos[3 * R + 1] - pos[3 * Cc + 1], pos[3 * R + 2] - pos[3 * Cc + 2]};
      double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double th = r ? acos(d[2] / r) : M_PI_2, ph = atan2(d[1], d[0]);
      orc_trans_calculator_get_AB_arrays_ext(c, A, B, ne, 1, r * k, th, ph, 0, 3);
      for (int ti = 0; ti < 2; ++ti)
        for (int yi = 0; yi < ne; ++yi)
          for (int tj = 0; tj < 2; ++tj)
            for (int yj = 0; yj < ne; ++yj)
              S[(ti * ne + yi) * n + tj * ne + yj] = (ti == tj) ? A[yi * ne + yj] : B[yi * ne + yj];
      const double complex *TR = T + (size_t)R * n * n;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double complex s = 0;
          for (int q = 0; q < n; ++q) s += TR[i * n + q] * S[q * n + j];
          M[((size_t)R * n + i) * N + (size_t)Cc * n + j] = -s;
        }
    }
  }
  for (size_t i = 0; i < N; ++i) M[i * N + i] += 1;
  free(A);
  free(B);
  free(S);
  return 0;
}

/* LAPACK zgetrf semantics (row-major storage, unblocked): A = P L U. ipiv[i]
 * is the 0-based row swapped with row i at step i. Returns 0 or i+1 if U(i,i)
 * is exactly zero. */
int orc_lu_factor(size_t n, double complex *a, int *ipiv) {
  int info = 0;
  for (size_t k = 0; k < n; ++k) {
    size_t p = k;
    double best = -1;
    for (size_t i = k; i < n; ++i) {
      double v = fabs(creal(a[i * n + k])) + fabs(cimag(a[i * n + k]));
      if (v > best) { best = v; p = i; }
    }
    ipiv[k] = (int)p;
    if (a[p * n + k] == 0) {
      if (!info) info = (int)k + 1;
      continue;
    }
    if (p != k)
      for (size_t j = 0; j < n; ++j) {
        double complex t = a[k * n + j];
        a[k * n + j] = a[p * n + j];
        a[p * n + j] = t;
      }
    double complex inv = 1.0 / a[k * n + k];
    for (size_t i = k + 1; i < n; ++i) {
      double complex l = a[i * n + k] * inv;
      a[i * n + k] = l;
      if (l != 0)
        for (size_t j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
    }
  }
  return info;
}

/* zgetrs, trans = 'N': b (n x nrhs, row-major) overwritten with A^{-1} b. */
void orc_lu_solve(size_t n, const double complex *a, const int *ipiv, double complex *b, size_t nrhs) {
  for (size_t k = 0; k < n; ++k)
    if ((size_t)ipiv[k] != k)
      for (size_t j = 0; j < nrhs; ++j) {
        double complex t = b[k * nrhs + j];
        b[k * nrhs + j] = b[(size_t)ipiv[k] * nrhs + j];
        b[(size_t)ipiv[k] * nrhs + j] = t;
      }
  for (size_t i = 0; i < n; ++i)
    for (size_t k = 0; k < i; ++k) {
      double complex l = a[i * n + k];
      if (l != 0)
        for (size_t j = 0; j < nrhs; ++j) b[i * nrhs + j] -= l * b[k * nrhs + j];
    }
  for (size_t ii = n; ii-- > 0;) {
    for (size_t k = ii + 1; k < n; ++k) {
      double complex u = a[ii * n + k];
      if (u != 0)
        for (size_t j = 0; j < nrhs; ++j) b[ii * nrhs + j] -= u * b[k * nrhs + j];
    }
    double complex inv = 1.0 / a[ii * n + ii];
    for (size_t j = 0; j < nrhs; ++j) b[ii * nrhs + j] *= inv;
  }
}

/* One frequency of the finite plane-wave scattering workflow
 * (misc/finiterectlat-scatter.py:70-111 with the full, unpacked system):
 * spheres (common radius, eps_i) in a medium eps_e, incidence k_dir (unit),
 * E_cart.  Outputs f (N), a_inc (N) and sigma_ext. */
int orc_finite_sphere_scatter(const orc_trans_calculator *c, int np, const double *pos, double radius,
                              double complex eps_i, double complex eps_e, double omega,
                              const double k_dir[3], const double complex E_cart[3],
                              double complex *f_out, double complex *a_out, double *sigma_ext,
                              double complex *M_out) {
  const int lMax = c->lMax, ne = c->nelem, n = 2 * ne;
  const size_t N = (size_t)np * n;
  double complex kk = csqrt(eps_e) * omega / ORC_C0;
  double complex *Td = malloc(sizeof(double complex) * n);
  orc_tmatrix_sphere_diag(lMax, radius, omega, eps_i, eps_e, Td);
  double complex *T = calloc((size_t)np * n * n, sizeof(double complex));
  for (int p = 0; p < np; ++p)
    for (int i = 0; i < n; ++i) T[(size_t)p * n * n + i * n + i] = Td[i];
  double complex *M = M_out ? M_out : malloc(sizeof(double complex) * N * N);
  orc_finite_modeproblem(c, np, pos, T, kk, M);
  double complex *LU = malloc(sizeof(double complex) * N * N);
  memcpy(LU, M, sizeof(double complex) * N * N);
  int *ipiv = malloc(sizeof(int) * N);
  int info = orc_lu_factor(N, LU, ipiv);
  double kr = creal(kk);
  double kc[3] = {kr * k_dir[0], kr * k_dir[1], kr * k_dir[2]};
  orc_planewave_full(lMax, np, pos, kc, E_cart, a_out);
  for (int p = 0; p < np; ++p)
    for (int i = 0; i < n; ++i) f_out[(size_t)p * n + i] = Td[i] * a_out[(size_t)p * n + i];
  orc_lu_solve(N, LU, ipiv, f_out, 1);
  double complex dot = 0;
  for (size_t i = 0; i < N; ++i) dot += conj(a_out[i]) * f_out[i];
  *sigma_ext = -creal(dot) / (kr * kr);
  free(Td);
  free(T);
  free(LU);
  free(ipiv);
  if (!M_out) free(M);
  return info;
}

/* qpms_scatsys_build_translation_matrix_e_full (scatsystem.c:1180-1217):
 * S(R <- C) blocks of kind J for R != C, zero diagonal blocks. */
int orc_finite_translation_matrix(const orc_trans_calculator *c, int np, const double *pos,
                                  double complex k, int J, double complex *S_out) {
  const int ne = c->nelem, n = 2 * ne;
  const size_t N = (size_t)np * n;
  memset(S_out, 0, N * N * sizeof(double complex));
  double complex *A = malloc(sizeof(double complex) * ne * ne), *B = malloc(sizeof(double complex) * ne * ne);
  for (int R = 0; R < np; ++R)
    for (int Cc = 0; Cc < np; ++Cc) {
      if (R == Cc) continue;
      double d[3] = {pos[3 * R] - pos[3 * Cc], pos[3 * R + 1] - pos[3 * Cc + 1], pos[3 * R + 2] - pos[3 * Cc + 2]};
      double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double th = r ? acos(d[2] / r) : M_PI_2, ph = atan2(d[1], d[0]);
      orc_trans_calculator_get_AB_arrays_ext(c, A, B, ne, 1, r * k, th, ph, 0, J);
      for (int ti = 0; ti < 2; ++ti)
        for (int yi = 0; yi < ne; ++yi)
          for (int tj = 0; tj < 2; ++tj)
            for (int yj = 0; yj < ne; ++yj)
              S_out[((size_t)R * n + ti * ne + yi) * N + (size_t)Cc * n + tj * ne + yj] =
                  (ti == tj) ? A[yi * ne + yj] : B[yi * ne + yj];
    }
  free(A);
  free(B);
  return 0;
}

/* ---- plain-argument shims for ctypes ---- */
void orc_tmatrix_sphere_diag_ri(int lMax, double radius, double omr, double omi, double eir, double eii,
                                double eer, double eei, double complex *Tdiag) {
  orc_tmatrix_sphere_diag(lMax, radius, omr + I * omi, eir + I * eii, eer + I * eei, Tdiag);
}
int orc_finite_modeproblem_ri(const orc_trans_calculator *c, int np, const double *pos,
                              const double complex *T, double kr, double ki, double complex *M) {
  return orc_finite_modeproblem(c, np, pos, T, kr + I * ki, M);
}
int orc_finite_translation_matrix_ri(const orc_trans_calculator *c, int np, const double *pos, double kr,
                                     double ki, int J, double complex *S) {
  return orc_finite_translation_matrix(c, np, pos, kr + I * ki, J, S);
}
int orc_finite_sphere_scatter_ri(const orc_trans_calculator *c, int np, const double *pos, double radius,
                                 double eir, double eii, double eer, double eei, double omega,
                                 const double *k_dir, const double complex *E_cart, double complex *f_out,
                                 double complex *a_out, double *sigma_ext, double complex *M_out) {
  return orc_finite_sphere_scatter(c, np, pos, radius, eir + I * eii, eer + I * eei, omega, k_dir, E_cart,
                                   f_out, a_out, sigma_ext, M_out);
}

/* ---- scattered field of a finite system ----
 * qpms_scatsys_scattered_E (scatsystem.c:2013-2039): for every particle,
 * kr = k * cart2sph(where - pos) (vectors.h:134-140, sph_cscale :262-265), the
 * field of its outgoing-wave coefficients by qpms_eval_uvswf (vswf.c:611-650)
 * -> qpms_eval_vswf_csph (vswf.c:533-560: Kahan sums over y of the electric and
 * the magnetic terms, then esum += msum) with the VSWFs of qpms_vswf_fill_csph
 * (vswf.c:230-288), turned to cartesian by csphvec2ccart (vectors.h:272-303) and
 * Kahan-summed over the particles.  QPMS_NORMALISATION_DEFAULT (qpms_types.h:167):
 * Condon-Shortley phase, azimuthal part e^{i m phi} and derivative / m = i e^{i m phi}
 * (normalisation.h:159-212), all normalisation factors 1.  Coefficients per particle
 * in bspec order (electric block, then magnetic). */
static void ckadd(double complex *s, double complex *c, double complex in) {
  double complex y = in - *c, t = *s + y;
  *c = (t - *s) - y;
  *s = t;
}

void orc_scattered_E(int lMax, int np, const double *pos, int J, double complex k, const double complex *cvf,
                     int npts, const double *where, double complex *E) {
  const int ne = lMax * (lMax + 2);
  double leg[ne], pi[ne], tau[ne];
  double complex bes[lMax + 1];
  for (int q = 0; q < npts; ++q) {
    double complex res[3] = {0, 0, 0}, rc[3] = {0, 0, 0};
    for (int p = 0; p < np; ++p) {
      const double dx = where[3 * q] - pos[3 * p], dy = where[3 * q + 1] - pos[3 * p + 1],
                   dz = where[3 * q + 2] - pos[3 * p + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const double theta = r ? acos(dz / r) : M_PI_2, phi = atan2(dy, dx);
      const double complex kr = k * r;
      orc_sph_bessel_fill(J, lMax, kr, bes);
      orc_pitau(theta, lMax, -1.0, leg, pi, tau);
      const double complex *cv = cvf + (size_t)p * 2 * ne;
      double complex es[3] = {0, 0, 0}, ec[3] = {0, 0, 0}, ms[3] = {0, 0, 0}, mc[3] = {0, 0, 0};
      for (int l = 1, y = 0; l <= lMax; ++l) {
        double complex besfac = r ? bes[l] / kr : ((1 == l) ? 1 / 3. : 0);
        double complex besderfac = bes[l - 1] - l * besfac;
        for (int m = -l; m <= l; ++m, ++y) {
          double complex eimf = cexp(I * m * phi), deimf = m ? I * cexp(I * m * phi) : 0;
          double complex N[3] = {l * (l + 1) * leg[y] * besfac * eimf, tau[y] * besderfac * eimf,
                                 pi[y] * besderfac * deimf};
          double complex M[3] = {0, pi[y] * bes[l] * deimf, -tau[y] * bes[l] * eimf};
          for (int c = 0; c < 3; ++c) {
            ckadd(&es[c], &ec[c], cv[y] * N[c]);
            ckadd(&ms[c], &mc[c], cv[ne + y] * M[c]);
          }
        }
      }
      for (int c = 0; c < 3; ++c) ckadd(&es[c], &ec[c], ms[c]);
      const double st = sin(theta), ct = cos(theta), sf = sin(phi), cf = cos(phi);
      double complex Ec[3];
      Ec[0] = st * cf * es[0] + ct * cf * es[1] - sf * es[2];
      Ec[1] = st * sf * es[0] + ct * sf * es[1] + cf * es[2];
      Ec[2] = ct * es[0] - st * es[1];
      for (int c = 0; c < 3; ++c) ckadd(&res[c], &rc[c], Ec[c]);
    }
    for (int c = 0; c < 3; ++c) E[3 * q + c] = res[c];
  }
}

void orc_scattered_E_ri(int lMax, int np, const double *pos, int J, double kr_, double ki_,
                        const double complex *cvf, int npts, const double *where, double complex *E) {
  orc_scattered_E(lMax, np, pos, J, kr_ + I * ki_, cvf, npts, where, E);
}
