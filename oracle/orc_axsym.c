/*
 * Oracle T-matrices of axially symmetric particles (test infrastructure only;
 * see orc.h).  Restates the reference's extended-boundary-condition method
 * (tmatrices.c:615-894, tmatrices.h:415-523):
 *   arc parametrisations     qpms_arc_sphere, qpms_arc_cylinder (tmatrices.c:620-646):
 *                            r(theta) and beta = angle between the surface normal
 *                            and the radial direction
 *   integrand                tmatrix_axialsym_integrand (tmatrices.c:659-696):
 *                            for the outgoing (Q) or regular (R) wave y of
 *                            (type t, l, m) at k r and the regular wave v of the
 *                            inside medium of (t', l', -m) at k_in r,
 *                            jac (z / z_in n.(y_t x v_t'bar) + n.(y_tbar x v_t')),
 *                            jac = r^2 sin(theta) / cos(beta), n = (cos beta, sin beta, 0)
 *   quadrature               gsl_integration_qag over [0, pi] per entry
 *                            (tmatrices.c:708-744, epsabs 1e-8, epsrel 1e-5):
 *                            here one adaptive 15-point Gauss-Kronrod bisection
 *                            over all entries of an m block at once, to a
 *                            tighter tolerance (the entries are the same integrals)
 *   T = -R Q^-1              tmatrices.c:864-884 (Q^T X = R^T, X = -T^T),
 *                            trimmed from lMaxQR to lMax
 * VSWFs: QPMS_NORMALISATION_DEFAULT (power-normalised, Condon-Shortley phase),
 * evaluated as the field oracle of orc_scatsys.c does (phi = 0).
 */
#include "orc.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static int m1pow(int p) { return (p % 2) ? -1 : 1; }

/* tmatrices.c:620-646 */
void orc_arc(int shape, const double *par, double theta, double *r, double *beta) {
  if (shape == 0) { /* sphere, par = {R} */
    *r = par[0];
    *beta = 0;
  } else if (shape == 1) { /* cylinder, par = {R, h} */
    const double R = par[0], h = par[1];
    const double thresh = atan(2 * R / h);
    if (theta < thresh) {
      *r = 0.5 * h / cos(theta);
      *beta = -theta;
    } else if (theta <= M_PI - thresh) {
      *r = R / cos(theta - M_PI_2);
      *beta = -theta + M_PI_2;
    } else {
      *r = 0.5 * h / cos(theta - M_PI);
      *beta = -theta + M_PI;
    }
  } else { /* spheroid, par = {a (equatorial semi-axis), c (polar semi-axis)} */
    const double a = par[0], c = par[1], s = sin(theta), co = cos(theta);
    const double q = s * s / (a * a) + co * co / (c * c);
    *r = 1 / sqrt(q);
    /* normal direction ~ grad (x^2/a^2 + z^2/c^2): angle to r-hat */
    const double dr = 0.5 * pow(q, -1.5) * 2 * s * co * (1 / (c * c) - 1 / (a * a)); /* dr/dtheta */
    *beta = atan2(-dr, *r);
  }
}

typedef struct {
  int L, m, l0, nl;
  double complex k, kin, zr;
  int shape;
  const double *par;
} ax_par;

/* Wave components (r, theta, phi) at phi = 0 for l = l0..L:
 * W[((l - l0) * 2 + t) * 3 + c], t = 0 electric (N), 1 magnetic (M). */
static void waves(const ax_par *P, int J, double complex x, int m, double theta, double complex *W) {
  const int L = P->L;
  double complex z[L + 2];
  orc_sph_bessel_fill(J, L, x, z);
  const int ne = L * (L + 2);
  double leg[ne], pi[ne], tau[ne];
  /* orc_pitau lives in orc_scatsys.c (static); restated here through the
   * public Legendre array */
  double P_[(L + 2) * (L + 3) / 2];
  const double ct = cos(theta), st = sin(theta);
  orc_legendre_array(L + 1, ct, -1.0, P_);
  for (int l = 1; l <= L; ++l)
    for (int mm = 0; mm <= l; ++mm) {
      double plm = P_[l * (l + 1) / 2 + mm];
      double plm1 = (l - 1 >= mm) ? P_[(l - 1) * l / 2 + mm] : 0.0;
      double dplm = (l * ct * plm - (l + mm) * plm1) / (ct * ct - 1);
      double nf = sqrt((2 * l + 1) / (4 * M_PI) * exp(lgamma(l - mm + 1) - lgamma(l + mm + 1)));
      double pref = 1. / sqrt(l * (l + 1.));
      double Lv = nf * plm * pref, Dv = nf * dplm * pref;
      int yp = l * (l + 1) + mm - 1, ym = l * (l + 1) - mm - 1;
      leg[yp] = Lv;
      pi[yp] = mm / st * Lv;
      tau[yp] = -st * Dv;
      if (mm > 0) {
        double f = m1pow(mm);
        leg[ym] = f * Lv;
        pi[ym] = -mm / st * f * Lv;
        tau[ym] = -st * f * Dv;
      }
    }
  for (int l = P->l0; l <= L; ++l) {
    const int y = l * (l + 1) + m - 1;
    const double complex besfac = z[l] / x, besder = z[l - 1] - l * besfac;
    const double complex di = m ? I : 0;
    double complex *w = W + (size_t)(l - P->l0) * 6;
    w[0] = l * (l + 1) * leg[y] * besfac; /* N */
    w[1] = tau[y] * besder;
    w[2] = pi[y] * besder * di;
    w[3] = 0; /* M */
    w[4] = pi[y] * z[l] * di;
    w[5] = -tau[y] * z[l];
  }
}

static double complex tp(double nr, double nt, const double complex *y, const double complex *v) {
  return nr * (y[1] * v[2] - y[2] * v[1]) + nt * (y[2] * v[0] - y[0] * v[2]);
}

/* all Q (first nb^2) and R (next nb^2) integrands of the m block at theta;
 * entry (i, j), i = (t, l) outside index, j = (t', l') inside index */
static void ax_integrand(double theta, const ax_par *P, double complex *out) {
  double r, beta;
  orc_arc(P->shape, P->par, theta, &r, &beta);
  const int nl = P->nl, nb = 2 * nl;
  double complex Yq[nl * 6], Yr[nl * 6], V[nl * 6];
  waves(P, 3, P->k * r, P->m, theta, Yq);
  waves(P, 1, P->k * r, P->m, theta, Yr);
  waves(P, 1, P->kin * r, -P->m, theta, V);
  const double nr = cos(beta), nt = sin(beta);
  const double jac = r * r * sin(theta) / nr;
  for (int qr = 0; qr < 2; ++qr) {
    const double complex *Y = qr ? Yr : Yq;
    for (int i = 0; i < nb; ++i) {
      const int t = i / nl, l = i % nl;
      for (int j = 0; j < nb; ++j) {
        const int t2 = j / nl, l2 = j % nl;
        const double complex *yt = Y + (l * 2 + t) * 3, *ytb = Y + (l * 2 + (1 - t)) * 3;
        const double complex *vt = V + (l2 * 2 + t2) * 3, *vtb = V + (l2 * 2 + (1 - t2)) * 3;
        out[(size_t)qr * nb * nb + i * nb + j] = jac * (P->zr * tp(nr, nt, yt, vtb) + tp(nr, nt, ytb, vt));
      }
    }
  }
}

/* 15-point Gauss-Kronrod constants (QUADPACK qk15) */
static const double xk[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                             0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                             0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                             0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
static const double wk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                             0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                             0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                             0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
static const double wgs[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                              0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

static double vqk15(const ax_par *P, int nv, double a, double b, double complex *res, double complex *f1,
                    double complex *f2, double complex *rg) {
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  ax_integrand(c, P, f1);
  for (int v = 0; v < nv; ++v) {
    res[v] = f1[v] * wk[7];
    rg[v] = f1[v] * wgs[3];
  }
  for (int j = 0; j < 7; ++j) {
    const double x = h * xk[j];
    ax_integrand(c - x, P, f1);
    ax_integrand(c + x, P, f2);
    for (int v = 0; v < nv; ++v) {
      res[v] += wk[j] * (f1[v] + f2[v]);
      if (j % 2 == 1) rg[v] += wgs[j / 2] * (f1[v] + f2[v]);
    }
  }
  double e = 0;
  for (int v = 0; v < nv; ++v) {
    res[v] *= h;
    const double d = cabs(res[v] - rg[v] * h);
    if (d > e) e = d;
  }
  return e;
}

/* adaptive bisection over [a, b] (split at the given breakpoints) until the
 * summed error estimate is below rtol x the largest |entry| */
static void vqag(const ax_par *P, int nv, int nbp, const double *bp, double rtol, double complex *out) {
  enum { MAXIV = 3000 };
  double *lo = malloc(sizeof(double) * MAXIV), *hi = malloc(sizeof(double) * MAXIV),
         *er = malloc(sizeof(double) * MAXIV);
  double complex *rs = malloc(sizeof(double complex) * (size_t)MAXIV * nv);
  double complex *f1 = malloc(sizeof(double complex) * nv * 3);
  double complex *f2 = f1 + nv, *rg = f1 + 2 * nv;
  int n = 0;
  for (int i = 0; i + 1 < nbp; ++i) {
    lo[n] = bp[i];
    hi[n] = bp[i + 1];
    er[n] = vqk15(P, nv, lo[n], hi[n], rs + (size_t)n * nv, f1, f2, rg);
    ++n;
  }
  for (;;) {
    double terr = 0, scale = 0;
    int worst = 0;
    for (int v = 0; v < nv; ++v) {
      double complex s = 0;
      for (int i = 0; i < n; ++i) s += rs[(size_t)i * nv + v];
      out[v] = s;
      if (cabs(s) > scale) scale = cabs(s);
    }
    for (int i = 0; i < n; ++i) {
      terr += er[i];
      if (er[i] > er[worst]) worst = i;
    }
    if (terr <= rtol * scale || n >= MAXIV - 1) break;
    const double mid = 0.5 * (lo[worst] + hi[worst]);
    lo[n] = mid;
    hi[n] = hi[worst];
    hi[worst] = mid;
    er[worst] = vqk15(P, nv, lo[worst], hi[worst], rs + (size_t)worst * nv, f1, f2, rg);
    er[n] = vqk15(P, nv, lo[n], hi[n], rs + (size_t)n * nv, f1, f2, rg);
    ++n;
  }
  free(lo);
  free(hi);
  free(er);
  free(rs);
  free(f1);
}

/* T (default normalisation, bspec order at lMax: electric block, then
 * magnetic; n = 2 lMax (lMax + 2)) of the axially symmetric particle, from Q
 * and R at lMaxQR >= lMax.  k, kin: wavenumbers outside / inside; zr = z / z_in
 * (wave impedance ratio).  Q, R (optional): the full matrices at lMaxQR in the
 * same order, row = outside wave (t, l, m), column = inside wave (t', l', -m)
 * stored at the column of (t', l', m). */
int orc_tmatrix_axialsym(int lMax, int lMaxQR, double complex k, double complex kin, double complex zr, int shape,
                         const double *par, double rtol, double complex *T, double complex *Qout,
                         double complex *Rout) {
  if (lMaxQR < lMax) lMaxQR = lMax;
  const int L = lMaxQR, neQ = L * (L + 2), nQ = 2 * neQ, ne = lMax * (lMax + 2), n = 2 * ne;
  double complex *TQ = calloc((size_t)nQ * nQ, sizeof(double complex));
  if (Qout) memset(Qout, 0, sizeof(double complex) * nQ * nQ);
  if (Rout) memset(Rout, 0, sizeof(double complex) * nQ * nQ);
  double bp[4] = {0, M_PI, 0, 0};
  int nbp = 2;
  if (shape == 1) {
    const double th = atan(2 * par[0] / par[1]);
    bp[0] = 0;
    bp[1] = th;
    bp[2] = M_PI - th;
    bp[3] = M_PI;
    nbp = 4;
  }
  int rc = 0;
  for (int m = -L; m <= L; ++m) {
    ax_par P;
    P.L = L;
    P.m = m;
    P.l0 = abs(m) > 1 ? abs(m) : 1;
    P.nl = L - P.l0 + 1;
    P.k = k;
    P.kin = kin;
    P.zr = zr;
    P.shape = shape;
    P.par = par;
    const int nb = 2 * P.nl, nv = 2 * nb * nb;
    double complex *QR = malloc(sizeof(double complex) * nv);
    vqag(&P, nv, nbp, bp, rtol, QR);
    const double complex *Q = QR, *R = QR + nb * nb;
    /* solve Q^T X = R^T, X = -T^T */
    double complex *A = malloc(sizeof(double complex) * nb * nb), *B = malloc(sizeof(double complex) * nb * nb);
    int *piv = malloc(sizeof(int) * nb);
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        A[i * nb + j] = Q[j * nb + i];
        B[i * nb + j] = R[j * nb + i];
      }
    if (orc_lu_factor(nb, A, piv)) rc = 1;
    orc_lu_solve(nb, A, piv, B, nb);
    for (int i = 0; i < nb; ++i) {
      const int t = i / P.nl, l = P.l0 + i % P.nl;
      const int gi = t * neQ + l * (l + 1) + m - 1;
      for (int j = 0; j < nb; ++j) {
        const int t2 = j / P.nl, l2 = P.l0 + j % P.nl;
        const int gj = t2 * neQ + l2 * (l2 + 1) + m - 1;
        TQ[(size_t)gi * nQ + gj] = -B[j * nb + i];
        if (Qout) Qout[(size_t)gi * nQ + gj] = Q[i * nb + j];
        if (Rout) Rout[(size_t)gi * nQ + gj] = R[i * nb + j];
      }
    }
    free(A);
    free(B);
    free(piv);
    free(QR);
  }
  for (int t = 0; t < 2; ++t)
    for (int y = 0; y < ne; ++y)
      for (int t2 = 0; t2 < 2; ++t2)
        for (int y2 = 0; y2 < ne; ++y2)
          T[(size_t)(t * ne + y) * n + t2 * ne + y2] = TQ[(size_t)(t * neQ + y) * nQ + t2 * neQ + y2];
  free(TQ);
  return rc;
}

void orc_tmatrix_axialsym_ri(int lMax, int lMaxQR, const double *kk, int shape, const double *par, double rtol,
                             double complex *T, double complex *Q, double complex *R, int *rc) {
  /* kk = {Re k, Im k, Re k_in, Im k_in, Re zr, Im zr} */
  *rc = orc_tmatrix_axialsym(lMax, lMaxQR, kk[0] + I * kk[1], kk[2] + I * kk[3], kk[4] + I * kk[5], shape, par, rtol,
                             T, Q, R);
}

void orc_arc_ri(int shape, const double *par, double theta, double *rb) { orc_arc(shape, par, theta, rb, rb + 1); }
