/*
 * Oracle: CPU restatement of the QPMS mode-problem hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library (qpms_gb300/) links,
 * loads or calls this code; only the tests, the smoke check and the CPU
 * baseline leg of bench.py do, and there only to check results.
 *
 * Every function restates one function of the reference (kostyfisik/qpms) and
 * cites the reference file:line it follows.  The reference's third-party
 * numerics (GSL special functions, AMOS complex Bessel, GSL 3j) are replaced
 * by self-written equivalents from the mathematics; each is pinned in the
 * CPU tests against mpmath / sympy, and the Gaunt coefficients against the
 * reference's own gaunt.c compiled from its sources (oracle/_ref).
 *
 * Prefix: orc_.  Complex numbers are C99 `double complex`, which has the
 * same layout as the reference's `complex double` and numpy complex128.
 */
#ifndef QPMS_ORACLE_H
#define QPMS_ORACLE_H
#include <complex.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- special functions (orc_specfunc.c) ---- */

/* Wigner 3j symbol with integer arguments (replaces gsl_sf_coupling_3j with
 * doubled arguments, translations.c:375-376).  Racah formula in long double. */
double orc_wigner3j(int j1, int j2, int j3, int m1, int m2, int m3);

/* Gaunt coefficients a_q(m,n,mu,nu), q = 0..qmax, of the product expansion
 * P_n^m P_nu^mu = sum_q a_q P_{n+nu-2q}^{m+mu} (replaces gaunt_xu, gaunt.c:396).
 * Returns qmax = gaunt_q_max(m,n,mu,nu) (gaunt.h:6-8). */
int orc_gaunt(int m, int n, int mu, int nu, double *aq);
int orc_gaunt_q_max(int m, int n, int mu, int nu);

/* Unnormalised associated Legendre P_l^m(x), 0<=m<=l<=L, in GSL layout
 * l(l+1)/2+m, with Condon-Shortley factor csphase^m (replaces
 * gsl_sf_legendre_array_e(GSL_SF_LEGENDRE_NONE, ...), translations.c:651-653). */
void orc_legendre_array(int L, double x, double csphase, double *out);

/* Spherical Bessel functions z_l(x), l = 0..lmax, of kind J
 * (1 = j, 2 = y, 3 = h+, 4 = h-).  Follows qpms_sph_bessel_fill
 * (bessel.c:86-147, :52-83): real x and complex x branches. */
int orc_sph_bessel_fill(int J, int lmax, double complex x, double complex *res);

/* ---- translation operator (orc_trans.c) ---- */

typedef struct orc_trans_calculator {
  int normalisation;            /* qpms_normalisation_t bits */
  int lMax;
  int nelem;                    /* lMax (lMax + 2) */
  double complex **A_multipliers; /* nelem^2 + 1 pointers into one block */
  double complex **B_multipliers;
} orc_trans_calculator;

/* translations.c:439-508 */
orc_trans_calculator *orc_trans_calculator_init(int lMax, int normalisation);
void orc_trans_calculator_free(orc_trans_calculator *c);
/* Total number of A / B multipliers (ragged table sizes). */
size_t orc_trans_calculator_nA(const orc_trans_calculator *c);
size_t orc_trans_calculator_nB(const orc_trans_calculator *c);

/* translations.c:610-698, 1124-1132 (the _ext form, kd = (r, theta, phi)). */
int orc_trans_calculator_get_AB_arrays_ext(const orc_trans_calculator *c,
    double complex *Adest, double complex *Bdest,
    size_t deststride, size_t srcstride,
    double complex kdlj_r, double kdlj_theta, double kdlj_phi,
    int r_ge_d, int J);

/* Batched loop over n vectors (the numpy loop of translations_python.c:24-132,
 * extended to complex kr): A,B at [i][nelem][nelem]. */
int orc_trans_AB_batch(const orc_trans_calculator *c, size_t n,
    const double complex *kr, const double *theta, const double *phi,
    int J, double complex *A, double complex *B);

/* Closed-form single coefficients (translations.c:135-286), used by the
 * single-vs-array property test (tests/single_translations_vs_calc.c). */
double complex orc_trans_single_A(int norm, int m, int n, int mu, int nu,
    double complex kr, double theta, double phi, int r_ge_d, int J);
double complex orc_trans_single_B(int norm, int m, int n, int mu, int nu,
    double complex kr, double theta, double phi, int r_ge_d, int J);

/* ---- finite scattering system (orc_scatsys.c) ---- */
void orc_mie_coefficients(int lMax, double a, double complex k_i, double complex k_e,
                          double complex mu_i, double complex mu_e, int J_ext, int J_scat,
                          double complex *RV, double complex *RH);
void orc_tmatrix_sphere_diag(int lMax, double radius, double complex omega, double complex eps_i,
                             double complex eps_e, double complex *Tdiag);
void orc_planewave_full(int lMax, int np, const double *pos, const double k_cart[3],
                        const double complex E_cart[3], double complex *out);
int orc_finite_modeproblem(const orc_trans_calculator *c, int np, const double *pos,
                           const double complex *T, double complex k, double complex *M);
int orc_finite_translation_matrix(const orc_trans_calculator *c, int np, const double *pos,
                                  double complex k, int J, double complex *S_out);
int orc_lu_factor(size_t n, double complex *a, int *ipiv);
void orc_lu_solve(size_t n, const double complex *a, const int *ipiv, double complex *b, size_t nrhs);
int orc_finite_sphere_scatter(const orc_trans_calculator *c, int np, const double *pos, double radius,
                              double complex eps_i, double complex eps_e, double omega,
                              const double k_dir[3], const double complex E_cart[3],
                              double complex *f_out, double complex *a_out, double *sigma_ext,
                              double complex *M_out);

/* Scattered field at npts points where[q][3] of the full coefficient vector
 * cvf (np particles, common lMax); E[q][3] (scatsystem.c:2013-2039). */
void orc_scattered_E(int lMax, int np, const double *pos, int J, double complex k, const double complex *cvf,
                     int npts, const double *where, double complex *E);

/* ---- axially symmetric particles (orc_axsym.c) ---- */
/* shape 0 sphere {R}, 1 cylinder {R, h}, 2 spheroid {a, c} */
void orc_arc(int shape, const double *par, double theta, double *r, double *beta);
int orc_tmatrix_axialsym(int lMax, int lMaxQR, double complex k, double complex kin, double complex zr, int shape,
                         const double *par, double rtol, double complex *T, double complex *Qout,
                         double complex *Rout);

/* ---- interpolation (orc_interp.c) ---- */
/* kind 0 linear, 1 natural cubic spline; out[q] = S(xq[q]), NaN outside the knots */
void orc_spline_eval(int kind, int n, const double *x, const double *y, int nq, const double *xq, double *out);

/* ---- 2D Ewald sums and the lattice translation operator (orc_ewald.c) ---- */
typedef struct orc_c2 { double x, y; } orc_c2;
void orc_l2d_reduceBasis(orc_c2 b1, orc_c2 b2, orc_c2 *o1, orc_c2 *o2);
double orc_l2d_unitcell_area(orc_c2 b1, orc_c2 b2);
void orc_l2d_reciprocalBasis2pi(orc_c2 b1, orc_c2 b2, orc_c2 *rb1, orc_c2 *rb2);
double complex orc_complex_gamma_inc(double a, double complex x, int m);
double complex orc_ewald_sr_integral(double r, double complex k, int n, double eta);
typedef double (*orc_fn_t)(double, const void *);
double orc_qagiu(orc_fn_t f, const void *p, double a, double epsabs, double epsrel, double *abserr);
/* shift_z: height of the shift above the lattice plane (0: the xy sums) */
void orc_ewald3_sigma_xy(int lMax_e, int csphase, double eta, double complex k, orc_c2 b1, orc_c2 b2, orc_c2 beta,
                         orc_c2 shift, double shift_z, double maxR, double maxK, int parts, double complex *sigma_out,
                         double complex *sigma_short_out, double complex *sigma_long_out);
void orc_sigma_direct(int lMax_e, int csphase, double complex k, orc_c2 b1, orc_c2 b2, orc_c2 beta, orc_c2 shift,
                      double shift_z, int nlayers, double complex *out);
int orc_trans_calculator_get_AB_arrays_e32(const orc_trans_calculator *c, double complex *Adest,
                                           double complex *Bdest, size_t deststride, size_t srcstride, double eta,
                                           double complex k, orc_c2 b1, orc_c2 b2, orc_c2 beta, orc_c2 shift,
                                           double shift_z, double maxR, double maxK, int parts);
double orc_adjusted_eta(double unitcell_area, double complex wavenumber, const double kvec[3], int lMax);
int orc_periodic_modeproblem(const orc_trans_calculator *c, int np, const double *pos, const double complex *T,
                             double complex k, orc_c2 b1, orc_c2 b2, const double kvec[2], double eta,
                             double complex *M);

#ifdef __cplusplus
}
#endif
#endif
