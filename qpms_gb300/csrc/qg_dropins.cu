// Reference-API convenience entry points that sit beside the hot path:
// sphere T-matrices and their generators (tmatrices.c:49-75, 257-271,
// 500-622, 980-989), material helpers (materials.h:28-55, 151-158,
// materials.c:166-177), plane-wave expansion coefficients (vswf.c:445-530),
// the incident-field vector of a system (scatsystem.c:1970-1983), single
// translation coefficients (translations.h:40-44, 93-126) and the
// half-ellipse / kidney integration contours (beyn.c:88-226).
//
// All of these are O(n) or O(n^2) set-up work per particle or per contour;
// the O(N^2) / O(N^3) work of the mode problem stays on the GPU (the single
// translation coefficients are taken from one GPU evaluation of the whole
// A / B arrays).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <complex>
#include <vector>

#include "qg_internal.h"

namespace qg {
const qpms_vswf_set_spec_t *scatsys_spec(const qpms_scatsys_t *ss);  // qg_scatsys.cu
void mie_reflection(int lMax, double a, qpms_complex_t k_i, qpms_complex_t k_e, qpms_complex_t mu_i,
                    qpms_complex_t mu_e, int Je, int Js, qpms_complex_t *RV, qpms_complex_t *RH);
void planewave_sph_coeffs(int lMax, double theta, double phi, const qpms_complex_t Es[3], qpms_complex_t *el,
                          qpms_complex_t *mg);
qg_c uvswfi_norm_factor(int norm, qpms_uvswfi_t ui);  // qg_interp.cu
namespace {

typedef std::complex<double> cd;
constexpr double kC0 = 2.99792458e8;  // materials.h:11
constexpr int kMieMaxL = 10;          // Bessel orders up to 11 are compiled in

cd to_cd(qpms_complex_t z) { return cd(z.re, z.im); }
qpms_complex_t from_cd(cd z) {
  qpms_complex_t r;
  r.re = z.real();
  r.im = z.imag();
  return r;
}
void uvswfi_split(qpms_uvswfi_t ui, int *t, int *l, int *m) {
  *t = (int)(ui % 4);
  const long ysc = (long)(ui / 4);
  *l = (int)floor(sqrt((double)ysc) + 1e-9);
  *m = (int)(ysc - (long)*l * (*l + 1));
}
// a coefficient of a regular-wave expansion in the default normalisation,
// converted to normalisation norm (the waves scale by f_norm / f_default)
cd coeff_to_norm(int norm, int t, int l, int m, cd a) {
  if (norm == QPMS_NORMALISATION_DEFAULT) return a;
  const qpms_uvswfi_t ui = (qpms_uvswfi_t)t + 4 * (qpms_uvswfi_t)(l * (l + 1) + m);
  const qg_c fx = uvswfi_norm_factor(norm, ui), fd = uvswfi_norm_factor(QPMS_NORMALISATION_DEFAULT, ui);
  return a * cd(fd.re, fd.im) / cd(fx.re, fx.im);
}

// Plane-wave coefficients (vswf.c:445-476) in normalisation norm; long
// coefficients are zero for a transverse amplitude (amplitude.rc == 0 up to
// rounding) and not available otherwise.
int planewave_fill(double theta, double phi, const qpms_complex_t Es[3], qpms_complex_t *lc, qpms_complex_t *mc,
                   qpms_complex_t *ec, int lMax, int norm) {
  if (lMax < 1 || lMax > 16) {
    set_error("plane wave: lMax %d outside 1..16", lMax);
    return QPMS_EINVAL;
  }
  const int ne = lMax * (lMax + 2);
  if (lc) {
    // transverse up to rounding: |E_r| <= 1e-12 |E|
    const double amp = std::abs(to_cd(Es[0])) + std::abs(to_cd(Es[1])) + std::abs(to_cd(Es[2]));
    if (std::abs(to_cd(Es[0])) > 1e-12 * amp) {
      set_error("plane wave: longitudinal coefficients of a non-transverse amplitude are not supported");
      return QPMS_EINVAL;
    }
    for (int y = 0; y < ne; ++y) lc[y] = from_cd(0);
  }
  std::vector<qpms_complex_t> e(ne), g(ne);
  planewave_sph_coeffs(lMax, theta, phi, Es, e.data(), g.data());
  for (int l = 1, y = 0; l <= lMax; ++l)
    for (int m = -l; m <= l; ++m, ++y) {
      if (ec) ec[y] = from_cd(coeff_to_norm(norm, 2, l, m, to_cd(e[y])));
      if (mc) mc[y] = from_cd(coeff_to_norm(norm, 1, l, m, to_cd(g[y])));
    }
  return QPMS_SUCCESS;
}

// cartesian vector to the local spherical basis at direction (theta, phi) (vectors.h:306-330)
void cart_to_local(const qpms_complex_t E[3], double th, double ph, qpms_complex_t Es[3]) {
  const double st = sin(th), ct = cos(th), sf = sin(ph), cf = cos(ph);
  const cd x = to_cd(E[0]), y = to_cd(E[1]), z = to_cd(E[2]);
  Es[0] = from_cd(x * st * cf + y * st * sf + z * ct);
  Es[1] = from_cd(x * ct * cf + y * ct * sf - z * st);
  Es[2] = from_cd(-x * sf + y * cf);
}
void direction_of(double x, double y, double z, double *th, double *ph) {
  const double r = sqrt(x * x + y * y + z * z);
  *th = r > 0 ? acos(z / r) : 0.0;
  *ph = atan2(y, x);
}

// z with the sign of its zero component made to match the orientation (beyn.c:88-115)
qpms_complex_t align_zero(cd z, int orient) {
  qpms_complex_t r = from_cd(z);
  if (orient == 3 && r.re == 0) r.re = 0.0;
  if (orient == 1 && r.re == 0) r.re = -0.0;
  if (orient == 0 && r.im == 0) r.im = 0.0;
  if (orient == 2 && r.im == 0) r.im = -0.0;
  return r;
}
// the rotation and the axes of a half-ellipse orientation (beyn.c:134-152)
int orientation(int orient, double rRe, double rIm, cd *faktor, double *l, double *h) {
  *l = rRe;
  *h = rIm;
  switch (orient) {
    case 3: *faktor = cd(0, -1); *l = rIm; *h = rRe; return 0;
    case 1: *faktor = cd(0, 1); *l = rIm; *h = rRe; return 0;
    case 0: *faktor = 1; return 0;
    case 2: *faktor = -1; return 0;
    default: set_error("half-ellipse contour: unknown orientation %d", orient); return QPMS_EINVAL;
  }
}
beyn_contour_t *contour_alloc(size_t n, qpms_complex_t centre) {
  // n nodes, one entry of half-axes, and room for the orientation after it
  beyn_contour_t *c = (beyn_contour_t *)malloc(sizeof(beyn_contour_t) + (n + 2) * sizeof(c->z_dz[0]));
  if (!c) {
    set_error("out of host memory");
    return nullptr;
  }
  c->centre = centre;
  c->n = n;
  c->inside_test = nullptr;
  return c;
}

int single_AB(const qpms_trans_calculator *c, qpms_complex_t *A, qpms_complex_t *B, int m, int n, int mu, int nu,
              qpms_complex_t kr, double th, double ph, int r_ge_d, int J) {
  if (n < 1 || nu < 1 || n > c->lMax || nu > c->lMax || abs(m) > n || abs(mu) > nu) {
    set_error("translation coefficient (m %d, n %d; mu %d, nu %d) outside the calculator's lMax %d", m, n, mu, nu,
              (int)c->lMax);
    return QPMS_EINVAL;
  }
  const size_t ne = (size_t)c->lMax * (c->lMax + 2);
  std::vector<qpms_complex_t> a(ne * ne), b(ne * ne);
  const int rc = qpms_trans_calculator_get_AB_arrays_ext(c, a.data(), b.data(), ne, 1, kr, th, ph, r_ge_d, J);
  if (rc) return rc;
  const size_t i = (size_t)(n * (n + 1) + m - 1) * ne + (size_t)(nu * (nu + 1) + mu - 1);
  if (A) *A = a[i];
  if (B) *B = b[i];
  return QPMS_SUCCESS;
}
qpms_complex_t nan_c() {
  qpms_complex_t z;
  z.re = z.im = NAN;
  return z;
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

// ---------------- materials ----------------
qpms_complex_t qpms_refindex(qpms_epsmu_t em) { return from_cd(std::sqrt(to_cd(em.eps) * to_cd(em.mu))); }
qpms_complex_t qpms_wavenumber(qpms_complex_t omega, qpms_epsmu_t em) {
  return from_cd(to_cd(qpms_refindex(em)) * to_cd(omega) / kC0);
}
qpms_complex_t qpms_waveimpedance(qpms_epsmu_t em) { return from_cd(std::sqrt(to_cd(em.mu) / to_cd(em.eps))); }
qpms_epsmu_t qpms_epsmu_generator_eval(qpms_epsmu_generator_t gen, qpms_complex_t omega) {
  return gen.function(omega, gen.params);
}
qpms_complex_t qpms_drude_epsilon(qpms_complex_t eps_inf, qpms_complex_t omega_p, qpms_complex_t gamma_p,
                                  qpms_complex_t omega) {
  const cd w = to_cd(omega), wp = to_cd(omega_p);
  return from_cd(to_cd(eps_inf) - wp * wp / (w * (w + cd(0, 1) * to_cd(gamma_p))));
}
qpms_epsmu_t qpms_lorentzdrude_epsmu(qpms_complex_t omega, const qpms_ldparams_t *p) {
  qpms_epsmu_t em;
  em.eps = qpms_lorentzdrude_eps(omega, p);
  em.mu = from_cd(1.0);
  return em;
}
qpms_epsmu_t qpms_lorentzdrude_epsmu_g(qpms_complex_t omega, const void *p) {
  return qpms_lorentzdrude_epsmu(omega, (const qpms_ldparams_t *)p);
}

// ---------------- sphere T-matrices and generators ----------------
qpms_complex_t *qpms_mie_coefficients_reflection(qpms_complex_t *target, const qpms_vswf_set_spec_t *bspec, double a,
                                                 qpms_complex_t k_i, qpms_complex_t k_e, qpms_complex_t mu_i,
                                                 qpms_complex_t mu_e, qpms_bessel_t J_ext, qpms_bessel_t J_scat) {
  if (J_ext == J_scat || J_ext < 1 || J_ext > 4 || J_scat < 1 || J_scat > 4) {
    set_error("Mie coefficients: J_ext %d and J_scat %d must be distinct Bessel kinds 1..4", J_ext, J_scat);
    return nullptr;
  }
  const int lMax = (int)bspec->lMax;
  if (lMax < 1 || lMax > kMieMaxL) {
    set_error("Mie coefficients: lMax %d outside 1..%d", lMax, kMieMaxL);
    return nullptr;
  }
  std::vector<qpms_complex_t> RV(lMax + 1), RH(lMax + 1);
  mie_reflection(lMax, a, k_i, k_e, mu_i, mu_e, J_ext, J_scat, RV.data(), RH.data());
  std::vector<qpms_complex_t> out(bspec->n);
  for (size_t i = 0; i < bspec->n; ++i) {
    int t, l, m;
    uvswfi_split(bspec->ilist[i], &t, &l, &m);
    if ((t != 1 && t != 2) || l < 1 || l > lMax) {
      set_error("Mie coefficients: basis element %llu is not a transverse wave of the basis",
                (unsigned long long)bspec->ilist[i]);
      return nullptr;
    }
    out[i] = t == 2 ? RV[l] : RH[l];
  }
  if (!target) target = (qpms_complex_t *)malloc(std::max<size_t>(bspec->n, 1) * sizeof(qpms_complex_t));
  if (!target) {
    set_error("out of host memory");
    return nullptr;
  }
  memcpy(target, out.data(), bspec->n * sizeof(qpms_complex_t));
  return target;
}

int qpms_tmatrix_spherical_fill(qpms_tmatrix_t *t, double a, qpms_complex_t k_i, qpms_complex_t k_e,
                                qpms_complex_t mu_i, qpms_complex_t mu_e) {
  const size_t n = t->spec->n;
  std::vector<qpms_complex_t> d(n);
  if (!qpms_mie_coefficients_reflection(d.data(), t->spec, a, k_i, k_e, mu_i, mu_e, QPMS_BESSEL_REGULAR,
                                        QPMS_HANKEL_PLUS))
    return QPMS_EINVAL;
  memset(t->m, 0, n * n * sizeof(qpms_complex_t));
  for (size_t i = 0; i < n; ++i) t->m[i * n + i] = d[i];
  return QPMS_SUCCESS;
}
qpms_tmatrix_t *qpms_tmatrix_spherical(const qpms_vswf_set_spec_t *bspec, double a, qpms_complex_t k_i,
                                       qpms_complex_t k_e, qpms_complex_t mu_i, qpms_complex_t mu_e) {
  qpms_tmatrix_t *t = qpms_tmatrix_init(bspec);
  if (t && qpms_tmatrix_spherical_fill(t, a, k_i, k_e, mu_i, mu_e)) {
    qpms_tmatrix_free(t);
    return nullptr;
  }
  return t;
}
int qpms_tmatrix_spherical_mu0_fill(qpms_tmatrix_t *t, double a, double omega, qpms_complex_t eps_fg,
                                    qpms_complex_t eps_bg) {
  const qpms_complex_t k_i = from_cd(std::sqrt(to_cd(eps_fg)) * omega / kC0);
  const qpms_complex_t k_e = from_cd(std::sqrt(to_cd(eps_bg)) * omega / kC0);
  return qpms_tmatrix_spherical_fill(t, a, k_i, k_e, from_cd(1.0), from_cd(1.0));
}
qpms_tmatrix_t *qpms_tmatrix_spherical_mu0(const qpms_vswf_set_spec_t *bspec, double a, double omega,
                                           qpms_complex_t eps_fg, qpms_complex_t eps_bg) {
  qpms_tmatrix_t *t = qpms_tmatrix_init(bspec);
  if (t && qpms_tmatrix_spherical_mu0_fill(t, a, omega, eps_fg, eps_bg)) {
    qpms_tmatrix_free(t);
    return nullptr;
  }
  return t;
}
int qpms_tmatrix_generator_sphere(qpms_tmatrix_t *t, qpms_complex_t omega, const void *params) {
  const qpms_tmatrix_generator_sphere_param_t *p = (const qpms_tmatrix_generator_sphere_param_t *)params;
  const qpms_epsmu_t out = p->outside.function(omega, p->outside.params);
  const qpms_epsmu_t in = p->inside.function(omega, p->inside.params);
  return qpms_tmatrix_spherical_fill(t, p->radius, qpms_wavenumber(omega, in), qpms_wavenumber(omega, out), in.mu,
                                     out.mu);
}
int qpms_tmatrix_generator_constant(qpms_tmatrix_t *t, qpms_complex_t omega, const void *orig_v) {
  (void)omega;
  const qpms_tmatrix_t *orig = (const qpms_tmatrix_t *)orig_v;
  const size_t n = t->spec->n, no = orig->spec->n;
  const size_t copy = std::min(n, no) * std::min(n, no);
  memcpy(t->m, orig->m, copy * sizeof(qpms_complex_t));
  memset(t->m + copy, 0, (n * n - copy) * sizeof(qpms_complex_t));
  return QPMS_SUCCESS;
}
qpms_tmatrix_t *qpms_tmatrix_init_from_generator(const qpms_vswf_set_spec_t *bspec, qpms_tmatrix_generator_t gen,
                                                 qpms_complex_t omega) {
  qpms_tmatrix_t *t = qpms_tmatrix_init(bspec);
  if (t && gen.function(t, omega, gen.params)) {
    qpms_tmatrix_free(t);
    return nullptr;
  }
  return t;
}
qpms_tmatrix_t *qpms_tmatrix_copy(const qpms_tmatrix_t *T) {
  qpms_tmatrix_t *t = qpms_tmatrix_init(T->spec);
  if (t) memcpy(t->m, T->m, T->spec->n * T->spec->n * sizeof(qpms_complex_t));
  return t;
}
qpms_tmatrix_t *qpms_tmatrix_mv(qpms_tmatrix_t *dest, const qpms_tmatrix_t *orig) {
  if (dest->spec->n != orig->spec->n) {
    set_error("qpms_tmatrix_mv: bases of %zu and %zu elements", dest->spec->n, orig->spec->n);
    return nullptr;
  }
  memcpy(dest->m, orig->m, orig->spec->n * orig->spec->n * sizeof(qpms_complex_t));
  return dest;
}
bool qpms_tmatrix_isclose(const qpms_tmatrix_t *A, const qpms_tmatrix_t *B, double rtol, double atol) {
  // identical bases (vswf.c:37-49): same normalisation and element list
  if (A->spec != B->spec) {
    if (A->spec->n != B->spec->n || A->spec->norm != B->spec->norm) return false;
    for (size_t i = 0; i < A->spec->n; ++i)
      if (A->spec->ilist[i] != B->spec->ilist[i]) return false;
  }
  if (A->m == B->m) return true;
  const size_t nn = A->spec->n * A->spec->n;
  for (size_t i = 0; i < nn; ++i)
    if (std::abs(to_cd(B->m[i]) - to_cd(A->m[i])) > atol + rtol * std::abs(to_cd(B->m[i]))) return false;
  return true;
}
qpms_complex_t *qpms_apply_tmatrix(qpms_complex_t *f, const qpms_complex_t *a, const qpms_tmatrix_t *T) {
  const size_t n = T->spec->n;
  std::vector<cd> out(n);
  for (size_t i = 0; i < n; ++i) {
    cd s = 0;
    for (size_t j = 0; j < n; ++j) s += to_cd(T->m[i * n + j]) * to_cd(a[j]);
    out[i] = s;
  }
  if (!f) f = (qpms_complex_t *)malloc(std::max<size_t>(n, 1) * sizeof(qpms_complex_t));
  if (!f) {
    set_error("out of host memory");
    return nullptr;
  }
  for (size_t i = 0; i < n; ++i) f[i] = from_cd(out[i]);
  return f;
}

// ---------------- plane waves ----------------
int qpms_planewave2vswf_fill_sph(sph_t wavedir, csphvec_t amplitude, qpms_complex_t *target_longcoeff,
                                 qpms_complex_t *target_mgcoeff, qpms_complex_t *target_elcoeff, qpms_l_t lMax,
                                 qpms_normalisation_t norm) {
  const qpms_complex_t Es[3] = {amplitude.rc, amplitude.thetac, amplitude.phic};
  return planewave_fill(wavedir.theta, wavedir.phi, Es, target_longcoeff, target_mgcoeff, target_elcoeff,
                        (int)lMax, (int)norm);
}
int qpms_planewave2vswf_fill_cart(cart3_t wavedir, ccart3_t amplitude, qpms_complex_t *target_longcoeff,
                                  qpms_complex_t *target_mgcoeff, qpms_complex_t *target_elcoeff, qpms_l_t lMax,
                                  qpms_normalisation_t norm) {
  double th, ph;
  direction_of(wavedir.x, wavedir.y, wavedir.z, &th, &ph);
  const qpms_complex_t E[3] = {amplitude.x, amplitude.y, amplitude.z};
  qpms_complex_t Es[3];
  cart_to_local(E, th, ph, Es);
  return planewave_fill(th, ph, Es, target_longcoeff, target_mgcoeff, target_elcoeff, (int)lMax, (int)norm);
}
int qpms_incfield_planewave(qpms_complex_t *target, const qpms_vswf_set_spec_t *bspec, const cart3_t evalpoint,
                            const void *args, bool add) {
  const qpms_incfield_planewave_params_t *p = (const qpms_incfield_planewave_params_t *)args;
  cd kc[3];
  if (p->use_cartesian) {
    kc[0] = to_cd(p->k.cart.x);
    kc[1] = to_cd(p->k.cart.y);
    kc[2] = to_cd(p->k.cart.z);
  } else {
    const cd r = to_cd(p->k.sph.r);
    const double st = sin(p->k.sph.theta);
    kc[0] = r * st * cos(p->k.sph.phi);
    kc[1] = r * st * sin(p->k.sph.phi);
    kc[2] = r * cos(p->k.sph.theta);
  }
  // e^{i k.r} at the expansion point; the direction is that of Re k
  const cd phasefac = std::exp(cd(0, 1) * (kc[0] * evalpoint.x + kc[1] * evalpoint.y + kc[2] * evalpoint.z));
  double th, ph;
  direction_of(kc[0].real(), kc[1].real(), kc[2].real(), &th, &ph);
  qpms_complex_t Es[3];
  if (p->use_cartesian) {
    const qpms_complex_t E[3] = {p->E.cart.x, p->E.cart.y, p->E.cart.z};
    cart_to_local(E, th, ph, Es);
  } else {
    Es[0] = p->E.sph.rc;
    Es[1] = p->E.sph.thetac;
    Es[2] = p->E.sph.phic;
  }
  for (int i = 0; i < 3; ++i) Es[i] = from_cd(phasefac * to_cd(Es[i]));
  const int lMax = (int)bspec->lMax, ne = lMax * (lMax + 2);
  std::vector<qpms_complex_t> lc(ne), mc(ne), ec(ne);
  int rc = planewave_fill(th, ph, Es, bspec->lMax_L > 0 ? lc.data() : nullptr, mc.data(), ec.data(), lMax,
                          (int)bspec->norm);
  if (rc) return rc;
  if (!add) memset(target, 0, bspec->n * sizeof(qpms_complex_t));
  for (size_t i = 0; i < bspec->n; ++i) {
    int t, l, m;
    uvswfi_split(bspec->ilist[i], &t, &l, &m);
    if (l < 1 || l > lMax) continue;  // L00 and out-of-range elements get no contribution
    const int y = l * (l + 1) + m - 1;
    const qpms_complex_t v = t == 2 ? ec[y] : t == 1 ? mc[y] : lc[y];
    target[i] = from_cd(to_cd(target[i]) + to_cd(v));
  }
  return QPMS_SUCCESS;
}
qpms_complex_t *qpms_scatsys_incident_field_vector_full(qpms_complex_t *target_full, const qpms_scatsys_t *ss,
                                                        qpms_incfield_t f, const void *args, bool add) {
  const qpms_vswf_set_spec_t *bspec = scatsys_spec(ss);
  const bool own = !target_full;
  if (own) target_full = (qpms_complex_t *)calloc(std::max<size_t>(ss->fecv_size, 1), sizeof(qpms_complex_t));
  if (!target_full) {
    set_error("out of host memory");
    return nullptr;
  }
  for (qpms_ss_pi_t pi = 0; pi < ss->p_count; ++pi) {
    const size_t start = ss->fecv_pstarts ? ss->fecv_pstarts[pi] : (size_t)pi * bspec->n;
    if (f(target_full + start, bspec, ss->p[pi].pos, args, add)) {
      if (own) free(target_full);
      return nullptr;
    }
  }
  return target_full;
}

// ---------------- single translation coefficients ----------------
int qpms_trans_calculator_get_AB_p_ext(const qpms_trans_calculator *c, qpms_complex_t *Adest, qpms_complex_t *Bdest,
                                       int m, int n, int mu, int nu, qpms_complex_t kdlj_r, double kdlj_th,
                                       double kdlj_phi, int r_ge_d, int J) {
  return single_AB(c, Adest, Bdest, m, n, mu, nu, kdlj_r, kdlj_th, kdlj_phi, r_ge_d, J);
}
qpms_complex_t qpms_trans_calculator_get_A_ext(const qpms_trans_calculator *c, int m, int n, int mu, int nu,
                                               qpms_complex_t kdlj_r, double kdlj_th, double kdlj_phi, int r_ge_d,
                                               int J) {
  qpms_complex_t A;
  return single_AB(c, &A, nullptr, m, n, mu, nu, kdlj_r, kdlj_th, kdlj_phi, r_ge_d, J) ? nan_c() : A;
}
qpms_complex_t qpms_trans_calculator_get_B_ext(const qpms_trans_calculator *c, int m, int n, int mu, int nu,
                                               qpms_complex_t kdlj_r, double kdlj_th, double kdlj_phi, int r_ge_d,
                                               int J) {
  qpms_complex_t B;
  return single_AB(c, nullptr, &B, m, n, mu, nu, kdlj_r, kdlj_th, kdlj_phi, r_ge_d, J) ? nan_c() : B;
}
int qpms_trans_calculator_get_AB_p(const qpms_trans_calculator *c, qpms_complex_t *Adest, qpms_complex_t *Bdest,
                                   qpms_m_t m, qpms_l_t n, qpms_m_t mu, qpms_l_t nu, csph_t kdlj, bool r_ge_d,
                                   qpms_bessel_t J) {
  return single_AB(c, Adest, Bdest, m, n, mu, nu, kdlj.r, kdlj.theta, kdlj.phi, r_ge_d, J);
}
qpms_complex_t qpms_trans_calculator_get_A(const qpms_trans_calculator *c, qpms_m_t m, qpms_l_t n, qpms_m_t mu,
                                           qpms_l_t nu, csph_t kdlj, bool r_ge_d, qpms_bessel_t J) {
  return qpms_trans_calculator_get_A_ext(c, m, n, mu, nu, kdlj.r, kdlj.theta, kdlj.phi, r_ge_d, J);
}
qpms_complex_t qpms_trans_calculator_get_B(const qpms_trans_calculator *c, qpms_m_t m, qpms_l_t n, qpms_m_t mu,
                                           qpms_l_t nu, csph_t kdlj, bool r_ge_d, qpms_bessel_t J) {
  return qpms_trans_calculator_get_B_ext(c, m, n, mu, nu, kdlj.r, kdlj.theta, kdlj.phi, r_ge_d, J);
}
// A one-off calculator of lMax max(n, nu) per call, as the reference's
// single-coefficient functions recompute their factors per call.
qpms_complex_t qpms_trans_single_A(qpms_normalisation_t norm, qpms_m_t m, qpms_l_t n, qpms_m_t mu, qpms_l_t nu,
                                   csph_t kdlj, bool r_ge_d, qpms_bessel_t J) {
  qpms_trans_calculator *c = qpms_trans_calculator_init(std::max(n, nu), norm);
  if (!c) return nan_c();
  const qpms_complex_t r = qpms_trans_calculator_get_A(c, m, n, mu, nu, kdlj, r_ge_d, J);
  qpms_trans_calculator_free(c);
  return r;
}
qpms_complex_t qpms_trans_single_B(qpms_normalisation_t norm, qpms_m_t m, qpms_l_t n, qpms_m_t mu, qpms_l_t nu,
                                   csph_t kdlj, bool r_ge_d, qpms_bessel_t J) {
  qpms_trans_calculator *c = qpms_trans_calculator_init(std::max(n, nu), norm);
  if (!c) return nan_c();
  const qpms_complex_t r = qpms_trans_calculator_get_B(c, m, n, mu, nu, kdlj, r_ge_d, J);
  qpms_trans_calculator_free(c);
  return r;
}

// ---------------- Beyn contours ----------------
beyn_contour_t *beyn_contour_halfellipse(qpms_complex_t centre, double rRe, double rIm, size_t n,
                                         beyn_contour_halfellipse_orientation orient) {
  cd fk;
  double l, h;
  if (orientation(orient, rRe, rIm, &fk, &l, &h)) return nullptr;
  beyn_contour_t *c = contour_alloc(n, centre);
  if (!c) return nullptr;
  const cd z0 = to_cd(centre), I(0, 1);
  const size_t nline = n / 2, narc = n - nline;
  for (size_t i = 0; i < narc; ++i) {  // the arc, node i at t = (i + 1/2) pi / narc
    const double t = (i + 0.5) * M_PI / narc, st = sin(t), ct = cos(t);
    c->z_dz[i][0] = from_cd(z0 + fk * (ct * l + I * st * h));
    c->z_dz[i][1] = from_cd(fk * (-l * st + I * h * ct) * (M_PI / narc));
  }
  for (size_t i = 0; i < nline; ++i) {  // the straight side through the centre
    const double t = 0.5 * (1 - (double)nline) + i;
    c->z_dz[narc + i][0] = align_zero(z0 + fk * t * 2.0 * l / (double)nline, orient);
    c->z_dz[narc + i][1] = from_cd(fk * 2.0 * l / (double)nline);
  }
  c->z_dz[n][0] = from_cd(rRe);
  c->z_dz[n][1] = from_cd(rIm);
  memcpy(&c->z_dz[n + 1][0], &orient, sizeof orient);
  return c;
}
beyn_contour_t *beyn_contour_kidney(qpms_complex_t centre, double rRe, double rIm, double rounding, size_t n,
                                    beyn_contour_halfellipse_orientation orient) {
  if (!(rounding >= 0 && rounding < 0.5)) {
    set_error("kidney contour: rounding %g outside [0, 0.5)", rounding);
    return nullptr;
  }
  cd fk;
  double l, h;
  if (orientation(orient, rRe, rIm, &fk, &l, &h)) return nullptr;
  beyn_contour_t *c = contour_alloc(n, centre);
  if (!c) return nullptr;
  const cd z0 = to_cd(centre), I(0, 1);
  // corner circles of radius y centred at (+-x, y); the big arc of radius h
  const double y = rounding * h, x = sqrt((h - y) * (h - y) - y * y);
  const double alpha = asin(y / (h - y)), ar = l / h;
  const double tmax = 2 * (x + (M_PI_2 + alpha) * y + (M_PI_2 - alpha) * h), dt = tmax / n;
  size_t i = 0;
  double t, t_lo = 0, t_hi = x;
  for (; t = i * dt, t <= t_hi && i < n; ++i) {  // straight side, right half
    c->z_dz[i][0] = align_zero(z0 + (t - t_lo) * ar * fk, orient);
    c->z_dz[i][1] = from_cd(dt * ar * fk);
  }
  t_lo = t_hi;
  t_hi = t_lo + (M_PI_2 + alpha) * y;
  for (; t = i * dt, t < t_hi && i < n; ++i) {  // first corner
    const double phi = (t - t_lo) / y - M_PI_2;
    c->z_dz[i][0] = from_cd(z0 + (ar * (x + y * cos(phi)) + y * (1 + sin(phi)) * I) * fk);
    c->z_dz[i][1] = from_cd(dt * (-ar * sin(phi) + cos(phi) * I) * fk);
  }
  t_lo = t_hi;
  t_hi = t_lo + (M_PI - 2 * alpha) * h;
  for (; t = i * dt, t < t_hi && i < n; ++i) {  // big arc
    const double phi = (t - t_lo) / h + alpha;
    c->z_dz[i][0] = from_cd(z0 + (ar * (h * cos(phi)) + h * sin(phi) * I) * fk);
    c->z_dz[i][1] = from_cd(dt * (-ar * sin(phi) + cos(phi) * I) * fk);
  }
  t_lo = t_hi;
  t_hi = t_lo + (M_PI_2 + alpha) * y;
  for (; t = i * dt, t < t_hi && i < n; ++i) {  // second corner
    const double phi = (t - t_lo) / y + M_PI - alpha;
    c->z_dz[i][0] = from_cd(z0 + (ar * (-x + y * cos(phi)) + y * (1 + sin(phi)) * I) * fk);
    c->z_dz[i][1] = from_cd(dt * (-ar * sin(phi) + cos(phi) * I) * fk);
  }
  t_lo = t_hi;
  for (; t = i * dt, i < n; ++i) {  // straight side, left half
    c->z_dz[i][0] = align_zero(z0 + (t - t_lo - x) * ar * fk, orient);
    c->z_dz[i][1] = from_cd(dt * ar * fk);
  }
  c->z_dz[n][0] = from_cd(rRe);
  c->z_dz[n][1] = from_cd(rIm);
  memcpy(&c->z_dz[n + 1][0], &orient, sizeof orient);
  return c;
}

}  // extern "C"
