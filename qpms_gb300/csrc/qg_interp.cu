// Tabulated optical data: permittivity interpolators (materials.h:101-145,
// materials.c:11-153), T-matrix interpolators (tmatrices.h:285-330,
// tmatrices.c:287-350) and the SCUFF-EM T-matrix file reader
// (tmatrices.c:367-490).
//
// The reference interpolates with GSL (gsl_interp / gsl_spline); its Python
// layer always asks for gsl_interp_cspline (cymaterials.pyx:259,
// cytmatrices.pyx:38-39) and declares gsl_interp_linear.  Both are restated
// here from their published definitions: piecewise-linear interpolation, and
// the natural cubic spline (second derivative zero at both ends; the
// tridiagonal system for the knot curvatures solved by the Thomas algorithm).
// Outside the tabulated range an evaluation returns NaN (GSL's
// gsl_interp_eval reports GSL_EDOM there).
//
// Device side: qpms_gpu_tmatrix_interpolator_eval_batch evaluates all
// elements of T(omega) for a batch of frequencies in one kernel (one thread
// per (omega, element); the interval search is per thread over the shared
// knots), the T-matrix generation of a frequency sweep.
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <complex>
#include <mutex>
#include <string>
#include <vector>

#include "qg_internal.h"

typedef std::complex<double> cd;

struct qpms_interp_type_t {
  int kind;  // 0 linear, 1 natural cubic spline
  const char *name;
};

namespace qg {

// One tabulated function on strictly increasing knots x[0..n-1].
struct Spline {
  int kind = 0;
  std::vector<double> y, c;  // c[i] = S''(x_i) / 2 (cubic only)

  // Returns false if the data do not suit the kind (n < 2, or n < 3 for cubic).
  bool init(int kind_, size_t n, const double *x, const double *yv) {
    kind = kind_;
    y.assign(yv, yv + n);
    if (n < 2 || (kind == 1 && n < 3)) return false;
    c.assign(n, 0.0);
    if (kind == 1) {
      // h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i + h_i c_{i+1} = 3 (D_i - D_{i-1}), c_0 = c_{n-1} = 0
      const size_t m = n - 2;
      std::vector<double> diag(m), off(m), rhs(m);
      for (size_t j = 0; j < m; ++j) {
        const size_t i = j + 1;
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        diag[j] = 2 * (h0 + h1);
        off[j] = h1;  // coupling of c_i and c_{i+1}
        rhs[j] = 3 * ((yv[i + 1] - yv[i]) / h1 - (yv[i] - yv[i - 1]) / h0);
      }
      // Thomas algorithm on the symmetric tridiagonal system
      for (size_t j = 1; j < m; ++j) {
        const double w = off[j - 1] / diag[j - 1];
        diag[j] -= w * off[j - 1];
        rhs[j] -= w * rhs[j - 1];
      }
      for (size_t j = m; j-- > 0;) {
        double v = rhs[j];
        if (j + 1 < m) v -= off[j] * c[j + 2];
        c[j + 1] = v / diag[j];
      }
    }
    return true;
  }
};

// i with x[i] <= xq <= x[i+1], i in [0, n-2] (xq inside the range).
QG_HD size_t interval(const double *x, size_t n, double xq) {
  size_t lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const size_t mid = (lo + hi) / 2;
    if (x[mid] > xq) hi = mid;
    else lo = mid;
  }
  return lo;
}

QG_HD double spline_eval(int kind, const double *x, size_t n, const double *y, const double *c, double xq) {
  if (!(xq >= x[0] && xq <= x[n - 1])) return NAN;
  const size_t i = interval(x, n, xq);
  const double h = x[i + 1] - x[i], t = xq - x[i];
  const double D = (y[i + 1] - y[i]) / h;
  if (kind == 0) return y[i] + t * D;
  const double b = D - h * (c[i + 1] + 2 * c[i]) / 3;
  const double d = (c[i + 1] - c[i]) / (3 * h);
  return y[i] + t * (b + t * (c[i] + t * d));
}

namespace {
constexpr double kC0i = 299792458.0;      // materials.h:11
constexpr double kScuffOmegaUnit = 3e14;  // tmatrices.c:37

// qpms_normalisation_factor_{M,N} (normalisation.h:17-90) including the
// Condon-Shortley bit (normalisation.h:54-57, 118-131).
cd uvswfi_factor(int norm, qpms_uvswfi_t ui) {
  const int t = (int)(ui & 3);
  const long ysc = (long)(ui / 4);
  const int l = (int)floor(sqrt((double)ysc));
  const int m = (int)(ysc - (long)l * (l + 1));
  double nf = 1;
  switch (norm & (QPMS_NORMALISATION_NORM_POWER | QPMS_NORMALISATION_NORM_NONE)) {
    case QPMS_NORMALISATION_NORM_SPHARM: nf = sqrt((double)l * (l + 1)); break;
    case QPMS_NORMALISATION_NORM_NONE:
      nf = sqrt(l * (l + 1.0) * 4 * M_PI / (2 * l + 1)) * exp(0.5 * (lgamma(l + m + 1.0) - lgamma(l - m + 1.0)));
      break;
    default: break;
  }
  cd r(nf, 0);
  const bool mag = (t == 1);
  if (norm & (mag ? QPMS_NORMALISATION_M_MINUS : QPMS_NORMALISATION_N_MINUS)) r = -r;
  if (norm & (mag ? QPMS_NORMALISATION_M_I : QPMS_NORMALISATION_N_I)) r *= cd(0, 1);
  if (norm & QPMS_NORMALISATION_INVERSE) r = 1.0 / r;
  if ((norm & QPMS_NORMALISATION_CSPHASE) && (m % 2)) r = -r;
  return r;
}

__global__ void tmi_eval_kernel(int kind, const double *__restrict__ x, int nk, const double *__restrict__ yre,
                                const double *__restrict__ cre, const double *__restrict__ yim,
                                const double *__restrict__ cim, const unsigned char *__restrict__ flags, int ne,
                                const double *__restrict__ freqs, int nf, qg_c *__restrict__ out) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)nf * ne) return;
  const int w = (int)(idx / ne), e = (int)(idx % ne);
  const double f = freqs[w];
  const unsigned char fl = flags[e];
  double re = 0, im = 0;
  if (fl & 1) re = spline_eval(kind, x, nk, yre + (size_t)e * nk, cre + (size_t)e * nk, f);
  if (fl & 2) im = spline_eval(kind, x, nk, yim + (size_t)e * nk, cim + (size_t)e * nk, f);
  out[idx] = cmk(re, im);
}
}  // namespace

// the factor of the wave ui in normalisation norm (other translation units)
qg_c uvswfi_norm_factor(int norm, qpms_uvswfi_t ui) {
  const cd f = uvswfi_factor(norm, ui);
  return cmk(f.real(), f.imag());
}
}  // namespace qg

using namespace qg;

struct qpms_permittivity_interpolator_t {
  std::vector<double> wl, n, k;  // wavelength in metres, refractive index, extinction coefficient
  Spline sn, sk;
  int kind = 1;
};

struct qpms_tmatrix_interpolator_t {
  qpms_vswf_set_spec_t spec;
  std::vector<qpms_uvswfi_t> ilist;
  size_t n = 0, nf = 0;
  int kind = 1;
  std::vector<double> freqs;
  std::vector<unsigned char> flags;        // per element: 1 real part tabulated non-zero, 2 imaginary
  std::vector<double> yre, cre, yim, cim;  // [element][knot]
  struct DevCopy {
    int dev;
    double *x, *yre, *cre, *yim, *cim;
    unsigned char *flags;
  };
  std::vector<DevCopy> devs;
  std::mutex mu;
  ~qpms_tmatrix_interpolator_t() {
    if (devs.empty()) return;  // never used on a device: no CUDA call
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto &d : devs) {
      cudaSetDevice(d.dev);
      for (void *p : {(void *)d.x, (void *)d.yre, (void *)d.cre, (void *)d.yim, (void *)d.cim, (void *)d.flags})
        cudaFree(p);
    }
    cudaSetDevice(cur);
  }
};

static const qpms_interp_type_t g_linear = {0, "linear"}, g_cspline = {1, "cspline"};

namespace qg {
// Accessors for the scattering-system code (qg_scatsys.cu).
cd permittivity_interp_eps(const qpms_permittivity_interpolator_t *ip, double omega);
void tmatrix_interp_eval(const qpms_tmatrix_interpolator_t *ip, double freq, qg_c *out);
const qpms_vswf_set_spec_t *tmatrix_interp_spec(const qpms_tmatrix_interpolator_t *ip);

cd permittivity_interp_eps(const qpms_permittivity_interpolator_t *ip, double omega) {
  // materials.c:120-129: n, k at the vacuum wavelength, eps = (n + i k)^2
  const double lambda = 2 * M_PI * kC0i / omega;
  const size_t N = ip->wl.size();
  const double n = spline_eval(ip->kind, ip->wl.data(), N, ip->n.data(), ip->sn.c.data(), lambda);
  const double k = spline_eval(ip->kind, ip->wl.data(), N, ip->k.data(), ip->sk.c.data(), lambda);
  return cd(n * n - k * k, 2 * n * k);
}

// T(freq), row-major n x n; elements without tabulated data are zero
// (tmatrices.c:339-349 writes only the tabulated ones into a fresh T-matrix).
void tmatrix_interp_eval(const qpms_tmatrix_interpolator_t *ip, double freq, qg_c *out) {
  const size_t ne = ip->n * ip->n, nk = ip->nf;
  for (size_t e = 0; e < ne; ++e) {
    double re = 0, im = 0;
    if (ip->flags[e] & 1) re = spline_eval(ip->kind, ip->freqs.data(), nk, &ip->yre[e * nk], &ip->cre[e * nk], freq);
    if (ip->flags[e] & 2) im = spline_eval(ip->kind, ip->freqs.data(), nk, &ip->yim[e * nk], &ip->cim[e * nk], freq);
    out[e] = cmk(re, im);
  }
}

const qpms_vswf_set_spec_t *tmatrix_interp_spec(const qpms_tmatrix_interpolator_t *ip) { return &ip->spec; }
}  // namespace qg

extern "C" {

const qpms_interp_type_t *const qpms_interp_linear = &g_linear;
const qpms_interp_type_t *const qpms_interp_cspline = &g_cspline;

// ---------------- permittivity ----------------
qpms_permittivity_interpolator_t *qpms_permittivity_interpolator_create(size_t incount, const double *wavelength_m,
                                                                        const double *n, const double *k,
                                                                        const qpms_interp_type_t *iptype) {
  clear_error();
  if (incount == 0 || !wavelength_m || !n || !k || !iptype) {
    set_error("permittivity interpolator: empty or NULL input");
    return nullptr;
  }
  for (size_t i = 1; i < incount; ++i)
    if (!(wavelength_m[i] > wavelength_m[i - 1])) {
      set_error("permittivity interpolator: wavelengths must increase strictly");
      return nullptr;
    }
  auto *ip = new (std::nothrow) qpms_permittivity_interpolator_t();
  if (!ip) { set_error("out of host memory"); return nullptr; }
  ip->kind = iptype->kind;
  ip->wl.assign(wavelength_m, wavelength_m + incount);
  ip->n.assign(n, n + incount);
  ip->k.assign(k, k + incount);
  if (!ip->sn.init(ip->kind, incount, ip->wl.data(), n) || !ip->sk.init(ip->kind, incount, ip->wl.data(), k)) {
    set_error("permittivity interpolator: %zu points are too few for %s interpolation", incount, iptype->name);
    delete ip;
    return nullptr;
  }
  return ip;
}

// qpms_read_refractiveindex_yml (materials.c:43-87): the "data: |" block of a
// refractiveindex.info file, lines "wavelength_um n k" until the first line
// that is not such a triple; '#' lines are skipped.
int qpms_load_refractiveindex_yml(const char *path, size_t *count, double **lambdas_m, double **n, double **k) {
  clear_error();
  if (!path || !count || !lambdas_m || !n || !k) { set_error("NULL argument"); return QPMS_EINVAL; }
  FILE *f = fopen(path, "r");
  if (!f) { set_error("could not open refractive index file %s", path); return errno ? errno : QPMS_ERROR; }
  std::vector<double> L, N, K;
  char line[1024];
  bool started = false;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    if (!started) {
      if (strstr(line, "data: |")) started = true;
      continue;
    }
    double a, b, c;
    if (sscanf(line, "%lf %lf %lf", &a, &b, &c) == 3) {
      L.push_back(a * 1e-6);  // micrometres in the file
      N.push_back(b);
      K.push_back(c);
    } else {
      break;
    }
  }
  fclose(f);
  if (L.empty()) { set_error("no refractive index data in %s", path); return QPMS_ERROR; }
  *count = L.size();
  *lambdas_m = (double *)malloc(L.size() * 8);
  *n = (double *)malloc(L.size() * 8);
  *k = (double *)malloc(L.size() * 8);
  if (!*lambdas_m || !*n || !*k) { set_error("out of host memory"); return QPMS_ENOMEM; }
  memcpy(*lambdas_m, L.data(), L.size() * 8);
  memcpy(*n, N.data(), L.size() * 8);
  memcpy(*k, K.data(), L.size() * 8);
  return QPMS_SUCCESS;
}

qpms_permittivity_interpolator_t *qpms_permittivity_interpolator_from_yml(const char *path,
                                                                          const qpms_interp_type_t *iptype) {
  size_t cnt = 0;
  double *l = nullptr, *n = nullptr, *k = nullptr;
  if (qpms_load_refractiveindex_yml(path, &cnt, &l, &n, &k)) return nullptr;
  qpms_permittivity_interpolator_t *ip = qpms_permittivity_interpolator_create(cnt, l, n, k, iptype);
  free(l);
  free(n);
  free(k);
  return ip;
}

void qpms_permittivity_interpolator_free(qpms_permittivity_interpolator_t *ip) { delete ip; }

qpms_complex_t qpms_permittivity_interpolator_eps_at_omega(const qpms_permittivity_interpolator_t *ip,
                                                           double omega_SI) {
  qpms_complex_t r;
  r.re = r.im = NAN;
  if (!ip) return r;
  const cd e = permittivity_interp_eps(ip, omega_SI);
  r.re = e.real();
  r.im = e.imag();
  return r;
}

// materials.c:179-181: the constant medium *params as a qpms_epsmu_generator_t
qpms_epsmu_t qpms_epsmu_const_g(qpms_complex_t omega, const void *epsmu) {
  (void)omega;
  return *(const qpms_epsmu_t *)epsmu;
}

// qpms_epsmu_generator_t form (materials.c:131-142): Im omega is discarded.
qpms_epsmu_t qpms_permittivity_interpolator_epsmu_g(qpms_complex_t omega, const void *interp) {
  qpms_epsmu_t em;
  em.eps = qpms_permittivity_interpolator_eps_at_omega((const qpms_permittivity_interpolator_t *)interp, omega.re);
  em.mu.re = 1;
  em.mu.im = 0;
  return em;
}

double qpms_permittivity_interpolator_omega_max(const qpms_permittivity_interpolator_t *ip) {
  return 2 * M_PI * kC0i / ip->wl.front();
}

double qpms_permittivity_interpolator_omega_min(const qpms_permittivity_interpolator_t *ip) {
  return 2 * M_PI * kC0i / ip->wl.back();
}

// ---------------- VSWF sets and T-matrices ----------------
// vswf.c:76-92: electric block l = 1..lMax, m = -l..l, then the magnetic block.
qpms_vswf_set_spec_t *qpms_vswf_set_spec_from_lMax(qpms_l_t lMax, qpms_normalisation_t norm) {
  clear_error();
  if (lMax < 1) { set_error("lMax must be >= 1"); return nullptr; }
  auto *c = (qpms_vswf_set_spec_t *)malloc(sizeof(qpms_vswf_set_spec_t));
  const size_t ne = (size_t)lMax * (lMax + 2);
  if (!c) return nullptr;
  c->n = c->capacity = 2 * ne;
  c->ilist = (qpms_uvswfi_t *)malloc(sizeof(qpms_uvswfi_t) * 2 * ne);
  if (!c->ilist) { free(c); return nullptr; }
  size_t i = 0;
  for (int it = 0; it < 2; ++it)
    for (int l = 1; l <= lMax; ++l)
      for (int m = -l; m <= l; ++m) c->ilist[i++] = (it ? 1 : 2) + 4 * (qpms_uvswfi_t)(l * (l + 1) + m);
  c->norm = norm;
  c->lMax = c->lMax_M = c->lMax_N = lMax;
  c->lMax_L = -1;
  return c;
}

void qpms_vswf_set_spec_free(qpms_vswf_set_spec_t *s) {
  if (s) free(s->ilist);
  free(s);
}

qpms_tmatrix_t *qpms_tmatrix_init(const qpms_vswf_set_spec_t *bspec) {
  auto *t = (qpms_tmatrix_t *)malloc(sizeof(qpms_tmatrix_t));
  if (!t) return nullptr;
  t->spec = bspec;
  t->m = (qpms_complex_t *)calloc(bspec->n * bspec->n, sizeof(qpms_complex_t));
  t->owns_m = true;
  if (!t->m) { free(t); return nullptr; }
  return t;
}

void qpms_tmatrix_free(qpms_tmatrix_t *t) {
  if (t && t->owns_m) free(t->m);
  free(t);
}

static bool same_spec(const qpms_vswf_set_spec_t *a, const qpms_vswf_set_spec_t *b) {
  if (a == b) return true;
  if (a->n != b->n || a->norm != b->norm) return false;
  for (size_t i = 0; i < a->n; ++i)
    if (a->ilist[i] != b->ilist[i]) return false;
  return true;
}

qpms_tmatrix_interpolator_t *qpms_tmatrix_interpolator_create(size_t incount, const double *freqs,
                                                              const qpms_tmatrix_t *ta,
                                                              const qpms_interp_type_t *iptype) {
  clear_error();
  if (incount == 0 || !freqs || !ta || !iptype || !ta[0].spec) {
    set_error("T-matrix interpolator: empty or NULL input");
    return nullptr;
  }
  for (size_t i = 0; i < incount; ++i)
    if (!same_spec(ta[0].spec, ta[i].spec)) {
      set_error("All T-matrices for interpolation must have the same basis!");
      return nullptr;
    }
  for (size_t i = 1; i < incount; ++i)
    if (!(freqs[i] > freqs[i - 1])) {
      set_error("T-matrix interpolator: frequencies must increase strictly");
      return nullptr;
    }
  if (incount < 2 || (iptype->kind == 1 && incount < 3)) {
    set_error("T-matrix interpolator: %zu frequencies are too few for %s interpolation", incount, iptype->name);
    return nullptr;
  }
  auto *ip = new (std::nothrow) qpms_tmatrix_interpolator_t();
  if (!ip) { set_error("out of host memory"); return nullptr; }
  const size_t n = ta[0].spec->n, ne = n * n;
  ip->ilist.assign(ta[0].spec->ilist, ta[0].spec->ilist + n);
  ip->spec = *ta[0].spec;
  ip->spec.ilist = ip->ilist.data();
  ip->spec.capacity = n;
  ip->n = n;
  ip->nf = incount;
  ip->kind = iptype->kind;
  ip->freqs.assign(freqs, freqs + incount);
  ip->flags.assign(ne, 0);
  ip->yre.assign(ne * incount, 0.0);
  ip->cre.assign(ne * incount, 0.0);
  ip->yim.assign(ne * incount, 0.0);
  ip->cim.assign(ne * incount, 0.0);
  std::vector<double> yr(incount), yi(incount);
  Spline s;
  for (size_t e = 0; e < ne; ++e) {
    bool nzr = false, nzi = false;
    for (size_t i = 0; i < incount; ++i) {
      yr[i] = ta[i].m[e].re;
      yi[i] = ta[i].m[e].im;
      nzr |= yr[i] != 0;
      nzi |= yi[i] != 0;
    }
    // tmatrices.c:303-325: a spline only for elements that are non-zero somewhere
    if (nzr) {
      s.init(ip->kind, incount, freqs, yr.data());
      memcpy(&ip->yre[e * incount], yr.data(), incount * 8);
      memcpy(&ip->cre[e * incount], s.c.data(), incount * 8);
      ip->flags[e] |= 1;
    }
    if (nzi) {
      s.init(ip->kind, incount, freqs, yi.data());
      memcpy(&ip->yim[e * incount], yi.data(), incount * 8);
      memcpy(&ip->cim[e * incount], s.c.data(), incount * 8);
      ip->flags[e] |= 2;
    }
  }
  return ip;
}

void qpms_tmatrix_interpolator_free(qpms_tmatrix_interpolator_t *ip) { delete ip; }

// tmatrices.c:339-349: elements with tabulated data are overwritten (real
// part) and incremented (imaginary part); the others keep their value.
int qpms_tmatrix_interpolator_eval_fill(qpms_tmatrix_t *t, const qpms_tmatrix_interpolator_t *ip, double freq) {
  clear_error();
  if (!t || !ip || !t->spec || !same_spec(t->spec, &ip->spec)) {
    set_error("Tried to fill a T-matrix with an incompatible interpolator!");
    return QPMS_EINVAL;
  }
  const size_t ne = ip->n * ip->n, nk = ip->nf;
  for (size_t e = 0; e < ne; ++e) {
    if (ip->flags[e] & 1) {
      t->m[e].re = spline_eval(ip->kind, ip->freqs.data(), nk, &ip->yre[e * nk], &ip->cre[e * nk], freq);
      t->m[e].im = 0;
    }
    if (ip->flags[e] & 2)
      t->m[e].im += spline_eval(ip->kind, ip->freqs.data(), nk, &ip->yim[e * nk], &ip->cim[e * nk], freq);
  }
  return QPMS_SUCCESS;
}

qpms_tmatrix_t *qpms_tmatrix_interpolator_eval(const qpms_tmatrix_interpolator_t *ip, double freq) {
  if (!ip) return nullptr;
  qpms_tmatrix_t *t = qpms_tmatrix_init(&ip->spec);
  if (!t) { set_error("out of host memory"); return nullptr; }
  qpms_tmatrix_interpolator_eval_fill(t, ip, freq);
  return t;
}

// qpms_tmatrix_generator_t form (tmatrices.c:351-356): Re omega is the frequency.
int qpms_tmatrix_generator_interpolator(qpms_tmatrix_t *t, qpms_complex_t omega, const void *interp) {
  return qpms_tmatrix_interpolator_eval_fill(t, (const qpms_tmatrix_interpolator_t *)interp, omega.re);
}

const qpms_vswf_set_spec_t *qpms_tmatrix_interpolator_bspec(const qpms_tmatrix_interpolator_t *ip) {
  return ip ? &ip->spec : nullptr;
}

// T(freqs[w]) for nf frequencies into out[w][n][n] (row-major), DEVICE
// pointers, on `stream`.  The tabulated data go to the device on first use.
int qpms_gpu_tmatrix_interpolator_eval_batch(const qpms_tmatrix_interpolator_t *ipc, size_t nf, const double *d_freqs,
                                             qpms_complex_t *d_out, void *stream) {
  clear_error();
  if (!ipc || !d_freqs || !d_out) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (nf == 0) return QPMS_SUCCESS;
  auto *ip = const_cast<qpms_tmatrix_interpolator_t *>(ipc);
  const size_t ne = ip->n * ip->n, nk = ip->nf;
  if (nf > (size_t)(1u << 30) / (ne ? ne : 1)) { set_error("batch too large"); return QPMS_EINVAL; }
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  qpms_tmatrix_interpolator_t::DevCopy dc{};
  {
    std::lock_guard<std::mutex> g(ip->mu);
    bool found = false;
    for (auto &d : ip->devs)
      if (d.dev == dev) {
        dc = d;
        found = true;
      }
    if (!found) {
      dc.dev = dev;
      const size_t b = ne * nk * 8;
      QG_CUDA_TRY(cudaMalloc(&dc.x, nk * 8));
      QG_CUDA_TRY(cudaMalloc(&dc.yre, b));
      QG_CUDA_TRY(cudaMalloc(&dc.cre, b));
      QG_CUDA_TRY(cudaMalloc(&dc.yim, b));
      QG_CUDA_TRY(cudaMalloc(&dc.cim, b));
      QG_CUDA_TRY(cudaMalloc(&dc.flags, ne));
      QG_CUDA_TRY(cudaMemcpy(dc.x, ip->freqs.data(), nk * 8, cudaMemcpyHostToDevice));
      QG_CUDA_TRY(cudaMemcpy(dc.yre, ip->yre.data(), b, cudaMemcpyHostToDevice));
      QG_CUDA_TRY(cudaMemcpy(dc.cre, ip->cre.data(), b, cudaMemcpyHostToDevice));
      QG_CUDA_TRY(cudaMemcpy(dc.yim, ip->yim.data(), b, cudaMemcpyHostToDevice));
      QG_CUDA_TRY(cudaMemcpy(dc.cim, ip->cim.data(), b, cudaMemcpyHostToDevice));
      QG_CUDA_TRY(cudaMemcpy(dc.flags, ip->flags.data(), ne, cudaMemcpyHostToDevice));
      ip->devs.push_back(dc);
    }
  }
  const size_t tot = nf * ne;
  tmi_eval_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      ip->kind, dc.x, (int)nk, dc.yre, dc.cre, dc.yim, dc.cim, dc.flags, (int)ne, d_freqs, (int)nf, (qg_c *)d_out);
  g_launches.fetch_add(1);
  QG_CUDA_TRY(cudaGetLastError());
  return QPMS_SUCCESS;
}

// ---------------- SCUFF-EM T-matrix files ----------------
// qpms_read_scuff_tmatrix (tmatrices.c:367-465): lines
//   "freq_SU Alpha LAlpha MAlpha PAlpha Beta LBeta MBeta PBeta ReT ImT",
// P = 0 magnetic, 1 electric; a new frequency starts a new T-matrix (NaN
// until filled); the element goes to [Beta][Alpha] of the requested basis,
// converted from the SCUFF convention to bs->norm; freq = freq_SU * 3e14 rad/s.
int qpms_load_scuff_tmatrix(const char *path, const qpms_vswf_set_spec_t *bs, size_t *n_out, double **freqs,
                            double **freqs_su, qpms_tmatrix_t **tmatrices_array, qpms_complex_t **tmdata) {
  clear_error();
  if (!path || !bs || !n_out || !freqs || !tmdata) { set_error("NULL argument"); return QPMS_EINVAL; }
  if (bs->norm & (QPMS_NORMALISATION_REVERSE_AZIMUTHAL_PHASE | QPMS_NORMALISATION_SPHARM_REAL)) {
    set_error("only standard complex-spherical-harmonic waves are supported");
    return QPMS_EINVAL;
  }
  FILE *f = fopen(path, "r");
  if (!f) { set_error("Could not open T-matrix file %s", path); return errno ? errno : QPMS_ERROR; }
  const size_t bn = bs->n, nn = bn * bn;
  std::vector<double> F, Fsu;
  std::vector<qpms_complex_t> data;
  char line[1024];
  double last = NAN;
  int ret = QPMS_SUCCESS;
  const int scuff = QPMS_NORMALISATION_NORM_POWER | QPMS_NORMALISATION_CSPHASE | QPMS_NORMALISATION_M_I |
                    QPMS_NORMALISATION_N_MINUS;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    int A, LA, MA, PA, B, LB, MB, PB;
    double fr, tr, ti;
    if (sscanf(line, "%lf %d %d %d %d %d %d %d %d %lf %lf", &fr, &A, &LA, &MA, &PA, &B, &LB, &MB, &PB, &tr, &ti) != 11) {
      bool blank = true;
      for (const char *c = line; *c; ++c)
        if (*c != ' ' && *c != '\t' && *c != '\n' && *c != '\r') blank = false;
      if (blank) continue;
      set_error("Malformed T-matrix file %s", path);
      ret = QPMS_ERROR;
      break;
    }
    if (fr != last) {
      last = fr;
      Fsu.push_back(fr);
      F.push_back(fr * kScuffOmegaUnit);
      const qpms_complex_t nanc = {NAN, NAN};
      data.insert(data.end(), nn, nanc);
    }
    if ((PA != 0 && PA != 1) || (PB != 0 && PB != 1)) { set_error("bad polarisation index"); ret = QPMS_ERROR; break; }
    if (LA < 1 || LB < 1 || abs(MA) > LA || abs(MB) > LB) continue;  // not a transversal wave of any basis
    const qpms_uvswfi_t src = (PA ? 2 : 1) + 4 * (qpms_uvswfi_t)(LA * (LA + 1) + MA);
    const qpms_uvswfi_t dst = (PB ? 2 : 1) + 4 * (qpms_uvswfi_t)(LB * (LB + 1) + MB);
    long si = -1, di = -1;
    for (size_t i = 0; i < bn; ++i) {
      if (bs->ilist[i] == src) si = (long)i;
      if (bs->ilist[i] == dst) di = (long)i;
    }
    if (si < 0 || di < 0) continue;  // not in the requested basis
    const cd v = cd(tr, ti) * uvswfi_factor(bs->norm, src) / uvswfi_factor(bs->norm, dst) *
                 uvswfi_factor(scuff, dst) / uvswfi_factor(scuff, src);
    qpms_complex_t &o = data[(F.size() - 1) * nn + (size_t)di * bn + (size_t)si];
    o.re = v.real();
    o.im = v.imag();
  }
  fclose(f);
  if (ret) return ret;
  const size_t nf = F.size();
  *n_out = nf;
  *freqs = (double *)malloc(nf * 8 + 8);
  memcpy(*freqs, F.data(), nf * 8);
  if (freqs_su) {
    *freqs_su = (double *)malloc(nf * 8 + 8);
    memcpy(*freqs_su, Fsu.data(), nf * 8);
  }
  *tmdata = (qpms_complex_t *)malloc(data.size() * sizeof(qpms_complex_t) + 16);
  memcpy(*tmdata, data.data(), data.size() * sizeof(qpms_complex_t));
  if (tmatrices_array) {
    *tmatrices_array = (qpms_tmatrix_t *)malloc(nf * sizeof(qpms_tmatrix_t) + 8);
    for (size_t i = 0; i < nf; ++i) {
      (*tmatrices_array)[i].spec = bs;
      (*tmatrices_array)[i].m = *tmdata + i * nn;
      (*tmatrices_array)[i].owns_m = false;
    }
  }
  for (size_t i = 0; i < data.size(); ++i)
    if (isnan(data[i].re) || isnan(data[i].im)) {
      set_error("Encountered NAN in a loaded T-matrix");
      ret |= QPMS_NAN_ENCOUNTERED;
      break;
    }
  return ret;
}

}  // extern "C"
