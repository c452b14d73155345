// Scattering systems: constructors, T-matrices at omega, and the drop-in
// mode-problem entry points (assembly, LU, solve) over the GPU kernels.
//
// Host work here is O(particles) set-up only (T-matrix diagonals per omega,
// the plane wave's direction coefficients); every O(N^2) or O(N^3) step --
// translation blocks, M = I - T S, LU, solves, residuals -- runs on the GPU.
#include <cublas_v2.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <mutex>
#include <new>
#include <vector>

#include "qg_assembly.h"
#include "qg_internal.h"
#include "qg_specfunc.cuh"

namespace qg {
std::complex<double> permittivity_interp_eps(const qpms_permittivity_interpolator_t *ip, double omega);  // qg_interp.cu
void tmatrix_interp_eval(const qpms_tmatrix_interpolator_t *ip, double freq, qg_c *out);
const qpms_vswf_set_spec_t *tmatrix_interp_spec(const qpms_tmatrix_interpolator_t *ip);
namespace {

typedef std::complex<double> cd;
constexpr double kC0 = 2.99792458e8;  // materials.h:11

cd to_cd(qpms_complex_t z) { return cd(z.re, z.im); }
qpms_complex_t from_cd(cd z) {
  qpms_complex_t r;
  r.re = z.real();
  r.im = z.imag();
  return r;
}

// ---------------- cuBLAS handle (one per host thread and device) ----------------
struct BlasSlot {
  int dev = -1;
  cublasHandle_t h = nullptr;
};
thread_local BlasSlot t_blas;

int blas_handle(cublasHandle_t *h) {
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  if (t_blas.h && t_blas.dev == dev) {
    *h = t_blas.h;
    return QPMS_SUCCESS;
  }
  if (t_blas.h) cublasDestroy(t_blas.h);
  t_blas.h = nullptr;
  if (cublasCreate(&t_blas.h) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return QPMS_ERROR;
  }
  t_blas.dev = dev;
  *h = t_blas.h;
  return QPMS_SUCCESS;
}



// ---------------- Mie sphere T-matrix (tmatrices.c:500-561) ----------------
template <int L>
void bessel_fill_host(int J, cd x, cd *out) {
  qg_c z[L + 1];
  sph_bessel<L>(J, cmk(x.real(), x.imag()), z);
  for (int l = 0; l <= L; ++l) out[l] = cd(z[l].re, z[l].im);
}
void bessel_fill(int J, int L, cd x, cd *out) {
  switch (L) {
#define QG_C(LL) case LL: bessel_fill_host<LL>(J, x, out); break;
    QG_C(2) QG_C(3) QG_C(4) QG_C(5) QG_C(6) QG_C(7) QG_C(8) QG_C(9) QG_C(10) QG_C(11)
#undef QG_C
    default: for (int l = 0; l <= L; ++l) out[l] = cd(NAN, NAN);
  }
}

// Mie reflection coefficients RV (electric), RH (magnetic), l = 0..lMax;
// Je / Js the Bessel kinds of the exciting and scattered waves.
void mie_coefficients(int lMax, double a, cd k_i, cd k_e, cd mu_i, cd mu_e, cd *RV, cd *RH, int Je = 1, int Js = 3) {
  const cd x_i = k_i * a, x_e = k_e * a;
  const cd eta_inv_i = k_i / mu_i, eta_inv_e = k_e / mu_e;
  std::vector<cd> zi(lMax + 2), ze(lMax + 2), zs(lMax + 2);
  bessel_fill(1, lMax + 1, x_i, zi.data());
  bessel_fill(Je, lMax + 1, x_e, ze.data());
  bessel_fill(Js, lMax + 1, x_e, zs.data());
  for (int l = 0; l <= lMax; ++l) {
    const cd dzi = -zi[l + 1] + double(l) / x_i * zi[l];
    const cd dze = -ze[l + 1] + double(l) / x_e * ze[l];
    const cd dzs = -zs[l + 1] + double(l) / x_e * zs[l];
    const cd fi = zi[l] / x_i + dzi, fs = zs[l] / x_e + dzs, fe = ze[l] / x_e + dze;
    RV[l] = (-eta_inv_i * fe * zi[l] + eta_inv_e * ze[l] * fi) / (-eta_inv_e * fi * zs[l] + eta_inv_i * zi[l] * fs);
    RH[l] = (-eta_inv_e * fe * zi[l] + eta_inv_i * ze[l] * fi) / (-eta_inv_i * fi * zs[l] + eta_inv_e * zi[l] * fs);
  }
}

// ---------------- plane-wave coefficients (vswf.c:338-379, 445-530) ----------------
// Electric and magnetic coefficients of a plane wave with direction (theta,
// phi) and local-basis amplitude Es (r, theta, phi components), default
// normalisation (its dual: e^{-im phi}, Condon-Shortley phase).
void planewave_coeffs(int lMax, double theta, double phi, const cd Es[3], cd *el, cd *mg) {
  const double ct = cos(theta), st = sin(theta);
  const int ne = lMax * (lMax + 2);
  std::vector<double> pi(ne, 0.0), tau(ne, 0.0);
  const double csphase = -1.0;
  if (fabs(ct) == 1.0) {  // legendre.c:71-88
    for (int l = 1; l <= lMax; ++l) {
      const double fl = 0.25 * sqrt((2 * l + 1) / M_PI);
      const int lpar = (l % 2) ? -1 : 1;
      pi[l * (l + 1) + 1 - 1] = -((ct > 0) ? -1 : lpar) * fl * csphase;
      pi[l * (l + 1) - 1 - 1] = -((ct > 0) ? -1 : lpar) * fl * csphase;
      tau[l * (l + 1) + 1 - 1] = ((ct > 0) ? +1 : lpar) * fl * csphase;
      tau[l * (l + 1) - 1 - 1] = -((ct > 0) ? +1 : lpar) * fl * csphase;
    }
  } else {  // legendre.c:89-110 with GSL spharm normalisation
    std::vector<double> P((lMax + 2) * (lMax + 3) / 2);
    for (int m = 0; m <= lMax + 1; ++m) legendre_column(lMax + 1, m, ct, P.data());
    for (int l = 1; l <= lMax; ++l)
      for (int m = 0; m <= l; ++m) {
        const double plm = P[l * (l + 1) / 2 + m];
        const double plm1 = (l - 1 >= m) ? P[(l - 1) * l / 2 + m] : 0.0;
        const double dplm = (l * ct * plm - (l + m) * plm1) / (ct * ct - 1);
        const double nf = sqrt((2 * l + 1) / (4 * M_PI) * exp(lgamma(l - m + 1.0) - lgamma(l + m + 1.0))) /
                          sqrt(l * (l + 1.0));
        const int yp = l * (l + 1) + m - 1, ym = l * (l + 1) - m - 1;
        pi[yp] = m / st * nf * plm;
        tau[yp] = -st * nf * dplm;
        if (m > 0) {
          const double f = (m % 2) ? -1.0 : 1.0;
          pi[ym] = -m / st * f * nf * plm;
          tau[ym] = -st * f * nf * dplm;
        }
      }
  }
  static const cd ipw[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
  for (int l = 1, y = 0; l <= lMax; ++l) {
    const cd pre1 = 4 * M_PI * ipw[l % 4], pre23 = -4 * M_PI * ipw[(l + 1) % 4];
    for (int m = -l; m <= l; ++m, ++y) {
      const cd eimf = std::exp(cd(0, -m * phi));
      const cd deimf = (m == 0) ? cd(0, 0) : cd(0, -1) * eimf;
      mg[y] = pre1 * (pi[y] * deimf * Es[1] - tau[y] * eimf * Es[2]);
      el[y] = pre23 * (tau[y] * eimf * Es[1] + pi[y] * deimf * Es[2]);
    }
  }
}

// ---------------- system object ----------------
struct SphereKind {
  double radius;
  cd eps;                                 // constant permittivity, or
  std::vector<qpms_ldparams_triple_t> ld;  // Lorentz-Drude oscillators (non-empty: used), or
  double ld_omega_p = 0;
  const qpms_permittivity_interpolator_t *pint = nullptr;  // tabulated n, k (set: used)
  const qpms_tmatrix_interpolator_t *tmi = nullptr;        // set: tabulated T(omega), not a sphere
  std::vector<double> axnodes;  // non-empty: axially symmetric particle, surface quadrature nodes
  int ax_lext = 0;              // its lMax_extend
  int ax_zsym = 0;              // its surface is symmetric under z -> -z
};

// qpms_lorentzdrude_eps (materials.c:156-164): sum_j f_j wp^2 / (w_j^2 - w^2 - i w g_j).
// As there, eps_inf is not added (the parameter sets carry eps_inf = 1).
cd lorentzdrude_eps(cd omega, double omega_p, const qpms_ldparams_triple_t *d, size_t n) {
  cd eps = 0;
  for (size_t j = 0; j < n; ++j)
    eps += d[j].f * omega_p * omega_p / (d[j].omega * d[j].omega - omega * omega - cd(0, 1) * omega * d[j].gamma);
  return eps;
}
cd kind_eps(const SphereKind &k, cd omega) {
  if (k.pint) return permittivity_interp_eps(k.pint, omega.real());  // Im omega discarded, materials.c:131-142
  return k.ld.empty() ? k.eps : lorentzdrude_eps(omega, k.ld_omega_p, k.ld.data(), k.ld.size());
}

struct ScatsysPriv {
  qpms_scatsys_t pub;  // first member: the public, reference-layout view
  std::vector<qpms_particle_tid_t> p;
  std::vector<size_t> pstarts;
  qpms_vswf_set_spec_t spec;
  std::vector<qpms_uvswfi_t> ilist;
  std::vector<SphereKind> kinds;
  cd eps_medium;
  qpms_epsmu_t medium_const;  // params of the constant-medium generator
  int lMax = 0;
  bool dense = false;  // some kind has a tabulated (full) T-matrix: every T is passed dense
  // device copies
  double *d_pos = nullptr;
  int *d_tmid = nullptr;
};

struct SswPriv {
  qpms_scatsys_at_omega_t pub;
  std::vector<qpms_tmatrix_t> tms;
  std::vector<qpms_tmatrix_t *> tmp;
  std::vector<std::vector<qg_c>> tdata;  // dense n x n per type
};

ScatsysPriv *sspriv(const qpms_scatsys_t *ss) {
  return reinterpret_cast<ScatsysPriv *>(const_cast<qpms_scatsys_t *>(ss));
}

qpms_epsmu_t epsmu_const_fn(qpms_complex_t, const void *params) {
  return *reinterpret_cast<const qpms_epsmu_t *>(params);
}

// T diagonal (bspec order: electric block then magnetic block) of kind t at omega
void sphere_tdiag(const ScatsysPriv *s, int t, cd omega, std::vector<cd> &out) {
  const int lMax = s->lMax, ne = lMax * (lMax + 2);
  const cd k_i = std::sqrt(kind_eps(s->kinds[t], omega)) * omega / kC0, k_e = std::sqrt(s->eps_medium) * omega / kC0;
  std::vector<cd> RV(lMax + 1), RH(lMax + 1);
  mie_coefficients(lMax, s->kinds[t].radius, k_i, k_e, 1.0, 1.0, RV.data(), RH.data());
  out.assign(2 * ne, 0);
  for (int n = 1, i = 0; n <= lMax; ++n)
    for (int m = -n; m <= n; ++m, ++i) {
      out[i] = RV[n];
      out[ne + i] = RH[n];
    }
}

// Are all T-matrices of this ssw diagonal?
bool tm_all_diagonal(const qpms_scatsys_at_omega_t *ssw, size_t n) {
  for (int t = 0; t < ssw->ss->tm_count; ++t) {
    const qpms_complex_t *m = ssw->tm[t]->m;
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j)
        if (i != j && (m[i * n + j].re != 0 || m[i * n + j].im != 0)) return false;
  }
  return true;
}

// Validates that every particle uses one common default bspec (the kernels'
// layout), and returns its lMax and n.
int check_uniform_bspec(const qpms_scatsys_at_omega_t *ssw, int *lMax, size_t *n) {
  const qpms_scatsys_t *ss = ssw->ss;
  const qpms_vswf_set_spec_t *s0 = ssw->tm[0]->spec;
  for (int t = 0; t < ss->tm_count; ++t) {
    const qpms_vswf_set_spec_t *s = ssw->tm[t]->spec;
    if (s->n != s0->n || s->lMax != s0->lMax) {
      set_error("all particles must share one bspec");
      return QPMS_EINVAL;
    }
    const int L = s->lMax, ne = L * (L + 2);
    if (s->n != (size_t)2 * ne) { set_error("bspec must be the full lMax set"); return QPMS_EINVAL; }
    for (int it = 0, i = 0; it < 2; ++it)
      for (int nn = 1; nn <= L; ++nn)
        for (int m = -nn; m <= nn; ++m, ++i) {
          const qpms_uvswfi_t u = (it ? 1 : 2) + 4 * (qpms_uvswfi_t)(nn * (nn + 1) + m);
          if (s->ilist[i] != u) { set_error("bspec must be in qpms_vswf_set_spec_from_lMax order"); return QPMS_EINVAL; }
        }
  }
  if (!ss->c || ss->c->lMax < s0->lMax) { set_error("trans calculator lMax too small"); return QPMS_EINVAL; }
  if ((size_t)ss->p_count * s0->n != ss->fecv_size) { set_error("fecv_size mismatch"); return QPMS_EINVAL; }
  *lMax = s0->lMax;
  *n = s0->n;
  return QPMS_SUCCESS;
}

// Device workspace for one pipeline call (freed at the end).
struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

int dalloc(DevBuf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  QG_CUDA_TRY(cudaMalloc(&b.p, bytes));
  return QPMS_SUCCESS;
}

// Uploads positions and T-matrix ids of a system (any constructor) to dev.
int upload_particles(const qpms_scatsys_t *ss, DevBuf &dpos, DevBuf &dtm) {
  const int np = ss->p_count;
  std::vector<double> pos(3 * (size_t)np);
  std::vector<int> tm(np);
  for (int i = 0; i < np; ++i) {
    pos[3 * i] = ss->p[i].pos.x;
    pos[3 * i + 1] = ss->p[i].pos.y;
    pos[3 * i + 2] = ss->p[i].pos.z;
    tm[i] = ss->p[i].tmatrix_id;
  }
  int e;
  if ((e = dalloc(dpos, pos.size() * 8))) return e;
  if ((e = dalloc(dtm, tm.size() * 4))) return e;
  QG_CUDA_TRY(cudaMemcpy(dpos.p, pos.data(), pos.size() * 8, cudaMemcpyHostToDevice));
  QG_CUDA_TRY(cudaMemcpy(dtm.p, tm.data(), tm.size() * 4, cudaMemcpyHostToDevice));
  return QPMS_SUCCESS;
}

}  // namespace

// Lagrange-Gauss reduction of a 2D basis (lattices2d.c:635-655 semantics).
void lattice_reduce(double *b1, double *b2) {
  auto dot = [](const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1]; };
  double B1 = dot(b1, b1), mu = dot(b1, b2) / B1;
  b2[0] -= round(mu) * b1[0];
  b2[1] -= round(mu) * b1[1];
  double B2 = dot(b2, b2);
  while (B2 < B1) {
    double t0 = b1[0], t1 = b1[1];
    b1[0] = b2[0];
    b1[1] = b2[1];
    b2[0] = t0;
    b2[1] = t1;
    B1 = B2;
    mu = dot(b1, b2) / B1;
    b2[0] -= round(mu) * b1[0];
    b2[1] -= round(mu) * b1[1];
    B2 = dot(b2, b2);
  }
}

int axsym_nodes(qpms_arc_function_t shape, std::vector<double> &nodes, int *zsym);  // qg_axsym.cu
int axsym_tmatrix_device(const std::vector<double> &nodes, int zsym, int L, const qpms_vswf_set_spec_t *bspec,
                         int nw, const qg_c *k, const qg_c *kin, const qg_c *zr, qg_c *dT, qg_c *dQ, qg_c *dR,
                         cudaStream_t st);
void field_forget_system(const qpms_scatsys_t *ss);  // qg_field.cu
void sym_forget_system(const qpms_scatsys_t *ss);    // qg_sym.cu

// T-matrix of kind t at omega: the diagonal (n values) for a system of
// spheres, the full row-major n x n matrix when the system is dense.
void kind_tmat(const ScatsysPriv *s, int t, cd om, std::vector<qg_c> &out) {
  const size_t n = s->spec.n;
  const SphereKind &K = s->kinds[t];
  if (K.tmi) {  // tabulated: tmatrices.c:351-356 uses Re omega
    out.assign(n * n, cmk(0, 0));
    tmatrix_interp_eval(K.tmi, om.real(), out.data());
    return;
  }
  if (!K.axnodes.empty()) {  // axially symmetric: the EBCM kernel at om (NaN on failure)
    out.assign(n * n, cmk(NAN, NAN));
    const cd ei = kind_eps(K, om), em = s->eps_medium;
    const cd kin = std::sqrt(ei) * om / kC0, kout = std::sqrt(em) * om / kC0;
    const cd zr = std::sqrt(ei / em);  // z_out / z_in = sqrt(eps_in / eps_out) for mu = 1
    const qg_c k1 = cmk(kout.real(), kout.imag()), k2 = cmk(kin.real(), kin.imag()), z = cmk(zr.real(), zr.imag());
    qg_c *dT = nullptr;
    if (cudaMalloc(&dT, n * n * 16) != cudaSuccess) return;
    if (!axsym_tmatrix_device(K.axnodes, K.ax_zsym, std::max<int>(K.ax_lext, s->lMax), &s->spec, 1, &k1, &k2,
                              &z, dT, nullptr, nullptr, 0))
      cudaMemcpy(out.data(), dT, n * n * 16, cudaMemcpyDeviceToHost);
    cudaFree(dT);
    return;
  }
  std::vector<cd> d;
  sphere_tdiag(s, t, om, d);
  if (!s->dense) {
    out.resize(n);
    for (size_t i = 0; i < n; ++i) out[i] = cmk(d[i].real(), d[i].imag());
  } else {
    out.assign(n * n, cmk(0, 0));
    for (size_t i = 0; i < n; ++i) out[i * n + i] = cmk(d[i].real(), d[i].imag());
  }
}

int assemble_modeproblem_device(const qpms_scatsys_t *ss, int nw, const std::vector<qg_c> &T_host, bool dense,
                                const std::vector<qg_c> &k_host, int J, qg_c *dM, cudaStream_t st);

// M = I - T S of ssw (any T-matrices in one basis) on the device, row-major.
int ssw_modeproblem_device(const qpms_scatsys_at_omega_t *ssw, qg_c *dM, cudaStream_t st) {
  int lMax;
  size_t n;
  if (check_uniform_bspec(ssw, &lMax, &n)) return QPMS_EINVAL;
  const bool diag = tm_all_diagonal(ssw, n);
  std::vector<qg_c> T;
  for (int t = 0; t < ssw->ss->tm_count; ++t)
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j)
        if (!diag || i == j) T.push_back(*(const qg_c *)&ssw->tm[t]->m[i * n + j]);
  std::vector<qg_c> k(1, *(const qg_c *)&ssw->wavenumber);
  return assemble_modeproblem_device(ssw->ss, 1, T, !diag, k, 3, dM, st);
}

// I + S (translation matrix with Bessel kind J, zero self blocks) on the device:
// the assembly with T = -1.  Callers subtract I where they want S.
int ss_translation_device(const qpms_scatsys_t *ss, qg_c k, int J, qg_c *dM, cudaStream_t st) {
  const ScatsysPriv *s = sspriv(ss);
  std::vector<qg_c> T((size_t)ss->tm_count * s->spec.n, cmk(-1.0, 0.0));
  std::vector<qg_c> kk(1, k);
  // a dense system still takes the diagonal -1 here
  return assemble_modeproblem_device(ss, 1, T, false, kk, J, dM, st);
}

// Accessors used by qg_solve.cu.
bool scatsys_is_own(const qpms_scatsys_t *ss) { return ss && ss->medium.function == epsmu_const_fn; }
int scatsys_lmax(const qpms_scatsys_t *ss) { return sspriv(ss)->lMax; }
bool scatsys_dense(const qpms_scatsys_t *ss) { return sspriv(ss)->dense; }
// T of kind t at omega, diagonal or dense as scatsys_dense(ss) says.
void scatsys_tdiag(const qpms_scatsys_t *ss, int t, double om_re, double om_im, std::vector<qg_c> &out) {
  kind_tmat(sspriv(ss), t, cd(om_re, om_im), out);
}
qg_c scatsys_wavenumber(const qpms_scatsys_t *ss, double om_re, double om_im) {
  const cd k = std::sqrt(sspriv(ss)->eps_medium) * cd(om_re, om_im) / kC0;
  return cmk(k.real(), k.imag());
}
void planewave_direction_coeffs(int lMax, const double k_dir[3], const qpms_complex_t E_cart[3],
                                std::vector<qg_c> &coef) {
  const double kn = sqrt(k_dir[0] * k_dir[0] + k_dir[1] * k_dir[1] + k_dir[2] * k_dir[2]);
  const double th = kn ? acos(k_dir[2] / kn) : M_PI_2, ph = atan2(k_dir[1], k_dir[0]);
  const double st = sin(th), ct = cos(th), sf = sin(ph), cf = cos(ph);
  const cd E[3] = {to_cd(E_cart[0]), to_cd(E_cart[1]), to_cd(E_cart[2])};
  // ccart2csphvec (vectors.h:306-330)
  const cd Es[3] = {E[0] * st * cf + E[1] * st * sf + E[2] * ct, E[0] * ct * cf + E[1] * ct * sf - E[2] * st,
                    -E[0] * sf + E[1] * cf};
  const int ne = lMax * (lMax + 2);
  std::vector<cd> el(ne), mg(ne);
  planewave_coeffs(lMax, th, ph, Es, el.data(), mg.data());
  coef.resize(2 * ne);
  for (int y = 0; y < ne; ++y) {
    coef[y] = cmk(el[y].real(), el[y].imag());
    coef[ne + y] = cmk(mg[y].real(), mg[y].imag());
  }
}
int blas_handle_get(cublasHandle_t *h) { return blas_handle(h); }
// Host-side helpers of the reference-API convenience entry points (qg_dropins.cu).
const qpms_vswf_set_spec_t *scatsys_spec(const qpms_scatsys_t *ss) { return &sspriv(ss)->spec; }
void mie_reflection(int lMax, double a, qpms_complex_t k_i, qpms_complex_t k_e, qpms_complex_t mu_i,
                    qpms_complex_t mu_e, int Je, int Js, qpms_complex_t *RV, qpms_complex_t *RH) {
  std::vector<cd> v(lMax + 1), h(lMax + 1);
  mie_coefficients(lMax, a, to_cd(k_i), to_cd(k_e), to_cd(mu_i), to_cd(mu_e), v.data(), h.data(), Je, Js);
  for (int l = 0; l <= lMax; ++l) {
    RV[l] = from_cd(v[l]);
    RH[l] = from_cd(h[l]);
  }
}
// Plane-wave coefficients for direction (theta, phi) and local amplitude Es,
// default normalisation, el / mg of length lMax (lMax + 2).
void planewave_sph_coeffs(int lMax, double theta, double phi, const qpms_complex_t Es[3], qpms_complex_t *el,
                          qpms_complex_t *mg) {
  const int ne = lMax * (lMax + 2);
  const cd E[3] = {to_cd(Es[0]), to_cd(Es[1]), to_cd(Es[2])};
  std::vector<cd> e(ne), m(ne);
  planewave_coeffs(lMax, theta, phi, E, e.data(), m.data());
  for (int y = 0; y < ne; ++y) {
    el[y] = from_cd(e[y]);
    mg[y] = from_cd(m[y]);
  }
}

// Assemble M for nw frequencies of one system into device memory dM
// (the T-matrices per frequency are given host-side, dense or diagonal).
int assemble_modeproblem_device(const qpms_scatsys_t *ss, int nw, const std::vector<qg_c> &T_host, bool dense,
                                const std::vector<qg_c> &k_host, int J, qg_c *dM, cudaStream_t st) {
  DevBuf dpos, dtm, dT, dk;
  int e;
  if ((e = upload_particles(ss, dpos, dtm))) return e;
  if ((e = dalloc(dT, T_host.size() * 16))) return e;
  if ((e = dalloc(dk, k_host.size() * 16))) return e;
  QG_CUDA_TRY(cudaMemcpyAsync(dT.p, T_host.data(), T_host.size() * 16, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(dk.p, k_host.data(), k_host.size() * 16, cudaMemcpyHostToDevice, st));
  AsmArgs a;
  a.nw = nw;
  a.np = ss->p_count;
  a.ntm = ss->tm_count;
  a.dense = dense ? 1 : 0;
  a.J = J;
  a.pos = (const double *)dpos.p;
  a.tmid = (const int *)dtm.p;
  a.T = (const qg_c *)dT.p;
  a.k = (const qg_c *)dk.p;
  a.M = dM;
  if ((e = launch_assemble(a, priv(ss->c)->dev, st))) return e;
  QG_CUDA_TRY(cudaStreamSynchronize(st));
  return QPMS_SUCCESS;
}

}  // namespace qg

using namespace qg;

extern "C" {

static qpms_scatsys_t *create_spheres(int np, const double *pos_xyz, const int *kind, int nkinds,
                                      const double *radius, const qpms_complex_t *eps_inside,
                                      qpms_complex_t eps_medium, qpms_l_t lMax, const double *b1, const double *b2,
                                      const qpms_ldparams_t *const *ld_inside = nullptr);

// One translation calculator per lMax (default normalisation), built on first
// use and shared by every system of this library for the life of the process:
// its device tables stay resident, so making a system costs no device work.
static qpms_trans_calculator *shared_calculator(int lMax) {
  static std::mutex m;
  static qpms_trans_calculator *calc[16] = {nullptr};
  std::lock_guard<std::mutex> lk(m);
  if (lMax < 1 || lMax >= 16) return nullptr;
  if (!calc[lMax]) calc[lMax] = qpms_trans_calculator_init(lMax, QPMS_NORMALISATION_DEFAULT);
  return calc[lMax];
}

qpms_scatsys_t *qpms_gpu_scatsys_create_spheres(int np, const double *pos_xyz, const int *kind, int nkinds,
                                                const double *radius, const qpms_complex_t *eps_inside,
                                                qpms_complex_t eps_medium, qpms_l_t lMax) {
  return create_spheres(np, pos_xyz, kind, nkinds, radius, eps_inside, eps_medium, lMax, nullptr, nullptr);
}

qpms_scatsys_t *qpms_gpu_scatsys_create_spheres_ld(int np, const double *pos_xyz, const int *kind, int nkinds,
                                                   const double *radius, const qpms_complex_t *eps_inside,
                                                   const qpms_ldparams_t *const *ld_inside,
                                                   qpms_complex_t eps_medium, qpms_l_t lMax, const double *b1,
                                                   const double *b2) {
  if ((b1 == nullptr) != (b2 == nullptr)) {
    set_error("give both lattice vectors or neither");
    return nullptr;
  }
  if (!eps_inside && !ld_inside) {
    set_error("NULL permittivities");
    return nullptr;
  }
  std::vector<qpms_complex_t> eps(nkinds);
  for (int t = 0; t < nkinds; ++t) {
    eps[t].re = eps_inside ? eps_inside[t].re : 1.0;
    eps[t].im = eps_inside ? eps_inside[t].im : 0.0;
  }
  return create_spheres(np, pos_xyz, kind, nkinds, radius, eps.data(), eps_medium, lMax, b1, b2, ld_inside);
}

qpms_scatsys_t *qpms_gpu_scatsys_create(int np, const double *pos_xyz, const int *kind, int nkinds,
                                        const qpms_gpu_particle_kind_t *kinds, qpms_complex_t eps_medium,
                                        qpms_l_t lMax, const double *b1, const double *b2) {
  clear_error();
  if (!kinds || nkinds < 1) { set_error("no particle kinds"); return nullptr; }
  if ((b1 == nullptr) != (b2 == nullptr)) { set_error("give both lattice vectors or neither"); return nullptr; }
  std::vector<double> radius(nkinds);
  std::vector<qpms_complex_t> eps(nkinds);
  std::vector<const qpms_ldparams_t *> ld(nkinds, nullptr);
  bool dense = false;
  for (int t = 0; t < nkinds; ++t) {
    const qpms_gpu_particle_kind_t &K = kinds[t];
    if (K.type < 0 || K.type > 2) {
      set_error("kind %d: type must be 0 (sphere), 1 (T-matrix) or 2 (axially symmetric)", t);
      return nullptr;
    }
    radius[t] = K.type == 0 ? K.radius : 1.0;
    eps[t] = K.eps;
    ld[t] = K.type != 1 ? K.ld : nullptr;
    if (K.type == 2) {
      if (K.lMax_extend > 12) { set_error("kind %d: lMax_extend above 12", t); return nullptr; }
      dense = true;
      continue;
    }
    if (K.type == 1) {
      if (!K.tmatrix) { set_error("kind %d: NULL T-matrix interpolator", t); return nullptr; }
      const qpms_vswf_set_spec_t *sp = tmatrix_interp_spec(K.tmatrix);
      const int ne = lMax * (lMax + 2);
      bool ok = sp->n == (size_t)(2 * ne) && sp->norm == QPMS_NORMALISATION_DEFAULT;
      for (int it = 0, i = 0; ok && it < 2; ++it)
        for (int l = 1; ok && l <= lMax; ++l)
          for (int m = -l; ok && m <= l; ++m, ++i)
            ok = sp->ilist[i] == (qpms_uvswfi_t)((it ? 1 : 2) + 4 * (qpms_uvswfi_t)(l * (l + 1) + m));
      if (!ok) {
        set_error("kind %d: the T-matrix basis must be the default lMax = %d basis (qpms_vswf_set_spec_from_lMax)",
                  t, lMax);
        return nullptr;
      }
      dense = true;
    } else if (!(K.radius > 0)) {
      set_error("kind %d: sphere radius must be positive", t);
      return nullptr;
    }
  }
  qpms_scatsys_t *ss = create_spheres(np, pos_xyz, kind, nkinds, radius.data(), eps.data(), eps_medium, lMax, b1,
                                      b2, ld.data());
  if (!ss) return nullptr;
  ScatsysPriv *s = sspriv(ss);
  for (int t = 0; t < nkinds; ++t) {
    s->kinds[t].pint = kinds[t].type != 1 ? kinds[t].eps_interp : nullptr;
    s->kinds[t].tmi = kinds[t].type == 1 ? kinds[t].tmatrix : nullptr;
    if (kinds[t].type == 2) {
      if (axsym_nodes(kinds[t].shape, s->kinds[t].axnodes, &s->kinds[t].ax_zsym)) {
        qpms_gpu_scatsys_free(ss);
        return nullptr;
      }
      s->kinds[t].ax_lext = kinds[t].lMax_extend;
    }
  }
  s->dense = dense;
  return ss;
}

qpms_complex_t qpms_lorentzdrude_eps(qpms_complex_t omega, const qpms_ldparams_t *p) {
  qpms_complex_t r;
  r.re = r.im = 0;
  if (!p) return r;
  const cd e = lorentzdrude_eps(to_cd(omega), p->omega_p, p->data, p->n);
  r.re = e.real();
  r.im = e.imag();
  return r;
}

qpms_scatsys_t *qpms_gpu_scatsys_create_spheres_2d(int np, const double *pos_xyz, const int *kind, int nkinds,
                                                   const double *radius, const qpms_complex_t *eps_inside,
                                                   qpms_complex_t eps_medium, qpms_l_t lMax, const double b1[2],
                                                   const double b2[2]) {
  if (!b1 || !b2) {
    set_error("NULL lattice basis");
    return nullptr;
  }
  return create_spheres(np, pos_xyz, kind, nkinds, radius, eps_inside, eps_medium, lMax, b1, b2);
}

static qpms_scatsys_t *create_spheres(int np, const double *pos_xyz, const int *kind, int nkinds,
                                      const double *radius, const qpms_complex_t *eps_inside,
                                      qpms_complex_t eps_medium, qpms_l_t lMax, const double *b1, const double *b2,
                                      const qpms_ldparams_t *const *ld_inside) {
  clear_error();
  if (np < 1 || !pos_xyz || nkinds < 1 || !radius || !eps_inside || lMax < 1 || lMax > 6) {
    set_error("invalid arguments (np >= 1, 1 <= lMax <= 6)");
    return nullptr;
  }
  ScatsysPriv *s = new (std::nothrow) ScatsysPriv();
  if (!s) { set_error("out of host memory"); return nullptr; }
  memset(&s->pub, 0, sizeof(s->pub));
  s->lMax = lMax;
  s->eps_medium = to_cd(eps_medium);
  for (int t = 0; t < nkinds; ++t) {
    SphereKind k;
    k.radius = radius[t];
    k.eps = to_cd(eps_inside[t]);
    if (ld_inside && ld_inside[t]) {  // copied: the caller's parameter block may go away
      k.ld.assign(ld_inside[t]->data, ld_inside[t]->data + ld_inside[t]->n);
      k.ld_omega_p = ld_inside[t]->omega_p;
    }
    s->kinds.push_back(k);
  }
  const int ne = lMax * (lMax + 2);
  for (int it = 0; it < 2; ++it)
    for (int n = 1; n <= lMax; ++n)
      for (int m = -n; m <= n; ++m) s->ilist.push_back((it ? 1 : 2) + 4 * (qpms_uvswfi_t)(n * (n + 1) + m));
  s->spec.n = s->spec.capacity = 2 * ne;
  s->spec.ilist = s->ilist.data();
  s->spec.lMax = s->spec.lMax_M = s->spec.lMax_N = lMax;
  s->spec.lMax_L = -1;
  s->spec.norm = QPMS_NORMALISATION_DEFAULT;
  s->p.resize(np);
  s->pstarts.resize(np + 1);
  for (int i = 0; i < np; ++i) {
    const int t = kind ? kind[i] : 0;
    if (t < 0 || t >= nkinds) { set_error("particle kind out of range"); delete s; return nullptr; }
    s->p[i].pos.x = pos_xyz[3 * i];
    s->p[i].pos.y = pos_xyz[3 * i + 1];
    s->p[i].pos.z = pos_xyz[3 * i + 2];
    s->p[i].tmatrix_id = t;
    s->pstarts[i] = (size_t)i * 2 * ne;
  }
  s->pstarts[np] = (size_t)np * 2 * ne;
  qpms_scatsys_t &P = s->pub;
  P.lattice_dimension = 0;
  s->medium_const.eps = eps_medium;
  s->medium_const.mu = from_cd(1.0);
  P.medium.function = epsmu_const_fn;
  P.medium.params = &s->medium_const;
  P.tm_count = P.tm_capacity = nkinds;
  P.tmg_count = nkinds;
  P.p = s->p.data();
  P.p_count = P.p_capacity = np;
  P.fecv_size = (size_t)np * 2 * ne;
  P.fecv_pstarts = s->pstarts.data();
  P.max_bspecn = 2 * ne;
  P.lenscale = 0;
  for (int i = 0; i < np; ++i) {
    double r = sqrt(pos_xyz[3 * i] * pos_xyz[3 * i] + pos_xyz[3 * i + 1] * pos_xyz[3 * i + 1] +
                    pos_xyz[3 * i + 2] * pos_xyz[3 * i + 2]);
    if (r > P.lenscale) P.lenscale = r;
  }
  if (b1) {
    // scatsystem.c:187-214: reduced basis, reciprocal basis (without 2 pi),
    // unit-cell area and the default Ewald eta = sqrt(pi / A)
    double u1[2] = {b1[0], b1[1]}, u2[2] = {b2[0], b2[1]};
    lattice_reduce(u1, u2);
    const double det = u1[0] * u2[1] - u1[1] * u2[0];
    if (det == 0) { set_error("degenerate lattice basis"); delete s; return nullptr; }
    P.lattice_dimension = 2;
    P.per.lattice_basis[0] = {u1[0], u1[1], 0};
    P.per.lattice_basis[1] = {u2[0], u2[1], 0};
    P.per.reciprocal_basis[0] = {u2[1] / det, -u2[0] / det, 0};
    P.per.reciprocal_basis[1] = {-u1[1] / det, u1[0] / det, 0};
    P.per.unitcell_volume = fabs(det);
    P.per.eta = sqrt(M_PI) / sqrt(fabs(det));
  }
  P.c = shared_calculator(lMax);
  if (!P.c) {
    delete s;
    return nullptr;
  }
  return &s->pub;
}

void qpms_gpu_scatsys_free(qpms_scatsys_t *ss) {
  if (!ss) return;
  field_forget_system(ss);
  sym_forget_system(ss);
  delete sspriv(ss);  // the translation calculator is shared (shared_calculator)
}

qpms_scatsys_at_omega_t *qpms_gpu_scatsys_at_omega(const qpms_scatsys_t *ss, qpms_complex_t omega) {
  clear_error();
  if (!ss) { set_error("NULL system"); return nullptr; }
  const ScatsysPriv *s = sspriv(ss);
  SswPriv *w = new (std::nothrow) SswPriv();
  if (!w) { set_error("out of host memory"); return nullptr; }
  const size_t n = s->spec.n;
  const cd om = to_cd(omega);
  w->tms.resize(ss->tm_count);
  w->tmp.resize(ss->tm_count);
  w->tdata.resize(ss->tm_count);
  for (int t = 0; t < ss->tm_count; ++t) {
    std::vector<qg_c> d;
    kind_tmat(s, t, om, d);
    if (d.size() == n * n) {
      w->tdata[t] = d;
    } else {
      w->tdata[t].assign(n * n, cmk(0, 0));
      for (size_t i = 0; i < n; ++i) w->tdata[t][i * n + i] = d[i];
    }
    w->tms[t].spec = &s->spec;
    w->tms[t].m = (qpms_complex_t *)w->tdata[t].data();
    w->tms[t].owns_m = false;
    w->tmp[t] = &w->tms[t];
  }
  w->pub.ss = ss;
  w->pub.tm = w->tmp.data();
  w->pub.omega = omega;
  w->pub.medium.eps = from_cd(s->eps_medium);
  w->pub.medium.mu = from_cd(1.0);
  w->pub.wavenumber = from_cd(std::sqrt(s->eps_medium) * om / kC0);  // qpms_wavenumber, materials.h:46-48
  return &w->pub;
}

void qpms_gpu_scatsys_at_omega_free(qpms_scatsys_at_omega_t *ssw) {
  if (ssw) delete reinterpret_cast<SswPriv *>(ssw);
}

qpms_complex_t *qpms_scatsysw_build_modeproblem_matrix_full(qpms_complex_t *target,
                                                            const qpms_scatsys_at_omega_t *ssw) {
  clear_error();
  if (!ssw || !ssw->ss) { set_error("NULL ssw"); return nullptr; }
  if (ssw->ss->lattice_dimension != 0) { set_error("periodic system: use qpms_scatsyswk_build_modeproblem_matrix_full"); return nullptr; }
  const size_t N = ssw->ss->fecv_size;
  DevBuf dM;
  if (dalloc(dM, N * N * 16)) return nullptr;
  if (ssw_modeproblem_device(ssw, (qg_c *)dM.p, 0)) return nullptr;
  bool own = false;
  if (!target) {
    target = (qpms_complex_t *)malloc(N * N * 16);
    own = true;
    if (!target) { set_error("out of host memory"); return nullptr; }
  }
  if (cudaMemcpy(target, dM.p, N * N * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    if (own) free(target);
    return nullptr;
  }
  return target;
}

// The reference's names of the system lifetime functions (scatsystem.h:297-306).
void qpms_scatsys_free(qpms_scatsys_t *ss) { qpms_gpu_scatsys_free(ss); }
qpms_scatsys_at_omega_t *qpms_scatsys_at_omega(const qpms_scatsys_t *ss, qpms_complex_t omega) {
  return qpms_gpu_scatsys_at_omega(ss, omega);
}
void qpms_scatsys_at_omega_free(qpms_scatsys_at_omega_t *ssw) { qpms_gpu_scatsys_at_omega_free(ssw); }
// scatsystem.h:20: the reference's thread count for its CPU builders; the
// GPU paths have no such knob (accepted and ignored).
void qpms_scatsystem_set_nthreads(long n) { (void)n; }

// S with outgoing waves (scatsystem.h:357-362): qpms_scatsys_build_translation_matrix_e_full
// with J = QPMS_HANKEL_PLUS.
qpms_complex_t *qpms_scatsys_build_translation_matrix_full(qpms_complex_t *target, const qpms_scatsys_t *ss,
                                                           qpms_complex_t k) {
  return qpms_scatsys_build_translation_matrix_e_full(target, ss, k, QPMS_HANKEL_PLUS);
}

qpms_complex_t *qpms_scatsys_build_translation_matrix_e_full(qpms_complex_t *target, const qpms_scatsys_t *ss,
                                                             qpms_complex_t k, qpms_bessel_t J) {
  clear_error();
  if (!ss) { set_error("NULL system"); return nullptr; }
  if (J < 1 || J > 4) { set_error("invalid J"); return nullptr; }
  const ScatsysPriv *s = sspriv(ss);
  const size_t n = s->spec.n, N = ss->fecv_size;
  (void)n;
  DevBuf dM;
  if (dalloc(dM, N * N * 16)) return nullptr;
  if (ss_translation_device(ss, cmk(k.re, k.im), J, (qg_c *)dM.p, 0)) return nullptr;
  bool own = false;
  if (!target) {
    target = (qpms_complex_t *)malloc(N * N * 16);
    own = true;
    if (!target) { set_error("out of host memory"); return nullptr; }
  }
  if (cudaMemcpy(target, dM.p, N * N * 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("device to host copy failed");
    if (own) free(target);
    return nullptr;
  }
  for (size_t i = 0; i < N; ++i) target[i * N + i].re -= 1.0;
  return target;
}

}  // extern "C"
