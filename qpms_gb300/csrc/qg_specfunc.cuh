// FP64 special functions for the translation kernels (host + device).
//
// Spherical Bessel / Hankel functions z_l(x), l = 0..L, of the four kinds
// used by qpms_sph_bessel_fill (qpms/bessel.c:86-147; kinds qpms_types.h:176-182):
//   J = 1  j_l   regular      Miller backward recurrence (|x| <= L + 1) or forward
//                             recurrence (|x| > L + 1, where every order is still
//                             in the oscillatory regime), DLMF 10.51.1;
//                             normalised with j_0 = sin x / x or j_1.
//   J = 2  y_l   singular     forward recurrence (dominant solution).
//   J = 3  h+_l  = j + i y    real x: j and y separately (the reference's GSL path,
//                             bessel.c:52-83); complex x: forward recurrence from
//                             h_0 = -i e^{ix}/x, h_1 = -e^{ix}(x+i)/x^2 (AMOS
//                             zbesh in the reference, bessel.c:121-127).
//   J = 4  h-_l  = j - i y    likewise with e^{-ix}.
// Associated Legendre P_l^m(x) (unnormalised, Condon-Shortley phase -1, the GSL
// GSL_SF_LEGENDRE_NONE array that translations.c:651-653 requests), by the
// three-term recurrence in l (DLMF 14.10.3) from P_m^m = (-1)^m (2m-1)!! u^m.
#pragma once
#include "qg_complex.cuh"

namespace qg {

// Miller start offset above L for |x| <= L + 1: the minimal-solution error
// decays like (|x| / 2N)^(2(N-L)); 16 extra orders give < 1e-17 for L <= 17.
constexpr int kMillerExtra = 16;

template <int L>
QG_HD void sph_j(qg_c x, bool real_x, qg_c *z) {
  const double ax = real_x ? fabs(x.re) : cabsd(x);
  if (ax == 0.0) {
    z[0] = cmk(1.0, 0.0);
#pragma unroll
    for (int l = 1; l <= L; ++l) z[l] = cmk(0.0, 0.0);
    return;
  }
  if (real_x) {
    const double xr = x.re, ri = 1.0 / xr;
    double s, c;
    sincos(xr, &s, &c);
    const double j0 = s * ri, j1 = (s * ri - c) * ri;
    if (ax > L + 1) {
      double a = j0, b = j1;
      z[0] = cmk(a, 0.0);
      if (L >= 1) z[1] = cmk(b, 0.0);
#pragma unroll
      for (int l = 1; l < L; ++l) {
        double nx = (2 * l + 1) * ri * b - a;
        z[l + 1] = cmk(nx, 0.0);
        a = b;
        b = nx;
      }
      return;
    }
    // Miller: f_{N+1} = 0, f_N = tiny, downward to 0.
    double f1 = 0.0, f0 = 1e-200;
    const int N = L + kMillerExtra;
    double keep[L + 1];
    for (int l = N; l >= 1; --l) {
      double fm = (2 * l + 1) * ri * f0 - f1;
      f1 = f0;
      f0 = fm;
      if (l - 1 <= L) keep[l - 1] = fm;
      if (fabs(fm) > 1e200) {  // rescale to stay finite
        f0 *= 1e-200;
        f1 *= 1e-200;
        for (int k = l - 1; k <= L; ++k) keep[k] *= 1e-200;
      }
    }
    const double scale = (fabs(j0) >= fabs(j1)) ? j0 / keep[0] : j1 / keep[1];
#pragma unroll
    for (int l = 0; l <= L; ++l) z[l] = cmk(keep[l] * scale, 0.0);
    return;
  }
  const qg_c ri = crecip(x);
  const qg_c s = csin_(x), c = ccos_(x);
  const qg_c j0 = cmul(s, ri);
  const qg_c j1 = cmul(csub(j0, c), ri);
  if (ax > L + 1) {
    qg_c a = j0, b = j1;
    z[0] = a;
    if (L >= 1) z[1] = b;
#pragma unroll
    for (int l = 1; l < L; ++l) {
      qg_c nx = csub(cscale(cmul(ri, b), 2 * l + 1), a);
      z[l + 1] = nx;
      a = b;
      b = nx;
    }
    return;
  }
  qg_c f1 = cmk(0.0, 0.0), f0 = cmk(1e-200, 0.0);
  const int N = L + kMillerExtra;
  qg_c keep[L + 1];
  for (int l = N; l >= 1; --l) {
    qg_c fm = csub(cscale(cmul(ri, f0), 2 * l + 1), f1);
    f1 = f0;
    f0 = fm;
    if (l - 1 <= L) keep[l - 1] = fm;
    if (fabs(fm.re) + fabs(fm.im) > 1e200) {
      f0 = cscale(f0, 1e-200);
      f1 = cscale(f1, 1e-200);
      for (int k = l - 1; k <= L; ++k) keep[k] = cscale(keep[k], 1e-200);
    }
  }
  const qg_c scale = (cabs2(j0) >= cabs2(j1)) ? cdiv(j0, keep[0]) : cdiv(j1, keep[1]);
#pragma unroll
  for (int l = 0; l <= L; ++l) z[l] = cmul(keep[l], scale);
}

// Forward recurrence from z0, z1 with 1/x given.
template <int L>
QG_HD void sph_forward(qg_c ri, qg_c z0, qg_c z1, qg_c *z) {
  z[0] = z0;
  if (L >= 1) z[1] = z1;
  qg_c a = z0, b = z1;
#pragma unroll
  for (int l = 1; l < L; ++l) {
    qg_c nx = csub(cscale(cmul(ri, b), 2 * l + 1), a);
    z[l + 1] = nx;
    a = b;
    b = nx;
  }
}

// z_l(x), l = 0..L, of kind J (1..4).  Returns false for an invalid kind.
template <int L>
QG_HD bool sph_bessel(int J, qg_c x, qg_c *z) {
  const bool real_x = (x.im == 0.0);
  if (J == 1) {
    sph_j<L>(x, real_x, z);
    return true;
  }
  if (J < 1 || J > 4) return false;
  if (real_x) {
    const double xr = x.re, ri = 1.0 / xr;
    double s, c;
    sincos(xr, &s, &c);
    // y_l forward (real), y_0 = -cos x / x, y_1 = -(cos x / x + sin x) / x
    double ya = -c * ri, yb = (-c * ri - s) * ri;
    if (J == 2) {
      z[0] = cmk(ya, 0.0);
      if (L >= 1) z[1] = cmk(yb, 0.0);
#pragma unroll
      for (int l = 1; l < L; ++l) {
        double nx = (2 * l + 1) * ri * yb - ya;
        z[l + 1] = cmk(nx, 0.0);
        ya = yb;
        yb = nx;
      }
      return true;
    }
    sph_j<L>(x, true, z);
    const double sg = (J == 3) ? 1.0 : -1.0;
    z[0].im = sg * ya;
    if (L >= 1) z[1].im = sg * yb;
#pragma unroll
    for (int l = 1; l < L; ++l) {
      double nx = (2 * l + 1) * ri * yb - ya;
      z[l + 1].im = sg * nx;
      ya = yb;
      yb = nx;
    }
    return true;
  }
  const qg_c ri = crecip(x);
  if (J == 2) {
    const qg_c s = csin_(x), c = ccos_(x);
    const qg_c y0 = cscale(cmul(c, ri), -1.0);
    const qg_c y1 = cmul(csub(y0, s), ri);
    sph_forward<L>(ri, y0, y1, z);
    return true;
  }
  if (J == 3) {
    const qg_c e = cexpi(x);  // e^{ix}
    const qg_c h0 = cmul(cmk(0.0, -1.0), cmul(e, ri));
    const qg_c h1 = cscale(cmul(cmul(e, cadd(x, cmk(0.0, 1.0))), cmul(ri, ri)), -1.0);
    sph_forward<L>(ri, h0, h1, z);
  } else {
    const qg_c e = cexpi(cmk(-x.re, -x.im));  // e^{-ix}
    const qg_c h0 = cmul(cmk(0.0, 1.0), cmul(e, ri));
    const qg_c h1 = cscale(cmul(cmul(e, csub(x, cmk(0.0, 1.0))), cmul(ri, ri)), -1.0);
    sph_forward<L>(ri, h0, h1, z);
  }
  return true;
}

// One column m of the unnormalised Legendre table, P_l^m(x) for l = m..L,
// written at out[l(l+1)/2 + m] (GSL array layout), csphase = -1.
QG_HD void legendre_column(int L, int m, double x, double *out) {
  const double u = sqrt((1.0 - x) * (1.0 + x));
  double pmm = 1.0;
  for (int k = 1; k <= m; ++k) pmm *= -(2 * k - 1) * u;
  out[m * (m + 1) / 2 + m] = pmm;
  if (m + 1 > L) return;
  double pm1 = x * (2 * m + 1) * pmm;
  out[(m + 1) * (m + 2) / 2 + m] = pm1;
  double a = pmm, b = pm1;
  for (int l = m + 2; l <= L; ++l) {
    double pl = ((2 * l - 1) * x * b - (l + m - 1) * a) / (l - m);
    out[l * (l + 1) / 2 + m] = pl;
    a = b;
    b = pl;
  }
}

// Reciprocals 1/k, k = 1..kRecipMax, for division-free recurrences (FP64
// division costs an order of magnitude more than an FMA on the FP64 pipe).
constexpr int kRecipMax = 48;
#if defined(__CUDACC__)
static __constant__ double c_recip[kRecipMax + 1] = {
    0.0, 1.0 / 1, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7, 1.0 / 8, 1.0 / 9, 1.0 / 10,
    1.0 / 11, 1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15, 1.0 / 16, 1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20,
    1.0 / 21, 1.0 / 22, 1.0 / 23, 1.0 / 24, 1.0 / 25, 1.0 / 26, 1.0 / 27, 1.0 / 28, 1.0 / 29, 1.0 / 30,
    1.0 / 31, 1.0 / 32, 1.0 / 33, 1.0 / 34, 1.0 / 35, 1.0 / 36, 1.0 / 37, 1.0 / 38, 1.0 / 39, 1.0 / 40,
    1.0 / 41, 1.0 / 42, 1.0 / 43, 1.0 / 44, 1.0 / 45, 1.0 / 46, 1.0 / 47, 1.0 / 48};

// legendre_column with the division by (l - m) replaced by a product with
// the correctly rounded reciprocal (L <= kRecipMax).
__device__ __forceinline__ void legendre_column_rt(int L, int m, double x, double *out) {
  const double u = sqrt((1.0 - x) * (1.0 + x));
  double pmm = 1.0;
  for (int k = 1; k <= m; ++k) pmm *= -(2 * k - 1) * u;
  out[m * (m + 1) / 2 + m] = pmm;
  if (m + 1 > L) return;
  double pm1 = x * (2 * m + 1) * pmm;
  out[(m + 1) * (m + 2) / 2 + m] = pm1;
  double a = pmm, b = pm1;
  for (int l = m + 2; l <= L; ++l) {
    double pl = ((2 * l - 1) * x * b - (l + m - 1) * a) * c_recip[l - m];
    out[l * (l + 1) / 2 + m] = pl;
    a = b;
    b = pl;
  }
}
#endif

}  // namespace qg
