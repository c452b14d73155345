// Complex double helpers shared by host and device code of libqpms_gb300.
// The layout {re, im} matches C99 `complex double`, numpy complex128 and
// cuDoubleComplex, so buffers pass through the C ABI unchanged.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define QG_HD __host__ __device__ __forceinline__
#else
#define QG_HD inline
#endif

struct __align__(16) qg_c {
  double re, im;
};

QG_HD qg_c cmk(double r, double i) { qg_c z; z.re = r; z.im = i; return z; }
QG_HD qg_c cadd(qg_c a, qg_c b) { return cmk(a.re + b.re, a.im + b.im); }
QG_HD qg_c csub(qg_c a, qg_c b) { return cmk(a.re - b.re, a.im - b.im); }
QG_HD qg_c cmul(qg_c a, qg_c b) {
  return cmk(fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re));
}
QG_HD qg_c cscale(qg_c a, double s) { return cmk(a.re * s, a.im * s); }
QG_HD qg_c cconj(qg_c a) { return cmk(a.re, -a.im); }
QG_HD double cabs2(qg_c a) { return a.re * a.re + a.im * a.im; }
QG_HD double cabsd(qg_c a) { return hypot(a.re, a.im); }
// Smith's algorithm for a / b.
QG_HD qg_c cdiv(qg_c a, qg_c b) {
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, den = b.re + b.im * r;
    return cmk((a.re + a.im * r) / den, (a.im - a.re * r) / den);
  } else {
    double r = b.re / b.im, den = b.im + b.re * r;
    return cmk((a.re * r + a.im) / den, (a.im * r - a.re) / den);
  }
}
QG_HD qg_c crecip(qg_c b) { return cdiv(cmk(1.0, 0.0), b); }
// exp(i z) for complex z
QG_HD qg_c cexpi(qg_c z) {
  double s, c;
  sincos(z.re, &s, &c);
  double e = exp(-z.im);
  return cmk(e * c, e * s);
}
QG_HD qg_c csin_(qg_c z) {
  double s, c;
  sincos(z.re, &s, &c);
  return cmk(s * cosh(z.im), c * sinh(z.im));
}
QG_HD qg_c ccos_(qg_c z) {
  double s, c;
  sincos(z.re, &s, &c);
  return cmk(c * cosh(z.im), -s * sinh(z.im));
}
