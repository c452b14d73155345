// Faddeeva function w(z) = exp(-z^2) erfc(-i z) and the complex erfc, FP64,
// host and device.
//
// Method: J.A.C. Weideman, "Computation of the complex error function",
// SIAM J. Numer. Anal. 31 (1994) 1497-1518: for Im z >= 0,
//   w(z) ~ 2 p(Z) / (L - i z)^2 + pi^{-1/2} / (L - i z),  Z = (L + i z)/(L - i z),
// with a degree-(N-1) polynomial p whose coefficients are the Fourier
// coefficients of exp(-t^2)(L^2 + t^2) on t = L tan(theta/2), L = (N/sqrt 2)^{1/2}.
// N = 40 gives a relative error of a few 1e-15 over Re z in [-4, 4],
// Im z in [0, 25] (checked against scipy.special.wofz in the tests); the
// lower half plane follows from w(-z) = 2 exp(-z^2) - w(z).
#pragma once
#include "qg_complex.cuh"

namespace qg {

constexpr int kWeidemanN = 40;

// Coefficients a_1..a_N in Horner order (highest power first); filled once by
// weideman_coeffs() on the host and copied to device constant memory.
struct WeidemanCoeffs {
  double a[kWeidemanN];
  double L;
};

// Host: computes the coefficients by a direct DFT (2M = 4N points).
void weideman_coeffs(WeidemanCoeffs *c);

QG_HD qg_c faddeeva_w_upper(qg_c z, const WeidemanCoeffs &C) {
  // Im z >= 0
  const qg_c iz = cmk(-z.im, z.re);
  const qg_c den = cmk(C.L - iz.re, -iz.im);  // L - i z
  const qg_c num = cmk(C.L + iz.re, iz.im);   // L + i z
  const qg_c rden = crecip(den);
  const qg_c Z = cmul(num, rden);
  qg_c p = cmk(C.a[0], 0.0);
#pragma unroll 8
  for (int n = 1; n < kWeidemanN; ++n) p = cadd(cmul(p, Z), cmk(C.a[n], 0.0));
  const qg_c r2 = cmul(rden, rden);
  const double isqpi = 0.56418958354775628694807945156077;  // 1/sqrt(pi)
  return cadd(cscale(cmul(p, r2), 2.0), cscale(rden, isqpi));
}

// erfc(u) for complex u (any half plane): erfc(u) = exp(-u^2) w(i u) for Re u >= 0,
// erfc(u) = 2 - erfc(-u) otherwise.
QG_HD qg_c cerfc(qg_c u, const WeidemanCoeffs &C) {
  const bool neg = u.re < 0;
  const qg_c v = neg ? cmk(-u.re, -u.im) : u;
  const qg_c w = faddeeva_w_upper(cmk(-v.im, v.re), C);  // w(i v), Im(i v) = Re v >= 0
  const qg_c e = cexpi(cmk(-2.0 * v.re * v.im, v.re * v.re - v.im * v.im));  // exp(-v^2) = exp(i * (i v^2))
  // exp(-v^2): -v^2 = -(vr^2 - vi^2) - 2 i vr vi; cexpi(z) = exp(i z) so pass z = -i(-v^2) = i v^2
  const qg_c r = cmul(e, w);
  return neg ? cmk(2.0 - r.re, -r.im) : r;
}

}  // namespace qg
