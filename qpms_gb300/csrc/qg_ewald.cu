// 2D Ewald lattice sums and the periodic mode-problem assembly on sm_103a.
//
// For every unit (frequency w, Bloch vector beta, particle pair R <- C) of a
// batch, ewald_assemble_kernel evaluates the scalar lattice sums
//   sigma_{n,m} = sigma^S_{n,m} + sigma^L_{n,m} (+ sigma0 for R == C),
// 0 <= n <= lMax_e = 2 lMax + 1, n + m even (2D lattice in the xy plane),
// as the reference's ewald3_sigma_short / ewald3_21_xy_sigma_long /
// ewald3_sigma0 (qpms/ewald.c:260-273, 286-503, 742-920), contracts them with
// the translation multipliers into the lattice translation operator W
// (translations.c:926-1078, including its B sum over q <= qmax_A) and writes
// the block M[R, C] = delta_RC I - T_R W(R <- C) into the row-major matrix.
//
// Method, FP64 throughout:
//  * short range: per direct-lattice point R (R - particle_shift, origin
//    excluded for the self pair), the integrals
//      I_n = int_eta^inf exp(-R^2 xi^2 + k^2/(4 xi^2)) xi^(2n) dxi
//    in closed form,  I_0 = sqrt(pi)/(4R) [e^{ikR} erfc(R eta + ik/2eta) + e^{-ikR} erfc(R eta - ik/2eta)],
//    I_{-1} = sqrt(pi)/(2ik) [e^{-ikR} erfc(R eta - ik/2eta) - e^{ikR} erfc(R eta + ik/2eta)],
//    and upward by the integration-by-parts recurrence
//      I_n = [(2n-1) I_{n-1} - (k^2/2) I_{n-2} + eta^(2n-1) e^{-R^2 eta^2 + k^2/4eta^2}] / (2 R^2),
//    replacing the reference's per-point adaptive quadrature (gsl qagiu, 1e-13);
//  * long range: per reciprocal point K, Gamma(1/2 - j, x^2), x = gamma k / 2eta,
//    from Gamma(1/2, z) = sqrt(pi) erfc(sqrt z) and the downward recurrence
//    Gamma(a-1, z) = (Gamma(a, z) - z^(a-1) e^{-z}) / (a-1), on the branch the
//    reference selects (ewald.c:390-393; for real k: the limit from below the
//    negative real axis);
//  * both sums run over all lattice points whose terms exceed ~e^{-56} of the
//    leading scale (|R| eta <= 7.5, x^2 <= 56): the reference's automatic
//    cut-off (EWALD_AUTO_CUTOFF) stops at relative contributions below
//    DBL_EPSILON, so both truncate below double precision.
// One CTA per unit; each thread accumulates the (n, m) sums of a strided
// subset of lattice points in registers; a shuffle + shared-memory reduction
// gives sigma in shared memory, where the contraction reads it exactly as the
// finite assembly reads its Bessel/Legendre factor table.
//
// Pairs of particles at different heights (shift.z = z_R - z_C != 0, layers of
// the lattice; the reference's LAT_2D_IN_3D short-range branch and the
// shifted long-range branch of ewald.c:441-469) have sums of every parity:
//  * short range: Legendre P_n^|m|(cos theta) of R - shift by the upward
//    recurrences, all (n, m);
//  * long range: per reciprocal point the double sum over (j, s) of
//      S1[y][j, s] (k w)^(2j - s) (|beta + K| / k)^(n - s) gamma^(2j - 1) Delta_j,
//    w = -shift.z, with Kambe's Delta_j(X, z) = int_X^inf t^(-1/2-j) e^{-t + z^2/4t} dt,
//    z^2 = -(gamma k w)^2, by the series sum_q (z^2/4)^q / q! Gamma(1/2 - j - q, X)
//    (ewaldsf.c:344-402), written as X^-j sum_q r_q g_(j+q) with
//    g_i = X^i Gamma(1/2 - i, X) (upward: g_i = (X g_(i-1) - sqrt(X) e^-X) / (1/2 - i))
//    and r_q = (-w^2 eta^2)^q / q!;
//  * eta is lowered to 1 / |w| where eta |w| > 1, which keeps the cancellation
//    in the series below e^2 (the sums do not depend on eta);
//  * distant layers, |k w| >= 2.5 (where eta <= 1 / |w| would let the short-
//    and long-range parts cancel by e^(k^2 / 4 eta^2)): the eta -> infinity
//    limit, a pure reciprocal-lattice sum (no short range) with
//    Delta_j(0, z) = 2 (a/2)^(1/2-j) K_(j-1/2)(a), a = gamma k |w|, in closed
//    form by the half-integer Bessel K recurrence; it converges like
//    e^(-|beta + K| |w|);
//  * the (n, m) accumulators are split into passes of at most 36 entries to
//    stay in registers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "qg_assembly.h"
#include "qg_ewald.h"
#include "qg_faddeeva.cuh"
#include "qg_internal.h"
#include "qg_ktimer.h"

namespace qg {

void weideman_coeffs(WeidemanCoeffs *c) {
  const int N = kWeidemanN, M = 2 * N, M2 = 2 * M;
  const double L = sqrt(N / sqrt(2.0));
  std::vector<double> f(M2, 0.0);
  for (int k = -M + 1; k <= M - 1; ++k) {
    const double th = k * M_PI / M, t = L * tan(th / 2);
    f[k + M] = exp(-t * t) * (L * L + t * t);  // index 0 stays 0
  }
  std::vector<double> g(M2);
  for (int j = 0; j < M2; ++j) g[j] = f[(j + M2 / 2) % M2];  // fftshift
  double an[kWeidemanN + 1];
  for (int n = 1; n <= N; ++n) {
    double re = 0;
    for (int j = 0; j < M2; ++j) re += g[j] * cos(2 * M_PI * (double)j * n / M2);
    an[n] = re / M2;
  }
  for (int i = 0; i < N; ++i) c->a[i] = an[N - i];
  c->L = L;
}

namespace {

__constant__ WeidemanCoeffs c_wd;
__constant__ EwaldConst c_ew;

constexpr int kEThreads = 128;

// Gamma(1/2 - j, z), j = 0..jmax, on the branch given by u = "sqrt(z)" (the
// caller chooses the sign of u); z = u^2.
__device__ __forceinline__ void gamma_half_down(qg_c u, int jmax, qg_c *G) {
  const double sqpi = 1.7724538509055160273;
  const qg_c z = cmul(u, u);
  G[0] = cscale(cerfc(u, c_wd), sqpi);
  // exp(-z) = exp(i w) with w = i z = (-zi, zr)
  const qg_c emz = cexpi(cmk(-z.im, z.re));
  qg_c zp = crecip(u);  // z^(-1/2) on the branch of u
  const qg_c rz = crecip(z);
  for (int j = 1; j <= jmax; ++j) {
    const double a = 0.5 - j;  // Gamma(a, z) = (Gamma(a+1, z) - z^a e^{-z}) / a
    G[j] = cscale(csub(G[j - 1], cmul(zp, emz)), 1.0 / a);
    zp = cmul(zp, rz);
  }
}

// clilgamma (ewald.h:157-170) with the branch rules of the reference
__device__ __forceinline__ qg_c csqrt_(qg_c z) {
  const double r = hypot(z.re, z.im);
  double a = sqrt(0.5 * (r + fabs(z.re)));
  if (a == 0.0) return cmk(0.0, z.im);
  double b = 0.5 * z.im / a;
  if (z.re >= 0) return cmk(a, b);
  return cmk(fabs(b), copysign(a, z.im));
}

template <int LMAX>
struct EwShape {
  static constexpr int LE = 2 * LMAX + 1;
  static constexpr int S = (LE + 1) * (LE + 1);  // nelem_sc
  static constexpr int NE = LMAX * (LMAX + 2);
  static constexpr int NE2 = NE * NE;
  static constexpr int NB = 2 * NE;
  static constexpr int NEVEN = (LE + 1) * (LE + 2) / 2;  // (n, m) with n + m even
  static constexpr int ZP = S < 36 ? S : 36;               // accumulators per shifted pass
  static constexpr int RED = NEVEN > ZP ? NEVEN : ZP;      // reduction buffer width
};

// (n, m) of the k-th even pair, in n-major order
__device__ __forceinline__ void even_nm(int k, int &n, int &m) {
  n = (int)((sqrtf(8.0f * k + 1.0f) - 1.0f) * 0.5f);
  if ((n + 1) * (n + 2) / 2 <= k) ++n;
  if (n * (n + 1) / 2 > k) --n;
  m = -n + 2 * (k - n * (n + 1) / 2);
}


// Unit data shared by the passes of one shifted pair.
struct ZUnit {
  qg_c k;
  double eta, bx, by, sx, sy, w;
  int KM;         // terms of the Delta series
  int spectral;   // 1: pure reciprocal-lattice sum (distant layers, |k w| >= 2.5)
};

// One pass of the shifted sums: sigma_y for Y0 <= y < Y0 + NY into sig[].
// s1u[e] = S1[e] (k w)^(2j - s) (2 eta / k)^(2j) (unit constants), rr[q] = r_q.
template <int LMAX, int Y0, int NY>
__device__ __forceinline__ void shifted_pass(const ZUnit &u, const qg_c *s1u, const double *rr, qg_c *sig,
                                             qg_c (*red)[EwShape<LMAX>::RED], int *errflag) {
  constexpr int LE = EwShape<LMAX>::LE;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const qg_c k = u.k;
  const double eta = u.eta, w = u.w;
  const bool kreal = (k.im == 0.0);
  qg_c acc[NY];
#pragma unroll
  for (int i = 0; i < NY; ++i) acc[i] = cmk(0, 0);
  const double sqpi = 1.7724538509055160273;

  // ---------------- short range (none for the reciprocal-lattice sum) ----------------
  if (!u.spectral) {
    const double rc = 7.5 / eta;
    const double smax = sqrt(u.sx * u.sx + u.sy * u.sy);
    const int I1 = (int)ceil((rc + smax) * c_ew.rbn[0] / (2 * M_PI)) + 1;
    const int I2 = (int)ceil((rc + smax) * c_ew.rbn[1] / (2 * M_PI)) + 1;
    const int W1 = 2 * I1 + 1, W2 = 2 * I2 + 1;
    const bool sr_ok = (long)W1 * W2 <= kEwMaxPoints && I1 >= 0 && I2 >= 0;
    if (!sr_ok && tid == 0) atomicOr(errflag, 1);
    const qg_c k2h = cscale(cmul(k, k), 0.5);
    const qg_c ik2eta = cmk(-k.im / (2 * eta), k.re / (2 * eta));
    const qg_c rk = crecip(k);
    for (int t = tid; sr_ok && t < W1 * W2; t += kEThreads) {
      const int i = t / W2 - I1, j = t % W2 - I2;
      const double Rx = i * c_ew.b[0] + j * c_ew.b[2] - u.sx, Ry = i * c_ew.b[1] + j * c_ew.b[3] - u.sy;
      const double rho2 = Rx * Rx + Ry * Ry, r2 = rho2 + w * w, r = sqrt(r2);
      if (r * eta > 7.5) continue;
      const qg_c zp = cmk(r * eta + ik2eta.re, ik2eta.im), zm = cmk(r * eta - ik2eta.re, -ik2eta.im);
      const qg_c Ep = cmul(cexpi(cscale(k, r)), cerfc(zp, c_wd)), Em = cmul(cexpi(cscale(k, -r)), cerfc(zm, c_wd));
      const qg_c d = csub(Em, Ep);
      qg_c pm2 = cscale(cmul(cmk(d.im, -d.re), rk), sqpi / 2);  // I_{-1}
      qg_c pm1 = cscale(cadd(Ep, Em), sqpi / (4 * r));           // I_0
      const qg_c ex = cmk(-r2 * eta * eta + (k.re * k.re - k.im * k.im) / (4 * eta * eta),
                          2 * k.re * k.im / (4 * eta * eta));
      const qg_c E = cexpi(cmk(ex.im, -ex.re));
      double sb, cb;
      sincos(u.bx * Rx + u.by * Ry, &sb, &cb);
      // base_n = -i (2/k)^(n+1) / sqrt(pi) r^n I_n e^{i beta.(R - s)}
      qg_c base[LE + 1];
      {
        qg_c pf = cscale(cmul(cmk(0.0, -1.0), cscale(rk, 2.0)), 1.0 / sqpi);
        const qg_c twok = cscale(rk, 2.0);
        const qg_c eb = cmk(cb, sb);
        double rn = 1.0, etap = eta;
        const double inv2r2 = 1.0 / (2 * r2);
#pragma unroll
        for (int n = 0; n <= LE; ++n) {
          qg_c In;
          if (n == 0) {
            In = pm1;
          } else {
            In = cscale(cadd(csub(cscale(pm1, 2 * n - 1), cmul(k2h, pm2)), cscale(E, etap)), inv2r2);
            pm2 = pm1;
            pm1 = In;
            etap *= eta * eta;
          }
          base[n] = cmul(cmul(cscale(pf, rn), In), eb);
          pf = cmul(pf, twok);
          rn *= r;
        }
      }
      const double rho = sqrt(rho2);
      const double ct = w / r, st = rho / r;
      const qg_c e1 = rho > 0 ? cmk(Rx / rho, Ry / rho) : cmk(1.0, 0.0);
      double pmm = 1.0;  // P_mu^mu(ct) with the Condon-Shortley phase
      qg_c em = cmk(1.0, 0.0);
#pragma unroll
      for (int mu = 0; mu <= LE; ++mu) {
        if (mu > 0) {
          pmm *= -(2 * mu - 1) * st;
          em = cmul(em, e1);
        }
        double p0 = 0.0, p1 = pmm;
#pragma unroll
        for (int n = mu; n <= LE; ++n) {
          double P;
          if (n == mu) {
            P = pmm;
          } else {
            P = ((2 * n - 1) * ct * p1 - (n + mu - 1) * p0) / (n - mu);
            p0 = p1;
            p1 = P;
          }
#pragma unroll
          for (int sg = 0; sg < 2; ++sg) {
            if (sg == 1 && mu == 0) continue;
            const int m = sg ? -mu : mu, y = n * (n + 1) + m;
            if (y < Y0 || y >= Y0 + NY) continue;
            const qg_c e = sg ? cconj(em) : em;
            acc[y - Y0] = cadd(acc[y - Y0], cscale(cmul(base[n], e), P * c_ew.legs[y]));
          }
        }
      }
    }
  }
  // ---------------- long range ----------------
  {
    const double kap2 = k.re * k.re + k.im * k.im;
    const double aw = fabs(w);
    // Ewald: terms below e^-56 past x^2 = 56; reciprocal-lattice sum: the terms
    // fall like e^(-|beta + K| |w|) (|beta + K|/k)^(2 lMax + 1), below 1e-17 past |beta + K| |w| = 80
    const double pmax = u.spectral ? 80.0 / aw : sqrt(kap2 + 56.0 * 4 * eta * eta);
    const double Kc = pmax + sqrt(u.bx * u.bx + u.by * u.by);
    const int I1 = (int)ceil(Kc * c_ew.bn[0] / (2 * M_PI)) + 1;
    const int I2 = (int)ceil(Kc * c_ew.bn[1] / (2 * M_PI)) + 1;
    const int W1 = 2 * I1 + 1, W2 = 2 * I2 + 1;
    const bool lr_ok = (long)W1 * W2 <= kEwMaxPoints && I1 >= 0 && I2 >= 0;
    if (!lr_ok && tid == 0) atomicOr(errflag, 1);
    const qg_c rk = crecip(k);
    const qg_c lrfac = crecip(cscale(cmul(k, k), c_ew.area));
    const qg_c kaw = cscale(k, aw);
    const qg_c rkaw = crecip(kaw);
    const int KM = u.KM;
    for (int t = tid; lr_ok && t < W1 * W2; t += kEThreads) {
      const int i = t / W2 - I1, j = t % W2 - I2;
      const double Kx = i * c_ew.rb[0] + j * c_ew.rb[2], Ky = i * c_ew.rb[1] + j * c_ew.rb[3];
      const double qx = Kx + u.bx, qy = Ky + u.by;
      const double rb = sqrt(qx * qx + qy * qy);
      if (u.spectral && rb > pmax) continue;
      qg_c gam, uu;
      if (kreal) {
        const double tt = rb / k.re;
        if (tt >= 1.0) {
          gam = cmk(sqrt(tt - 1.0) * sqrt(tt + 1.0), 0.0);
          const double x = gam.re * k.re / (2 * eta);
          if (!u.spectral && x * x > 56.0) continue;
          uu = cmk(x, 0.0);
        } else {
          const double g = sqrt(1.0 - tt) * sqrt(1.0 + tt);
          gam = cmk(0.0, -g);
          uu = cmk(0.0, -g * k.re / (2 * eta));
        }
      } else {
        const double kk2 = k.re * k.re + k.im * k.im;
        const qg_c z = cmk((rb * k.re + 0.0 * k.im) / kk2, (0.0 * k.re - rb * k.im) / kk2);
        qg_c a1 = cmk(z.re - 1, z.im), a2 = cmk(z.re + 1, z.im);
        a2 = (a2.re < 0 && a2.im <= 0) ? cscale(csqrt_(a2), -1.0) : csqrt_(a2);
        a1 = (a1.re < 0 && a1.im >= 0) ? cscale(csqrt_(a1), -1.0) : csqrt_(a1);
        gam = cmul(a1, a2);
        const qg_c x = cscale(cmul(gam, k), 1.0 / (2 * eta));
        const qg_c x2 = cmul(x, x);
        if (!u.spectral && x2.re > 56.0) continue;
        uu = csqrt_(x2);
        if (x2.re < 0 && !signbit(x2.im)) uu = cscale(uu, -1.0);
      }
      qg_c D[LE + 1];
      if (u.spectral) {
        // gamma^(2j-1) Delta_j(0, z) = sqrt(pi) 2^j (k|w|)^-j e^-a Kt_j, a = gamma k |w|,
        // Kt_j = gamma^(j-1) kappa_j(a) (half-integer Bessel K); sqrt(pi) 2^j (k|w|)^-j is in s1u
        const qg_c a = cmul(gam, kaw);
        const qg_c ea = cexpi(cmk(-a.im, a.re));  // e^-a
        const qg_c g2 = cmul(gam, gam);
        qg_c km1 = crecip(gam), kc = cmk(1.0, 0.0);
        D[0] = cmul(km1, ea);
        if (LE >= 1) D[1] = ea;
#pragma unroll
        for (int jq = 1; jq < LE; ++jq) {
          const qg_c kn = cadd(cmul(g2, km1), cscale(cmul(kc, rkaw), 2 * jq - 1));
          km1 = kc;
          kc = kn;
          D[jq + 1] = cmul(kn, ea);
        }
      } else {
        // D_a = sum_q r_q g_(a+q), g_i = X^i Gamma(1/2 - i, X)
        const qg_c X = cmul(uu, uu);
        const qg_c emX = cexpi(cmk(-X.im, X.re));
        const qg_c uemX = cmul(uu, emX);
#pragma unroll
        for (int a2i = 0; a2i <= LE; ++a2i) D[a2i] = cmk(0, 0);
        qg_c g = cscale(cerfc(uu, c_wd), sqpi);
        for (int jj = 0; jj <= LE + KM; ++jj) {
          if (jj > 0) g = cscale(csub(cmul(X, g), uemX), 1.0 / (0.5 - jj));
#pragma unroll
          for (int a2i = 0; a2i <= LE; ++a2i) {
            const int q = jj - a2i;
            if (q >= 0 && q <= KM) D[a2i] = cadd(D[a2i], cscale(g, rr[q]));
          }
        }
        // gamma^(2j-1) Delta_j = (2 eta / k)^(2j) D_j / gamma; the (2 eta / k)^(2j) is in s1u
        const qg_c rg = crecip(gam);
#pragma unroll
        for (int a2i = 0; a2i <= LE; ++a2i) D[a2i] = cmul(D[a2i], rg);
      }
      qg_c tpow[LE + 1];
      tpow[0] = cmk(1, 0);
      const qg_c tk = cscale(rk, rb);
#pragma unroll
      for (int p = 1; p <= LE; ++p) tpow[p] = cmul(tpow[p - 1], tk);
      double sK, cK;
      sincos(Kx * u.sx + Ky * u.sy, &sK, &cK);
      const qg_c phasefac = cmul(cmk(cK, sK), lrfac);
      const qg_c e1 = rb > 0 ? cmk(qx / rb, qy / rb) : cmk(1.0, 0.0);
      qg_c em = cmk(1.0, 0.0);
#pragma unroll
      for (int mu = 0; mu <= LE; ++mu) {
        if (mu > 0) em = cmul(em, e1);
        const qg_c emp = cmul(em, phasefac), emn = cmul(cconj(em), phasefac);
#pragma unroll
        for (int n = mu; n <= LE; ++n) {
#pragma unroll
          for (int sg = 0; sg < 2; ++sg) {
            if (sg == 1 && mu == 0) continue;
            const int m = sg ? -mu : mu, y = n * (n + 1) + m;
            if (y < Y0 || y >= Y0 + NY) continue;
            const int LM = n - mu;
            int e = c_ew.zoff[y];
            qg_c js = cmk(0, 0);
#pragma unroll
            for (int jq = 0; jq <= LM; ++jq)
#pragma unroll
              for (int sv = jq + (LM - jq) % 2; sv <= 2 * jq && sv <= LM; sv += 2) {
                js = cadd(js, cmul(cmul(s1u[e], tpow[n - sv]), D[jq]));
                ++e;
              }
            acc[y - Y0] = cadd(acc[y - Y0], cmul(js, sg ? emn : emp));
          }
        }
      }
    }
  }
  // ---------------- reduction into sig[Y0 .. Y0 + NY) ----------------
#pragma unroll
  for (int i = 0; i < NY; ++i) {
    double re = acc[i].re, im = acc[i].im;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) red[warp][i] = cmk(re, im);
  }
  __syncthreads();
  if (tid < NY) {
    qg_c v = cmk(0, 0);
    for (int wq = 0; wq < kEThreads / 32; ++wq) v = cadd(v, red[wq][tid]);
    sig[Y0 + tid] = v;
  }
  __syncthreads();
}

template <int LMAX, int Y0>
__device__ __forceinline__ void shifted_passes(const ZUnit &u, const qg_c *s1u, const double *rr, qg_c *sig,
                                               qg_c (*red)[EwShape<LMAX>::RED], int *errflag) {
  constexpr int S = EwShape<LMAX>::S, ZP = EwShape<LMAX>::ZP;
  constexpr int NY = (S - Y0 < ZP) ? S - Y0 : ZP;
  shifted_pass<LMAX, Y0, NY>(u, s1u, rr, sig, red, errflag);
  if constexpr (Y0 + NY < S) shifted_passes<LMAX, Y0 + NY>(u, s1u, rr, sig, red, errflag);
}

constexpr int kELChunks = 8;  // reciprocal-point chunks classified per batch

// Class of a reciprocal point |beta + K| = rb: 0 past the cutoff (x^2 > 56),
// 1 evanescent at real k (gamma and x real), 2 otherwise; gamma and the branch
// of x = gamma k / 2 eta (clilgamma, ewald.h:157-170, and ewald.c:390-393).
__device__ __forceinline__ int lr_class(qg_c k, bool kreal, double eta, double rb, qg_c &gam, qg_c &uu) {
  if (kreal) {
    // clilgamma(rb / k) for real k: sqrt(t - 1) sqrt(t + 1) with t - 1 exact;
    // near a Rayleigh anomaly (t -> 1) the 1/gamma terms dominate, so gamma is
    // formed from the exact differences as there
    const double tt = rb / k.re;
    if (tt >= 1.0) {
      gam = cmk(sqrt(tt - 1.0) * sqrt(tt + 1.0), 0.0);
      const double x = gam.re * k.re / (2 * eta);
      if (x * x > 56.0) return 0;
      uu = cmk(x, 0.0);
      return 1;
    }
    const double g = sqrt(1.0 - tt) * sqrt(1.0 + tt);
    gam = cmk(0.0, -g);  // -i sqrt(1 - t^2)
    // x^2 = -(g k / 2 eta)^2, approached from below the negative axis: sqrt -> -i c
    uu = cmk(0.0, -g * k.re / (2 * eta));
    return 2;
  }
  // z = rb / k as C's real / complex division forms it: (rb + 0i)(conj k) / |k|^2.
  // The sign of a zero imaginary part (rb = 0, i.e. beta on a reciprocal
  // lattice point) picks the branch of a1 below, so it must be +0 as there.
  const double kk2 = k.re * k.re + k.im * k.im;
  const qg_c z = cmk((rb * k.re + 0.0 * k.im) / kk2, (0.0 * k.re - rb * k.im) / kk2);
  qg_c a1 = cmk(z.re - 1, z.im), a2 = cmk(z.re + 1, z.im);
  a2 = (a2.re < 0 && a2.im <= 0) ? cscale(csqrt_(a2), -1.0) : csqrt_(a2);
  a1 = (a1.re < 0 && a1.im >= 0) ? cscale(csqrt_(a1), -1.0) : csqrt_(a1);
  gam = cmul(a1, a2);
  const qg_c x = cscale(cmul(gam, k), 1.0 / (2 * eta));
  const qg_c x2 = cmul(x, x);
  if (x2.re > 56.0) return 0;
  uu = csqrt_(x2);
  if (x2.re < 0 && !signbit(x2.im)) uu = cscale(uu, -1.0);  // branch m = -1 (ewald.c:390-393)
  return 2;
}

// M[R, C] = delta_RC I - T_R W(R <- C) from sigma in shared memory
// (translations.c:926-1078 contraction; the B sum runs over q <= qmax_A).
template <int LMAX>
__device__ __forceinline__ void contract_block(const EwaldArgs &a, const TransDevTables &T, const qg_c *sig,
                                               size_t wk, size_t per, int pr, int R, int C, int iw) {
  using Sh = EwShape<LMAX>;
  constexpr int NE = Sh::NE, NE2 = Sh::NE2, NB = Sh::NB;
  const int tid = threadIdx.x;
  const size_t N = (size_t)a.np * NB;
  // full matrix: block (R, C) of the N x N matrix wk; pair list: block pr alone (ld NB)
  qg_c *M = a.npairs ? a.M + (wk * per + pr) * NB * NB : a.M + wk * N * N;
  const size_t ldm = a.npairs ? (size_t)NB : N;
  const size_t row0 = a.npairs ? 0 : (size_t)R * NB, col0 = a.npairs ? 0 : (size_t)C * NB;
  const qg_c *TR = a.T + ((size_t)iw * a.ntm + a.tmid[R]) * NB;
#pragma unroll 1
  for (int which = 0; which < 2; ++which) {
    const uint8_t *cnt = which ? T.cntBe : T.cntA;
    const double *coef = which ? T.coefB : T.coefA;
    const uint16_t *slot = which ? T.slotB : T.slotA;
    const int32_t *perm = which ? T.permB : T.perm;
    for (int kx = tid; kx < NE2; kx += kEThreads) {
      const int c = cnt[kx];
      double sr = 0, si = 0;
      for (int q = 0; q < c; ++q) {
        const double cf = __ldg(coef + q * NE2 + kx);
        const qg_c x = sig[__ldg(slot + q * NE2 + kx)];
        sr = fma(cf, x.re, sr);
        si = fma(cf, x.im, si);
      }
      const qg_c v = which ? cmk(-si, sr) : cmk(sr, si);
      const int e = __ldg(perm + kx);
      const int yi = e / NE, yj = e - yi * NE;
      const int r1 = yi, c1 = which ? NE + yj : yj;
      const int r2 = NE + yi, c2 = which ? yj : NE + yj;
      const qg_c m1 = cscale(cmul(TR[r1], v), -1.0), m2 = cscale(cmul(TR[r2], v), -1.0);
      M[(row0 + r1) * ldm + col0 + c1] = (R == C && r1 == c1) ? cadd(m1, cmk(1, 0)) : m1;
      M[(row0 + r2) * ldm + col0 + c2] = (R == C && r2 == c2) ? cadd(m2, cmk(1, 0)) : m2;
    }
  }
  __syncthreads();
}

template <int LMAX>
__global__ void __launch_bounds__(kEThreads) ewald_assemble_kernel(EwaldArgs a, TransDevTables T) {
  using Sh = EwShape<LMAX>;
  constexpr int LE = Sh::LE, S = Sh::S, NEV = Sh::NEVEN;
  __shared__ qg_c sig[S];
  __shared__ qg_c red[kEThreads / 32][Sh::RED];
  __shared__ int lstA[kEThreads * kELChunks], lstB[kEThreads * kELChunks];
  __shared__ int lw[2][kEThreads / 32], lcnt[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int np = a.np;
  const size_t per = a.npairs ? (size_t)a.npairs : (size_t)np * np;  // blocks per matrix
  const size_t units = (size_t)a.nw * a.nk * per;
  for (size_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int pr = (int)(u % per);
    const size_t wk = u / per;
    const int iw = (int)(wk / a.nk), ik = a.paired ? iw : (int)(wk % a.nk);
    const int R = a.npairs ? a.pairs[2 * pr] : pr / np;
    const int C = a.npairs ? a.pairs[2 * pr + 1] : pr - R * np;
    const qg_c k = a.k[iw];
    const double eta = a.eta[wk];
    const double bx = a.beta[2 * ik], by = a.beta[2 * ik + 1];
    const double sx = a.pos[3 * R] - a.pos[3 * C], sy = a.pos[3 * R + 1] - a.pos[3 * C + 1];
    const double sz = a.pos[3 * R + 2] - a.pos[3 * C + 2];
    if (sz != 0.0) {
      // a pair of layers: ewald_layers_kernel forms it (launched when a.layered)
      if (!a.layered && tid == 0) atomicOr(a.err, 2);
      continue;
    }
    const bool self = (sx == 0.0 && sy == 0.0);
    const bool kreal = (k.im == 0.0);
    qg_c acc[NEV];
#pragma unroll
    for (int i = 0; i < NEV; ++i) acc[i] = cmk(0, 0);

    // ---------------- short range (direct lattice) ----------------
    if (a.srtab) {  // the tabulated terms of (frequency, pair) with the Bloch phase
      const size_t ti = (size_t)iw * per + pr;
      const int cnt = a.srcnt[ti];
      const qg_c *tab = a.srtab + ti * NEV * (size_t)a.srmax;
      const double *pts = a.srpts + ti * 2 * (size_t)a.srmax;
      for (int p = tid; p < cnt; p += kEThreads) {
        double sb, cb;
        sincos(bx * pts[2 * p] + by * pts[2 * p + 1], &sb, &cb);
#pragma unroll
        for (int kk = 0; kk < NEV; ++kk) {
          const qg_c c = tab[(size_t)kk * a.srmax + p];
          acc[kk].re = fma(cb, c.re, fma(-sb, c.im, acc[kk].re));
          acc[kk].im = fma(cb, c.im, fma(sb, c.re, acc[kk].im));
        }
      }
    } else {
      const double rc = 7.5 / eta;  // |R - shift| eta <= 7.5
      const double smax = sqrt(sx * sx + sy * sy);
      const int I1 = (int)ceil((rc + smax) * c_ew.rbn[0] / (2 * M_PI)) + 1;
      const int I2 = (int)ceil((rc + smax) * c_ew.rbn[1] / (2 * M_PI)) + 1;
      const int W1 = 2 * I1 + 1, W2 = 2 * I2 + 1;
      const bool sr_ok = (long)W1 * W2 <= kEwMaxPoints && I1 >= 0 && I2 >= 0;
      if (!sr_ok && tid == 0) atomicOr(a.err, 1);
      const qg_c k2h = cscale(cmul(k, k), 0.5);
      const qg_c ik2eta = cmk(-k.im / (2 * eta), k.re / (2 * eta));  // i k / (2 eta)
      const qg_c rk = crecip(k);
      // direct-lattice points in batches, compacted as the reciprocal ones below
      const int WS = sr_ok ? W1 * W2 : 0;
      for (int t0 = 0; t0 < WS; t0 += kEThreads * kELChunks) {
        __syncthreads();
        if (tid == 0) lcnt[0] = 0;
        __syncthreads();
        for (int c = 0; c < kELChunks; ++c) {
          const int t = t0 + c * kEThreads + tid;
          bool ok = false;
          if (t < WS) {
            const int i = t / W2 - I1, j = t % W2 - I2;
            const double Rx = i * c_ew.b[0] + j * c_ew.b[2] - sx, Ry = i * c_ew.b[1] + j * c_ew.b[3] - sy;
            ok = !(self && i == 0 && j == 0) && sqrt(Rx * Rx + Ry * Ry) * eta <= 7.5;
          }
          const unsigned bA = __ballot_sync(0xffffffffu, ok);
          if (lane == 0) lw[0][warp] = __popc(bA);
          __syncthreads();
          int oA = lcnt[0];
          for (int w = 0; w < warp; ++w) oA += lw[0][w];
          if (ok) lstA[oA + __popc(bA & ((1u << lane) - 1u))] = t;
          __syncthreads();
          if (tid == 0)
            for (int w = 0; w < kEThreads / 32; ++w) lcnt[0] += lw[0][w];
          __syncthreads();
        }
        const int nS = lcnt[0];
      for (int pidx = tid; pidx < nS; pidx += kEThreads) {
        const int t = lstA[pidx];
        const int i = t / W2 - I1, j = t % W2 - I2;
        const double Rx = i * c_ew.b[0] + j * c_ew.b[2] - sx, Ry = i * c_ew.b[1] + j * c_ew.b[3] - sy;
        const double r2 = Rx * Rx + Ry * Ry, r = sqrt(r2);
        // e^{i beta.(R - s)} folded into E+-, E: the I_n recurrence is linear, so
        // it yields I_n e^{i beta.(R - s)} directly
        double sb, cb;
        sincos(bx * Rx + by * Ry, &sb, &cb);
        const qg_c ebeta = cmk(cb, sb);
        const qg_c zp = cmk(r * eta + ik2eta.re, ik2eta.im);
        const qg_c ekr = cexpi(cscale(k, r)), erp = cerfc(zp, c_wd);
        qg_c emkr, erm;
        if (kreal) {  // z- = conj(z+), e^{-ikr} = conj(e^{ikr}) for real k
          emkr = cconj(ekr);
          erm = cconj(erp);
        } else {
          emkr = cexpi(cscale(k, -r));
          erm = cerfc(cmk(r * eta - ik2eta.re, -ik2eta.im), c_wd);
        }
        const qg_c Ep = cmul(cmul(ekr, erp), ebeta), Em = cmul(cmul(emkr, erm), ebeta);
        const double sqpi = 1.7724538509055160273;
        const qg_c I0 = cscale(cadd(Ep, Em), sqpi / (4 * r));
        // I_{-1} = sqrt(pi)/(2 i k) (Em - Ep)
        const qg_c d = csub(Em, Ep);
        const qg_c Im1 = cscale(cmul(cmk(d.im, -d.re), rk), sqpi / 2);  // (Em-Ep)/(i) = -i (Em-Ep)
        // E = exp(-r^2 eta^2 + k^2 / (4 eta^2)) e^{i beta.(R - s)}
        const qg_c ex = cmk(-r2 * eta * eta + (k.re * k.re - k.im * k.im) / (4 * eta * eta),
                            2 * k.re * k.im / (4 * eta * eta));
        const qg_c E = cmul(cexpi(cmk(ex.im, -ex.re)), ebeta);
        qg_c pm2 = Im1, pm1 = I0;
        double etap = eta;  // eta^(2n-1)
        const double inv2r2 = 1.0 / (2 * r2);
        const qg_c e1 = cmk(Rx / r, Ry / r), e2 = cmul(e1, e1), e1c = cconj(e1);  // e^{i phi}
        // c_n = prefac_n r^n = -i (2/k)^{n+1} r^n / sqrt(pi)
        qg_c cn = cscale(cmk(rk.im, -rk.re), 2.0 / sqpi);  // -i (2/k) / sqrt(pi)
        const qg_c twor_k = cscale(rk, 2.0 * r);
        qg_c emn = cmk(1, 0);  // e^{-i n phi}
#pragma unroll
        for (int n = 0; n <= LE; ++n) {
          qg_c In;
          if (n == 0) {
            In = I0;
          } else {
            In = cscale(cadd(csub(cscale(pm1, 2 * n - 1), cmul(k2h, pm2)), cscale(E, etap)), inv2r2);
            pm2 = pm1;
            pm1 = In;
            etap *= eta * eta;
          }
          const qg_c base = cmul(cn, In);
          // m = -n, -n+2, ..., n: acc += leg0m (base e^{i m phi})
          qg_c em = emn;
#pragma unroll
          for (int q = 0; q <= n; ++q) {
            const int m = -n + 2 * q;
            const int kk = n * (n + 1) / 2 + q;
            const qg_c pr = cmul(base, em);
            const double lg = c_ew.leg0m[n * (n + 1) + m];
            acc[kk].re = fma(lg, pr.re, acc[kk].re);
            acc[kk].im = fma(lg, pr.im, acc[kk].im);
            em = cmul(em, e2);
          }
          emn = cmul(emn, e1c);
          cn = cmul(cn, twor_k);
        }
      }
      }
    }
    // ---------------- long range (reciprocal lattice) ----------------
    {
      const double kap2 = k.re * k.re + k.im * k.im;
      const double Kc = sqrt(kap2 + 56.0 * 4 * eta * eta) + sqrt(bx * bx + by * by);
      const int I1 = (int)ceil(Kc * c_ew.bn[0] / (2 * M_PI)) + 1;
      const int I2 = (int)ceil(Kc * c_ew.bn[1] / (2 * M_PI)) + 1;
      const int W1 = 2 * I1 + 1, W2 = 2 * I2 + 1;
      const bool lr_ok = (long)W1 * W2 <= kEwMaxPoints && I1 >= 0 && I2 >= 0;
      if (!lr_ok && tid == 0) atomicOr(a.err, 1);
      const qg_c rk = crecip(k);
      const qg_c lrfac = crecip(cscale(cmul(k, k), c_ew.area));  // commonfac 1 / (k^2 A), ewald.c:344
      // reciprocal points in batches: classified (outside the cutoff / evanescent
      // at real k / other) and compacted in grid order with a block prefix sum,
      // so the warps process dense lists (FP64 lanes masked off by divergence
      // are lost time on the FP64 pipe)
      const int WW = lr_ok ? W1 * W2 : 0;
      for (int t0 = 0; t0 < WW; t0 += kEThreads * kELChunks) {
        __syncthreads();
        if (tid == 0) {
          lcnt[0] = 0;
          lcnt[1] = 0;
        }
        __syncthreads();
        for (int c = 0; c < kELChunks; ++c) {
          const int t = t0 + c * kEThreads + tid;
          int cls = 0;
          if (t < WW) {
            const int i = t / W2 - I1, j = t % W2 - I2;
            const double qx = i * c_ew.rb[0] + j * c_ew.rb[2] + bx, qy = i * c_ew.rb[1] + j * c_ew.rb[3] + by;
            qg_c g_, u_;
            cls = lr_class(k, kreal, eta, sqrt(qx * qx + qy * qy), g_, u_);
          }
          const unsigned bA = __ballot_sync(0xffffffffu, cls == 1), bB = __ballot_sync(0xffffffffu, cls == 2);
          if (lane == 0) {
            lw[0][warp] = __popc(bA);
            lw[1][warp] = __popc(bB);
          }
          __syncthreads();
          int oA = lcnt[0], oB = lcnt[1];
          for (int w = 0; w < warp; ++w) {
            oA += lw[0][w];
            oB += lw[1][w];
          }
          const unsigned lt = (1u << lane) - 1u;
          if (cls == 1) lstA[oA + __popc(bA & lt)] = t;
          if (cls == 2) lstB[oB + __popc(bB & lt)] = t;
          __syncthreads();
          if (tid == 0)
            for (int w = 0; w < kEThreads / 32; ++w) {
              lcnt[0] += lw[0][w];
              lcnt[1] += lw[1][w];
            }
          __syncthreads();
        }
        const int nA = lcnt[0], nB = lcnt[1];
        for (int pidx = tid; pidx < nA + nB; pidx += kEThreads) {
          const int t = pidx < nA ? lstA[pidx] : lstB[pidx - nA];
          const int i = t / W2 - I1, j = t % W2 - I2;
          const double Kx = i * c_ew.rb[0] + j * c_ew.rb[2], Ky = i * c_ew.rb[1] + j * c_ew.rb[3];
          const double qx = Kx + bx, qy = Ky + by;
          const double rb = sqrt(qx * qx + qy * qy);
          qg_c gam, uu;
          lr_class(k, kreal, eta, rb, gam, uu);
          double sK, cK;
          sincos(Kx * sx + Ky * sy, &sK, &cK);
          const qg_c phasefac = cmul(cmk(cK, sK), lrfac);  // e^{i K.s} / (k^2 A)
          // e^{i alpha}, alpha = arg(beta + K) (0 at the origin, as atan2(0, 0))
          const qg_c e1 = rb > 0 ? cmk(qx / rb, qy / rb) : cmk(1.0, 0.0), e2 = cmul(e1, e1), e1c = cconj(e1);
          if (pidx < nA) {
            // evanescent order at real k: gamma, x = gamma k / 2 eta, Gamma(1/2 - j, x^2),
            // rb / k are real, so is every P_nj; only e^{i m alpha} and the phase are complex
            const double x = uu.re, X = x * x, emX = exp(-X);
            double Gr[LE / 2 + 1];
            Gr[0] = 1.7724538509055160273 * erfc(x);  // Gamma(1/2, x^2)
            double zp = 1.0 / x;                      // x^(1-2j)
            const double rX = 1.0 / X;
  #pragma unroll
            for (int j = 1; j <= LE / 2; ++j) {
              Gr[j] = (Gr[j - 1] - zp * emX) / (0.5 - j);
              zp *= rX;
            }
            double gpr[LE / 2 + 1];
            {
              double g = 1.0 / gam.re;
              const double gsq = gam.re * gam.re;
  #pragma unroll
              for (int j = 0; j <= LE / 2; ++j) {
                gpr[j] = g * Gr[j];
                g *= gsq;
              }
            }
            double tp[LE + 1];
            tp[0] = 1.0;
            const double tkr = rb / k.re;
  #pragma unroll
            for (int p = 1; p <= LE; ++p) tp[p] = tp[p - 1] * tkr;
            qg_c emn = phasefac;
  #pragma unroll
            for (int n = 0; n <= LE; ++n) {
              double P[LE / 2 + 1];
  #pragma unroll
              for (int j = 0; j <= n / 2; ++j) P[j] = tp[n - 2 * j] * gpr[j];
              qg_c em = emn;
  #pragma unroll
              for (int q = 0; q <= n; ++q) {
                const int m = -n + 2 * q;
                const int y = n * (n + 1) + m;
                const int jmax = (n - (m < 0 ? -m : m)) / 2;
                double jr = 0;
  #pragma unroll
                for (int j = 0; j <= jmax; ++j) jr = fma(c_ew.s1r[c_ew.s1off[y] + j], P[j], jr);
                // acc += i^(n+1) jr em
                const int kk = n * (n + 1) / 2 + q;
                switch ((n + 1) & 3) {
                  case 0: acc[kk].re = fma(jr, em.re, acc[kk].re); acc[kk].im = fma(jr, em.im, acc[kk].im); break;
                  case 1: acc[kk].re = fma(-jr, em.im, acc[kk].re); acc[kk].im = fma(jr, em.re, acc[kk].im); break;
                  case 2: acc[kk].re = fma(-jr, em.re, acc[kk].re); acc[kk].im = fma(-jr, em.im, acc[kk].im); break;
                  default: acc[kk].re = fma(jr, em.im, acc[kk].re); acc[kk].im = fma(-jr, em.re, acc[kk].im); break;
                }
                em = cmul(em, e2);
              }
              emn = cmul(emn, e1c);
            }
          } else {
            qg_c G[LE / 2 + 1];
            gamma_half_down(uu, LE / 2, G);
            // powers: (rb/k)^(n - 2j) and gamma^(2j - 1)
            const qg_c tk = cscale(rk, rb);
            qg_c gp[LE / 2 + 1];  // gamma^(2j-1) G_j
            {
              qg_c g = crecip(gam);  // gamma^-1
              const qg_c gsq = cmul(gam, gam);
              for (int j = 0; j <= LE / 2; ++j) {
                gp[j] = cmul(g, G[j]);
                g = cmul(g, gsq);
              }
            }
            qg_c tpow[LE + 1];
            tpow[0] = cmk(1, 0);
            for (int p = 1; p <= LE; ++p) tpow[p] = cmul(tpow[p - 1], tk);
            // s1[y][j] = i^(n+1) s1r[y][j]: js = i^(n+1) sum_j s1r P_nj, P_nj = tpow[n-2j] gp[j]
            qg_c emn = phasefac;  // e^{-i n alpha} e^{i K.s} / (k^2 A)
    #pragma unroll
            for (int n = 0; n <= LE; ++n) {
              qg_c P[LE / 2 + 1];
    #pragma unroll
              for (int j = 0; j <= n / 2; ++j) P[j] = cmul(tpow[n - 2 * j], gp[j]);
              qg_c em = emn;
    #pragma unroll
              for (int q = 0; q <= n; ++q) {
                const int m = -n + 2 * q;
                const int y = n * (n + 1) + m;
                const int jmax = (n - (m < 0 ? -m : m)) / 2;
                double jr = 0, ji = 0;
    #pragma unroll
                for (int j = 0; j <= jmax; ++j) {
                  const double c = c_ew.s1r[c_ew.s1off[y] + j];
                  jr = fma(c, P[j].re, jr);
                  ji = fma(c, P[j].im, ji);
                }
                qg_c js;  // times i^(n+1)
                switch ((n + 1) & 3) {
                  case 0: js = cmk(jr, ji); break;
                  case 1: js = cmk(-ji, jr); break;
                  case 2: js = cmk(-jr, -ji); break;
                  default: js = cmk(ji, -jr); break;
                }
                const int kk = n * (n + 1) / 2 + q;
                const qg_c pr = cmul(js, em);
                acc[kk].re += pr.re;
                acc[kk].im += pr.im;
                em = cmul(em, e2);
              }
              emn = cmul(emn, e1c);
            }
          }
        }
      }
    }
    // ---------------- reduction into sig[] ----------------
#pragma unroll
    for (int i = 0; i < NEV; ++i) {
      double re = acc[i].re, im = acc[i].im;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
      }
      if (lane == 0) red[warp][i] = cmk(re, im);
    }
    __syncthreads();
    for (int s = tid; s < S; s += kEThreads) sig[s] = cmk(0, 0);
    __syncthreads();
    if (tid < NEV) {
      qg_c v = cmk(0, 0);
      for (int w = 0; w < kEThreads / 32; ++w) v = cadd(v, red[w][tid]);
      int n, m;
      even_nm(tid, n, m);
      sig[n * (n + 1) + m] = v;
    }
    __syncthreads();
    if (tid == 0 && self) {
      // sigma0 = Gamma(-1/2, -(k/2eta)^2) / (2 sqrt(pi)) on the branch from below (ewald.c:260-273)
      const qg_c kk2 = cscale(k, 1.0 / (2 * eta));
      qg_c z = cmul(kk2, kk2);
      z = cmk(-z.re, -z.im);
      qg_c uu;
      if (kreal) {
        uu = cmk(0.0, -k.re / (2 * eta));
      } else {
        uu = csqrt_(z);
        if (z.re < 0 && !signbit(z.im)) uu = cscale(uu, -1.0);  // ewald.c:266-268
      }
      qg_c G[2];
      gamma_half_down(uu, 1, G);
      sig[0] = cadd(sig[0], cscale(G[1], 1.0 / (2 * 1.7724538509055160273)));
    }
    __syncthreads();
    contract_block<LMAX>(a, T, sig, wk, per, pr, R, C, iw);
  }
}

// Short-range tables: one CTA per (frequency w, pair) at the common eta of w.
// Lattice points are taken in grid order, compacted with a block prefix sum
// (deterministic order); every valid point stores R - s and its terms
// c_nm = prefac_n |R - s|^n I_n leg0m e^{i m phi} (n + m even).
template <int LMAX>
__global__ void __launch_bounds__(kEThreads) ewald_sr_table_kernel(EwaldArgs a) {
  using Sh = EwShape<LMAX>;
  constexpr int LE = Sh::LE, NEV = Sh::NEVEN;
  __shared__ int wsum[kEThreads / 32];
  __shared__ int base_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int np = a.np;
  const size_t per = (size_t)np * np;
  const size_t units = (size_t)a.nw * per;
  for (size_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int pr = (int)(u % per), iw = (int)(u / per);
    const int R = pr / np, C = pr - R * np;
    const double sx = a.pos[3 * R] - a.pos[3 * C], sy = a.pos[3 * R + 1] - a.pos[3 * C + 1];
    const double sz = a.pos[3 * R + 2] - a.pos[3 * C + 2];
    const qg_c k = a.k[iw];
    const double eta = a.eta[(size_t)iw * a.nk];
    const bool self = (sx == 0.0 && sy == 0.0), kreal = (k.im == 0.0);
    qg_c *tab = a.srtab + u * NEV * (size_t)a.srmax;
    double *pts = a.srpts + u * 2 * (size_t)a.srmax;
    if (tid == 0) base_s = 0;
    __syncthreads();
    if (sz == 0.0) {
      const double rc = 7.5 / eta;
      const double smax = sqrt(sx * sx + sy * sy);
      const int I1 = (int)ceil((rc + smax) * c_ew.rbn[0] / (2 * M_PI)) + 1;
      const int I2 = (int)ceil((rc + smax) * c_ew.rbn[1] / (2 * M_PI)) + 1;
      const int W1 = 2 * I1 + 1, W2 = 2 * I2 + 1;
      const bool sr_ok = (long)W1 * W2 <= kEwMaxPoints && I1 >= 0 && I2 >= 0;
      if (!sr_ok && tid == 0) atomicOr(a.err, 1);
      const qg_c k2h = cscale(cmul(k, k), 0.5);
      const qg_c ik2eta = cmk(-k.im / (2 * eta), k.re / (2 * eta));
      const qg_c rk = crecip(k);
      const int tot = sr_ok ? W1 * W2 : 0;
      for (int t0 = 0; t0 < tot; t0 += kEThreads) {
        const int t = t0 + tid;
        double Rx = 0, Ry = 0, r2 = 0, r = 0;
        bool valid = false;
        if (t < tot) {
          const int i = t / W2 - I1, j = t % W2 - I2;
          Rx = i * c_ew.b[0] + j * c_ew.b[2] - sx;
          Ry = i * c_ew.b[1] + j * c_ew.b[3] - sy;
          r2 = Rx * Rx + Ry * Ry;
          r = sqrt(r2);
          valid = !(self && i == 0 && j == 0) && r * eta <= 7.5;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, valid);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        int off = base_s;
        for (int w = 0; w < warp; ++w) off += wsum[w];
        const int pos = off + __popc(bal & ((1u << lane) - 1u));
        __syncthreads();
        if (tid == 0) {
          int s2 = base_s;
          for (int w = 0; w < kEThreads / 32; ++w) s2 += wsum[w];
          base_s = s2;
        }
        if (valid && pos < a.srmax) {
          pts[2 * pos] = Rx;
          pts[2 * pos + 1] = Ry;
          const qg_c zp = cmk(r * eta + ik2eta.re, ik2eta.im);
          const qg_c ekr = cexpi(cscale(k, r)), erp = cerfc(zp, c_wd);
          qg_c emkr, erm;
          if (kreal) {
            emkr = cconj(ekr);
            erm = cconj(erp);
          } else {
            emkr = cexpi(cscale(k, -r));
            erm = cerfc(cmk(r * eta - ik2eta.re, -ik2eta.im), c_wd);
          }
          const qg_c Ep = cmul(ekr, erp), Em = cmul(emkr, erm);
          const double sqpi = 1.7724538509055160273;
          const qg_c I0 = cscale(cadd(Ep, Em), sqpi / (4 * r));
          const qg_c d = csub(Em, Ep);
          const qg_c Im1 = cscale(cmul(cmk(d.im, -d.re), rk), sqpi / 2);
          const qg_c ex = cmk(-r2 * eta * eta + (k.re * k.re - k.im * k.im) / (4 * eta * eta),
                              2 * k.re * k.im / (4 * eta * eta));
          const qg_c E = cexpi(cmk(ex.im, -ex.re));
          qg_c pm2 = Im1, pm1 = I0;
          double etap = eta;
          const double inv2r2 = 1.0 / (2 * r2);
          const qg_c e1 = cmk(Rx / r, Ry / r), e2 = cmul(e1, e1), e1c = cconj(e1);
          qg_c cn = cscale(cmk(rk.im, -rk.re), 2.0 / sqpi);
          const qg_c twor_k = cscale(rk, 2.0 * r);
          qg_c emn = cmk(1, 0);
#pragma unroll
          for (int n = 0; n <= LE; ++n) {
            qg_c In;
            if (n == 0) {
              In = I0;
            } else {
              In = cscale(cadd(csub(cscale(pm1, 2 * n - 1), cmul(k2h, pm2)), cscale(E, etap)), inv2r2);
              pm2 = pm1;
              pm1 = In;
              etap *= eta * eta;
            }
            const qg_c base = cmul(cn, In);
            qg_c em = emn;
#pragma unroll
            for (int q = 0; q <= n; ++q) {
              const int m = -n + 2 * q;
              const int kk = n * (n + 1) / 2 + q;
              tab[(size_t)kk * a.srmax + pos] = cscale(cmul(base, em), c_ew.leg0m[n * (n + 1) + m]);
              em = cmul(em, e2);
            }
            emn = cmul(emn, e1c);
            cn = cmul(cn, twor_k);
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (tid == 0) {
      if (base_s > a.srmax) atomicOr(a.err, 1);
      a.srcnt[u] = base_s < a.srmax ? base_s : a.srmax;
    }
    __syncthreads();
  }
}

template <int LMAX>
__global__ void __launch_bounds__(kEThreads) ewald_layers_kernel(EwaldArgs a, TransDevTables T) {
  using Sh = EwShape<LMAX>;
  constexpr int S = Sh::S;
  __shared__ qg_c sig[S];
  __shared__ qg_c red[kEThreads / 32][Sh::RED];
  __shared__ qg_c s1u[kEwZ];
  __shared__ double rr[48];
  const int tid = threadIdx.x;
  const int np = a.np;
  const size_t per = a.npairs ? (size_t)a.npairs : (size_t)np * np;  // blocks per matrix
  const size_t units = (size_t)a.nw * a.nk * per;
  for (size_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int pr = (int)(u % per);
    const size_t wk = u / per;
    const int iw = (int)(wk / a.nk), ik = a.paired ? iw : (int)(wk % a.nk);
    const int R = a.npairs ? a.pairs[2 * pr] : pr / np;
    const int C = a.npairs ? a.pairs[2 * pr + 1] : pr - R * np;
    const qg_c k = a.k[iw];
    const double eta = a.eta[wk];
    const double bx = a.beta[2 * ik], by = a.beta[2 * ik + 1];
    const double sx = a.pos[3 * R] - a.pos[3 * C], sy = a.pos[3 * R + 1] - a.pos[3 * C + 1];
    const double sz = a.pos[3 * R + 2] - a.pos[3 * C + 2];
    if (sz == 0.0) continue;  // ewald_assemble_kernel
    // ---------------- layers at different heights ----------------
    ZUnit zu;
    zu.k = k;
    zu.w = -sz;
    // distant layers (|k sz| >= 2.5): the pure reciprocal-lattice sum; else
    // eta <= 1 / |sz| for the Delta series, which keeps k / (2 eta) <= 1.25
    zu.spectral = hypot(k.re, k.im) * fabs(sz) >= 2.5;
    zu.eta = fmin(eta, 1.0 / fabs(sz));
    zu.bx = bx;
    zu.by = by;
    zu.sx = sx;
    zu.sy = sy;
    const double x2e = sz * sz * zu.eta * zu.eta;
    {
      int q = 0;
      double tq = 1.0;
      while (q < 46 && tq > 1e-18) {
        ++q;
        tq *= x2e / q;
      }
      zu.KM = q;
    }
    if (tid == 0) {
      double tq = 1.0;
      for (int q = 0; q <= zu.KM; ++q) {
        rr[q] = tq;
        tq *= -x2e / (q + 1);
      }
    }
    {
      // Ewald: S1 (k w)^(2j - s) (2 eta / k)^(2j);
      // reciprocal-lattice sum: S1 sqrt(pi) 2^j sgn(w)^s (k |w|)^(j - s)
      const qg_c kw = cscale(k, zu.w), te = cscale(crecip(k), 2 * zu.eta);
      const qg_c te2 = cmul(te, te);
      const qg_c rkaw = crecip(cscale(k, fabs(zu.w)));
      for (int e = tid; e < c_ew.zoff[S]; e += kEThreads) {
        const int jq = c_ew.zj[e], sv = c_ew.zsv[e];
        qg_c f = c_ew.zs1[e];
        if (zu.spectral) {
          f = cscale(f, 1.7724538509055160273 * (double)(1 << jq) * ((zu.w < 0 && (sv & 1)) ? -1.0 : 1.0));
          for (int q = 0; q < sv - jq; ++q) f = cmul(f, rkaw);
        } else {
          for (int q = 0; q < 2 * jq - sv; ++q) f = cmul(f, kw);
          for (int q = 0; q < jq; ++q) f = cmul(f, te2);
        }
        s1u[e] = f;
      }
    }
    __syncthreads();
    shifted_passes<LMAX, 0>(zu, s1u, rr, sig, red, a.err);
    contract_block<LMAX>(a, T, sig, wk, per, pr, R, C, iw);
    __syncthreads();
  }
}

template <int LMAX>
int launch_ew(const EwaldArgs &a, const TransDevTables &T, cudaStream_t st) {
  const size_t units = (size_t)a.nw * a.nk * (a.npairs ? (size_t)a.npairs : (size_t)a.np * a.np);
  if (!units) return QPMS_SUCCESS;
  int dev = 0, nsm = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  QG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  size_t grid = std::min<size_t>(units, (size_t)nsm * 16);
  const double nblk = 2.0 * LMAX * (LMAX + 2);
  KtScope kt(KT_EWALD, st, 16.0 * nblk * nblk * (double)units);
  if (a.srtab) {
    const size_t tunits = (size_t)a.nw * a.np * a.np;
    ewald_sr_table_kernel<LMAX><<<(unsigned)std::min<size_t>(tunits, (size_t)nsm * 16), kEThreads, 0, st>>>(a);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  }
  ewald_assemble_kernel<LMAX><<<(unsigned)grid, kEThreads, 0, st>>>(a, T);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  if (a.layered) {
    ewald_layers_kernel<LMAX><<<(unsigned)grid, kEThreads, 0, st>>>(a, T);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  }
  return QPMS_SUCCESS;
}

}  // namespace

int ewald_upload_constants(const EwaldConst &c, cudaStream_t st) {
  // the Faddeeva coefficients: once per device (callers hold the Ewald lock)
  static bool wd_done[64] = {false};
  int dev = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("device index %d out of range", dev);
    return QPMS_EINVAL;
  }
  if (!wd_done[dev]) {
    WeidemanCoeffs w;
    weideman_coeffs(&w);
    QG_CUDA_TRY(cudaMemcpyToSymbol(c_wd, &w, sizeof w));
    wd_done[dev] = true;
  }
  QG_CUDA_TRY(cudaMemcpyToSymbolAsync(c_ew, &c, sizeof c, 0, cudaMemcpyHostToDevice, st));
  return QPMS_SUCCESS;
}

int launch_ewald_assemble(const EwaldArgs &a, const TransDevTables &T, cudaStream_t st) {
  switch (T.lMax) {
    case 1: return launch_ew<1>(a, T, st);
    case 2: return launch_ew<2>(a, T, st);
    case 3: return launch_ew<3>(a, T, st);
    case 4: return launch_ew<4>(a, T, st);
    default: set_error("Ewald assembly: lMax %d not compiled (1..4)", T.lMax); return QPMS_EINVAL;
  }
}

}  // namespace qg

extern "C" int qpms_gpu_debug_cerfc(double re, double im, double *out) {
  static qg::WeidemanCoeffs w;
  static bool init = false;
  if (!init) {
    qg::weideman_coeffs(&w);
    init = true;
  }
  const qg_c r = qg::cerfc(cmk(re, im), w);
  out[0] = r.re;
  out[1] = r.im;
  return 0;
}
