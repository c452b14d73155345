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
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "qg_assembly.h"
#include "qg_ewald.h"
#include "qg_faddeeva.cuh"
#include "qg_internal.h"

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
};

// (n, m) of the k-th even pair, in n-major order
__device__ __forceinline__ void even_nm(int k, int &n, int &m) {
  n = (int)((sqrtf(8.0f * k + 1.0f) - 1.0f) * 0.5f);
  if ((n + 1) * (n + 2) / 2 <= k) ++n;
  if (n * (n + 1) / 2 > k) --n;
  m = -n + 2 * (k - n * (n + 1) / 2);
}

template <int LMAX>
__global__ void __launch_bounds__(kEThreads) ewald_assemble_kernel(EwaldArgs a, TransDevTables T) {
  using Sh = EwShape<LMAX>;
  constexpr int LE = Sh::LE, S = Sh::S, NE = Sh::NE, NE2 = Sh::NE2, NB = Sh::NB, NEV = Sh::NEVEN;
  __shared__ qg_c sig[S];
  __shared__ qg_c red[kEThreads / 32][NEV];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int np = a.np;
  const size_t per = a.npairs ? (size_t)a.npairs : (size_t)np * np;  // blocks per matrix
  const size_t units = (size_t)a.nw * a.nk * per;
  const size_t N = (size_t)np * NB;
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
    const bool self = (sx == 0.0 && sy == 0.0);
    const bool kreal = (k.im == 0.0);
    qg_c acc[NEV];
#pragma unroll
    for (int i = 0; i < NEV; ++i) acc[i] = cmk(0, 0);

    // ---------------- short range (direct lattice) ----------------
    {
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
      for (int t = tid; sr_ok && t < W1 * W2; t += kEThreads) {
        const int i = t / W2 - I1, j = t % W2 - I2;
        if (self && i == 0 && j == 0) continue;
        const double Rx = i * c_ew.b[0] + j * c_ew.b[2] - sx, Ry = i * c_ew.b[1] + j * c_ew.b[3] - sy;
        const double r2 = Rx * Rx + Ry * Ry, r = sqrt(r2);
        if (r * eta > 7.5) continue;
        const double phi = atan2(Ry, Rx);
        // e^{i beta.R} e^{i m phi} handled below
        const qg_c zp = cmk(r * eta + ik2eta.re, ik2eta.im), zm = cmk(r * eta - ik2eta.re, -ik2eta.im);
        const qg_c ekr = cexpi(cscale(k, r)), emkr = cexpi(cscale(k, -r));
        const qg_c Ep = cmul(ekr, cerfc(zp, c_wd)), Em = cmul(emkr, cerfc(zm, c_wd));
        const double sqpi = 1.7724538509055160273;
        qg_c In[LE + 1];
        const qg_c I0 = cscale(cadd(Ep, Em), sqpi / (4 * r));
        // I_{-1} = sqrt(pi)/(2 i k) (Em - Ep)
        const qg_c d = csub(Em, Ep);
        const qg_c Im1 = cscale(cmul(cmk(d.im, -d.re), rk), sqpi / 2);  // (Em-Ep)/(i) = -i (Em-Ep)
        // E = exp(-r^2 eta^2 + k^2 / (4 eta^2))
        const qg_c ex = cmk(-r2 * eta * eta + (k.re * k.re - k.im * k.im) / (4 * eta * eta),
                            2 * k.re * k.im / (4 * eta * eta));
        const qg_c E = cexpi(cmk(ex.im, -ex.re));
        In[0] = I0;
        qg_c pm2 = Im1, pm1 = I0;
        double etap = eta;  // eta^(2n-1)
        const double inv2r2 = 1.0 / (2 * r2);
#pragma unroll
        for (int n = 1; n <= LE; ++n) {
          const qg_c v = cscale(cadd(csub(cscale(pm1, 2 * n - 1), cmul(k2h, pm2)), cscale(E, etap)), inv2r2);
          In[n] = v;
          pm2 = pm1;
          pm1 = v;
          etap *= eta * eta;
        }
        double sb, cb;
        sincos(bx * Rx + by * Ry, &sb, &cb);
        const qg_c ebeta = cmk(cb, sb);
        double s1, c1;
        sincos(phi, &s1, &c1);
        const qg_c e1 = cmk(c1, s1);
        // prefac_n r^n I_n e^{i beta R}: prefac_n = -i (2/k)^{n+1} / sqrt(pi)
        qg_c pf = cscale(cmul(cmk(0.0, -1.0), cscale(rk, 2.0)), 1.0 / sqpi);  // -i (2/k) / sqrt(pi)
        const qg_c twok = cscale(rk, 2.0);
        double rn = 1.0;
#pragma unroll
        for (int n = 0; n <= LE; ++n) {
          const qg_c base = cmul(cmul(cscale(pf, rn), In[n]), ebeta);
          // m = -n, -n+2, ..., n: e^{i m phi}
          qg_c em = cmk(1, 0);
          for (int q = 0; q < n; ++q) em = cmul(em, cconj(e1));  // e^{-i n phi}
          const qg_c e2 = cmul(e1, e1);
#pragma unroll
          for (int q = 0; q <= n; ++q) {
            const int m = -n + 2 * q;
            const int kk = n * (n + 1) / 2 + q;
            acc[kk] = cadd(acc[kk], cscale(cmul(base, em), c_ew.leg0m[n * (n + 1) + m]));
            em = cmul(em, e2);
          }
          pf = cmul(pf, twok);
          rn *= r;
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
      for (int t = tid; lr_ok && t < W1 * W2; t += kEThreads) {
        const int i = t / W2 - I1, j = t % W2 - I2;
        const double Kx = i * c_ew.rb[0] + j * c_ew.rb[2], Ky = i * c_ew.rb[1] + j * c_ew.rb[3];
        const double qx = Kx + bx, qy = Ky + by;
        const double rb = sqrt(qx * qx + qy * qy);
        qg_c gam, uu;
        if (kreal) {
          // clilgamma(rb / k) (ewald.h:157-170) for real k: sqrt(t - 1) sqrt(t + 1)
          // with t - 1 exact; near a Rayleigh anomaly (t -> 1) the 1/gamma terms
          // dominate, so gamma is formed from the exact differences as there
          const double tt = rb / k.re;
          if (tt >= 1.0) {
            gam = cmk(sqrt(tt - 1.0) * sqrt(tt + 1.0), 0.0);
            const double x = gam.re * k.re / (2 * eta);
            if (x * x > 56.0) continue;
            uu = cmk(x, 0.0);
          } else {
            const double g = sqrt(1.0 - tt) * sqrt(1.0 + tt);
            gam = cmk(0.0, -g);  // -i sqrt(1 - t^2)
            // x^2 = -(g k / 2 eta)^2, approached from below the negative axis: sqrt -> -i c
            uu = cmk(0.0, -g * k.re / (2 * eta));
          }
        } else {
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
          if (x2.re > 56.0) continue;
          uu = csqrt_(x2);
          if (x2.re < 0 && !signbit(x2.im)) uu = cscale(uu, -1.0);  // branch m = -1 (ewald.c:390-393)
        }
        qg_c G[LE / 2 + 1];
        gamma_half_down(uu, LE / 2, G);
        double sK, cK;
        sincos(Kx * sx + Ky * sy, &sK, &cK);
        const qg_c phasefac = cmul(cmk(cK, sK), lrfac);  // e^{i K.s} / (k^2 A)
        const double alpha = atan2(qy, qx);
        double s1, c1;
        sincos(alpha, &s1, &c1);
        const qg_c e1 = cmk(c1, s1), e2 = cmul(e1, e1);
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
#pragma unroll
        for (int n = 0; n <= LE; ++n) {
          qg_c em = cmk(1, 0);
          for (int q = 0; q < n; ++q) em = cmul(em, cconj(e1));
#pragma unroll
          for (int q = 0; q <= n; ++q) {
            const int m = -n + 2 * q;
            const int y = n * (n + 1) + m;
            const int jmax = (n - (m < 0 ? -m : m)) / 2;
            qg_c js = cmk(0, 0);
            for (int j = 0; j <= jmax; ++j)
              js = cadd(js, cmul(cmul(tpow[n - 2 * j], gp[j]), c_ew.s1[c_ew.s1off[y] + j]));
            const int kk = n * (n + 1) / 2 + q;
            acc[kk] = cadd(acc[kk], cmul(cmul(js, em), phasefac));
            em = cmul(em, e2);
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
    // ---------------- contraction into the M block ----------------
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
}

template <int LMAX>
int launch_ew(const EwaldArgs &a, const TransDevTables &T, cudaStream_t st) {
  const size_t units = (size_t)a.nw * a.nk * (a.npairs ? (size_t)a.npairs : (size_t)a.np * a.np);
  if (!units) return QPMS_SUCCESS;
  int dev = 0, nsm = 0;
  QG_CUDA_TRY(cudaGetDevice(&dev));
  QG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  size_t grid = std::min<size_t>(units, (size_t)nsm * 16);
  ewald_assemble_kernel<LMAX><<<(unsigned)grid, kEThreads, 0, st>>>(a, T);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
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
