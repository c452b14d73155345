// Host-side construction of the VSWF translation multiplier tables.
//
// Semantics follow the reference's qpms_trans_calculator_init
// (qpms/translations.c:439-508) with the multiplier formulas of
// qpms_trans_calculator_multipliers_A (:313-368, Xu's (61) with the AN1 phase,
// :29-32) and qpms_trans_calculator_multipliers_B (:382-437, Cruzan form with
// the BN1 phase, :37-40), the normalisation factors of normalisation.h:17-90
// and the index map y = n(n+1)+m-1 of indexing.h:13-27.
//
// Differences in method (not in meaning): the Gaunt coefficients a_q(m,n,mu,nu)
// are obtained by projecting P_n^m P_nu^mu onto P_p^{m+mu} with Gauss-Legendre
// quadrature in long double (the integrand is a polynomial, so the rule is
// exact), instead of Xu's recurrences (gaunt.c); the Wigner 3j symbols of the
// B form come from the Racah sum in long double instead of GSL.  All factor
// products are formed in long double and rounded once.
//
// Structural facts used by the kernel: for every normalisation the A
// multipliers are real and the B multipliers purely imaginary (the phase
// factors i^(n+nu) i^(n-nu) = (-1)^n and i^(p+1) i^(n-nu) = i (-1)^(n-q), and the
// reference stores the normalisation ratio in a double, i.e. its real part).
#include <math.h>
#include <algorithm>
#include <complex>
#include <numeric>

#include "qg_internal.h"

namespace qg {
namespace {

typedef long double ld;

int m1pow(int p) { return (p % 2) ? -1 : 1; }

ld lfact(int n) { return lgammal((ld)n + 1); }

// Gauss-Legendre nodes/weights on [-1, 1] (Newton on P_K), long double.
void gauss_legendre(int K, std::vector<ld> &x, std::vector<ld> &w) {
  x.resize(K);
  w.resize(K);
  const ld pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < K; ++i) {
    ld z = cosl(pi * (i + 0.75L) / (K + 0.5L)), dp = 0;
    for (int it = 0; it < 100; ++it) {
      ld p0 = 1, p1 = z;
      for (int k = 2; k <= K; ++k) {
        ld p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = K * (z * p1 - p0) / (z * z - 1);
      ld dz = p1 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-30L) break;
    }
    ld p0 = 1, p1 = z;
    for (int k = 2; k <= K; ++k) {
      ld p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = K * (z * p1 - p0) / (z * z - 1);
    x[i] = z;
    w[i] = 2 / ((1 - z * z) * dp * dp);
  }
}

// Ferrers P_l^m(x) (Condon-Shortley phase), any integer |m| <= l.
ld ferrers(int l, int m, ld x) {
  int am = m < 0 ? -m : m;
  ld u = sqrtl((1 - x) * (1 + x));
  ld pmm = 1;
  for (int k = 1; k <= am; ++k) pmm *= -(2 * k - 1) * u;
  ld val;
  if (l == am) {
    val = pmm;
  } else {
    ld a = pmm, b = x * (2 * am + 1) * pmm;
    for (int k = am + 2; k <= l; ++k) {
      ld c = ((2 * k - 1) * x * b - (k + am - 1) * a) / (k - am);
      a = b;
      b = c;
    }
    val = b;
  }
  if (m < 0) val *= m1pow(am) * expl(lfact(l - am) - lfact(l + am));
  return val;
}

// Gaunt coefficients of P_n^m P_nu^mu = sum_q a_q P_{n+nu-2q}^{m+mu}.
int gaunt_gl(int m, int n, int mu, int nu, std::vector<ld> &aq) {
  const int M = m + mu;
  const int qmax = std::min(n, std::min(nu, (n + nu - abs(M)) / 2));
  const int K = n + nu + 4;  // degree <= 2(n+nu): exact for K >= n+nu+1
  std::vector<ld> x, w;
  gauss_legendre(K, x, w);
  aq.assign(qmax + 1, 0);
  for (int q = 0; q <= qmax; ++q) {
    const int p = n + nu - 2 * q;
    ld s = 0;
    for (int k = 0; k < K; ++k) s += w[k] * ferrers(n, m, x[k]) * ferrers(nu, mu, x[k]) * ferrers(p, M, x[k]);
    aq[q] = s * (2 * p + 1) / 2 * expl(lfact(p - M) - lfact(p + M));
  }
  return qmax;
}

// Wigner 3j by the Racah sum (long double).
ld wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0;
  if (j3 < abs(j1 - j2) || j3 > j1 + j2) return 0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0;
  ld lpre = 0.5L * (lfact(j1 + j2 - j3) + lfact(j1 - j2 + j3) + lfact(-j1 + j2 + j3) - lfact(j1 + j2 + j3 + 1) +
                    lfact(j1 + m1) + lfact(j1 - m1) + lfact(j2 + m2) + lfact(j2 - m2) + lfact(j3 + m3) +
                    lfact(j3 - m3));
  int kmin = std::max(0, std::max(j2 - j3 - m1, j1 - j3 + m2));
  int kmax = std::min(j1 + j2 - j3, std::min(j1 - m1, j2 + m2));
  ld s = 0;
  for (int k = kmin; k <= kmax; ++k) {
    ld lden = lfact(k) + lfact(j3 - j2 + k + m1) + lfact(j3 - j1 + k - m2) + lfact(j1 + j2 - j3 - k) +
              lfact(j1 - k - m1) + lfact(j2 - k + m2);
    s += (k % 2 ? -1 : 1) * expl(lpre - lden);
  }
  return m1pow(j1 - j2 - m3) * s;
}

// normalisation.h:17-31 and :39-73 (factor_M_noCS / factor_N_noCS)
std::complex<ld> norm_factor(int norm, int l, int m, bool magnetic) {
  ld f;
  switch (norm & QPMS_NORMALISATION_NORM_SPHARM) {  // the two norm bits
    case QPMS_NORMALISATION_NORM_POWER: f = 1; break;
    case QPMS_NORMALISATION_NORM_SPHARM: f = sqrtl((ld)l * (l + 1)); break;
    case QPMS_NORMALISATION_NORM_NONE:
      f = sqrtl((ld)l * (l + 1) * 4 * 3.141592653589793238462643383279502884L / (2 * l + 1)) *
          expl(0.5L * (lfact(l + m) - lfact(l - m)));
      break;
    default: return std::complex<ld>(NAN, NAN);
  }
  std::complex<ld> c(f, 0);
  const int minus = magnetic ? 32 : 128, imag = magnetic ? 16 : 64;
  if (norm & minus) c = -c;
  if (norm & imag) c *= std::complex<ld>(0, 1);
  if (norm & 1) c = ld(1) / c;  // QPMS_NORMALISATION_INVERSE
  return c;
}

// common factor of translations.c:116-133 with the per-type ratio (real part)
ld common_normfac(int norm, int m, int n, int mu, int nu, bool B) {
  const int csphase = (norm & QPMS_NORMALISATION_CSPHASE) ? -1 : 1;
  ld f = (csphase == 1) ? m1pow(m - mu) : 1;
  f *= sqrtl((ld)n * (n + 1) / ((ld)nu * (nu + 1)));
  f *= sqrtl((ld)(2 * n + 1) / (2 * nu + 1));
  std::complex<ld> ratio = norm_factor(norm, nu, mu, B) / norm_factor(norm, n, m, false);
  return f * ratio.real();
}

ld normlogfac(int m, int n, int mu, int nu) {
  return -0.5L * (lfact(n + m) - lfact(n - m) + lfact(nu - mu) - lfact(nu + mu));
}

}  // namespace

bool build_trans_tables(int lMax, int norm, TransHostTables *t) {
  if (lMax < 1 || lMax > kTransLmaxMax) return false;
  if (norm & (2 | 4)) return false;  // real / reversed-phase harmonics: not implemented in the reference either
  switch (norm & QPMS_NORMALISATION_NORM_SPHARM) {
    case QPMS_NORMALISATION_NORM_POWER:
    case QPMS_NORMALISATION_NORM_SPHARM:
    case QPMS_NORMALISATION_NORM_NONE: break;
    default: return false;
  }
  const int ne = lMax * (lMax + 2), ne2 = ne * ne;
  t->lMax = lMax;
  t->nelem = ne;
  t->tq = lMax + 1;
  t->A_off.assign(ne2 + 1, 0);
  t->B_off.assign(ne2 + 1, 0);
  t->A_mult.clear();
  t->B_mult.clear();
  std::vector<std::vector<ld>> cA(ne2), cB(ne2);
  std::vector<std::vector<int>> sA(ne2), sB(ne2);
  std::vector<ld> aq;
  for (int y = 0; y < ne; ++y) {
    const int n = (int)sqrt((double)y + 1), m = y - (n * (n + 1) - 1);
    for (int yu = 0; yu < ne; ++yu) {
      const int nu = (int)sqrt((double)yu + 1), mu = yu - (nu * (nu + 1) - 1);
      const int e = y * ne + yu, d = mu - m;
      // ---- A (translations.c:313-368) ----
      const int qmaxA = gaunt_gl(-m, n, mu, nu, aq);
      {
        const ld nf = common_normfac(norm, m, n, mu, nu, false) * m1pow(m);
        const ld ex = lfact(2 * n) - lfact(n + 1) + lfact(2 * nu + 2) - lfact(nu + 1) + lfact(n + nu + m - mu) -
                      lfact(n - m) - lfact(nu + mu) + lfact(n + nu) - lfact(2 * (n + nu)) + normlogfac(m, n, mu, nu);
        const ld presum = expl(ex) * nf / (4 * n) * m1pow(n);  // i^(n+nu) i^(n-nu) = (-1)^n
        for (int q = 0; q <= qmaxA; ++q) {
          const int p = n + nu - 2 * q;
          const ld ppfac = (d >= 0) ? 1 : m1pow(d) * expl(lfact(p + d) - lfact(p - d));
          const ld sf = (ld)(n * (n + 1) + nu * (nu + 1) - p * (p + 1)) * m1pow(q) * (aq[q] / aq[0]);
          cA[e].push_back(presum * sf * ppfac);
          sA[e].push_back(p * p + p + d);
        }
      }
      // ---- B (translations.c:372-437) ----
      const int qmaxB = std::min(n, std::min(nu, (n + nu + 1 - abs(d)) / 2));
      {
        const ld nf = common_normfac(norm, m, n, mu, nu, true);
        const ld presum = m1pow(1 - m) * (ld)(2 * nu + 1) / (2 * (ld)(n * (n + 1))) *
                          expl(lfact(n + m) - lfact(n - m) + lfact(nu - mu) - lfact(nu + mu) +
                               normlogfac(m, n, mu, nu)) * nf;
        const int Mc = -m;
        for (int q = 0; q <= qmaxB; ++q) {
          const int p = n + nu - 2 * q;
          const ld ppfac = (d >= 0) ? 1 : m1pow(d) * expl(lfact(p + 1 + d) - lfact(p + 1 - d));
          const ld tt = sqrtl((ld)((p + 1) * (p + 1) - (n - nu) * (n - nu)) *
                              (ld)((n + nu + 1) * (n + nu + 1) - (p + 1) * (p + 1)));
          const ld cz = m1pow(mu + Mc) * (2 * p + 3) *
                        expl(0.5L * (lfact(n + Mc) - lfact(n - Mc) + lfact(nu + mu) - lfact(nu - mu) +
                                     lfact(p - Mc - mu + 1) - lfact(p + Mc + mu + 1))) *
                        wigner3j(n, nu, p + 1, Mc, mu, -Mc - mu) * wigner3j(n, nu, p, 0, 0, 0);
          // i^(p+1) i^(n-nu) = i (-1)^(n-q): store the imaginary coefficient
          cB[e].push_back(presum * tt * ppfac * cz * m1pow(n - q));
          sB[e].push_back((p + 1) * (p + 1) + (p + 1) + d);
        }
      }
    }
  }
  // reference-layout ragged tables
  for (int e = 0; e < ne2; ++e) {
    t->A_off[e + 1] = t->A_off[e] + cA[e].size();
    t->B_off[e + 1] = t->B_off[e] + cB[e].size();
    for (ld v : cA[e]) t->A_mult.push_back(cmk((double)v, 0.0));
    for (ld v : cB[e]) t->B_mult.push_back(cmk(0.0, (double)v));
  }
  // kernel order: A and B elements each sorted by their own term count
  // (descending), so the lanes of a warp share trip counts
  t->perm.resize(ne2);
  t->permB.resize(ne2);
  std::iota(t->perm.begin(), t->perm.end(), 0);
  std::iota(t->permB.begin(), t->permB.end(), 0);
  std::stable_sort(t->perm.begin(), t->perm.end(), [&](int a, int b) { return cA[a].size() > cA[b].size(); });
  std::stable_sort(t->permB.begin(), t->permB.end(), [&](int a, int b) { return cB[a].size() > cB[b].size(); });
  const int tq = t->tq;
  t->cntA.assign(ne2, 0);
  t->cntB.assign(ne2, 0);
  t->cntBe.assign(ne2, 0);
  t->coefA.assign((size_t)tq * ne2, 0.0);
  t->coefB.assign((size_t)tq * ne2, 0.0);
  t->slotA.assign((size_t)tq * ne2, 0);
  t->slotB.assign((size_t)tq * ne2, 0);
  for (int k = 0; k < ne2; ++k) {
    const int e = t->perm[k], eb = t->permB[k];
    t->cntA[k] = (uint8_t)cA[e].size();
    t->cntB[k] = (uint8_t)cB[eb].size();
    t->cntBe[k] = (uint8_t)std::min(cB[eb].size(), cA[eb].size());
    for (size_t q = 0; q < cA[e].size(); ++q) {
      t->coefA[q * ne2 + k] = (double)cA[e][q];
      t->slotA[q * ne2 + k] = (uint16_t)sA[e][q];
    }
    for (size_t q = 0; q < cB[eb].size(); ++q) {
      t->coefB[q * ne2 + k] = (double)cB[eb][q];
      t->slotB[q * ne2 + k] = (uint16_t)sB[eb][q];
    }
  }
  return true;
}

}  // namespace qg
