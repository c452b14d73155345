// Host dense complex linear algebra for the Beyn post-processing (see qg_hostla.h).
// Textbook algorithms (Golub & Van Loan, "Matrix Computations", 4th ed.:
// Householder QR 5.2, one-sided Jacobi SVD 8.6.3, Hessenberg reduction 7.4.3,
// shifted QR 7.5, eigenvectors of the Schur form 7.6.4), written for the
// sizes Beyn needs (L up to a few hundred); parallel over columns with OpenMP
// where the work is O(m L^2).
#include <math.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <numeric>
#include <vector>

#include "qg_hostla.h"

namespace qg {
namespace hostla {

namespace {
inline double abs1(cd z) { return fabs(z.real()) + fabs(z.imag()); }
inline cd phase(cd z) {
  const double a = std::abs(z);
  return a > 0 ? z / a : cd(1, 0);
}
}  // namespace

int svd_thin(int m, int n, const cd *A, int lda, cd *U, double *s, cd *V) {
  // ---- Householder QR: W = A, reflectors stored in W below the diagonal ----
  std::vector<cd> W((size_t)m * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) W[i + (size_t)j * m] = A[i + (size_t)j * lda];
  std::vector<double> beta(n, 0.0);
  std::vector<cd> alpha(n);
  for (int j = 0; j < n; ++j) {
    cd *x = &W[j + (size_t)j * m];
    const int len = m - j;
    double nx = 0;
    for (int i = 0; i < len; ++i) nx += std::norm(x[i]);
    nx = sqrt(nx);
    if (nx == 0) {
      alpha[j] = 0;
      beta[j] = 0;
      continue;
    }
    const cd a = -phase(x[0]) * nx;
    x[0] -= a;  // v = x - a e1, kept in place
    double vn = 0;
    for (int i = 0; i < len; ++i) vn += std::norm(x[i]);
    beta[j] = vn > 0 ? 2.0 / vn : 0.0;
    alpha[j] = a;
#pragma omp parallel for schedule(static) if ((size_t)len * (n - j) > 32768)
    for (int k = j + 1; k < n; ++k) {
      cd *y = &W[j + (size_t)k * m];
      cd d = 0;
      for (int i = 0; i < len; ++i) d += std::conj(x[i]) * y[i];
      d *= beta[j];
      for (int i = 0; i < len; ++i) y[i] -= d * x[i];
    }
  }
  // R (n x n, upper) -> G, the matrix the Jacobi sweeps orthogonalise
  std::vector<cd> G((size_t)n * n, cd(0, 0));
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < j; ++i) G[i + (size_t)j * n] = W[i + (size_t)j * m];
    G[j + (size_t)j * n] = alpha[j];
  }
  // Q (m x n) = H_0 ... H_{n-1} [I; 0]
  std::vector<cd> Q((size_t)m * n, cd(0, 0));
  for (int j = 0; j < n; ++j) Q[j + (size_t)j * m] = 1;
  for (int j = n - 1; j >= 0; --j) {
    if (beta[j] == 0) continue;
    const cd *v = &W[j + (size_t)j * m];
    const int len = m - j;
#pragma omp parallel for schedule(static) if ((size_t)len * n > 32768)
    for (int k = 0; k < n; ++k) {
      cd *y = &Q[j + (size_t)k * m];
      cd d = 0;
      for (int i = 0; i < len; ++i) d += std::conj(v[i]) * y[i];
      d *= beta[j];
      for (int i = 0; i < len; ++i) y[i] -= d * v[i];
    }
  }
  // ---- one-sided Jacobi on G: G J_1 J_2 ... -> columns mutually orthogonal ----
  std::vector<cd> Vm((size_t)n * n, cd(0, 0));
  for (int j = 0; j < n; ++j) Vm[j + (size_t)j * n] = 1;
  const double tol = 4 * DBL_EPSILON;
  bool converged = false;
  for (int sweep = 0; sweep < 80 && !converged; ++sweep) {
    converged = true;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        cd *gp = &G[(size_t)p * n], *gq = &G[(size_t)q * n];
        double a = 0, b = 0;
        cd g = 0;
        for (int i = 0; i < n; ++i) {
          a += std::norm(gp[i]);
          b += std::norm(gq[i]);
          g += std::conj(gp[i]) * gq[i];
        }
        const double ag = std::abs(g);
        if (ag == 0 || ag <= tol * sqrt(a * b)) continue;
        converged = false;
        // D = diag(1, e^{-i phi}) makes the 2x2 Gram matrix real; then the
        // symmetric Schur rotation [c s; -s c] diagonalises it.
        const cd eph = std::conj(g) / ag;  // e^{-i phi}
        const double tau = (b - a) / (2 * ag);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1 + tau * tau));
        const double c = 1 / sqrt(1 + t * t), sn = c * t;
        for (int i = 0; i < n; ++i) {
          const cd x = gp[i], y = eph * gq[i];
          gp[i] = c * x - sn * y;
          gq[i] = sn * x + c * y;
        }
        cd *vp = &Vm[(size_t)p * n], *vq = &Vm[(size_t)q * n];
        for (int i = 0; i < n; ++i) {
          const cd x = vp[i], y = eph * vq[i];
          vp[i] = c * x - sn * y;
          vq[i] = sn * x + c * y;
        }
      }
  }
  // singular values, sorted descending
  std::vector<double> sv(n);
  for (int j = 0; j < n; ++j) {
    double a = 0;
    for (int i = 0; i < n; ++i) a += std::norm(G[i + (size_t)j * n]);
    sv[j] = sqrt(a);
  }
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return sv[x] > sv[y]; });
  // U = Q (G_j / s_j), V columns permuted alike
  std::vector<cd> UR((size_t)n * n);
  for (int jj = 0; jj < n; ++jj) {
    const int j = ord[jj];
    s[jj] = sv[j];
    for (int i = 0; i < n; ++i) {
      UR[i + (size_t)jj * n] = sv[j] > 0 ? G[i + (size_t)j * n] / sv[j] : cd(i == jj ? 1 : 0, 0);
      V[i + (size_t)jj * n] = Vm[i + (size_t)j * n];
    }
  }
#pragma omp parallel for schedule(static) if ((size_t)m * n * n > 65536)
  for (int jj = 0; jj < n; ++jj)
    for (int i = 0; i < m; ++i) {
      cd acc = 0;
      for (int k = 0; k < n; ++k) acc += Q[i + (size_t)k * m] * UR[k + (size_t)jj * n];
      U[i + (size_t)jj * m] = acc;
    }
  return converged ? 0 : -1;
}

int eig(int n, const cd *A, int lda, cd *w, cd *X) {
  if (n <= 0) return 0;
  std::vector<cd> H((size_t)n * n), Z((size_t)n * n, cd(0, 0));
  auto h = [&](int i, int j) -> cd & { return H[i + (size_t)j * n]; };
  auto z = [&](int i, int j) -> cd & { return Z[i + (size_t)j * n]; };
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) h(i, j) = A[i + (size_t)j * lda];
    z(j, j) = 1;
  }
  // ---- Hessenberg reduction H = P^H A P, Z = P ----
  std::vector<cd> v(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int len = n - k - 1;
    double nx = 0;
    for (int i = 0; i < len; ++i) nx += std::norm(h(k + 1 + i, k));
    nx = sqrt(nx);
    if (nx == 0) continue;
    const cd a = -phase(h(k + 1, k)) * nx;
    for (int i = 0; i < len; ++i) v[i] = h(k + 1 + i, k);
    v[0] -= a;
    double vn = 0;
    for (int i = 0; i < len; ++i) vn += std::norm(v[i]);
    if (vn == 0) continue;
    const double bt = 2.0 / vn;
    for (int j = k; j < n; ++j) {  // left: (I - bt v v^H) H
      cd d = 0;
      for (int i = 0; i < len; ++i) d += std::conj(v[i]) * h(k + 1 + i, j);
      d *= bt;
      for (int i = 0; i < len; ++i) h(k + 1 + i, j) -= d * v[i];
    }
    for (int i = 0; i < n; ++i) {  // right: H (I - bt v v^H), Z likewise
      cd d = 0, e = 0;
      for (int jj = 0; jj < len; ++jj) {
        d += h(i, k + 1 + jj) * v[jj];
        e += z(i, k + 1 + jj) * v[jj];
      }
      d *= bt;
      e *= bt;
      for (int jj = 0; jj < len; ++jj) {
        h(i, k + 1 + jj) -= d * std::conj(v[jj]);
        z(i, k + 1 + jj) -= e * std::conj(v[jj]);
      }
    }
    h(k + 1, k) = a;
    for (int i = k + 2; i < n; ++i) h(i, k) = 0;
  }
  // ---- single-shift complex QR to the Schur form T, Z accumulates ----
  const double eps = DBL_EPSILON, small = DBL_MIN * n / DBL_EPSILON;
  int ihi = n - 1, iter = 0, total = 0;
  while (ihi > 0) {
    if (++total > 60 * n + 100) return -1;
    int l = ihi;
    for (; l > 0; --l) {
      const double tst = abs1(h(l - 1, l - 1)) + abs1(h(l, l));
      if (abs1(h(l, l - 1)) <= eps * tst || abs1(h(l, l - 1)) <= small) {
        h(l, l - 1) = 0;
        break;
      }
    }
    if (l == ihi) {  // 1 x 1 block deflated
      --ihi;
      iter = 0;
      continue;
    }
    ++iter;
    cd mu;
    if (iter % 10 == 0) {  // exceptional shift
      mu = h(ihi, ihi) + 0.75 * std::abs(h(ihi, ihi - 1));
    } else {  // Wilkinson: eigenvalue of the trailing 2 x 2 nearer h(ihi, ihi)
      const cd a = h(ihi - 1, ihi - 1), b = h(ihi - 1, ihi), c = h(ihi, ihi - 1), d = h(ihi, ihi);
      const cd hm = 0.5 * (a + d), hd = 0.5 * (a - d);
      const cd disc = std::sqrt(hd * hd + b * c);
      const cd m1 = hm + disc, m2 = hm - disc;
      mu = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
    }
    cd x = h(l, l) - mu, y = h(l + 1, l);
    for (int k = l; k < ihi; ++k) {
      // Givens [c s; -conj(s) c] with c real taking (x, y) to (r, 0)
      double c;
      cd s;
      const double ax = std::abs(x), ay = std::abs(y);
      if (ay == 0) {
        c = 1;
        s = 0;
      } else if (ax == 0) {
        c = 0;
        s = std::conj(y) / ay;
      } else {
        const double r = hypot(ax, ay);
        c = ax / r;
        s = (x / ax) * std::conj(y) / r;
      }
      for (int j = (k == l ? l : k - 1); j < n; ++j) {
        const cd h1 = h(k, j), h2 = h(k + 1, j);
        h(k, j) = c * h1 + s * h2;
        h(k + 1, j) = -std::conj(s) * h1 + c * h2;
      }
      const int imax = std::min(k + 2, ihi);
      for (int i = 0; i <= imax; ++i) {
        const cd h1 = h(i, k), h2 = h(i, k + 1);
        h(i, k) = c * h1 + std::conj(s) * h2;
        h(i, k + 1) = -s * h1 + c * h2;
      }
      for (int i = 0; i < n; ++i) {
        const cd z1 = z(i, k), z2 = z(i, k + 1);
        z(i, k) = c * z1 + std::conj(s) * z2;
        z(i, k + 1) = -s * z1 + c * z2;
      }
      if (k + 1 < ihi) {
        x = h(k + 1, k);
        y = h(k + 2, k);
      }
    }
  }
  // ---- eigenvalues and eigenvectors of T, back-transformed by Z ----
  for (int k = 0; k < n; ++k) w[k] = h(k, k);
  std::vector<cd> yv(n);
  for (int k = 0; k < n; ++k) {
    const cd lam = h(k, k);
    const double smin = std::max(eps * abs1(lam), DBL_MIN / eps);
    std::fill(yv.begin(), yv.end(), cd(0, 0));
    yv[k] = 1;
    for (int i = k - 1; i >= 0; --i) {
      cd acc = 0;
      for (int j = i + 1; j <= k; ++j) acc += h(i, j) * yv[j];
      cd d = h(i, i) - lam;
      if (abs1(d) < smin) d = smin;
      yv[i] = -acc / d;
    }
    double nrm = 0, best = -1;
    int ib = 0;
    for (int i = 0; i < n; ++i) {
      cd acc = 0;
      for (int j = 0; j <= k; ++j) acc += z(i, j) * yv[j];
      X[i + (size_t)k * n] = acc;
      const double a2 = std::norm(acc);
      nrm += a2;
      if (a2 > best) {
        best = a2;
        ib = i;
      }
    }
    // unit 2-norm, largest component real (zgeev's normalisation)
    const cd sc = std::conj(X[ib + (size_t)k * n]) / (sqrt(best) * sqrt(nrm));
    for (int i = 0; i < n; ++i) X[i + (size_t)k * n] *= sc;
    X[ib + (size_t)k * n] = cd(X[ib + (size_t)k * n].real(), 0);
  }
  return 0;
}

void probe_matrix(size_t m, size_t l, unsigned long long seed, cd *out) {
  uint64_t st = seed;
  auto next = [&]() {  // splitmix64
    uint64_t zz = (st += 0x9e3779b97f4a7c15ULL);
    zz = (zz ^ (zz >> 30)) * 0xbf58476d1ce4e5b9ULL;
    zz = (zz ^ (zz >> 27)) * 0x94d049bb133111ebULL;
    return zz ^ (zz >> 31);
  };
  auto unif = [&]() { return ((next() >> 11) + 1) * (1.0 / 9007199254740992.0); };  // (0, 1]
  auto gauss = [&]() { return sqrt(-2 * log(unif())) * cos(2 * M_PI * unif()); };  // Box-Muller
  for (size_t i = 0; i < m * l; ++i) {
    const double re = gauss();
    out[i] = cd(re, gauss());
  }
}

}  // namespace hostla
}  // namespace qg
