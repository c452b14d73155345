// T-matrices of axially symmetric particles (cylinders, spheroids, any
// surface r(theta) with C_inf symmetry) by the extended-boundary-condition
// method on sm_103a: the reference's qpms_tmatrix_axialsym_fill and its
// relatives (tmatrices.c:615-976, tmatrices.h:415-523).
//
// For every m the outside waves (t, l, m) and the inside regular waves
// (t', l', -m) couple through the surface integrals
//   Q, R [(t,l), (t',l')] = int_0^pi jac (z/z_in n.(y_t x v_t'bar) + n.(y_tbar x v_t')) dtheta,
// y the outgoing (Q) or regular (R) wave at k r(theta), v the regular wave at
// k_in r(theta), n = (cos beta, sin beta, 0) in (r, theta, phi), jac =
// r^2 sin(theta) / cos(beta) (tmatrices.c:659-696), and T = -R Q^-1 per m
// block (tmatrices.c:864-884), trimmed from lMax_extend to the bspec.
//
// GPU design: the radial factors (spherical Bessel/Hankel recurrences of
// qg_specfunc.cuh) are formed once per (frequency, node) and the angular ones
// (normalised Legendre recurrences) once per (|m|, node), by two small
// kernels.  Then one CTA per (frequency, m): quadrature nodes (composite
// Gauss-Legendre on panels that break at the kinks of the surface, e.g. the
// cylinder's rims) are staged kAxChunk at a time, all threads forming the
// weighted n x y of the outside waves and the inside waves v in shared
// memory; since n . (y x v) = (n x y) . v, every Q / R entry is then a
// combination of dot products of those staged vectors (3 complex FMAs per
// entry and node, accumulated in FP64 registers; GB300's FP64 pipe is the
// bound).  The m block (at most 24 x 24) is solved in shared memory by
// Gauss-Jordan elimination with partial pivoting (Q^T X = R^T, X = -T^T).  The reference
// integrates each entry separately by adaptive quadrature (GSL qag, epsrel
// 1e-5); the fixed rule here is the same integral to double precision on
// smooth panels.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <complex>
#include <vector>

#include "qg_internal.h"
#include "qg_specfunc.cuh"

namespace qg {

qg_c uvswfi_norm_factor(int norm, qpms_uvswfi_t ui);  // qg_interp.cu

namespace {

constexpr int kAxThreads = 128;
constexpr int kAxChunk = 16;     // quadrature nodes staged per pass
constexpr int kAxMaxL = 12;      // largest lMax_extend
constexpr int kAxPerThread = 9;  // Q and R entries per thread: 2 * 24^2 / 128
constexpr int kAxGauss = 32;     // Gauss-Legendre nodes per panel
constexpr double kC0 = 299792458.0;  // materials.h:11

struct AxDev {
  int L, nw, nq;
  const double *nodes;       // [nq][5]: theta, weight * jac, r, cos beta, sin beta
  const qg_c *k, *kin, *zr;  // [nw]
  const qg_c *rad;           // [nw][nq][3 sets][L][3]: z_l, z_l / x, z_(l-1) - l z_l / x (l = 1..L)
  const double *ang;         // [L + 1 (mu)][nq][L][3]: leg, pi, tau at +mu (l = 1..L)
  qg_c *T;                   // [nw][nQ][nQ], default normalisation, m blocks only
  qg_c *Q, *R;               // optional, same layout (inside wave (t', l', -m) at the column of (t', l', m))
  int *err;                  // 1: a singular Q block
  int zsym;                  // 1: surface symmetric under z -> -z; nodes cover theta in [0, pi/2] (weights x2)
};

// Radial factors per (frequency, node): set 0 h+(k r), set 1 j(k r), set 2 j(k_in r).
template <int LQ>
__global__ void axsym_radial_kernel(AxDev a, qg_c *rad) {
  const int L = a.L;
  const size_t tot = (size_t)a.nw * a.nq * 3;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < tot; x += (size_t)gridDim.x * blockDim.x) {
    const int set = (int)(x % 3);
    const size_t wq = x / 3;
    const int q = (int)(wq % a.nq), w = (int)(wq / a.nq);
    const double r = a.nodes[5 * (size_t)q + 2];
    const qg_c xx = cscale(set == 2 ? a.kin[w] : a.k[w], r);
    qg_c z[LQ + 1];
    sph_bessel<LQ>(set == 0 ? 3 : 1, xx, z);
    const qg_c rx = crecip(xx);
    qg_c *o = rad + (wq * 3 + set) * (size_t)L * 3;
    for (int l = 1; l <= L; ++l) {
      const qg_c bf = cmul(z[l], rx);
      o[(l - 1) * 3] = z[l];
      o[(l - 1) * 3 + 1] = bf;
      o[(l - 1) * 3 + 2] = csub(z[l - 1], cscale(bf, (double)l));
    }
  }
}

// Angular factors per (mu, node): normalised Legendre (Condon-Shortley
// phase) leg = P / sqrt(l(l+1)), pi = mu leg / sin, tau = dP/dtheta / sqrt(l(l+1)).
__global__ void axsym_angular_kernel(int L, int nq, const double *__restrict__ nodes, double *__restrict__ ang) {
  const size_t tot = (size_t)(L + 1) * nq;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < tot; x += (size_t)gridDim.x * blockDim.x) {
    const int q = (int)(x % nq), mu = (int)(x / nq);
    double st, ct;
    sincos(nodes[5 * (size_t)q], &st, &ct);
    double *o = ang + x * (size_t)L * 3;
    double pmm = 0.28209479177387814347;  // 1 / sqrt(4 pi)
    for (int j = 1; j <= mu; ++j) pmm *= -sqrt((2.0 * j - 1) / (2.0 * j)) * st;
    pmm *= sqrt(2.0 * mu + 1);
    for (int l = 1; l < mu && l <= L; ++l) o[(l - 1) * 3] = o[(l - 1) * 3 + 1] = o[(l - 1) * 3 + 2] = 0.0;
    double p2 = 0.0, p1 = 0.0;
    for (int l = mu; l <= L; ++l) {
      double P;
      if (l == mu) {
        P = pmm;
      } else {
        const double al = sqrt((4.0 * l * l - 1) / ((double)l * l - (double)mu * mu));
        const double bl = sqrt(((l - 1.0) * (l - 1.0) - (double)mu * mu) / (4.0 * (l - 1.0) * (l - 1.0) - 1));
        P = al * (ct * p1 - bl * p2);
      }
      if (l >= 1) {
        const double rl = 1.0 / sqrt((double)l * (l + 1));
        o[(l - 1) * 3] = P * rl;
        o[(l - 1) * 3 + 1] = mu / st * P * rl;
        o[(l - 1) * 3 + 2] =
            (l * ct * P - sqrt((2.0 * l + 1) * ((double)l * l - (double)mu * mu) / (2.0 * l - 1)) * p1) / st * rl;
      }
      p2 = p1;
      p1 = P;
    }
  }
}

// The e-th formed entry of D: set qr (0 Q, 1 R), row (t, l), column (t2, l2)
// (l, l2 indices from l0).  With z-mirror symmetry only the entries with
// l + l2 + [t == t2] even are formed (the others integrate to zero): each row
// has nl of them, first t2 = t with l2 of the other parity, then t2 != t with
// l2 of the same parity.
__device__ __forceinline__ void d_entry(int e, int nb, int nl, int nb2, int zsym, int &qr, int &t, int &l, int &t2,
                                        int &l2) {
  if (!zsym) {
    qr = e / nb2;
    const int rem = e - qr * nb2, i = rem / nb, j = rem - i * nb;
    t = i / nl;
    l = i - t * nl;
    t2 = j / nl;
    l2 = j - t2 * nl;
    return;
  }
  const int per = nb * nl;
  qr = e / per;
  const int rem = e - qr * per, i = rem / nl, kk = rem - i * nl;
  t = i / nl;
  l = i - t * nl;
  const int p1 = (l + 1) & 1;               // parity of l2 when t2 == t
  const int c1 = p1 ? nl / 2 : (nl + 1) / 2;  // number of l2 in [0, nl) with that parity
  if (kk < c1) {
    t2 = t;
    l2 = 2 * kk + p1;
  } else {
    t2 = 1 - t;
    l2 = 2 * (kk - c1) + (l & 1);
  }
}

// One CTA per (frequency, m).  Staging: per node and l, the weighted
// n x y of the outgoing (Q) and regular (R) outside waves of both types,
// w = weight (n_theta y_phi, -n_r y_phi, n_r y_theta - n_theta y_r), and the
// inside regular waves v, since n . (y x v) = (n x y) . v.  Accumulation: the
// dot products D[(t,l),(s,l')] = sum_q w_(t,l) . v_(s,l') (3 complex FMAs per
// entry and node); then Q[(t,l),(t',l')] = z/z_in D[(t,l),(t'bar,l')] + D[(tbar,l),(t',l')].
template <int LQ>
__global__ void __launch_bounds__(kAxThreads) axsym_kernel(AxDev a) {
  extern __shared__ qg_c sh[];
  __shared__ double nd[kAxChunk][3];
  __shared__ int piv_s;
  __shared__ qg_c inv_s;
  __shared__ qg_c fac[2 * LQ];
  const int L = a.L;
  const int m = (int)blockIdx.x - L, iw = blockIdx.y;
  const int mu = m < 0 ? -m : m;
  const int l0 = mu > 1 ? mu : 1, nl = L - l0 + 1, nb = 2 * nl, nb2 = nb * nb, tot = 2 * nb2;
  const int ntd = a.zsym ? tot / 2 : tot;  // D entries formed (z-mirror: nl of each row's nb)
  const int tid = threadIdx.x;
  const qg_c zr = a.zr[iw];
  const double sgn_mu = (mu & 1) ? -1.0 : 1.0;
  // (leg, pi, tau) at -mu = (s leg, -s pi, s tau), s = (-1)^mu
  const double fo_l = m >= 0 ? 1.0 : sgn_mu, fo_p = m >= 0 ? 1.0 : -sgn_mu;  // outside waves at m
  const double fi_l = m >= 0 ? sgn_mu : 1.0, fi_p = m >= 0 ? -sgn_mu : 1.0;  // inside waves at -m
  qg_c acc[kAxPerThread];
#pragma unroll
  for (int s = 0; s < kAxPerThread; ++s) acc[s] = cmk(0, 0);
  const qg_c *radw = a.rad + (size_t)iw * a.nq * 3 * L * 3;
  const double *angm = a.ang + (size_t)mu * a.nq * L * 3;

  for (int q0 = 0; q0 < a.nq; q0 += kAxChunk) {
    const int cnt = min(kAxChunk, a.nq - q0);
    __syncthreads();
    if (tid < cnt) {
      const double *ndq = a.nodes + 5 * (size_t)(q0 + tid);
      nd[tid][0] = ndq[1];
      nd[tid][1] = ndq[3];
      nd[tid][2] = ndq[4];
    }
    __syncthreads();
    // ---- staging: items (node, l, set) ----
    for (int it = tid; it < cnt * nl * 3; it += kAxThreads) {
      const int set = it % 3, ql = it / 3, li = ql % nl, q = ql / nl;
      const int l = l0 + li, qg = q0 + q;
      const double *an = angm + ((size_t)qg * L + (l - 1)) * 3;
      const qg_c *rd = radw + (((size_t)qg * 3 + set) * L + (l - 1)) * 3;
      const double fl = set == 2 ? fi_l : fo_l, fp = set == 2 ? fi_p : fo_p;
      const double Lg = an[0] * fl, Pi = an[1] * fp, Ta = an[2] * fl;
      const qg_c z = rd[0], bf = rd[1], bd = rd[2];
      // N = (l(l+1) leg z/x, tau besder, i pi besder), M = (0, i pi z, -tau z)
      const qg_c N0 = cscale(bf, l * (l + 1.0) * Lg), N1 = cscale(bd, Ta), N2 = cmk(-bd.im * Pi, bd.re * Pi);
      const qg_c M1 = cmk(-z.im * Pi, z.re * Pi), M2 = cscale(z, -Ta);
      qg_c *o = sh + ((size_t)q * nl + li) * 18 + set * 6;
      if (set == 2) {
        o[0] = N0;
        o[1] = N1;
        o[2] = N2;
        o[3] = cmk(0, 0);
        o[4] = M1;
        o[5] = M2;
      } else {
        const double wq = nd[q][0], nr = nd[q][1] * wq, nt = nd[q][2] * wq;
        // weight (n x y): (nt y_phi, -nr y_phi, nr y_theta - nt y_r)
        o[0] = cscale(N2, nt);
        o[1] = cscale(N2, -nr);
        o[2] = csub(cscale(N1, nr), cscale(N0, nt));
        o[3] = cscale(M2, nt);
        o[4] = cscale(M2, -nr);
        o[5] = cscale(M1, nr);
      }
    }
    __syncthreads();
    // ---- D entries of this thread over the staged nodes ----
#pragma unroll
    for (int s = 0; s < kAxPerThread; ++s) {
      const int e = tid + s * kAxThreads;
      if (e >= ntd) break;
      int qr, t, l, t2, l2;
      d_entry(e, nb, nl, nb2, a.zsym, qr, t, l, t2, l2);
      double sr = acc[s].re, si = acc[s].im;
      for (int q = 0; q < cnt; ++q) {
        const qg_c *W = sh + ((size_t)q * nl + l) * 18 + qr * 6 + 3 * t;
        const qg_c *V = sh + ((size_t)q * nl + l2) * 18 + 12 + 3 * t2;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const qg_c w = W[c], v = V[c];
          sr = fma(w.re, v.re, sr);
          sr = fma(-w.im, v.im, sr);
          si = fma(w.re, v.im, si);
          si = fma(w.im, v.re, si);
        }
      }
      acc[s] = cmk(sr, si);
    }
  }
  __syncthreads();
  // ---- D into shared memory, then A = Q^T, B = R^T (optional global Q, R) ----
  qg_c *D = sh, *A = sh + 2 * nb2, *B = A + nb2;
  if (a.zsym)
    for (int e = tid; e < tot; e += kAxThreads) D[e] = cmk(0, 0);
  __syncthreads();
#pragma unroll
  for (int s = 0; s < kAxPerThread; ++s) {
    const int e = tid + s * kAxThreads;
    if (e >= ntd) break;
    int qr, t, l, t2, l2;
    d_entry(e, nb, nl, nb2, a.zsym, qr, t, l, t2, l2);
    D[qr * nb2 + (t * nl + l) * nb + t2 * nl + l2] = acc[s];
  }
  __syncthreads();
  const int neQ = L * (L + 2), nQ = 2 * neQ;
  for (int e = tid; e < tot; e += kAxThreads) {
    const int qr = e / nb2, rem = e - qr * nb2;
    const int i = rem / nb, j = rem - i * nb;
    const int t = i / nl, li = i - t * nl, t2 = j / nl, lj = j - t2 * nl;
    const qg_c *Dq = D + qr * nb2;
    const qg_c v1 = Dq[(t * nl + li) * nb + (1 - t2) * nl + lj];
    const qg_c v2 = Dq[((1 - t) * nl + li) * nb + t2 * nl + lj];
    const qg_c val = cadd(cmul(zr, v1), v2);
    (qr ? B : A)[j * nb + i] = val;
    qg_c *G = qr ? a.R : a.Q;
    if (G) {
      const int l = l0 + li, l2 = l0 + lj;
      const size_t gi = (size_t)t * neQ + l * (l + 1) + m - 1, gj = (size_t)t2 * neQ + l2 * (l2 + 1) + m - 1;
      G[((size_t)iw * nQ + gi) * nQ + gj] = val;
    }
  }
  __syncthreads();
  // ---- Gauss-Jordan with partial pivoting: A X = B ----
  bool singular = false;
  for (int c = 0; c < nb; ++c) {
    if (tid < 32) {
      double best = -1.0;
      int bi = c;
      for (int rr = c + tid; rr < nb; rr += 32) {
        const double v = fabs(A[rr * nb + c].re) + fabs(A[rr * nb + c].im);
        if (v > best) {
          best = v;
          bi = rr;
        }
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (tid == 0) piv_s = bi;
    }
    __syncthreads();
    const int p = piv_s;
    if (p != c)
      for (int x = tid; x < 2 * nb; x += kAxThreads) {
        qg_c *M = x < nb ? A : B;
        const int col = x < nb ? x : x - nb;
        const qg_c tmp = M[c * nb + col];
        M[c * nb + col] = M[p * nb + col];
        M[p * nb + col] = tmp;
      }
    __syncthreads();
    if (tid == 0) {
      const qg_c d = A[c * nb + c];
      if (d.re == 0.0 && d.im == 0.0) {
        inv_s = cmk(0, 0);
        atomicOr(a.err, 1);
      } else {
        inv_s = crecip(d);
      }
    }
    __syncthreads();
    if (inv_s.re == 0.0 && inv_s.im == 0.0) singular = true;
    for (int x = tid; x < 2 * nb; x += kAxThreads) {
      qg_c *M = x < nb ? A : B;
      const int col = x < nb ? x : x - nb;
      M[c * nb + col] = cmul(M[c * nb + col], inv_s);
    }
    __syncthreads();
    if (tid < nb) fac[tid] = tid == c ? cmk(0, 0) : A[tid * nb + c];
    __syncthreads();
    for (int x = tid; x < nb * 2 * nb; x += kAxThreads) {
      const int rr = x / (2 * nb), cc = x - rr * 2 * nb;
      if (rr == c) continue;
      qg_c *M = cc < nb ? A : B;
      const int col = cc < nb ? cc : cc - nb;
      M[rr * nb + col] = csub(M[rr * nb + col], cmul(fac[rr], M[c * nb + col]));
    }
    __syncthreads();
  }
  // ---- T[i][i'] = -X[i'][i] into the full matrix ----
  qg_c *Tw = a.T + (size_t)iw * nQ * nQ;
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  for (int x = tid; x < nb2; x += kAxThreads) {
    const int i = x / nb, j = x - i * nb;
    const int t = i / nl, l = l0 + i % nl, t2 = j / nl, l2 = l0 + j % nl;
    const size_t gi = (size_t)t * neQ + l * (l + 1) + m - 1, gj = (size_t)t2 * neQ + l2 * (l2 + 1) + m - 1;
    Tw[gi * nQ + gj] = singular ? cmk(nan, nan) : cscale(B[j * nb + i], -1.0);
  }
}

// Full default-order T at lMax_extend -> the bspec (index map, -1 where the
// bspec element is not in the full set), T'_ab = T_(map a)(map b) f_b / f_a
// with f the bspec normalisation factors relative to the default ones.
__global__ void axsym_gather_kernel(int nw, int nQ, int n, const qg_c *__restrict__ Tf, const int *__restrict__ map,
                                    const qg_c *__restrict__ f, qg_c *__restrict__ T) {
  const size_t tot = (size_t)nw * n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < tot; x += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(x % n), a = (int)((x / n) % n);
    const size_t w = x / ((size_t)n * n);
    const int ia = map[a], ib = map[b];
    qg_c v = cmk(0, 0);
    if (ia >= 0 && ib >= 0) v = cmul(Tf[(w * nQ + ia) * nQ + ib], cdiv(f[b], f[a]));
    T[x] = v;
  }
}

template <int LQ>
int launch_axsym(AxDev a, qg_c *rad, double *ang, cudaStream_t st) {
  {
    const size_t tot = (size_t)a.nw * a.nq * 3;
    axsym_radial_kernel<LQ><<<(unsigned)std::min<size_t>((tot + 127) / 128, 8192), 128, 0, st>>>(a, rad);
    QG_CUDA_TRY(cudaGetLastError());
    const size_t tot2 = (size_t)(a.L + 1) * a.nq;
    axsym_angular_kernel<<<(unsigned)((tot2 + 127) / 128), 128, 0, st>>>(a.L, a.nq, a.nodes, ang);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(2);
  }
  a.rad = rad;
  a.ang = ang;
  const size_t wave_bytes = (size_t)kAxChunk * LQ * 18 * sizeof(qg_c);
  const size_t solve_bytes = (size_t)4 * (2 * LQ) * (2 * LQ) * sizeof(qg_c);
  const size_t shmem = std::max(wave_bytes, solve_bytes);
  QG_CUDA_TRY(cudaFuncSetAttribute(axsym_kernel<LQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem));
  dim3 grid(2 * a.L + 1, a.nw);
  axsym_kernel<LQ><<<grid, kAxThreads, shmem, st>>>(a);
  QG_CUDA_TRY(cudaGetLastError());
  g_launches.fetch_add(1);
  return QPMS_SUCCESS;
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n from the
// Chebyshev-like initial guesses, Abramowitz & Stegun 25.4.29).
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2 / ((1 - z * z) * pp * pp);
  }
}

struct DevMem {
  void *p = nullptr;
  ~DevMem() {
    if (p) cudaFree(p);
  }
};

}  // namespace

// qpms_arc_sphere / qpms_arc_cylinder are exported below; the node builder
// recognises them to break the panels at the cylinder's rims.
}  // namespace qg

extern "C" {

qpms_arc_function_retval_t qpms_arc_sphere(double theta, const void *R) {
  (void)theta;
  qpms_arc_function_retval_t r;
  r.r = *(const double *)R;
  r.beta = 0;
  return r;
}

// tmatrices.c:625-646: caps at theta < atan(2R/h) and theta > pi - atan(2R/h)
qpms_arc_function_retval_t qpms_arc_cylinder(double theta, const void *params) {
  const qpms_arc_cylinder_params_t *p = (const qpms_arc_cylinder_params_t *)params;
  const double thresh = atan(2 * p->R / p->h);
  qpms_arc_function_retval_t res;
  if (!(theta >= 0 && theta <= M_PI)) {
    res.r = res.beta = NAN;
    return res;
  }
  if (theta < thresh) {
    res.r = 0.5 * p->h / cos(theta);
    res.beta = -theta;
  } else if (theta <= M_PI - thresh) {
    res.r = p->R / sin(theta);
    res.beta = M_PI_2 - theta;
  } else {
    res.r = -0.5 * p->h / cos(theta);
    res.beta = M_PI - theta;
  }
  return res;
}

// Spheroid x^2/a^2 + y^2/a^2 + z^2/c^2 = 1 (not in the reference, which takes
// such shapes as user arc functions): r(theta) and the angle of the outward
// normal from the radial direction.
qpms_arc_function_retval_t qpms_arc_spheroid(double theta, const void *params) {
  const qpms_arc_spheroid_params_t *p = (const qpms_arc_spheroid_params_t *)params;
  const double s = sin(theta), c = cos(theta);
  const double q = s * s / (p->a * p->a) + c * c / (p->c * p->c);
  qpms_arc_function_retval_t res;
  res.r = 1 / sqrt(q);
  const double dr = pow(q, -1.5) * s * c * (1 / (p->c * p->c) - 1 / (p->a * p->a));  // dr / dtheta
  res.beta = atan2(-dr, res.r);
  return res;
}

qpms_arc_function_retval_t qpms_arc_callback(double theta, const void *params) {
  const qpms_arc_callback_params_t *p = (const qpms_arc_callback_params_t *)params;
  qpms_arc_function_retval_t res;
  res.r = res.beta = NAN;
  if (p && p->fn) p->fn(theta, &res.r, &res.beta, p->user);
  return res;
}

}  // extern "C"

namespace qg {

// Quadrature nodes [nq][5] (theta, weight * jac, r, cos beta, sin beta) of
// the surface: panels of kAxGauss Gauss-Legendre nodes, broken at the
// cylinder rims.  The library's sphere, cylinder and spheroid are symmetric
// under z -> -z (*zsym = 1): the integrands are then even or odd under
// theta -> pi - theta, so the nodes cover [0, pi/2] with doubled weights and
// the odd entries are not formed; other arcs take 16 panels over [0, pi].
int axsym_nodes(qpms_arc_function_t shape, std::vector<double> &nodes, int *zsym) {
  if (!shape.function) {
    set_error("NULL arc function");
    return QPMS_EINVAL;
  }
  // the library's shapes are symmetric under z -> -z: half the range, weights x 2
  std::vector<double> bp;
  std::vector<int> panels;
  double wfac = 1.0;
  *zsym = 0;
  if (shape.function == qpms_arc_cylinder) {
    const qpms_arc_cylinder_params_t *p = (const qpms_arc_cylinder_params_t *)shape.params;
    if (!p || !(p->R > 0) || !(p->h > 0)) {
      set_error("cylinder needs R > 0, h > 0");
      return QPMS_EINVAL;
    }
    const double th = atan(2 * p->R / p->h);
    bp = {0.0, th, M_PI_2};
    panels = {6, 3};
    *zsym = 1;
  } else if (shape.function == qpms_arc_sphere || shape.function == qpms_arc_spheroid) {
    bp = {0.0, M_PI_2};
    panels = {shape.function == qpms_arc_sphere ? 2 : 8};
    *zsym = 1;
  } else {
    bp = {0.0, M_PI};
    panels = {16};
  }
  if (*zsym) wfac = 2.0;
  std::vector<double> gx, gw;
  gauss_legendre(kAxGauss, gx, gw);
  nodes.clear();
  for (size_t pc = 0; pc + 1 < bp.size(); ++pc) {
    const int per_piece = panels[pc];
    const double a0 = bp[pc], a1 = bp[pc + 1], hw = (a1 - a0) / per_piece;
    for (int pn = 0; pn < per_piece; ++pn) {
      const double lo = a0 + pn * hw, c = lo + 0.5 * hw;
      for (int g = 0; g < kAxGauss; ++g) {
        const double th = c + 0.5 * hw * gx[g];
        const qpms_arc_function_retval_t rb = shape.function(th, shape.params);
        const double cb = cos(rb.beta);
        if (!(rb.r > 0) || !(cb > 0)) {
          set_error("arc function: r = %g, beta = %g at theta = %g (need r > 0, |beta| < pi/2)", rb.r, rb.beta, th);
          return QPMS_EINVAL;
        }
        nodes.push_back(th);
        nodes.push_back(wfac * 0.5 * hw * gw[g] * rb.r * rb.r * sin(th) / cb);
        nodes.push_back(rb.r);
        nodes.push_back(cb);
        nodes.push_back(sin(rb.beta));
      }
    }
  }
  return QPMS_SUCCESS;
}

// T-matrices of one shape at nw frequencies (host k, k_in, z / z_in) into
// dT [nw][bspec n][bspec n] on the device; optionally the full Q, R at L into
// dQ, dR ([nw][nQ][nQ], default normalisation).
int axsym_tmatrix_device(const std::vector<double> &nodes, int zsym, int L, const qpms_vswf_set_spec_t *bspec,
                         int nw, const qg_c *k, const qg_c *kin, const qg_c *zr, qg_c *dT, qg_c *dQ, qg_c *dR,
                         cudaStream_t st) {
  if (L < 1 || L > kAxMaxL) {
    set_error("lMax_extend %d outside 1..%d", L, kAxMaxL);
    return QPMS_EINVAL;
  }
  const int nq = (int)(nodes.size() / 5);
  const int neQ = L * (L + 2), nQ = 2 * neQ;
  const int n = bspec ? (int)bspec->n : 0;
  std::vector<int> map(n);
  std::vector<qg_c> f(n);
  for (int i = 0; i < n; ++i) {
    const qpms_uvswfi_t u = bspec->ilist[i];
    const int t = (int)(u & 3);
    const long ysc = (long)(u / 4);
    const int l = (int)floor(sqrt((double)ysc) + 1e-9);
    const int m = (int)(ysc - (long)l * (l + 1));
    if (t != 1 && t != 2) {
      set_error("axially symmetric T-matrix: longitudinal waves are not supported");
      return QPMS_EINVAL;
    }
    map[i] = (l >= 1 && l <= L) ? (t == 2 ? 0 : neQ) + l * (l + 1) + m - 1 : -1;
    const qg_c fx = uvswfi_norm_factor(bspec->norm, u), fd = uvswfi_norm_factor(QPMS_NORMALISATION_DEFAULT, u);
    f[i] = cdiv(fx, fd);
  }
  DevMem dn, dk, dTf, dmap, df, derr;
  QG_CUDA_TRY(cudaMalloc(&dn.p, nodes.size() * 8));
  QG_CUDA_TRY(cudaMalloc(&dk.p, (size_t)nw * 48));
  QG_CUDA_TRY(cudaMalloc(&dTf.p, (size_t)nw * nQ * nQ * 16));
  QG_CUDA_TRY(cudaMalloc(&dmap.p, (size_t)std::max(n, 1) * 4));
  QG_CUDA_TRY(cudaMalloc(&df.p, (size_t)std::max(n, 1) * 16));
  QG_CUDA_TRY(cudaMalloc(&derr.p, 4));
  std::vector<qg_c> kk((size_t)nw * 3);
  for (int w = 0; w < nw; ++w) {
    kk[w] = k[w];
    kk[nw + w] = kin[w];
    kk[2 * nw + w] = zr[w];
  }
  QG_CUDA_TRY(cudaMemcpyAsync(dn.p, nodes.data(), nodes.size() * 8, cudaMemcpyHostToDevice, st));
  QG_CUDA_TRY(cudaMemcpyAsync(dk.p, kk.data(), (size_t)nw * 48, cudaMemcpyHostToDevice, st));
  if (n) {
    QG_CUDA_TRY(cudaMemcpyAsync(dmap.p, map.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    QG_CUDA_TRY(cudaMemcpyAsync(df.p, f.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st));
  }
  QG_CUDA_TRY(cudaMemsetAsync(dTf.p, 0, (size_t)nw * nQ * nQ * 16, st));
  QG_CUDA_TRY(cudaMemsetAsync(derr.p, 0, 4, st));
  if (dQ) QG_CUDA_TRY(cudaMemsetAsync(dQ, 0, (size_t)nw * nQ * nQ * 16, st));
  if (dR) QG_CUDA_TRY(cudaMemsetAsync(dR, 0, (size_t)nw * nQ * nQ * 16, st));
  AxDev a;
  a.L = L;
  a.nw = nw;
  a.nq = nq;
  a.nodes = (const double *)dn.p;
  a.k = (const qg_c *)dk.p;
  a.kin = a.k + nw;
  a.zr = a.k + 2 * nw;
  a.T = (qg_c *)dTf.p;
  a.Q = dQ;
  a.R = dR;
  a.err = (int *)derr.p;
  a.zsym = zsym;
  DevMem drad, dang;
  QG_CUDA_TRY(cudaMalloc(&drad.p, (size_t)nw * nq * 3 * L * 3 * 16));
  QG_CUDA_TRY(cudaMalloc(&dang.p, (size_t)(L + 1) * nq * L * 3 * 8));
  int e;
  if (L <= 4) e = launch_axsym<4>(a, (qg_c *)drad.p, (double *)dang.p, st);
  else if (L <= 8) e = launch_axsym<8>(a, (qg_c *)drad.p, (double *)dang.p, st);
  else e = launch_axsym<kAxMaxL>(a, (qg_c *)drad.p, (double *)dang.p, st);
  if (e) return e;
  if (n && dT) {
    const size_t tot = (size_t)nw * n * n;
    const unsigned grid = (unsigned)std::min<size_t>((tot + 255) / 256, 4096);
    axsym_gather_kernel<<<grid, 256, 0, st>>>(nw, nQ, n, (const qg_c *)dTf.p, (const int *)dmap.p,
                                              (const qg_c *)df.p, dT);
    QG_CUDA_TRY(cudaGetLastError());
    g_launches.fetch_add(1);
  }
  int herr = 0;
  QG_CUDA_TRY(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, st));
  QG_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    set_error("axially symmetric T-matrix: singular Q block");
    return QPMS_ERROR;
  }
  return QPMS_SUCCESS;
}

namespace {
qg_c wavenumber_of(qpms_complex_t omega, qpms_epsmu_t em) {
  // qpms_wavenumber (materials.h:46-48): sqrt(eps mu) omega / c
  const std::complex<double> e(em.eps.re, em.eps.im), mu(em.mu.re, em.mu.im), w(omega.re, omega.im);
  const std::complex<double> k = std::sqrt(e * mu) * w / kC0;
  return cmk(k.real(), k.imag());
}
qg_c impedance_ratio(qpms_epsmu_t out, qpms_epsmu_t in) {
  // qpms_waveimpedance (materials.h:52-55): z = sqrt(mu / eps); z_out / z_in
  const std::complex<double> eo(out.eps.re, out.eps.im), mo(out.mu.re, out.mu.im), ei(in.eps.re, in.eps.im),
      mi(in.mu.re, in.mu.im);
  const std::complex<double> r = std::sqrt(mo / eo) / std::sqrt(mi / ei);
  return cmk(r.real(), r.imag());
}
}  // namespace

// Host-facing batch: nw frequencies, T into host memory [nw][n][n].
int axsym_tmatrix_batch_host(qpms_arc_function_t shape, int lMax_extend, const qpms_vswf_set_spec_t *bspec, int nw,
                             const qpms_complex_t *omega, const qpms_epsmu_t *outside, const qpms_epsmu_t *inside,
                             qpms_complex_t *T_out) {
  if (!bspec || nw < 0 || (nw && (!omega || !outside || !inside || !T_out))) {
    set_error("NULL argument");
    return QPMS_EINVAL;
  }
  if (!nw) return QPMS_SUCCESS;
  std::vector<double> nodes;
  int zsym = 0;
  int e = axsym_nodes(shape, nodes, &zsym);
  if (e) return e;
  const int L = std::max<int>(lMax_extend, bspec->lMax);
  std::vector<qg_c> k(nw), kin(nw), zr(nw);
  for (int w = 0; w < nw; ++w) {
    k[w] = wavenumber_of(omega[w], outside[w]);
    kin[w] = wavenumber_of(omega[w], inside[w]);
    zr[w] = impedance_ratio(outside[w], inside[w]);
  }
  const size_t n = bspec->n;
  DevMem dT;
  QG_CUDA_TRY(cudaMalloc(&dT.p, (size_t)nw * n * n * 16 + 16));
  if ((e = axsym_tmatrix_device(nodes, zsym, L, bspec, nw, k.data(), kin.data(), zr.data(), (qg_c *)dT.p, nullptr,
                                nullptr, 0)))
    return e;
  QG_CUDA_TRY(cudaMemcpy(T_out, dT.p, (size_t)nw * n * n * 16, cudaMemcpyDeviceToHost));
  return QPMS_SUCCESS;
}

}  // namespace qg

using namespace qg;

extern "C" {

int qpms_gpu_tmatrix_axialsym_batch(const qpms_vswf_set_spec_t *bspec, qpms_l_t lMax_extend,
                                    qpms_arc_function_t shape, size_t nw, const qpms_complex_t *omega,
                                    const qpms_epsmu_t *outside, const qpms_epsmu_t *inside, qpms_complex_t *T_out) {
  clear_error();
  return axsym_tmatrix_batch_host(shape, lMax_extend, bspec, (int)nw, omega, outside, inside, T_out);
}

int qpms_tmatrix_axialsym_fill(qpms_tmatrix_t *t, qpms_complex_t omega, qpms_epsmu_t outside, qpms_epsmu_t inside,
                               qpms_arc_function_t shape, qpms_l_t lMax_extend) {
  clear_error();
  if (!t || !t->spec || !t->m) {
    set_error("NULL T-matrix");
    return QPMS_EINVAL;
  }
  return axsym_tmatrix_batch_host(shape, lMax_extend, t->spec, 1, &omega, &outside, &inside, t->m);
}

qpms_tmatrix_t *qpms_tmatrix_axialsym(const qpms_vswf_set_spec_t *bspec, qpms_complex_t omega, qpms_epsmu_t outside,
                                      qpms_epsmu_t inside, qpms_arc_function_t shape, qpms_l_t lMax_extend) {
  qpms_tmatrix_t *t = qpms_tmatrix_init(bspec);
  if (!t) return nullptr;
  if (qpms_tmatrix_axialsym_fill(t, omega, outside, inside, shape, lMax_extend)) {
    qpms_tmatrix_free(t);
    return nullptr;
  }
  return t;
}

int qpms_tmatrix_generator_axialsym(qpms_tmatrix_t *t, qpms_complex_t omega, const void *params) {
  clear_error();
  const qpms_tmatrix_generator_axialsym_param_t *p = (const qpms_tmatrix_generator_axialsym_param_t *)params;
  if (!p || !p->outside.function || !p->inside.function) {
    set_error("NULL generator parameters");
    return QPMS_EINVAL;
  }
  return qpms_tmatrix_axialsym_fill(t, omega, p->outside.function(omega, p->outside.params),
                                    p->inside.function(omega, p->inside.params), p->shape, p->lMax_extend);
}

// tmatrices.c:896-956: target[i1 + i2 n] = Q (J = QPMS_HANKEL_PLUS) or R
// (J = QPMS_BESSEL_REGULAR) of the lMaxQR basis in normalisation norm, row i1
// the outside wave (t, l, m), column i2 the inside wave (t', l', m') with
// m' = -m (zero elsewhere).
int qpms_tmatrix_axialsym_RQ_transposed_fill(qpms_complex_t *target, qpms_complex_t omega, qpms_epsmu_t outside,
                                             qpms_epsmu_t inside, qpms_arc_function_t shape, qpms_l_t lMaxQR,
                                             qpms_normalisation_t norm, qpms_bessel_t J) {
  clear_error();
  if (!target) {
    set_error("NULL target");
    return QPMS_EINVAL;
  }
  if (J != QPMS_HANKEL_PLUS && J != QPMS_BESSEL_REGULAR) {
    set_error("J must be QPMS_HANKEL_PLUS (Q) or QPMS_BESSEL_REGULAR (R)");
    return QPMS_EINVAL;
  }
  std::vector<double> nodes;
  int zsym = 0;
  int e = axsym_nodes(shape, nodes, &zsym);
  if (e) return e;
  const int L = lMaxQR;
  if (L < 1 || L > 12) {
    set_error("lMaxQR %d outside 1..12", L);
    return QPMS_EINVAL;
  }
  const int neQ = L * (L + 2), nQ = 2 * neQ;
  const qg_c k = wavenumber_of(omega, outside), kin = wavenumber_of(omega, inside), zr = impedance_ratio(outside, inside);
  DevMem dG;
  QG_CUDA_TRY(cudaMalloc(&dG.p, (size_t)nQ * nQ * 16));
  if ((e = axsym_tmatrix_device(nodes, zsym, L, nullptr, 1, &k, &kin, &zr, nullptr,
                                J == QPMS_HANKEL_PLUS ? (qg_c *)dG.p : nullptr,
                                J == QPMS_HANKEL_PLUS ? nullptr : (qg_c *)dG.p, 0)))
    return e;
  std::vector<qg_c> G((size_t)nQ * nQ);
  QG_CUDA_TRY(cudaMemcpy(G.data(), dG.p, G.size() * 16, cudaMemcpyDeviceToHost));
  // the library's basis of lMaxQR: electric block, then magnetic (vswf.c:76-92)
  qpms_vswf_set_spec_t *spec = qpms_vswf_set_spec_from_lMax(L, norm);
  if (!spec) return QPMS_ERROR;
  for (int i1 = 0; i1 < nQ; ++i1)
    for (int i2 = 0; i2 < nQ; ++i2) {
      const qpms_uvswfi_t u1 = spec->ilist[i1], u2 = spec->ilist[i2];
      const int y1 = (int)(u1 / 4), y2 = (int)(u2 / 4);
      const int l1 = (int)floor(sqrt((double)y1) + 1e-9), l2 = (int)floor(sqrt((double)y2) + 1e-9);
      const int m1 = y1 - l1 * (l1 + 1), m2 = y2 - l2 * (l2 + 1);
      qg_c v = cmk(0, 0);
      if (m1 + m2 == 0) {
        // stored at the column of (t', l', m1); waves in norm = factor x default waves
        const int gi = ((u1 & 3) == 2 ? 0 : neQ) + l1 * (l1 + 1) + m1 - 1;
        const int gj = ((u2 & 3) == 2 ? 0 : neQ) + l2 * (l2 + 1) + m1 - 1;
        const qg_c f1 = cdiv(uvswfi_norm_factor(norm, u1), uvswfi_norm_factor(QPMS_NORMALISATION_DEFAULT, u1));
        const qg_c f2 = cdiv(uvswfi_norm_factor(norm, u2), uvswfi_norm_factor(QPMS_NORMALISATION_DEFAULT, u2));
        v = cmul(cmul(G[(size_t)gi * nQ + gj], f1), f2);
      }
      target[i1 + (size_t)i2 * nQ] = *(const qpms_complex_t *)&v;
    }
  qpms_vswf_set_spec_free(spec);
  return QPMS_SUCCESS;
}

int qpms_tmatrix_generator_axialsym_RQ_transposed_fill(qpms_complex_t *target, qpms_complex_t omega,
                                                       const qpms_tmatrix_generator_axialsym_param_t *p,
                                                       qpms_normalisation_t norm, qpms_bessel_t J) {
  clear_error();
  if (!p || !p->outside.function || !p->inside.function) {
    set_error("NULL generator parameters");
    return QPMS_EINVAL;
  }
  return qpms_tmatrix_axialsym_RQ_transposed_fill(target, omega, p->outside.function(omega, p->outside.params),
                                                  p->inside.function(omega, p->inside.params), p->shape,
                                                  p->lMax_extend, norm, J);
}

}  // extern "C"
